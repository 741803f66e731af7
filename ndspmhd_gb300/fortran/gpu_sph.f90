!-----------------------------------------------------------------------------
! gpu_sph.f90 -- Fortran side of the drop-in boundary to libndsph_gpu.so.
!
! A maintainer adds this file to the reference's SOURCES and replaces the
! bodies of set_linklist (linkND.f90:45), iterate_density
! (iterate_density.f90:43) and get_rates (ratesND_mhd.f90:29) -- or derivs
! (derivs.f90:27) as a whole -- with calls to the gpu_* routines below.  The
! subroutine names, their callers (derivs.f90:82,92,156,
! stepND_leapfrog_mhd.f90:167, conservative2primitive.f90:556-560) and the
! module arrays stay as they are: the shim passes c_loc() of the module
! arrays, npart, and the options the hot path reads.
!
! Not compiled in this repository's CI (no Fortran compiler in the build
! image); the C side it binds is include/ndsph.h.
!-----------------------------------------------------------------------------
module gpu_sph
 use iso_c_binding
 implicit none

 type, bind(C) :: ndsph_opts_t
    integer(c_int32_t) :: ndim
    integer(c_int32_t) :: ibound(3)
    real(c_double)     :: xmin(3), xmax(3)
    real(c_double)     :: hfact, tolh, psep
    integer(c_int32_t) :: maxdensits, imhd, imagforce, iener, iav
    integer(c_int32_t) :: iavlim(3)
    real(c_double)     :: alphamin, alphaumin, alphaBmin, beta, avdecayconst, gamma, polyk
    integer(c_int32_t) :: idust, idrag_nature
    real(c_double)     :: Kdrag, C_cour, C_force
    integer(c_int32_t) :: precision, learned_h
 end type

 type, bind(C) :: ndsph_particles_t
    type(c_ptr) :: x, vel, Bevol, en, hh, pmass, alpha, itype, ireal
    type(c_ptr) :: rho, rhoalt, drhodt, dhdt, gradh, gradhn, gradgradh, numneigh
    type(c_ptr) :: dens, uu, pr, spsound, Bfield
    type(c_ptr) :: force, dBevoldt, dudt, dendt, daldt, divB, curlB, del2u, graddivv
 end type

 type, bind(C) :: ndsph_dt_t
    real(c_double)     :: dtcourant, dtforce, dtav, dtdrag, dtvisc, vsigmax, stressmax, hhmax, dt, time
    integer(c_int32_t) :: its, ncalctotal, nsteps, nrelink
 end type

 ! neighbour-search settings (ndsph_tuning); optional, see ndsph_set_tuning
 type, bind(C) :: ndsph_tuning_t
    real(c_float)      :: nl_skin
    integer(c_int32_t) :: nl_reuse
    real(c_float)      :: nl_grow, graph_cell_margin
    integer(c_int32_t) :: stencil
    integer(c_int32_t) :: step_pieces
 end type

 interface
    integer(c_int) function ndsph_init(ctx, opts, nmax) bind(C, name="ndsph_init")
      import :: c_ptr, c_int, c_int32_t, ndsph_opts_t
      type(c_ptr), intent(out)       :: ctx
      type(ndsph_opts_t), intent(in) :: opts
      integer(c_int32_t), value      :: nmax
    end function
    integer(c_int) function ndsph_finalize(ctx) bind(C, name="ndsph_finalize")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function ndsph_iterate_density(ctx, p, npart, dts) bind(C, name="ndsph_iterate_density")
      import :: c_ptr, c_int, c_int32_t, ndsph_particles_t, ndsph_dt_t
      type(c_ptr), value                     :: ctx
      type(ndsph_particles_t), intent(inout) :: p
      integer(c_int32_t), value              :: npart
      type(ndsph_dt_t), intent(inout)        :: dts
    end function
    integer(c_int) function ndsph_get_rates(ctx, p, npart, dts) bind(C, name="ndsph_get_rates")
      import :: c_ptr, c_int, c_int32_t, ndsph_particles_t, ndsph_dt_t
      type(c_ptr), value                     :: ctx
      type(ndsph_particles_t), intent(inout) :: p
      integer(c_int32_t), value              :: npart
      type(ndsph_dt_t), intent(inout)        :: dts
    end function
    integer(c_int) function ndsph_derivs(ctx, p, npart, dts) bind(C, name="ndsph_derivs")
      import :: c_ptr, c_int, c_int32_t, ndsph_particles_t, ndsph_dt_t
      type(c_ptr), value                     :: ctx
      type(ndsph_particles_t), intent(inout) :: p
      integer(c_int32_t), value              :: npart
      type(ndsph_dt_t), intent(inout)        :: dts
    end function
    integer(c_int) function ndsph_set_linklist(ctx, p, npart, dts) bind(C, name="ndsph_set_linklist")
      import :: c_ptr, c_int, c_int32_t, ndsph_particles_t, ndsph_dt_t
      type(c_ptr), value                     :: ctx
      type(ndsph_particles_t), intent(inout) :: p
      integer(c_int32_t), value              :: npart
      type(ndsph_dt_t), intent(inout)        :: dts
    end function
    integer(c_int) function ndsph_step(ctx, p, npart, dts) bind(C, name="ndsph_step")
      import :: c_ptr, c_int, c_int32_t, ndsph_particles_t, ndsph_dt_t
      type(c_ptr), value                     :: ctx
      type(ndsph_particles_t), intent(inout) :: p
      integer(c_int32_t), value              :: npart
      type(ndsph_dt_t), intent(inout)        :: dts
    end function
    integer(c_int) function ndsph_set_tuning(ctx, t) bind(C, name="ndsph_set_tuning")
      import :: c_ptr, c_int, ndsph_tuning_t
      type(c_ptr), value                :: ctx
      type(ndsph_tuning_t), intent(in)  :: t
    end function
    integer(c_int) function ndsph_get_tuning(ctx, t) bind(C, name="ndsph_get_tuning")
      import :: c_ptr, c_int, ndsph_tuning_t
      type(c_ptr), value                :: ctx
      type(ndsph_tuning_t), intent(out) :: t
    end function
 end interface

 type(c_ptr), save :: ctx = c_null_ptr
 ! pair-sum form of the context: 0 plain FP64 (the parity form), 1 FP32 pairs
 integer, save :: gpu_precision = 0
 ! 1: the learned h predictor (an MLP trained online on the device) sets the
 ! starting h of each step's density iteration in gpu_step; the iteration and
 ! its tolerance are unchanged
 integer, save :: gpu_learned_h = 0
 ! gpu_step copies back only what the next step reads (x, vel, Bevol, en, hh,
 ! alpha and their rates: 25 doubles a particle) unless this is set; the
 ! caller sets it before a step whose results output or evwrite will read
 ! (evolve.f90:136-166), which then also gets rho, the density terms, the
 ! primitives, div B, curl B and the switch sources (47.5 doubles a particle)
 logical, save :: gpu_step_all_outputs = .false.

contains

 subroutine gpu_opts(o)
  use dimen_mhd,    only:ndim
  use options
  use bound,        only:xmin,xmax
  use setup_params, only:hfact,psep
  use artvi,        only:alphamin,alphaumin,alphaBmin,beta,avdecayconst
  use eos,          only:gamma,polyk
  use timestep,     only:C_cour,C_force
  type(ndsph_opts_t), intent(out) :: o
  o%ndim = ndim
  o%ibound = 0;  o%ibound(1:ndim) = ibound(1:ndim)
  o%xmin = 0.;   o%xmin(1:ndim) = xmin(1:ndim)
  o%xmax = 0.;   o%xmax(1:ndim) = xmax(1:ndim)
  o%hfact = hfact;  o%tolh = tolh;  o%psep = psep
  o%maxdensits = maxdensits;  o%imhd = imhd;  o%imagforce = imagforce
  o%iener = iener;  o%iav = iav;  o%iavlim = iavlim
  o%alphamin = alphamin;  o%alphaumin = alphaumin;  o%alphaBmin = alphaBmin
  o%beta = beta;  o%avdecayconst = avdecayconst;  o%gamma = gamma;  o%polyk = polyk
  o%idust = idust;  o%idrag_nature = idrag_nature;  o%Kdrag = Kdrag
  o%C_cour = C_cour;  o%C_force = C_force
  o%precision = gpu_precision;  o%learned_h = gpu_learned_h
 end subroutine gpu_opts

 subroutine gpu_particles(p)
  use part
  use rates
  use hterms
  use linklist, only:numneigh
  use derivB,   only:curlB
  type(ndsph_particles_t), intent(out) :: p
  p%x = c_loc(x);  p%vel = c_loc(vel);  p%Bevol = c_loc(Bevol);  p%en = c_loc(en)
  p%hh = c_loc(hh);  p%pmass = c_loc(pmass);  p%alpha = c_loc(alpha)
  p%itype = c_loc(itype);  p%ireal = c_loc(ireal)
  p%rho = c_loc(rho);  p%rhoalt = c_loc(rhoalt);  p%drhodt = c_loc(drhodt);  p%dhdt = c_loc(dhdt)
  p%gradh = c_loc(gradh);  p%gradhn = c_loc(gradhn);  p%gradgradh = c_loc(gradgradh)
  p%numneigh = c_loc(numneigh)
  p%dens = c_loc(dens);  p%uu = c_loc(uu);  p%pr = c_loc(pr);  p%spsound = c_loc(spsound)
  p%Bfield = c_loc(Bfield)
  p%force = c_loc(force);  p%dBevoldt = c_loc(dBevoldt);  p%dudt = c_loc(dudt);  p%dendt = c_loc(dendt)
  p%daldt = c_loc(daldt);  p%divB = c_loc(divB);  p%curlB = c_loc(curlB)
  p%del2u = c_loc(del2u);  p%graddivv = c_loc(graddivv)
 end subroutine gpu_particles

 subroutine gpu_check(ierr, where)
  use loguns, only:iprint
  integer(c_int), intent(in) :: ierr
  character(len=*), intent(in) :: where
  if (ierr /= 0) then
     write(iprint,*) 'ERROR: libndsph_gpu ',where,' returned ',ierr
     call quit
  endif
 end subroutine gpu_check

 subroutine gpu_ensure()
  use part, only:npart
  type(ndsph_opts_t) :: o
  if (.not.c_associated(ctx)) then
     call gpu_opts(o)
     call gpu_check(ndsph_init(ctx, o, int(npart,c_int32_t)), 'init')
  endif
 end subroutine gpu_ensure

 ! replacement body of iterate_density (iterate_density.f90:43)
 subroutine gpu_iterate_density()
  use part,     only:npart
  use timestep, only:dtcourant
  type(ndsph_particles_t) :: p
  type(ndsph_dt_t) :: d
  call gpu_ensure()
  call gpu_particles(p)
  call gpu_check(ndsph_iterate_density(ctx, p, int(npart,c_int32_t), d), 'iterate_density')
 end subroutine gpu_iterate_density

 ! replacement body of get_rates (ratesND_mhd.f90:29)
 subroutine gpu_get_rates()
  use part,     only:npart
  use timestep, only:dtcourant,dtforce,dtav,dtdrag,dtvisc
  type(ndsph_particles_t) :: p
  type(ndsph_dt_t) :: d
  call gpu_ensure()
  call gpu_particles(p)
  call gpu_check(ndsph_get_rates(ctx, p, int(npart,c_int32_t), d), 'get_rates')
  dtcourant = d%dtcourant;  dtforce = d%dtforce;  dtav = d%dtav
  dtdrag = d%dtdrag;  dtvisc = d%dtvisc
 end subroutine gpu_get_rates

 ! replacement body of derivs (derivs.f90:27): boundary, link, density, EOS,
 ! rates in one host<->device round trip (no ghosts are needed)
 subroutine gpu_derivs()
  use part,     only:npart,ntotal
  use timestep, only:dtcourant,dtforce,dtav,dtdrag,dtvisc
  type(ndsph_particles_t) :: p
  type(ndsph_dt_t) :: d
  call gpu_ensure()
  call gpu_particles(p)
  call gpu_check(ndsph_derivs(ctx, p, int(npart,c_int32_t), d), 'derivs')
  ntotal = npart
  dtcourant = d%dtcourant;  dtforce = d%dtforce;  dtav = d%dtav
  dtdrag = d%dtdrag;  dtvisc = d%dtvisc
 end subroutine gpu_derivs

 ! replacement body of step (stepND_leapfrog_mhd.f90:31): predictor, derivs,
 ! corrector and the next dt on the device in one call; evolve.f90:93-96
 ! advances time and nsteps itself before calling step, so only dt and the
 ! timestep bounds come back
 subroutine gpu_step()
  use part,     only:npart,ntotal
  use timestep, only:dt,time,nsteps,dtcourant,dtforce,dtav,dtdrag,dtvisc
  type(ndsph_particles_t) :: p
  type(ndsph_dt_t) :: d
  call gpu_ensure()
  call gpu_particles(p)
  if (.not.gpu_step_all_outputs) then
     ! outputs no later step reads: left as they are on the host
     p%rho = c_null_ptr;  p%rhoalt = c_null_ptr;  p%drhodt = c_null_ptr
     p%gradh = c_null_ptr;  p%gradhn = c_null_ptr;  p%gradgradh = c_null_ptr
     p%numneigh = c_null_ptr;  p%dens = c_null_ptr;  p%uu = c_null_ptr
     p%pr = c_null_ptr;  p%spsound = c_null_ptr;  p%Bfield = c_null_ptr
     p%dudt = c_null_ptr;  p%divB = c_null_ptr;  p%curlB = c_null_ptr
     p%del2u = c_null_ptr;  p%graddivv = c_null_ptr
  endif
  d%dt = dt;  d%time = time;  d%nsteps = int(nsteps,c_int32_t)
  call gpu_check(ndsph_step(ctx, p, int(npart,c_int32_t), d), 'step')
  ntotal = npart
  dtcourant = d%dtcourant;  dtforce = d%dtforce;  dtav = d%dtav
  dtdrag = d%dtdrag;  dtvisc = d%dtvisc
  dt = d%dt
 end subroutine gpu_step

end module gpu_sph
