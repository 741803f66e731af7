"""CPU checks of the MLP oracle: hand-written backward == finite differences."""
import numpy as np

from oracle import mlp_oracle as M


def _params(seed=0):
    rng = np.random.default_rng(seed)
    p = rng.uniform(-0.5, 0.5, M.NPARAM)
    # exactly representable in BF16 so rounding does not enter the comparison
    return M.bf16(p.astype(np.float32)).astype(np.float64)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = _params()
    x = M.bf16(rng.normal(size=(64, M.NIN)).astype(np.float32)).astype(np.float64)
    y = rng.normal(size=64)
    loss, g = M.loss_and_grad(p, x, y)
    idx = list(range(0, M.NPARAM, 37)) + [M.OFF_B3, M.OFF_W3 + 5, M.OFF_B1 + 3]
    fd = M.fd_grad(p, x, y, idx=idx)
    for q in idx:
        assert abs(g[q] - fd[q]) <= 1e-6 * max(1.0, abs(fd[q])), (q, g[q], fd[q])
    assert abs(loss - M.loss_only(p, x, y)) < 1e-12


def test_bf16_rounding():
    # bf16 keeps 7 mantissa bits: 1 + 2^-7 is representable, 1 + 2^-8 is a tie
    v = np.array([1.0, 1.0078125, 1.00390625, 1.01171875, -3.14159], dtype=np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0078125
    assert r[2] == 1.0                     # tie to even (mantissa 0)
    assert r[3] == 1.015625                # tie to even (mantissa 2)
    assert abs(r[4] + 3.140625) < 1e-7
