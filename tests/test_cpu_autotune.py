"""Host logic of the autotuner (no GPU): candidate selection, cache keys and
cache round trip, with the timing function replaced by a fake."""
import numpy as np

from ndspmhd_gb300 import autotune as A
from ndspmhd_gb300 import configs


def test_picks_fastest_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("NDSPH_TUNE_CACHE", str(tmp_path / "t.json"))
    cost = {1.05: 9.0, 1.1: 7.5, 1.2: 8.0}
    calls = []

    def fake(opts, state, tuning, steps, warmup):
        calls.append(dict(tuning))
        return cost[tuning["nl_skin"]] + (3.0 if tuning["nl_reuse"] == 0 else 0.0)

    monkeypatch.setattr(A, "_time_device", fake)
    o, p = configs.mhd_box_3d(8, seed=1)
    st = configs.full_state(p, 3)
    cands = [{"nl_reuse": r, "nl_skin": s} for r in (0, 1) for s in (1.05, 1.1, 1.2)]
    r1 = A.tune_device(o, st, candidates=cands)
    assert not r1["cached"] and r1["tuning"] == {"nl_reuse": 1, "nl_skin": 1.1}
    assert len(calls) == len(cands) and len(r1["trials"]) == len(cands)
    r2 = A.tune_device(o, st, candidates=cands)
    assert r2["cached"] and r2["tuning"] == r1["tuning"] and len(calls) == len(cands)
    # another workload signature is tuned afresh
    o2 = dict(o, precision=1 - o["precision"])
    A.tune_device(o2, st, candidates=cands)
    assert len(calls) == 2 * len(cands)
    assert len(A.load_cache()) == 2


def test_signature_separates_workloads():
    o, p = configs.mhd_box_3d(8, seed=1)
    s1 = A.signature(o, 512)
    assert s1 == A.signature(dict(o), 500)            # same power-of-two bucket
    assert s1 != A.signature(o, 4096)
    assert s1 != A.signature(dict(o, idust=2), 512)
    assert s1 != A.signature(o, 512, batched=True)


def test_unwritable_cache_still_returns(tmp_path, monkeypatch):
    d = tmp_path / "ro"
    d.mkdir()
    d.chmod(0o500)
    monkeypatch.setenv("NDSPH_TUNE_CACHE", str(d / "sub" / "t.json"))
    monkeypatch.setattr(A, "_time_device", lambda *a: 1.0)
    o, p = configs.mhd_box_3d(8, seed=1)
    r = A.tune_device(o, configs.full_state(p, 3), candidates=[{"nl_reuse": 1, "nl_skin": 1.1}])
    assert r["tuning"]["nl_skin"] == 1.1
    assert np.isfinite(r["ms_per_step"])
