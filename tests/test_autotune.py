"""Autotuner logic (CPU, with a fake runner) and the gb_tune knobs (GPU)."""
import numpy as np
import pytest

from cucodeml_gb300 import _lib, api, autotune
from cucodeml_gb300.simulate import simulate_batch


def _grad(v):
    return {"blength": np.array([v, 2 * v]), "kappa": v, "omega0": 0.0, "omega2": 0.0, "p0": 0.0, "p1": 0.0}


def test_choose_fastest_agreeing(tmp_path):
    cands = [{"a": 0}, {"a": 1}, {"a": 2}, {"a": 3}]
    ms = {0: 5.0, 1: 3.0, 2: 1.0, 3: 2.0}

    def run(cfg):
        a = cfg["a"]
        if a == 2:                                  # fastest but wrong: never chosen
            return ms[a], ([10.5], [_grad(1.0)])
        return ms[a], ([10.0 + 1e-9 * a], [_grad(1.0 + 1e-8 * a)])

    path = str(tmp_path / "t.json")
    r = autotune.choose("k1", cands, run, cache_path=path)
    assert r["config"] == {"a": 3} and not r["cached"]
    assert [t["agrees"] for t in r["table"]] == [True, True, False, True]
    r2 = autotune.choose("k1", cands, lambda c: (_ for _ in ()).throw(AssertionError("ran")), cache_path=path)
    assert r2["cached"] and r2["config"] == {"a": 3}


def test_choose_reports_failures(tmp_path):
    def run(cfg):
        if cfg["a"] == 1:
            raise RuntimeError("refused")
        return 1.0, ([0.0], [_grad(0.0)])

    r = autotune.choose("k2", [{"a": 0}, {"a": 1}], run, cache_path=str(tmp_path / "t.json"))
    assert r["config"] == {"a": 0}
    assert r["table"][1]["error"] == "refused"


def test_signature_buckets():
    s1 = autotune.signature([(12, 1000), (30, 2000)], "batch-fast")
    s2 = autotune.signature([(12, 1001), (30, 2000)], "batch-fast")
    assert s1 == s2 and "genes=2" in s1 and "taxa=12-30" in s1


def test_tune_rejects_null_handle():
    L = _lib.load()
    assert L.gb_tune(None, 1, 1) == -1          # GB_ERR_ARG
    assert L.gb_batch_tune(None, 1, 1) == -1


@pytest.mark.gpu
def test_knobs_agree_and_lock():
    alns = simulate_batch(6, seed=7, taxa=(8, 20), codons=(150, 700))
    genes = []
    for a in alns:
        z, fp, pi = api.patterns(a.codons)
        genes.append((a.tree, z, fp, pi))
    prm = [{"blength": a.tree.branch, "kappa": a.model.kappa, "omega0": a.model.omega0,
            "omega2": a.model.omega2, "p0": a.model.p0, "p1": a.model.p1} for a in alns]
    ref = None
    for cfg in autotune.BATCH_CANDIDATES:
        b = api.Batch(genes, precision="fast", tuning=cfg)
        f, g, _ = b.evaluate(prm, grad=True)
        with pytest.raises(_lib.GBError):
            _lib.check(b._L.gb_batch_tune(b._h, _lib.TUNE["gchunk"], 256))
        b.close()
        if ref is None:
            ref = (f, g)
            continue
        assert autotune._agree(ref, (f, g), 1e-6, 1e-5), cfg
    a, z, fp, pi = alns[0], *genes[0][1:]
    lk = api.Likelihood(a.tree, z, fp, pi, precision="fast", tuning={"gchunk": 128, "grid": 40})
    r = lk.evaluate(a.tree.branch, a.model.kappa, a.model.omega0, a.model.omega2, a.model.p0, a.model.p1,
                    grad=True)
    assert np.isfinite(r.neg_lnL)
    with pytest.raises(_lib.GBError):
        _lib.check(lk._L.gb_tune(lk._h, _lib.TUNE["mma"], 0))
    lk.close()


@pytest.mark.gpu
def test_tune_batch_runs(tmp_path):
    alns = simulate_batch(4, seed=8, taxa=(8, 16), codons=(100, 400))
    genes = []
    for a in alns:
        z, fp, pi = api.patterns(a.codons)
        genes.append((a.tree, z, fp, pi))
    prm = [{"blength": a.tree.branch, "kappa": a.model.kappa, "omega0": a.model.omega0,
            "omega2": a.model.omega2, "p0": a.model.p0, "p1": a.model.p1} for a in alns]
    r = autotune.tune_batch(genes, prm, cache_path=str(tmp_path / "c.json"))
    assert r["config"] in autotune.BATCH_CANDIDATES
    assert all(t.get("agrees", True) for t in r["table"] if t.get("ms") is not None)
