"""Batched evaluation (gb_batch_*): many independent alignments in one CUDA
graph launch must give exactly what per-gene evaluation gives."""
import numpy as np
import pytest

from cucodeml_gb300 import api
from cucodeml_gb300.simulate import simulate_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def genes():
    alns = simulate_batch(12, seed=99, taxa=(6, 20), codons=(60, 400))
    out = []
    for a in alns:
        z, fpatt, pi = api.patterns(a.codons)
        out.append((a, z, fpatt, pi))
    return out


def params_of(a, scale=1.0):
    m = a.model
    return {"blength": a.tree.branch * scale, "kappa": m.kappa, "omega0": m.omega0, "omega2": m.omega2,
            "p0": m.p0, "p1": m.p1}


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_batch_equals_single(genes, precision):
    b = api.Batch([(a.tree, z, fp, pi) for a, z, fp, pi in genes], precision=precision)
    for rep, scale in enumerate((1.0, 1.2)):
        prm = [params_of(a, scale) for a, _, _, _ in genes]
        f, g, st = b.evaluate(prm, grad=True)
        assert st.kernels > 0
        for i, (a, z, fp, pi) in enumerate(genes):
            lk = api.Likelihood(a.tree, z, fp, pi, precision=precision)
            p = prm[i]
            r = lk.evaluate(p["blength"], p["kappa"], p["omega0"], p["omega2"], p["p0"], p["p1"], grad=True)
            assert abs(f[i] - r.neg_lnL) <= 1e-12 * abs(r.neg_lnL), (rep, i)
            assert np.allclose(g[i]["blength"], r.grad["blength"], rtol=1e-10, atol=1e-10)
            for k in ("kappa", "omega0", "omega2", "p0", "p1"):
                assert abs(g[i][k] - r.grad[k]) <= 1e-10 * max(1.0, abs(r.grad[k])), (rep, i, k)
            lk.close()
    f2, _, _ = b.evaluate([params_of(a) for a, _, _, _ in genes], grad=False)
    assert np.all(np.isfinite(f2))
    b.close()


def test_batch_fast_matches_fp64(genes):
    prm = [params_of(a) for a, _, _, _ in genes]
    b64 = api.Batch([(a.tree, z, fp, pi) for a, z, fp, pi in genes], precision="fp64")
    bf = api.Batch([(a.tree, z, fp, pi) for a, z, fp, pi in genes], precision="fast")
    f64, g64, _ = b64.evaluate(prm, grad=True)
    ff, gf, _ = bf.evaluate(prm, grad=True)
    assert np.max(np.abs(f64 - ff)) <= 1e-6
    for a, b in zip(g64, gf):
        va = np.concatenate([a["blength"], [a[k] for k in ("kappa", "omega0", "omega2", "p0", "p1")]])
        vb = np.concatenate([b["blength"], [b[k] for k in ("kappa", "omega0", "omega2", "p0", "p1")]])
        assert np.max(np.abs(va - vb) / np.maximum(1.0, np.abs(va))) <= 1e-5


def test_batch_fast_alternating_modes(genes):
    """lnL-only, then lnL + gradient, then lnL-only again on one batch (the
    batch-wide staging buffers and both captured graphs), each equal to the
    genes evaluated one by one."""
    b = api.Batch([(a.tree, z, fp, pi) for a, z, fp, pi in genes], precision="fast")
    singles = [api.Likelihood(a.tree, z, fp, pi, precision="fast") for a, z, fp, pi in genes]
    for rep, (scale, grad) in enumerate(((1.0, False), (1.1, True), (0.9, False), (1.2, True))):
        prm = [params_of(a, scale) for a, _, _, _ in genes]
        f, g, _ = b.evaluate(prm, grad=grad)
        for i, lk in enumerate(singles):
            p = prm[i]
            r = lk.evaluate(p["blength"], p["kappa"], p["omega0"], p["omega2"], p["p0"], p["p1"], grad=grad)
            assert abs(f[i] - r.neg_lnL) <= 1e-12 * abs(r.neg_lnL), (rep, i)
            if grad:
                assert np.allclose(g[i]["blength"], r.grad["blength"], rtol=1e-10, atol=1e-10), (rep, i)
                for k in ("kappa", "omega0", "omega2", "p0", "p1"):
                    assert abs(g[i][k] - r.grad[k]) <= 1e-10 * max(1.0, abs(r.grad[k])), (rep, i, k)
    for lk in singles:
        lk.close()
    b.close()


def test_batch_task_orders_agree(genes):
    """The persistent kernels' task order (critical path first, gene by gene,
    level by level) changes only the schedule: results are bit-identical."""
    prm = [params_of(a, 1.05) for a, _, _, _ in genes]
    out = []
    for order in (0, 1, 2):
        b = api.Batch([(a.tree, z, fp, pi) for a, z, fp, pi in genes], precision="fast",
                      tuning={"order": order})
        f, g, _ = b.evaluate(prm, grad=True)
        out.append((np.asarray(f), [np.concatenate([x["blength"], [x[k] for k in ("kappa", "omega0", "omega2",
                                                                                  "p0", "p1")]]) for x in g]))
        b.close()
    for f, g in out[1:]:
        assert np.array_equal(f, out[0][0])
        for a, b2 in zip(g, out[0][1]):
            assert np.array_equal(a, b2)


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_pipelined_halves_equal_one_batch(genes, precision):
    """gb_batch_submit / gb_batch_collect over two half-batches, with the host
    set-up of one overlapping the device work of the other, gives each gene
    what one gb_batch_eval gives, for a sequence of parameter sets."""
    gl = [(a.tree, z, fp, pi) for a, z, fp, pi in genes]
    sets = [[params_of(a, s) for a, _, _, _ in genes] for s in (1.0, 1.1, 0.9)]
    b = api.Batch(gl, precision=precision)
    ref = [b.evaluate(p, grad=True)[:2] for p in sets]
    b.close()
    pb = api.PipelinedBatch(gl, precision=precision)
    got = pb.evaluate_many(sets, grad=True)
    pb.close()
    for (f0, g0), (f1, g1) in zip(ref, got):
        assert np.max(np.abs(f0 - f1) / np.abs(f0)) <= 1e-12
        for a, c in zip(g0, g1):
            assert np.allclose(a["blength"], c["blength"], rtol=1e-10, atol=1e-10)
            for k in ("kappa", "omega0", "omega2", "p0", "p1"):
                assert abs(a[k] - c[k]) <= 1e-10 * max(1.0, abs(a[k]))


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_batch_model_b_equals_single(genes, precision):
    """Branch-site model B over a batch (gb_batch_submit_b, each gene's own
    free w1) against per-gene gb_eval_b: lnL to 1e-12, gradient including
    d/dw1 to 1e-10; then model A again on the same batch object (w1 = 1)."""
    b = api.Batch([(a.tree, z, fp, pi) for a, z, fp, pi in genes], precision=precision)
    prm = [dict(params_of(a), omega1=0.6 + 0.05 * i) for i, (a, _, _, _) in enumerate(genes)]
    f, g, _ = b.evaluate(prm, grad=True)
    for i, (a, z, fp, pi) in enumerate(genes):
        lk = api.Likelihood(a.tree, z, fp, pi, precision=precision)
        p = prm[i]
        r = lk.evaluate(p["blength"], p["kappa"], p["omega0"], p["omega2"], p["p0"], p["p1"], grad=True,
                        omega1=p["omega1"])
        assert abs(f[i] - r.neg_lnL) <= 1e-12 * abs(r.neg_lnL), i
        assert np.allclose(g[i]["blength"], r.grad["blength"], rtol=1e-10, atol=1e-10)
        for k in ("kappa", "omega0", "omega1", "omega2", "p0", "p1"):
            assert abs(g[i][k] - r.grad[k]) <= 1e-10 * max(1.0, abs(r.grad[k])), (i, k)
        lk.close()
    fa, ga, _ = b.evaluate([params_of(a) for a, _, _, _ in genes], grad=True)
    assert "omega1" not in ga[0]
    for i, (a, z, fp, pi) in enumerate(genes):
        lk = api.Likelihood(a.tree, z, fp, pi, precision=precision)
        p = params_of(a)
        r = lk.evaluate(p["blength"], p["kappa"], p["omega0"], p["omega2"], p["p0"], p["p1"])
        assert abs(fa[i] - r.neg_lnL) <= 1e-12 * abs(r.neg_lnL), i
        lk.close()
    b.close()
