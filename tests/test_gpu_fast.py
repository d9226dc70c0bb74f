"""Split-precision path (GB_PREC_FAST) against the FP64 path on the GPU.

The FP64 path equals the oracle to 1e-12 relative (test_gpu_fp64.py), so it
is the reference here.  Bar (the precision target of the fast path):
|delta lnL| <= 1e-6 absolute per alignment, per-pattern |delta log f| <= 1e-8.
"""
import numpy as np
import pytest

from cucodeml_gb300 import _lib, api
from cucodeml_gb300.simulate import simulate
from oracle import oracle as O
from tests.conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu


def node_blength(tree, x):
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = np.asarray(x)[: tree.nbranch]
    return bl


def both(tree, z, fpatt, pi, args):
    a = api.Likelihood(tree, z, fpatt, pi, precision="fp64").evaluate(*args, want_site=True)
    b = api.Likelihood(tree, z, fpatt, pi, precision="fast").evaluate(*args, want_site=True)
    return a, b


@pytest.mark.parametrize("name", golden_names())
def test_fast_lnL_golden(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    args = (node_blength(tree, x), x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2])
    a, b = both(tree, z, fpatt, pi, args)
    d = abs(a.neg_lnL - b.neg_lnL)
    dl = np.max(np.abs(a.lnf - b.lnf))
    print(f"{name}: |dlnL| = {d:.3e}  max |dlogf| = {dl:.3e}")
    assert d <= 1e-6
    assert dl <= 1e-8


@pytest.mark.parametrize("slices", [6, 7, 8])
def test_fast_lnL_64x5000(slices):
    aln = simulate(64, 5000, seed=2024)
    z, fpatt, pi = api.patterns(aln.codons)
    tree = aln.tree
    args = (tree.branch, 2.0, 0.3, 3.0, 0.5, 0.3)
    a = api.Likelihood(tree, z, fpatt, pi, precision="fp64").evaluate(*args, want_site=True)
    lk = api.Likelihood(tree, z, fpatt, pi, precision=16 + slices)
    b = lk.evaluate(*args, want_site=True)
    d = abs(a.neg_lnL - b.neg_lnL)
    dl = np.max(np.abs(a.lnf - b.lnf))
    print(f"64x5000 slices={slices}: lnL {-a.neg_lnL:.9f} |dlnL| = {d:.3e}  max |dlogf| = {dl:.3e} "
          f"fp64 {a.ms_device:.2f} ms  fast {b.ms_device:.2f} ms")
    if slices == 8:
        assert d <= 1e-6


def grad_vec(r):
    g = r.grad
    return np.concatenate([g["blength"], [g["kappa"], g["omega0"], g["omega2"], g["p0"], g["p1"]]])


@pytest.mark.parametrize("name", ["c8x300_s1", "c5x120_s5", "c24x400_s3", "c40x200_s4"])
def test_fast_gradient_golden(name):
    """Fast adjoint vs the FP64 adjoint (itself checked against finite differences)."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    args = (node_blength(tree, x), x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2])
    a = api.Likelihood(tree, z, fpatt, pi, precision="fp64").evaluate(*args, grad=True)
    b = api.Likelihood(tree, z, fpatt, pi, precision="fast").evaluate(*args, grad=True)
    ga, gb = grad_vec(a), grad_vec(b)
    err = np.max(np.abs(ga - gb) / np.maximum(1.0, np.abs(ga)))
    print(f"{name}: |dlnL| = {abs(a.neg_lnL - b.neg_lnL):.3e}  grad rel err = {err:.3e}")
    assert abs(a.neg_lnL - b.neg_lnL) <= 1e-6
    assert err <= 1e-5


def test_fast_gradient_64x5000():
    aln = simulate(64, 5000, seed=2024)
    z, fpatt, pi = api.patterns(aln.codons)
    tree = aln.tree
    args = (tree.branch, 2.0, 0.3, 3.0, 0.5, 0.3)
    a = api.Likelihood(tree, z, fpatt, pi, precision="fp64").evaluate(*args, grad=True)
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fast")
    b = lk.evaluate(*args, grad=True)
    b = lk.evaluate(*args, grad=True)
    ga, gb = grad_vec(a), grad_vec(b)
    err = np.max(np.abs(ga - gb) / np.maximum(1.0, np.abs(ga)))
    print(f"64x5000 lnL+grad: |dlnL| = {abs(a.neg_lnL - b.neg_lnL):.3e} grad rel err = {err:.3e} "
          f"fp64 {a.ms_device:.2f} ms fast {b.ms_device:.2f} ms")
    assert abs(a.neg_lnL - b.neg_lnL) <= 1e-6
    assert err <= 1e-5


@pytest.mark.parametrize("case", ["c24x400_s3", "c40x200_s4", "64x5000"])
def test_persistent_equals_levels(case, monkeypatch):
    """The persistent task-list kernels do the same arithmetic per (item, tile)
    as the one-launch-per-level kernels: results must be bit-identical, also
    when lnL-only and lnL+gradient evaluations alternate on one handle."""
    if case == "64x5000":
        aln = simulate(64, 5000, seed=2024)
        z, fpatt, pi = api.patterns(aln.codons)
        tree = aln.tree
        args = (tree.branch, 2.0, 0.3, 3.0, 0.5, 0.3)
    else:
        fx, tree, codons = load_golden(case)
        z, fpatt, pi = O.patterns(codons)
        x = np.array(fx["x"])
        nb = tree.nbranch
        args = (node_blength(tree, x), x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2])
    res = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("GBCODEML_PERSIST", mode)
        lk = api.Likelihood(tree, z, fpatt, pi, precision="fast")
        r0 = lk.evaluate(*args, want_site=True)
        r1 = lk.evaluate(*args, grad=True)
        r2 = lk.evaluate(*args)
        res[mode] = (r0, r1, r2)
        lk.close()
    p, l = res["1"], res["0"]
    assert p[0].neg_lnL == l[0].neg_lnL and np.array_equal(p[0].lnf, l[0].lnf)
    assert p[1].neg_lnL == l[1].neg_lnL and p[2].neg_lnL == l[0].neg_lnL
    assert np.array_equal(grad_vec(p[1]), grad_vec(l[1]))
    print(f"{case}: persistent == per-level; device ms (lnL+grad) {p[1].ms_device:.2f} vs {l[1].ms_device:.2f}")
