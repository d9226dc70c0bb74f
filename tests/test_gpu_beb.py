"""Bayes empirical Bayes (gb_beb) on the GPU, through the C ABI, against the
oracle's restatement of codeml's lfunNSsites_ACD and against codeml's own BEB
output (golden fixtures).

Bars: the 121 per-pattern log f(x_h | w) within 1e-10 + 2e-9 |log f| of the
oracle.  The GPU path and the oracle use different eigensolvers (Householder
+ QL as codeml, against cyclic Jacobi); at the grid's small omegas (w0 = 0.05)
the nonsynonymous entries of P(t) are sums that cancel to 1e-8 and below, and
the two solutions differ there by up to 5e-10 of log f (measured on the CPU
with the library's eigen solutions in a plain pruning).  Posteriors and grid
marginals within 1e-8 absolute (the same comparison moves them by 2e-11);
log f(X) within 1e-9 relative; against codeml, its printed rounding (5
decimals for site posteriors, 3 for the grid, 6 for log f(X)).
"""
import numpy as np
import pytest

from cucodeml_gb300 import api
from cucodeml_gb300.simulate import simulate
from oracle import oracle as O
from tests.conftest import golden_names, load_golden
from tests.test_beb_oracle import site_patterns

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_names())
def test_beb_matches_oracle_and_codeml(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    ref = O.Problem(tree, z, fpatt, pi, nthreads=4).beb(x)
    lk = api.Likelihood(tree, z, fpatt, pi)
    r = lk.beb_x(x, want_lnfw=True)
    assert np.all(np.abs(r["lnfw"] - ref["lnfw"]) <= 1e-10 + 2e-9 * np.abs(ref["lnfw"]))
    assert np.max(np.abs(r["post"] - ref["post"])) <= 1e-8
    assert np.max(np.abs(r["grid"] - ref["grid"])) <= 1e-8
    assert np.max(np.abs(r["p0p1"] - ref["p0p1"])) <= 1e-8
    assert abs(r["lnfX"] - ref["lnfX"]) <= 1e-9 * abs(ref["lnfX"])
    assert abs(r["S1"] - ref["S1"]) <= 1e-9 * abs(ref["S1"])
    g = fx["beb"]
    site = r["post"][:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(g["site_post_5dp"]))) <= 5.01e-6
    assert np.max(np.abs(r["grid"][2] - g["w0_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(r["grid"][3] - g["w2_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(r["p0p1"] - g["p0p1_post_3dp"])) <= 5.01e-4
    assert abs(r["lnfX"] - g["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["lnfX"])
    lk.close()


def test_beb_needs_fp64_handle():
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fast")
    with pytest.raises(api._lib.GBError) as e:
        lk.beb_x(np.array(fx["x"]))
    assert e.value.code == -6
    lk.close()


def test_beb_path_only_sets_match_full_evaluations():
    """At 64 taxa (node scaling on), the omega sets that gb_beb obtains by
    re-pruning only the foreground path equal full evaluations with the same
    eigen slots, and the posteriors are distributions.  (gb_eval_uvr forms
    P = U diag(e) V in general form, gb_beb from the symmetric part; at small
    omega the two roundings of the cancelling entries differ as two
    eigensolvers do, hence 2e-9 of log f.)"""
    aln = simulate(64, 1000, seed=21)
    z, fpatt, pi = O.patterns(aln.codons)
    tree = aln.tree
    kappa, p0, p1, w0, w2 = 2.0, 0.5, 0.3, 0.3, 3.0
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = tree.x_branch_lengths()
    lk = api.Likelihood(tree, z, fpatt, pi)
    assert lk.nscale > 0
    r = lk.beb(bl, kappa, w0, w2, p0, p1, want_lnfw=True)
    assert np.allclose(r["post"].sum(axis=0), 1.0, atol=1e-12)
    assert np.allclose(r["grid"][2:].sum(axis=1), 1.0, atol=1e-12)
    assert abs(r["p0p1"].sum() - 1.0) < 1e-12
    qf = api.model_setup(pi, kappa, w0, w2, p0, p1)[3]
    fk = np.array([0.25, 0.25, 0.25, 0.25])
    for i, j in [(0, 0), (3, 7), (9, 9)]:
        U, V, R, _, _ = api.model_setup(pi, kappa, (i + 0.5) / 10, 1 + (j + 0.5), p0, p1)
        e = lk.neg_lnL_uvr(U, V, R, qf, fk, bl)
        for row, s in ((0, i), (1, 10), (2, 11 + 10 * i + j), (3, 111 + j)):
            a, b = r["lnfw"][s], e.fhK[row]
            assert np.all(np.abs(a - b) <= 1e-10 + 2e-9 * np.abs(b)), (i, j, row)
    lk.close()


@pytest.mark.parametrize("name", ["mb8x300_s7", "mb24x400_s8"])
def test_beb_model_b_with_given_qfactors(name):
    """gb_beb_qf with model B's Qfactors (the oracle's set-up of model B)
    against the oracle's model-B BEB and codeml's output, same bars."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4, model_b=True)
    ref = pb.beb(x)
    qf = pb.set_params(x)[3]
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[: tree.nbranch]
    lk = api.Likelihood(tree, z, fpatt, pi)
    r = lk.beb_qf(bl, x[tree.nbranch], qf, want_lnfw=True)
    assert np.all(np.abs(r["lnfw"] - ref["lnfw"]) <= 1e-10 + 2e-9 * np.abs(ref["lnfw"]))
    assert np.max(np.abs(r["post"] - ref["post"])) <= 1e-8
    assert abs(r["lnfX"] - ref["lnfX"]) <= 1e-9 * abs(ref["lnfX"])
    site = r["post"][:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(fx["beb"]["site_post_5dp"]))) <= 5.01e-6
    lk.close()
