"""Pin the oracle's Bayes empirical Bayes (BEB) analysis of model A against the
reference codeml's own BEB output (golden fixtures, tests/golden/make_golden.py).

codeml runs lfunNSsites_ACD (codeml.c:6617-6826) after its fixed-parameter
evaluation; the fixtures hold its per-site posteriors of the four site classes
(5 decimals), the posteriors on the w0 / w2 grid and on the 100 (p0, p1)
triangles (3 decimals) and the printed log f(X), S1, S2 (6 decimals).
"""
import numpy as np
import pytest

from oracle import oracle as O


def site_patterns(z, codons):
    """pattern index of every site (columns of the codon matrix)."""
    key = {tuple(z[:, h]): h for h in range(z.shape[1])}
    return np.array([key[tuple(codons[:, i])] for i in range(codons.shape[1])])


def test_beb_matches_codeml(golden):
    fx, tree, codons = golden
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4)
    r = pb.beb(np.array(fx["x"]), lastround=True)
    g = fx["beb"]
    pose = site_patterns(z, codons)
    site = r["post"][:, pose].T
    assert np.max(np.abs(site - np.array(g["site_post_5dp"]))) <= 5.01e-6
    assert np.max(np.abs(r["grid"][2] - g["w0_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(r["grid"][3] - g["w2_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(r["p0p1"] - g["p0p1_post_3dp"])) <= 5.01e-4
    assert abs(r["lnfX"] - g["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["lnfX"])
    assert abs(r["S1"] - g["S1_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["S1"])
    assert abs(r["S2"] - g["S2_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["S2"])


def test_beb_posteriors_are_distributions():
    from tests.conftest import load_golden
    fx, tree, codons = load_golden("c24x400_s3")
    z, fpatt, pi = O.patterns(codons)
    r = O.Problem(tree, z, fpatt, pi, nthreads=4).beb(np.array(fx["x"]))
    assert np.allclose(r["post"].sum(axis=0), 1.0, atol=1e-12)
    assert np.allclose(r["grid"][2:].sum(axis=1), 1.0, atol=1e-12)
    assert abs(r["p0p1"].sum() - 1.0) < 1e-12
    assert np.all(r["grid"][:2] == -1)


def test_beb_class_sets_share_subtrees():
    """Sets with the same background omega differ only on the foreground
    branch: set 11 + 10 i + j (w0_i, w2_j) against set i (w0_i, w0_i) and
    set 111 + j (1, w2_j) against set 10 (1, 1); at a pattern they agree
    exactly when the foreground branch carries no information (t = 0)."""
    from tests.conftest import load_golden
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2)
    x = np.array(fx["x"])
    nb = tree.nbranch
    bn = tree.branch_nodes()
    fg = [ib for ib in range(nb) if tree.label[bn[ib]] == 1]
    assert len(fg) == 1
    x0 = x.copy()
    x0[fg[0]] = 0.0
    w = pb.beb(x0)["lnfw"]
    for i in range(10):
        for j in range(10):
            assert np.array_equal(w[11 + 10 * i + j], w[i])
    for j in range(10):
        assert np.array_equal(w[111 + j], w[10])


@pytest.mark.parametrize("nth", [1, 3])
def test_beb_thread_invariant(nth):
    from tests.conftest import load_golden
    fx, tree, codons = load_golden("c5x120_s5")
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    a = O.Problem(tree, z, fpatt, pi, nthreads=nth).beb(x)
    b = O.Problem(tree, z, fpatt, pi, nthreads=2).beb(x)
    assert np.array_equal(a["post"], b["post"]) and a["lnfX"] == b["lnfX"]


@pytest.mark.parametrize("name", ["mb8x300_s7", "mb24x400_s8"])
def test_beb_model_b_matches_codeml(name):
    """codeml runs model A's BEB grid for model B too (w1 = 1 in class 1),
    with model B's Qfactors (its free w1 in the mean rates)."""
    from tests.conftest import load_golden
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    r = O.Problem(tree, z, fpatt, pi, nthreads=4, model_b=True).beb(np.array(fx["x"]))
    g = fx["beb"]
    site = r["post"][:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(g["site_post_5dp"]))) <= 5.01e-6
    assert np.max(np.abs(r["grid"][2] - g["w0_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(r["grid"][3] - g["w2_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(r["p0p1"] - g["p0p1_post_3dp"])) <= 5.01e-4
    assert abs(r["lnfX"] - g["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["lnfX"])
