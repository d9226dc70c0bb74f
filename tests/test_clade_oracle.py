"""Clade model C (codeml model = 3, NSsites = 2, two branch types): the
oracle's restatement as two model-A class evaluations against the reference
codeml's fixed-parameter runs (tests/golden/mcC*.json).

Clade C's third class carries w2 on background and w3 on foreground
branches; that is model A's class 2a with eigen slots (w2, -, w3), while its
classes 0 and 1 are model A's with slots (w0, 1, -).  Bars as for model A.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import clade_d_names, clade_names, load_golden


@pytest.mark.parametrize("name", clade_names())
def test_clade_c_matches_codeml(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2)
    x = np.array(fx["x"])
    assert len(x) == fx["codeml_np"] == tree.nbranch + 6
    v, fhK, lnf = pb.clade_c(x)
    assert abs(-v - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(v)
    assert abs(-v - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))


@pytest.mark.parametrize("name", clade_names())
def test_clade_c_beb_matches_codeml(name):
    """codeml's BEB under clade C (lfunNSsites_ACD with modelACD = mC): the
    oracle's restatement against codeml's printed posteriors, grid marginals
    and log f(X).  (The library's device integral, fed the oracle's tables,
    is held to the oracle's integration in tests/test_gpu_clade.py.)"""
    from tests.test_beb_oracle import site_patterns
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    r = O.Problem(tree, z, fpatt, pi, nthreads=4).beb_clade(np.array(fx["x"]))
    g = fx["beb"]
    site = r["post"][:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(g["site_post_5dp"]))) <= 5.01e-6
    for row, key in ((2, "w0_post_3dp"), (3, "w2_post_3dp"), (4, "w3_post_3dp")):
        assert np.max(np.abs(r["grid"][row] - g[key])) <= 5.01e-4
    assert np.max(np.abs(r["p0p1"] - g["p0p1_post_3dp"])) <= 5.01e-4
    assert abs(r["lnfX"] - g["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["lnfX"])


@pytest.mark.parametrize("name", clade_d_names())
def test_clade_d_matches_codeml(name):
    """Clade model D (NSsites = 3, ncatG = 3): clade C with w1 free
    (SetParametersNSsites codeml.c:2427-2446, eigen slots w0, w1, w2, w3
    codeml.c:2535-2539), against codeml's fixed-parameter runs."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2, model_b=True)
    x = np.array(fx["x"])
    assert len(x) == fx["codeml_np"] == tree.nbranch + 7
    v, fhK, lnf = pb.clade_c(x)
    assert abs(-v - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(v)
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))


@pytest.mark.parametrize("name", clade_d_names())
def test_clade_d_beb_matches_codeml(name):
    """codeml's BEB under clade model D (lfunNSsites_ACD with modelACD = mD:
    120 omega sets, 10^6-point grid over the (p0, p1) triangles, w0, w1, w2,
    w3), restated in numpy over the oracle's pruning, against codeml's
    printed site posteriors (rst, 5 dp), grid posteriors and (p0, p1)
    posterior (out, 3 dp) and log f(X), S1 (stdout, 6 dp)."""
    from tests.test_beb_oracle import site_patterns
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    r = O.Problem(tree, z, fpatt, pi, nthreads=O.max_threads(), model_b=True).beb_clade_d(np.array(fx["x"]))
    b = fx["beb"]
    assert abs(r["lnfX"] - b["lnfX_6dp"]) <= 1e-6 + 1e-12 * abs(b["lnfX_6dp"])
    assert abs(r["S1"] - b["S1_6dp"]) <= 1e-6 + 1e-12 * abs(b["S1_6dp"])
    site = r["post"][:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(b["site_post_5dp"]))) <= 5.01e-6
    for row, key in enumerate(("w0_post_3dp", "w1_post_3dp", "w2_post_3dp", "w3_post_3dp")):
        assert np.max(np.abs(r["grid"][row] - np.array(b[key]))) <= 5.01e-4
    assert np.max(np.abs(r["p0p1"] - np.array(b["p0p1_post_3dp"]))) <= 5.01e-4
    assert np.allclose(r["post"].sum(axis=0), 1.0, atol=1e-12)


@pytest.mark.parametrize("name", clade_names() + clade_d_names())
def test_clade_neb_matches_codeml(name):
    """codeml's NEB under the clade models (lfunNSsites_rate
    codeml.c:5079-5129: freqK_c f_c normalised over the three classes),
    from the oracle's clade evaluation, against codeml's rst (5 dp)."""
    from tests.test_beb_oracle import site_patterns
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    d = name.startswith("mcD")
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2, model_b=d)
    x = np.array(fx["x"])
    nb = tree.nbranch
    v, fhK, lnf = pb.clade_c(x)
    p0, p1 = x[nb + 1], x[nb + 2]
    fk = np.array([p0, p1, 1 - p0 - p1])
    scaled = bool(np.any(fhK < 0))      # with scaled nodes fhK holds log f (f itself otherwise)
    f = np.exp(fhK - fhK.max(axis=0)) if scaled else fhK
    q = fk[:, None] * f
    post = q / q.sum(axis=0)
    site = post[:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(fx["neb_site_post_5dp"]))) <= 5.01e-6


def clade_opg_se(pb, x, small_diff):
    """codeml's getSE = 1 estimator (HessianSKT2004 treesub.c:6979-7048) over
    the oracle's clade evaluation: per-pattern scores from central
    differences of log f_h, step 2 small_diff (|x_i| + 1)."""
    n = len(x)
    eh = 2 * small_diff * (np.abs(x) + 1)
    D = []
    for i in range(n):
        f = []
        for s in (-1, 1):
            x1 = x.copy()
            x1[i] += s * eh[i]
            f.append(pb.clade_c(x1)[2])
        D.append((f[1] - f[0]) / (2 * eh[i]))
    D = np.array(D)
    H = -(D * pb.fpatt[None, :]) @ D.T
    V = np.linalg.inv(-0.5 * (H + H.T))
    dg = np.diag(V)
    return np.where(dg > 0, np.sqrt(np.abs(dg)), -1.0)


@pytest.mark.parametrize("name", [n for n in clade_names() + clade_d_names() if "8x300" in n])
def test_clade_se_matches_codeml(name):
    """codeml's SEs under the clade models (getSE = 1), restated over the
    oracle's clade evaluation: print rounding plus 5e-5 of the value (the
    8-taxon fixtures; the GPU test takes all four)."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=O.max_threads(), model_b=name.startswith("mcD"))
    se = clade_opg_se(pb, np.array(fx["x"]), fx["small_diff"])
    ref = np.array(fx["se_6dp"])
    assert se.shape == ref.shape
    assert np.all(np.abs(se - ref) <= 5.01e-7 + 5e-5 * np.abs(ref))
