"""Site models M2a and M1a (codeml model = 0, NSsites = 2 / 1) as branch-site
model A with every branch in the foreground.

Under M2a codeml mixes three classes, w0 < 1, w1 = 1 and w2, each on the whole
tree, with Qfactor_NS = 1 / meanrate(Q(kappa, p0 w0 + p1 + p2 w2))
(SetParametersNSsites codeml.c:2466-2487).  Model A with every branch
labelled #1 has the same mixture: classes 0 and 1 are w0 and 1 everywhere,
classes 2a and 2b are both w2 everywhere with weights summing to p2, and the
foreground Qfactor is the same mean-rate normalisation.  M1a is M2a with
p2 = 0.  So the model-A machinery (oracle, FP64 drop-in, adjoint, split
precision) evaluates them unchanged.  M3 with three classes (w0, w1, w2
free) is, the same way, model B on the all-foreground tree.  Pinned here:
the oracle under that mapping against the reference codeml's own
fixed-parameter runs of M2a, M1a and M3 (tests/golden/ms*.json).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import as_model_a, load_golden, site_model_names


@pytest.mark.parametrize("name", site_model_names())
def test_site_classes_match_codeml(name):
    """Every site model as K whole-tree classes on the all-foreground tree
    (three per evaluation of model A's class map), including M7 and M8 with
    ten beta categories."""
    from tests.conftest import site_model_classes
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, _ = as_model_a(fx, tree)
    om, pr = site_model_classes(fx, tree)
    x = np.array(fx["x"])
    nb = tree.nbranch
    v, fhK, lnf = O.Problem(t, z, fpatt, pi, nthreads=2).site_classes(x[:nb], x[nb], om, pr)
    assert abs(-v - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(v)
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))


@pytest.mark.parametrize("name", [n for n in site_model_names() if not n.startswith(("msM7", "msM8"))])
def test_site_model_as_model_a_matches_codeml(name):
    fx, tree, codons = load_golden(name)
    assert np.all(tree.label == 0)
    z, fpatt, pi = O.patterns(codons)
    t, x = as_model_a(fx, tree)
    pb = O.Problem(t, z, fpatt, pi, nthreads=2, model_b=fx["model"] == "M3")
    v, fhK, lnf, nscale = pb.neg_lnL(x, lastround=True, want_fhK=True)
    assert abs(-v - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(v)
    assert abs(-v - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))


@pytest.mark.parametrize("name", [n for n in site_model_names() if n.startswith("msM2a")])
def test_m2a_beb_as_model_a(name):
    """codeml's BEB for M2a (lfunNSsites_M2M8 codeml.c:6190-6415) has model
    A's grid (ternary (p0, p1), w0 in (0, 1), w2 in (1, 11), 10 points each)
    and prior; on the all-foreground tree model A's classes 2a and 2b both
    carry w2, so M2a's class-2 posterior is their sum."""
    from tests.test_beb_oracle import site_patterns
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, x = as_model_a(fx, tree)
    r = O.Problem(t, z, fpatt, pi, nthreads=4).beb(x)
    post = np.stack([r["post"][0], r["post"][1], r["post"][2] + r["post"][3]])
    g = fx["beb"]
    site = post[:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(g["site_post_5dp"]))) <= 5.01e-6
    assert np.max(np.abs(r["grid"][2] - g["w0_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(r["grid"][3] - g["w2_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(r["p0p1"] - g["p0p1_post_3dp"])) <= 5.01e-4
    assert abs(r["lnfX"] - g["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["lnfX"])
    # the posterior mean and SD of w codeml prints beside them (3 dp)
    ms = np.stack([r["wmean"], r["wsd"]])[:, site_patterns(z, codons)].T
    assert np.max(np.abs(ms - np.array(g["site_wmean_sd_3dp"]))) <= 5.01e-4


@pytest.mark.parametrize("name", site_model_names())
def test_site_model_neb_matches_codeml(name):
    """codeml's NEB under the site models (lfunNSsites_rate codeml.c:5079-5129:
    props_k f_k normalised over the K classes; M7 / M8 over the ten beta
    categories and w_s), from the oracle's K whole-tree classes, against
    codeml's rst (5 dp)."""
    from tests.conftest import site_model_classes
    from tests.test_beb_oracle import site_patterns
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, _ = as_model_a(fx, tree)
    om, pr = site_model_classes(fx, tree)
    x = np.array(fx["x"])
    nb = tree.nbranch
    v, fhK, lnf = O.Problem(t, z, fpatt, pi, nthreads=2).site_classes(x[:nb], x[nb], om, pr)
    scaled = bool(np.any(fhK < 0))      # with scaled nodes fhK holds log f
    f = np.exp(fhK - fhK.max(axis=0)) if scaled else fhK
    q = np.asarray(pr)[:, None] * f
    post = q / q.sum(axis=0)
    site = post[:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(fx["neb_site_post_5dp"]))) <= 5.01e-6


def _site_x_classes(x, nb, model):
    """(omegas, props) of a site model at codeml's x (oracle's quantiles)."""
    r = x[nb + 1:]
    if model == "M1a":
        return np.array([r[1], 1.0]), np.array([r[0], 1 - r[0]])
    if model == "M2a":
        return np.array([r[2], 1.0, r[3]]), np.array([r[0], r[1], 1 - r[0] - r[1]])
    if model == "M3":
        return np.array(r[2:5]), np.array([r[0], r[1], 1 - r[0] - r[1]])
    if model == "M7":
        return O.beta_classes(r[0], r[1])
    om, pr = O.beta_classes(r[1], r[2])
    return np.append(om, r[3]), np.append(pr * r[0], 1 - r[0])


@pytest.mark.parametrize("name", [n for n in site_model_names() if "24x400" not in n])
def test_site_model_se_generic_matches_codeml(name):
    """codeml's getSE = 1 SEs under the site models (M1a, M2a, M3, M7), by
    the estimator over the oracle's K whole-tree classes at the perturbed x:
    print rounding plus 5e-5 of the value (the smaller fixtures; the GPU test
    takes all six, M8 included, against codeml's SEs)."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, _ = as_model_a(fx, tree)
    x = np.array(fx["x"])
    nb = tree.nbranch
    pb = O.Problem(t, z, fpatt, pi, nthreads=O.max_threads())
    n = len(x)
    eh = 2 * fx["small_diff"] * (np.abs(x) + 1)
    D = np.zeros((n, len(fpatt)))
    for i in range(n):
        for sgn in (-1.0, 1.0):
            x1 = x.copy()
            x1[i] += sgn * eh[i]
            om, pr = _site_x_classes(x1, nb, fx["model"])
            D[i] += sgn * pb.site_classes(x1[:nb], x1[nb], om, pr)[2] / (2 * eh[i])
    H = -(D * fpatt[None, :]) @ D.T
    V = np.linalg.inv(-0.5 * (H + H.T))
    se = np.where(np.diag(V) > 0, np.sqrt(np.abs(np.diag(V))), -1.0)
    ref = np.array(fx["se_6dp"])
    assert np.all(np.abs(se - ref) <= 5.01e-7 + 5e-5 * np.abs(ref))
