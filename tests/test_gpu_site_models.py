"""Site models M2a / M1a on the GPU as branch-site model A with every branch
in the foreground (the equivalence is pinned on the CPU in
tests/test_site_models_oracle.py): the FP64 drop-in's lnL and per-pattern
log f against the reference codeml's own runs of M2a / M1a (1e-9 relative,
print rounding + 2e-11 |log f|) and the oracle, and for M2a the adjoint
gradient against 5-point differences of the oracle (1e-5, as for model A).
Every node of such a tree is on a foreground path, so all four classes are
pruned at every node: the schedule's other extreme from one foreground
branch.
"""
import numpy as np
import pytest

from cucodeml_gb300 import api
from oracle import oracle as O
from tests.conftest import as_model_a, load_golden, site_model_names
from tests.test_gpu_gradient import fd_grad

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", site_model_names())
def test_site_model_classes(name):
    """Likelihood.site_model: K whole-tree classes, three per gb_eval_uvr
    call, eigen solutions from the library; every site model including M7
    and M8 (ten beta categories) against codeml's printed lnL and log f, and
    for M7 / M8 Likelihood.m7 / m8 (the library's discretised beta) against
    the same classes from the oracle's quantiles; codeml's NEB over the K
    classes (Likelihood.site_neb)."""
    from tests.conftest import site_model_classes
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, _ = as_model_a(fx, tree)
    om, pr = site_model_classes(fx, tree)
    x = np.array(fx["x"])
    nb = t.nbranch
    bl = np.zeros(t.nnode)
    bl[t.branch_nodes()] = x[:nb]
    lk = api.Likelihood(t, z, fpatt, pi)
    f, fhK, lnf = lk.site_model(bl, x[nb], om, pr)
    if fx["model"] in ("M7", "M8"):          # the library's own discretised beta
        g = lk.m7(bl, x[nb], *x[nb + 1:nb + 3]) if fx["model"] == "M7" else lk.m8(bl, x[nb], *x[nb + 1:nb + 5])
        assert abs(g[0] - f) <= 1e-11 * abs(f)
        assert np.all(np.abs(g[2] - lnf) <= 5e-11 + 1e-12 * np.abs(lnf))   # quantiles agree to ~1e-13
    assert abs(-f - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))
    # codeml's NEB over the K classes (rst, 5 dp)
    from tests.test_beb_oracle import site_patterns
    post = lk.site_neb(fhK, pr)
    site = post[:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(fx["neb_site_post_5dp"]))) <= 5.01e-6
    lk.close()


@pytest.mark.parametrize("name", [n for n in site_model_names() if not n.startswith(("msM7", "msM8"))])
def test_site_model_fp64(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, x = as_model_a(fx, tree)
    m3 = fx["model"] == "M3"
    pb = O.Problem(t, z, fpatt, pi, nthreads=4, model_b=m3)
    lk = api.Likelihood(t, z, fpatt, pi)
    nb = t.nbranch
    bl = np.zeros(t.nnode)
    bl[t.branch_nodes()] = x[:nb]
    if m3:      # model B on the all-foreground tree: the drop-in's gb_eval_uvr
        U, V, R, qf, fk = pb.set_params(x)
        r = lk.neg_lnL_uvr(U, V, R, qf, fk, bl)
    else:
        r = lk.evaluate(bl, x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2], want_site=True)
    assert abs(-r.neg_lnL - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(r.lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))
    assert abs(r.neg_lnL - pb.neg_lnL(x)) <= 1e-9 * abs(r.neg_lnL)
    if fx["model"] == "M2a":
        f, g = lk.dfun_x(x, True)
        gfd = fd_grad(pb, x, True)
        assert np.max(np.abs(g - gfd) / np.maximum(1.0, np.abs(gfd))) <= 1e-5
    lk.close()


@pytest.mark.parametrize("name", [n for n in site_model_names() if n.startswith("msM2a")])
def test_m2a_beb(name):
    """gb_beb on the all-foreground tree is codeml's M2a BEB (class 2 = 2a + 2b;
    the equivalence is pinned on the CPU): against codeml's printed output."""
    from tests.test_beb_oracle import site_patterns
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, x = as_model_a(fx, tree)
    pb = O.Problem(t, z, fpatt, pi, nthreads=4)
    ref = pb.beb(x)
    qf = pb.set_params(x)[3]
    lk = api.Likelihood(t, z, fpatt, pi)
    nb = t.nbranch
    bl = np.zeros(t.nnode)
    bl[t.branch_nodes()] = x[:nb]
    r = lk.beb_qf(bl, x[nb], qf)
    post = np.stack([r["post"][0], r["post"][1], r["post"][2] + r["post"][3]])
    g = fx["beb"]
    pose = site_patterns(z, codons)
    site = post[:, pose].T
    assert np.max(np.abs(site - np.array(g["site_post_5dp"]))) <= 5.01e-6
    assert abs(r["lnfX"] - g["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["lnfX"])
    assert np.max(np.abs(r["wmean"] - ref["wmean"])) <= 1e-8
    assert np.max(np.abs(r["wsd"] - ref["wsd"])) <= 1e-6
    ms = np.stack([r["wmean"], r["wsd"]])[:, pose].T
    assert np.max(np.abs(ms - np.array(g["site_wmean_sd_3dp"]))) <= 5.01e-4
    lk.close()


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_m3_gradient_through_model_b(precision):
    """M3 with three classes (w0, w1, w2 free on every branch, proportions
    p0, p1, p2, Qfactor from p0 w0 + p1 w1 + p2 w2) is branch-site model B
    on the all-foreground tree, so gb_eval_b and its adjoint serve it: lnL
    against codeml's printed value, and the gradient in codeml's x (branch
    lengths, kappa, p0, p1, w0, w1, w2) against five-point differences of
    the oracle's model B on that tree (1e-5)."""
    name = "msM3k3x8x300_s14"
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, x = as_model_a(fx, tree)
    nb = t.nbranch
    lk = api.Likelihood(t, z, fpatt, pi, precision=precision)
    f, g = lk.dfun_x(x, True)
    assert abs(-f - fx["codeml_lnL"]) <= (1e-9 * abs(f) if precision == "fp64" else 1e-6) + 5.1e-7
    pb = O.Problem(t, z, fpatt, pi, nthreads=4, model_b=True)
    ref = fd_grad(pb, x, True)
    err = np.abs(g - ref) / np.maximum(1.0, np.abs(ref))
    print(f"M3 via model B ({precision}): max rel err {err.max():.2e}")
    assert err.max() <= 1e-5
    lk.close()


@pytest.mark.parametrize("name", [n for n in site_model_names() if n.startswith(("msM2a", "msM3"))])
def test_site_model_se_matches_codeml(name):
    """gb_se_opg on the all-foreground tree gives codeml's SEs under M2a
    (model A's x) and M3 (model B's x): print rounding plus 1e-4."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, x = as_model_a(fx, tree)
    lk = api.Likelihood(t, z, fpatt, pi)
    r = lk.se_opg(x, small_diff=fx["small_diff"])
    lk.close()
    ref = np.array(fx["se_6dp"])
    assert np.all(np.abs(r["se"] - ref) <= 5.01e-7 + 1e-4 * np.abs(ref))


@pytest.mark.parametrize("name", site_model_names())
def test_site_model_se_opg_site(name):
    """Likelihood.se_opg_site: codeml's getSE = 1 estimator under any site
    model from 2 n site_model evaluations on the device (the library's own
    beta categories for M7 / M8), against codeml's printed SEs: print
    rounding plus 1e-4 of the value."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    t, _ = as_model_a(fx, tree)
    lk = api.Likelihood(t, z, fpatt, pi)
    r = lk.se_opg_site(np.array(fx["x"]), fx["model"], small_diff=fx["small_diff"])
    lk.close()
    ref = np.array(fx["se_6dp"])
    assert np.all(np.abs(r["se"] - ref) <= 5.01e-7 + 1e-4 * np.abs(ref))
