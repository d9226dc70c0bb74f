"""Clade model C on the GPU: two gb_eval_uvr calls (classes 0, 1 with eigen
slots (w0, 1, -); class 2 as model A's class 2a with slots (w2, 1, w3)), the
route codeml's adapter takes for model = 3, against the oracle's restatement
(pinned to codeml in tests/test_clade_oracle.py) and codeml's printed lnL.

Bars as for model A's gb_eval_uvr test: with the oracle's eigen solutions,
lnL within 1e-12 relative and log f within 1e-11 of the oracle; 1e-9
relative of codeml's lnL.
"""
import numpy as np
import pytest

from cucodeml_gb300 import api
from oracle import oracle as O
from tests.conftest import clade_d_names, clade_names, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", clade_names())
def test_clade_c_eval_uvr(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    kappa, p0, p1, w0, w2, w3 = x[nb:nb + 6]
    p2 = 1 - p0 - p1
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4)
    v, fhK, lnf = pb.clade_c(x)
    Ua, Va, Ra, _, _ = pb.set_params(np.concatenate([x[:nb], [kappa, p0, p1, w0, w2]]))
    U3, V3, R3, _, _ = pb.set_params(np.concatenate([x[:nb], [kappa, p0, p1, w0, w3]]))
    U = [Ua[0], Ua[1], Ua[2], U3[2]]
    V = [Va[0], Va[1], Va[2], V3[2]]
    R = [Ra[0], Ra[1], Ra[2], R3[2]]
    qf = np.array([1.0 / O.build_q(pi, kappa, p0 * w0 + p1 + p2 * w)[1] for w in (w2, w3)])
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    lk = api.Likelihood(tree, z, fpatt, pi)
    f, g_fhK, g_lnf = lk.clade_uvr(U, V, R, qf, [p0, p1, p2], bl)
    assert abs(f - v) <= 1e-12 * abs(v)
    assert np.max(np.abs(g_lnf - lnf)) <= 1e-11
    assert abs(-f - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    lk.close()


@pytest.mark.parametrize("name", clade_names())
def test_clade_c_beb(name):
    """Likelihood.beb_clade_c: the 111 tables from two gb_beb_tables calls
    against the oracle's (1e-10 + 2e-9 |log f|, as for model A's BEB), the
    posteriors against codeml's printed clade-C BEB (print rounding)."""
    from tests.test_beb_oracle import site_patterns
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    kappa, p0, p1, w0, w2, w3 = x[nb:nb + 6]
    p2 = 1 - p0 - p1
    ref = O.Problem(tree, z, fpatt, pi, nthreads=4).beb_clade(x)
    qf = np.array([1.0 / O.build_q(pi, kappa, p0 * w0 + p1 + p2 * w)[1] for w in (w2, w3)])
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    lk = api.Likelihood(tree, z, fpatt, pi)
    g01 = (np.arange(10) + 0.5) / 10
    g03 = (np.arange(10) + 0.5) * 3 / 10
    a = lk.beb_tables(bl, kappa, qf, g01, g03)
    b = lk.beb_tables(bl, kappa, qf, g03, g03)
    tab = np.concatenate([a[:11], b[11:111]])
    assert np.all(np.abs(tab - ref["lnfw"]) <= 1e-10 + 2e-9 * np.abs(ref["lnfw"]))
    r = lk.beb_clade_c(bl, kappa, qf)
    site = r["post"][:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(fx["beb"]["site_post_5dp"]))) <= 5.01e-6
    assert abs(r["lnfX"] - fx["beb"]["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["lnfX"])
    lk.close()


@pytest.mark.parametrize("name", clade_d_names())
def test_clade_d_eval_uvr(name):
    """Clade model D (w1 free): the same two gb_eval_uvr calls with slot 1
    holding w1, against the oracle and codeml's printed lnL."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    kappa, p0, p1, w0, w1, w2, w3 = x[nb:nb + 7]
    p2 = 1 - p0 - p1
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4, model_b=True)
    v, fhK, lnf = pb.clade_c(x)
    Ua, Va, Ra, _, _ = pb.set_params(np.concatenate([x[:nb], [kappa, p0, p1, w0, w1, w2]]))
    U3, V3, R3, _, _ = pb.set_params(np.concatenate([x[:nb], [kappa, p0, p1, w0, w1, w3]]))
    U = [Ua[0], Ua[1], Ua[2], U3[2]]
    V = [Va[0], Va[1], Va[2], V3[2]]
    R = [Ra[0], Ra[1], Ra[2], R3[2]]
    qf = np.array([1.0 / O.build_q(pi, kappa, p0 * w0 + p1 * w1 + p2 * w)[1] for w in (w2, w3)])
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    lk = api.Likelihood(tree, z, fpatt, pi)
    f, g_fhK, g_lnf = lk.clade_uvr(U, V, R, qf, [p0, p1, p2], bl)
    assert abs(f - v) <= 1e-12 * abs(v)
    assert np.max(np.abs(g_lnf - lnf)) <= 1e-11
    assert abs(-f - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    lk.close()


@pytest.mark.parametrize("name", clade_names() + clade_d_names())
def test_clade_beb_integral_on_device_matches_oracle(name):
    """gb_beb_clade, fed the oracle's own log f(x_h | w) tables (111 for clade
    C, 120 for clade D), against the oracle's grid integration of the same
    tables: posteriors and grid marginals within 1e-12, log f(X) within 1e-12
    relative (the device sums patterns in another order)."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    d = name.startswith("mcD")
    pb = O.Problem(tree, z, fpatt, pi, nthreads=O.max_threads(), model_b=d)
    ref = pb.beb_clade_d(x) if d else pb.beb_clade(x)
    lk = api.Likelihood(tree, z, fpatt, pi)
    r = lk.beb_clade(ref["lnfw"], model_d=d)
    lk.close()
    assert np.max(np.abs(r["post"] - ref["post"])) <= 1e-12
    rows = ref["grid"] if d else ref["grid"][[2, 3, 4]]
    got = r["grid"] if d else r["grid"][[0, 2, 3]]
    assert np.max(np.abs(got - rows)) <= 1e-12
    assert np.max(np.abs(r["p0p1"] - ref["p0p1"])) <= 1e-12
    assert abs(r["lnfX"] - ref["lnfX"]) <= 1e-12 * abs(ref["lnfX"])
    if not d:
        assert np.all(r["grid"][1] == -1.0)
    print(f"{name}: device grid integral {r['ms_device']:.1f} ms, lnfX {r['lnfX']:.6f}")


@pytest.mark.parametrize("name", clade_d_names())
def test_clade_d_beb(name):
    """Likelihood.beb_clade_d: the 120 tables from three gb_beb_tables calls
    and the 10^6-point integral on the device, against codeml's printed
    clade-D BEB: site posteriors (5 dp), grid and (p0, p1) posteriors (3 dp),
    log f(X) (6 dp)."""
    from tests.test_beb_oracle import site_patterns
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    kappa, p0, p1, w0, w1, w2, w3 = x[nb:nb + 7]
    p2 = 1 - p0 - p1
    qf = np.array([1.0 / O.build_q(pi, kappa, p0 * w0 + p1 * w1 + p2 * w)[1] for w in (w2, w3)])
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    lk = api.Likelihood(tree, z, fpatt, pi)
    r = lk.beb_clade_d(bl, kappa, qf)
    lk.close()
    b = fx["beb"]
    site = r["post"][:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(b["site_post_5dp"]))) <= 5.01e-6
    for row, key in enumerate(("w0_post_3dp", "w1_post_3dp", "w2_post_3dp", "w3_post_3dp")):
        assert np.max(np.abs(r["grid"][row] - np.array(b[key]))) <= 5.01e-4
    assert np.max(np.abs(r["p0p1"] - np.array(b["p0p1_post_3dp"]))) <= 5.01e-4
    assert abs(r["lnfX"] - b["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(r["lnfX"])


def _clade_inputs(pb, x, nb, model_d):
    """codeml's four eigen solutions (w0, w1, w2, w3), Qfactors and class
    weights of clade model C (model_d False: w1 = 1) or D at x."""
    if model_d:
        kappa, p0, p1, w0, w1, w2, w3 = x[nb:nb + 7]
        head = [kappa, p0, p1, w0, w1]
    else:
        kappa, p0, p1, w0, w2, w3 = x[nb:nb + 6]
        w1 = 1.0
        head = [kappa, p0, p1, w0]
    p2 = 1 - p0 - p1
    Ua, Va, Ra, _, _ = pb.set_params(np.concatenate([x[:nb], head, [w2]]))
    U3, V3, R3, _, _ = pb.set_params(np.concatenate([x[:nb], head, [w3]]))
    qf = np.array([1.0 / O.build_q(pb.pi, kappa, p0 * w0 + p1 * w1 + p2 * w)[1] for w in (w2, w3)])
    return ([Ua[0], Ua[1], Ua[2], U3[2]], [Va[0], Va[1], Va[2], V3[2]], [Ra[0], Ra[1], Ra[2], R3[2]], qf,
            [p0, p1, p2])


@pytest.mark.parametrize("name", clade_names() + clade_d_names())
def test_clade_one_evaluation_matches_two_calls(name):
    """gb_eval_clade_uvr (three classes at every internal node, four eigen
    solutions, one graph) against the composition of two gb_eval_uvr calls:
    the same FP64 kernels on the same matrices, so fhK agrees to rounding of
    the mixture (1e-13) and -lnL to 1e-12 relative."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2, model_b=name.startswith("mcD"))
    U, V, R, qf, fk = _clade_inputs(pb, x, nb, name.startswith("mcD"))
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    lk = api.Likelihood(tree, z, fpatt, pi)
    f1, fhK1, lnf1 = lk.clade_uvr(U, V, R, qf, fk, bl)
    f2, fhK2, lnf2 = lk.clade_uvr(U, V, R, qf, fk, bl, two_calls=True)
    f1b, fhK1b, _ = lk.clade_uvr(U, V, R, qf, fk, bl)        # the graph replayed
    lk.close()
    assert np.max(np.abs(fhK1 - fhK2)) <= 1e-13 * np.max(np.abs(fhK2))
    assert np.max(np.abs(lnf1 - lnf2)) <= 1e-13 * np.max(np.abs(lnf2))
    assert abs(f1 - f2) <= 1e-12 * abs(f2)
    assert f1b == f1 and np.array_equal(fhK1b, fhK1)
    assert abs(-f1 - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9


def test_clade_one_evaluation_time():
    """64 taxa x 2000 codons with a foreground clade: one clade evaluation
    against the two model-A-shaped calls it replaces (times printed; the
    single evaluation prunes 3 classes per internal node where the pair
    prunes 2 + 2 at every node and 2 more at the clade's nodes twice)."""
    from cucodeml_gb300.simulate import simulate
    a = simulate(64, 2000, seed=2024)
    z, fpatt, pi = api.patterns(a.codons)
    nb = a.tree.nbranch
    pb = O.Problem(a.tree, z, fpatt, pi, nthreads=2)
    x = np.concatenate([a.tree.branch[a.tree.branch_nodes()], [2.0, 0.5, 0.3, 0.3, 2.5, 4.0]])
    U, V, R, qf, fk = _clade_inputs(pb, x, nb, False)
    lk = api.Likelihood(a.tree, z, fpatt, pi)
    t1, t2 = [], []
    for _ in range(5):
        f1, _, _ = lk.clade_uvr(U, V, R, qf, fk, a.tree.branch)
        t1.append(lk.last_ms)
        f2, _, _ = lk.clade_uvr(U, V, R, qf, fk, a.tree.branch, two_calls=True)
        t2.append(lk.last_ms)
    lk.close()
    assert abs(f1 - f2) <= 1e-12 * abs(f2)
    print(f"clade C 64x2000 ({len(fpatt)} patterns): one evaluation {min(t1):.2f} ms, two calls {min(t2):.2f} ms")


@pytest.mark.parametrize("name", clade_names() + clade_d_names())
def test_clade_own_setup_matches_codeml(name):
    """gb_eval_clade: the clade model from its parameters with the library's
    eigen solutions and Qfactors, against codeml's printed lnL and log f and
    against the same evaluation from the oracle's eigen solutions (the two
    eigensolvers agree to rounding: 1e-11 relative in lnL)."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    d = name.startswith("mcD")
    if d:
        kappa, p0, p1, w0, w1, w2, w3 = x[nb:nb + 7]
    else:
        kappa, p0, p1, w0, w2, w3 = x[nb:nb + 6]
        w1 = 1.0
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2, model_b=d)
    U, V, R, qf, fk = _clade_inputs(pb, x, nb, d)
    lk = api.Likelihood(tree, z, fpatt, pi)
    f, fhK, lnf = lk.clade(bl, kappa, p0, p1, w0, w2, w3, w1=w1)
    f2, _, _ = lk.clade_uvr(U, V, R, qf, fk, bl)
    with pytest.raises(Exception):
        lk.clade(bl, kappa, 0.7, 0.6, w0, w2, w3)              # p0 + p1 > 1
    lk.close()
    assert abs(f - f2) <= 1e-11 * abs(f2)
    assert abs(-f - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))


def _clade_neg_lnL(pb, x, nb, lastround):
    """The oracle's clade -lnL at codeml's x, proportions transformed as
    codeml's f_and_x does unless lastround."""
    x = np.array(x, dtype=np.float64)
    if not lastround:
        e1, e2 = np.exp(x[nb + 1]), np.exp(x[nb + 2])
        x[nb + 1], x[nb + 2] = e1 / (1 + e1 + e2), e2 / (1 + e1 + e2)
    return pb.clade_c(x)[0]


def _fd5(f, x, h=1e-4):
    g = np.zeros(len(x))
    for i in range(len(x)):
        e = h * (abs(x[i]) + 0.05)
        v = []
        for k in (-2, -1, 1, 2):
            xk = x.copy()
            xk[i] += k * e
            v.append(f(xk))
        g[i] = (v[0] - 8 * v[1] + 8 * v[2] - v[3]) / (12 * e)
    return g


@pytest.mark.parametrize("name", clade_names() + clade_d_names())
@pytest.mark.parametrize("lastround", [True, False])
def test_clade_gradient_matches_fd(name, lastround):
    """The clade models' analytic gradient (gb_dfun_clade_x: the FP64 adjoint
    over the three-class schedule, the chain rule through both branch types'
    Qfactors and the class weights) against five-point differences of the
    oracle's clade -lnL in codeml's x space, both of codeml's proportion
    spaces: 1e-5 relative, as for model A."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    d = name.startswith("mcD")
    nb = tree.nbranch
    x = np.array(fx["x"])
    if not lastround:
        p0, p1 = x[nb + 1], x[nb + 2]
        p2 = 1 - p0 - p1
        x[nb + 1], x[nb + 2] = np.log(p0 / p2), np.log(p1 / p2)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=O.max_threads(), model_b=d)
    lk = api.Likelihood(tree, z, fpatt, pi)
    f, g = lk.dfun_clade_x(x, lastround, model_d=d)
    lk.close()
    f0 = _clade_neg_lnL(pb, x, nb, lastround)
    assert abs(f - f0) <= 1e-12 * abs(f0)
    gfd = _fd5(lambda xx: _clade_neg_lnL(pb, xx, nb, lastround), x)
    err = np.abs(g - gfd) / np.maximum(1.0, np.abs(gfd))
    print(f"{name} lastround={lastround}: max rel err {err.max():.2e}")
    assert err.max() <= 1e-5


def test_clade_gradient_natural_parameters():
    """Likelihood.clade(grad=True) against the x-space entry: the same
    adjoint, branch lengths in node order and (kappa, p0, p1, w0, w2, w3)."""
    name = clade_names()[0]
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    nb = tree.nbranch
    x = np.array(fx["x"])
    kappa, p0, p1, w0, w2, w3 = x[nb:nb + 6]
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    lk = api.Likelihood(tree, z, fpatt, pi)
    f, _, _, g = lk.clade(bl, kappa, p0, p1, w0, w2, w3, grad=True)
    f2, gx = lk.dfun_clade_x(x, True)
    f3, _, _ = lk.clade(bl, kappa, p0, p1, w0, w2, w3)
    lk.close()
    assert f == f2 == f3
    assert np.allclose(g["blength"][tree.branch_nodes()], gx[:nb], rtol=1e-13, atol=0)
    assert np.allclose([g["kappa"], g["p0"], g["p1"], g["omega0"], g["omega2"], g["omega3"]], gx[nb:],
                       rtol=1e-13, atol=0)


@pytest.mark.parametrize("name", clade_names() + clade_d_names())
def test_clade_neb_matches_codeml(name):
    """gb_neb_clade: the mixture kernel's class posteriors of one clade
    evaluation against codeml's NEB (rst, 5 dp); they sum to 1."""
    from tests.test_beb_oracle import site_patterns
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    if name.startswith("mcD"):
        kappa, p0, p1, w0, w1, w2, w3 = x[nb:nb + 7]
    else:
        kappa, p0, p1, w0, w2, w3 = x[nb:nb + 6]
        w1 = 1.0
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    lk = api.Likelihood(tree, z, fpatt, pi)
    post, f = lk.neb_clade(bl, kappa, p0, p1, w0, w2, w3, w1=w1)
    lk.close()
    site = post[:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(fx["neb_site_post_5dp"]))) <= 5.01e-6
    assert np.allclose(post.sum(axis=0), 1.0, atol=1e-13)
    assert abs(-f - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9


@pytest.mark.parametrize("name", clade_names() + clade_d_names())
def test_clade_se_matches_codeml(name):
    """gb_se_opg_clade (codeml's getSE = 1 estimator over 2 np clade
    evaluations) against codeml's printed SEs: print rounding plus 1e-4 of
    the value, as for model A."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    lk = api.Likelihood(tree, z, fpatt, pi)
    r = lk.se_opg_clade(np.array(fx["x"]), model_d=name.startswith("mcD"), small_diff=fx["small_diff"])
    lk.close()
    ref = np.array(fx["se_6dp"])
    assert np.array_equal(r["H"], r["H"].T)
    assert np.all(np.abs(r["se"] - ref) <= 5.01e-7 + 1e-4 * np.abs(ref))
