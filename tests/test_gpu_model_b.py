"""Branch-site model B on the GPU through gb_eval_uvr, the entry codeml's
adapter uses (CUDA_ScheduleConditionalPNode hands over codeml's own U, V,
Root, Qfactors and class proportions): model B differs from model A only in
those inputs (w1 free), so the FP64 drop-in serves it unchanged.

Bars as for model A's gb_eval_uvr test: with the oracle's U, V, Root the GPU
lnL within 1e-12 relative of the oracle's and log f within 1e-11; against
codeml's printed lnL, 1e-9 relative.
"""
import numpy as np
import pytest

from cucodeml_gb300 import api
from oracle import oracle as O
from tests.conftest import load_golden, model_b_names

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", model_b_names())
def test_model_b_eval_uvr(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    pb = O.Problem(tree, z, fpatt, pi, model_b=True)
    U, V, R, qf, fk = pb.set_params(x)
    v, fhK, lnf, nsc = pb.neg_lnL(x, True, True)
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[: tree.nbranch]
    lk = api.Likelihood(tree, z, fpatt, pi)
    r = lk.neg_lnL_uvr(U, V, R, qf, fk, bl)
    assert lk.nscale == nsc
    assert abs(r.neg_lnL - v) <= 1e-12 * abs(v)
    assert np.max(np.abs(r.lnf - lnf)) <= 1e-11
    assert abs(-r.neg_lnL - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    lk.close()


@pytest.mark.parametrize("precision", ["fp64", "fast"])
@pytest.mark.parametrize("name", model_b_names())
def test_model_b_own_setup(name, precision):
    """gb_eval_b: the library's own model-B set-up (eigen solution of
    Q(kappa, w1), Qfactors with w1) against the oracle and codeml's printed
    lnL: FP64 within 1e-9 relative, split precision within 1e-6 absolute."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    kappa, p0, p1, w0, w1, w2 = x[nb:nb + 6]
    v = O.Problem(tree, z, fpatt, pi, model_b=True).neg_lnL(x)
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    lk = api.Likelihood(tree, z, fpatt, pi, precision=precision)
    r = lk.evaluate(bl, kappa, w0, w2, p0, p1, omega1=w1)
    bar = 1e-9 * abs(v) if precision == "fp64" else 1e-6
    assert abs(r.neg_lnL - v) <= bar
    assert abs(-r.neg_lnL - fx["codeml_lnL"]) <= max(bar, 5.1e-7)
    lk.close()


@pytest.mark.parametrize("lastround", [True, False])
@pytest.mark.parametrize("precision", ["fp64", "fast"])
@pytest.mark.parametrize("name", model_b_names())
def test_model_b_gradient(name, precision, lastround):
    """The adjoint gradient of model B in codeml's x space (gb_dfun_x with
    n = nbranch + 6: ..., w0, w1, w2), including d/dw1 through the second
    eigen solution and both Qfactors, against a five-point difference of the
    oracle: relative error <= 1e-5 of max(1, |g|)."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    if not lastround:
        p0, p1 = x[nb + 1], x[nb + 2]
        x[nb + 1] = np.log(p0 / (1 - p0 - p1))
        x[nb + 2] = np.log(p1 / (1 - p0 - p1))
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4, model_b=True)
    lk = api.Likelihood(tree, z, fpatt, pi, precision=precision)
    f, g = lk.dfun_x(x, lastround)
    assert len(g) == nb + 6
    assert abs(f - pb.neg_lnL(x, lastround)) <= (1e-9 * abs(f) if precision == "fp64" else 1e-6)
    ref = np.zeros(len(x))
    for i in range(len(x)):
        e = 1e-4 * (abs(x[i]) + 0.05)
        fs = []
        for k in (-2, -1, 1, 2):
            xk = x.copy()
            xk[i] += k * e
            fs.append(pb.neg_lnL(xk, lastround))
        ref[i] = (fs[0] - 8 * fs[1] + 8 * fs[2] - fs[3]) / (12 * e)
    err = np.abs(g - ref) / np.maximum(1.0, np.abs(ref))
    print(f"{name} {precision} lastround={lastround}: max rel err {err.max():.2e} (d/dw1 {g[nb + 4]:.6f} "
          f"fd {ref[nb + 4]:.6f})")
    assert err.max() <= 1e-5, (int(np.argmax(err)), err.max())
    lk.close()
