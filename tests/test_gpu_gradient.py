"""Adjoint gradient (FP64) through the C ABI against finite differences of the
oracle and against codeml's own numerical gradient (gradientB restated).

Bar: relative error <= 1e-5 against a 5-point central difference of the
oracle (step 1e-4 (|x_i| + 0.05), truncation O(h^4)), measured as
max |g - g_fd| / max(1, |g_fd|) over all np entries.
"""
import numpy as np
import pytest

from cucodeml_gb300 import api
from oracle import oracle as O
from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def fd_grad(pb, x, lastround, h=1e-4):
    g = np.zeros(len(x))
    for i in range(len(x)):
        e = h * (abs(x[i]) + 0.05)
        f = []
        for k in (-2, -1, 1, 2):
            xk = x.copy()
            xk[i] += k * e
            f.append(pb.neg_lnL(xk, lastround))
        g[i] = (f[0] - 8 * f[1] + 8 * f[2] - f[3]) / (12 * e)
    return g


def rel_err(g, ref):
    return float(np.max(np.abs(g - ref) / np.maximum(1.0, np.abs(ref))))


@pytest.mark.parametrize("name", ["c8x300_s1", "c8x300_s2", "c5x120_s5", "c24x400_s3"])
@pytest.mark.parametrize("lastround", [True, False])
def test_dfun_matches_fd(name, lastround):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4)
    x = np.array(fx["x"])
    nb = tree.nbranch
    if name.startswith("c5x120"):
        x[:nb] = np.maximum(x[:nb], 0.02)    # the FD needs every branch away from t = 0
    if not lastround:
        p0, p1 = x[nb + 1], x[nb + 2]
        x[nb + 1] = np.log(p0 / (1 - p0 - p1))
        x[nb + 2] = np.log(p1 / (1 - p0 - p1))
    lk = api.Likelihood(tree, z, fpatt, pi)
    f, g = lk.dfun_x(x, lastround)
    assert abs(f - pb.neg_lnL(x, lastround)) <= 1e-9 * abs(f)
    ref = fd_grad(pb, x, lastround)
    err = np.abs(g - ref) / np.maximum(1.0, np.abs(ref))
    i = int(np.argmax(err))
    assert err[i] <= 1e-5, (i, g[i], ref[i], err[i])
    lk.close()


def test_against_codeml_gradientB():
    fx, tree, codons = load_golden("c8x300_s2")
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4)
    x = np.array(fx["x"])
    lk = api.Likelihood(tree, z, fpatt, pi)
    f, g = lk.dfun_x(x, True)
    gb = pb.gradientB(x, True, central=True)
    # codeml's step (1e-6(|x|+1))^0.67 ~ 1e-4 limits its own accuracy
    assert rel_err(g, gb) <= 1e-4
    lk.close()
