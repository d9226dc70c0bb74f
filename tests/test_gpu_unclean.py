"""Gaps and ambiguous codons (codeml's cleandata = 0) on the GPU, FP64 path
(gb_create_unclean), against the oracle and the reference codeml.

Fixtures: tests/golden/u*.json (make_unclean_golden.py) keep the data as
codeml encoded it.  Bars as for clean data: with the oracle's U, V, Root the
lnL within 1e-12 relative and per-pattern log f within 1e-11; from natural
parameters codeml's printed lnL within 1e-9 relative; the adjoint gradient
within 1e-5 relative of a five-point difference of the oracle."""
import numpy as np
import pytest

from cucodeml_gb300 import _lib, api
from oracle import oracle as O
from tests.conftest import load_unclean, unclean_names

pytestmark = pytest.mark.gpu


def node_blength(tree, x):
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = np.asarray(x)[: tree.nbranch]
    return bl


@pytest.mark.parametrize("name", unclean_names())
def test_unclean_matches_oracle_and_codeml(name):
    fx, tree, z, fpatt, pi, amb = load_unclean(name)
    x = np.array(fx["x"])
    nb = tree.nbranch
    pb = O.Problem(tree, z, fpatt, pi, ambiguity=amb)
    U, V, R, qf, fk = pb.set_params(x)
    v, fhK, lnf, nsc = pb.neg_lnL(x, True, True)
    lk = api.Likelihood(tree, z, fpatt, pi, ambiguity=amb)
    r = lk.neg_lnL_uvr(U, V, R, qf, fk, node_blength(tree, x))
    assert abs(r.neg_lnL - v) <= 1e-12 * abs(v)
    assert np.max(np.abs(r.lnf - lnf)) <= 1e-11
    r2 = lk.evaluate(node_blength(tree, x), x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2], want_site=True)
    assert abs(-r2.neg_lnL - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(r2.lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))
    print(f"{name}: -lnL {r2.neg_lnL:.6f} codeml {-fx['codeml_lnL']:.6f}, {int((z >= 61).sum())} ambiguous cells")
    lk.close()


@pytest.mark.parametrize("name", unclean_names())
def test_unclean_gradient_matches_fd(name):
    fx, tree, z, fpatt, pi, amb = load_unclean(name)
    x = np.array(fx["x"])
    nb = tree.nbranch
    x[:nb] = np.maximum(x[:nb], 0.02)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4, ambiguity=amb)
    lk = api.Likelihood(tree, z, fpatt, pi, ambiguity=amb)
    f, g = lk.dfun_x(x, True)
    assert abs(f - pb.neg_lnL(x, True)) <= 1e-9 * abs(f)
    ref = np.zeros(len(x))
    for i in range(len(x)):
        e = 1e-4 * (abs(x[i]) + 0.05)
        fs = []
        for k in (-2, -1, 1, 2):
            xk = x.copy()
            xk[i] += k * e
            fs.append(pb.neg_lnL(xk, True))
        ref[i] = (fs[0] - 8 * fs[1] + 8 * fs[2] - fs[3]) / (12 * e)
    err = np.abs(g - ref) / np.maximum(1.0, np.abs(ref))
    assert err.max() <= 1e-5, (int(np.argmax(err)), err.max())
    lk.close()


def test_unclean_needs_fp64_and_valid_codes():
    fx, tree, z, fpatt, pi, amb = load_unclean(unclean_names()[0])
    with pytest.raises(_lib.GBError) as e:
        api.Likelihood(tree, z, fpatt, pi)                      # no tables: clean data only
    assert e.value.code == -1
    with pytest.raises(_lib.GBError) as e:
        api.Likelihood(tree, z, fpatt, pi, precision="fast", ambiguity=amb)
    assert e.value.code == -1
    nch, cmap = amb[0].copy(), amb[1]
    nch[int(z.max())] = 0                                       # a code standing for no sense codon
    with pytest.raises(_lib.GBError) as e:
        api.Likelihood(tree, z, fpatt, pi, ambiguity=(nch, cmap))
    assert e.value.code == -1
