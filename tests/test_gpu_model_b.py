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
