"""Pin the oracle's standard errors (codeml's getSE = 1 estimator,
HessianSKT2004 treesub.c:6979-7048) against codeml's own "SEs for
parameters" (golden fixtures, 6 decimals).

The estimator differentiates log f_h numerically with steps of 2e-6, so its
SEs inherit the conditioning of the approximate Hessian: where that is
near-singular (an SE of w2 in the hundreds, condition numbers up to 1e12) two
correct implementations differ by up to ~2e-5 relative.  The bar is print
rounding plus 5e-5 of the value.
"""
import numpy as np

from oracle import oracle as O


def test_opg_se_matches_codeml(golden):
    fx, tree, codons = golden
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4)
    g, H, se = pb.opg_se(np.array(fx["x"]), small_diff=fx["small_diff"])
    ref = np.array(fx["se_6dp"])
    assert se.shape == ref.shape
    assert np.all(np.abs(se - ref) <= 5.01e-7 + 5e-5 * np.abs(ref))
    assert np.array_equal(H, H.T)
    assert np.all(np.linalg.eigvalsh(-H) > -1e-8 * np.max(np.abs(H)))   # -H is a Gram matrix


import pytest

from tests.conftest import load_golden, model_b_names


@pytest.mark.parametrize("name", model_b_names())
def test_opg_se_matches_codeml_model_b(name):
    """The same estimator under branch-site model B (x ends w0, w1, w2)."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=4, model_b=True)
    g, H, se = pb.opg_se(np.array(fx["x"]), small_diff=fx["small_diff"])
    ref = np.array(fx["se_6dp"])
    assert se.shape == ref.shape
    assert np.all(np.abs(se - ref) <= 5.01e-7 + 5e-5 * np.abs(ref))
