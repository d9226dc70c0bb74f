"""Standard errors on the GPU (gb_se_opg, gb_hessian_x) through the C ABI.

gb_se_opg is codeml's getSE = 1 estimator (HessianSKT2004): against the
oracle's restatement, H within 1e-7 of its largest entry, g within
1e-4 (1 + |g|), SEs within 5e-5 relative -- the two eigensolvers move the
2e-6-step differences of log f by up to 5e-9 of max |H| and 5e-6 of an SE at
a Hessian condition number of 3.5e12 (measured on the CPU with the library's
eigen solutions); against codeml's printed SEs, print rounding plus 1e-4 of
the value.  gb_hessian_x (differences of the analytic gradient) against the
oracle's second differences of lnL, Richardson-extrapolated from steps
1e-4 (|x| + 1) and twice that, within 1e-4 of the largest entry.  (Plain
second differences at 1e-4 are off by 8e-4 of the largest entry, the
diagonal of a 0.003-long branch; the extrapolation and plain differences at
1e-5 agree to 1.2e-5.)
"""
import numpy as np
import pytest

from cucodeml_gb300 import api
from oracle import oracle as O
from tests.conftest import golden_names, load_golden, model_b_names

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_names() + model_b_names())
def test_se_opg_matches_oracle_and_codeml(name):
    """Models A and B (gb_se_opg takes model B's x, n = nbranch + 6)."""
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    go, Ho, seo = O.Problem(tree, z, fpatt, pi, nthreads=4,
                            model_b=name.startswith("mb")).opg_se(x, small_diff=fx["small_diff"])
    lk = api.Likelihood(tree, z, fpatt, pi)
    r = lk.se_opg(x, small_diff=fx["small_diff"])
    assert np.array_equal(r["H"], r["H"].T)
    assert np.max(np.abs(r["H"] - Ho)) <= 1e-7 * np.max(np.abs(Ho))
    assert np.all(np.abs(r["g"] - go) <= 1e-4 * (1 + np.abs(go)))
    assert np.all(np.abs(r["se"] - seo) <= 5e-5 * np.abs(seo))
    ref = np.array(fx["se_6dp"])
    assert np.all(np.abs(r["se"] - ref) <= 5.01e-7 + 1e-4 * np.abs(ref))
    lk.close()


def second_differences(pb, x, rel):
    n = len(x)
    h = rel * (np.abs(x) + 1)
    f = lambda v: pb.neg_lnL(v, True)
    f0 = f(x)
    H = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            def at(si, sj):
                v = x.copy()
                v[i] += si * h[i]
                v[j] += sj * h[j]
                return f(v)
            if i == j:
                H[i, i] = (at(1, 1) + at(-1, -1) - 2 * f0) / (4 * h[i] * h[i])
            else:
                H[i, j] = H[j, i] = (at(1, 1) + at(-1, -1) - at(1, -1) - at(-1, 1)) / (4 * h[i] * h[j])
    return H


def oracle_hessian(pb, x, rel=1e-4):
    return (4 * second_differences(pb, x, rel) - second_differences(pb, x, 2 * rel)) / 3


def test_hessian_from_adjoint_matches_second_differences():
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    Ho = oracle_hessian(O.Problem(tree, z, fpatt, pi, nthreads=4), x)
    lk = api.Likelihood(tree, z, fpatt, pi)
    H, se = lk.hessian_x(x, lastround=True)
    assert np.array_equal(H, H.T)
    assert np.max(np.abs(H - Ho)) <= 1e-4 * np.max(np.abs(Ho))
    C = np.linalg.inv(H)
    d = np.diag(C)
    assert np.allclose(se, np.where(d > 0, np.sqrt(np.abs(d)), -1.0), rtol=1e-8)
    lk.close()
