"""Branch-site model B (codeml NSsites = 3, ncatG = 3): the oracle against
the reference codeml's own fixed-parameter output (tests/golden/mb*.json).

Model B frees w1, which model A fixes at 1 (SetParametersNSsites
codeml.c:2427-2436); the site classes, their omega map (Set_UVR_BranchSite
codeml.c:2545-2568) and the pruning are model A's.  Bars as for model A:
patterns bit-exact, lnL within print rounding and 1e-9 relative, log f per
pattern within 5e-11 + 2e-11 |log f|.
"""
import numpy as np
import pytest

from cucodeml_gb300 import codon
from oracle import oracle as O
from tests.conftest import load_golden, model_b_names


@pytest.mark.parametrize("name", model_b_names())
def test_model_b_matches_codeml(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    got = [" ".join(codon.codon_string(int(c)) for c in z[:, h]) for h in range(z.shape[1])]
    assert got == fx["patterns"]
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2, model_b=True)
    x = np.array(fx["x"])
    assert len(x) == pb.np == fx["codeml_np"]
    v, fhK, lnf, nscale = pb.neg_lnL(x, lastround=True, want_fhK=True)
    assert abs(-v - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(v)
    assert abs(-v - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))


def test_model_b_with_w1_one_is_model_a():
    fx, tree, codons = load_golden("mb8x300_s7")
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    xb = x.copy()
    xb[nb + 4] = 1.0                                  # w1 = 1
    xa = np.delete(xb, nb + 4)
    a = O.Problem(tree, z, fpatt, pi, nthreads=2).neg_lnL(xa)
    b = O.Problem(tree, z, fpatt, pi, nthreads=2, model_b=True).neg_lnL(xb)
    assert a == b
