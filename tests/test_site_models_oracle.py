"""Site models M2a and M1a (codeml model = 0, NSsites = 2 / 1) as branch-site
model A with every branch in the foreground.

Under M2a codeml mixes three classes, w0 < 1, w1 = 1 and w2, each on the whole
tree, with Qfactor_NS = 1 / meanrate(Q(kappa, p0 w0 + p1 + p2 w2))
(SetParametersNSsites codeml.c:2466-2487).  Model A with every branch
labelled #1 has the same mixture: classes 0 and 1 are w0 and 1 everywhere,
classes 2a and 2b are both w2 everywhere with weights summing to p2, and the
foreground Qfactor is the same mean-rate normalisation.  M1a is M2a with
p2 = 0.  So the model-A machinery (oracle, FP64 drop-in, adjoint, split
precision) evaluates them unchanged.  Pinned here: the oracle under that
mapping against the reference codeml's own fixed-parameter runs of M2a and
M1a (tests/golden/ms*.json).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import as_model_a, load_golden, site_model_names


@pytest.mark.parametrize("name", site_model_names())
def test_site_model_as_model_a_matches_codeml(name):
    fx, tree, codons = load_golden(name)
    assert np.all(tree.label == 0)
    z, fpatt, pi = O.patterns(codons)
    t, x = as_model_a(fx, tree)
    pb = O.Problem(t, z, fpatt, pi, nthreads=2)
    v, fhK, lnf, nscale = pb.neg_lnL(x, lastround=True, want_fhK=True)
    assert abs(-v - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(v)
    assert abs(-v - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))
