"""Clade model C (codeml model = 3, NSsites = 2, two branch types): the
oracle's restatement as two model-A class evaluations against the reference
codeml's fixed-parameter runs (tests/golden/mcC*.json).

Clade C's third class carries w2 on background and w3 on foreground
branches; that is model A's class 2a with eigen slots (w2, -, w3), while its
classes 0 and 1 are model A's with slots (w0, 1, -).  Bars as for model A.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import clade_names, load_golden


@pytest.mark.parametrize("name", clade_names())
def test_clade_c_matches_codeml(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2)
    x = np.array(fx["x"])
    assert len(x) == fx["codeml_np"] == tree.nbranch + 6
    v, fhK, lnf = pb.clade_c(x)
    assert abs(-v - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(v)
    assert abs(-v - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))
