"""Pairwise Nei-Gojobori (1986) distances (gb_ng86, host code of the library)
against the table the reference codeml prints before its fit
(DistanceMatNG86 treesub.c:2270-2366; golden fixtures, 4 decimals)."""
import numpy as np
import pytest

from cucodeml_gb300 import api
from oracle import oracle as O
from tests.conftest import golden_names, load_golden, model_b_names


@pytest.mark.parametrize("name", golden_names() + model_b_names())
def test_ng86_matches_codeml(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    r = api.ng86(z, fpatt)
    ns = tree.ns
    iu = [(i, j) for i in range(ns) for j in range(i)]
    ref = fx["ng86_4dp"]
    for key in ("dS", "dN", "dN_dS"):
        got = np.array([r[key][i, j] for i, j in iu])
        assert np.max(np.abs(got - np.array(ref[key]))) <= 5.01e-5, key
    assert np.array_equal(r["dS"], r["dS"].T) and np.all(np.diag(r["dist"]) == 0)


def test_ng86_identical_sequences_are_zero():
    fx, tree, codons = load_golden("c8x300_s1")
    c = codons.copy()
    c[1] = c[0]
    z, fpatt, pi = O.patterns(c)
    r = api.ng86(z, fpatt)
    assert r["dS"][1, 0] == 0 and r["dN"][1, 0] == 0 and r["dist"][1, 0] == 0
