"""Pin the C oracle against the reference codeml's own outputs (golden fixtures).

The fixtures were produced by running the reference codeml (CPU build) at
fixed parameters; see tests/golden/make_golden.py.  They pin:
* pattern compression order and counts (bit-exact; lnf lists each pattern's
  codons and count in codeml's order);
* F3x4 codon frequencies (printed to 8 decimals);
* per-pattern log f (10 decimals) and lnL (6 decimals).
"""
import numpy as np

from cucodeml_gb300 import codon
from oracle import oracle as O


def test_patterns_bit_exact(golden):
    fx, tree, codons = golden
    z, fpatt, pi = O.patterns(codons)
    assert z.shape[1] == len(fx["patterns"])
    got = [" ".join(codon.codon_string(int(c)) for c in z[:, h]) for h in range(z.shape[1])]
    assert got == fx["patterns"]
    assert np.array_equal(fpatt, np.array(fx["fpatt"]))
    assert np.max(np.abs(pi - np.array(fx["pi_8dp"]))) <= 5.1e-9


def test_lnL_matches_codeml(golden):
    fx, tree, codons = golden
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2)
    x = np.array(fx["x"])
    v, fhK, lnf, nscale = pb.neg_lnL(x, lastround=True, want_fhK=True)
    assert abs(-v - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(v)
    assert abs(-v - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    assert np.max(np.abs(lnf - np.array(fx["lnf"]))) <= 5.1e-11 + 1e-12 * np.max(np.abs(lnf))
    if fx["ns"] > 16:
        assert nscale > 0          # node scaling is exercised


def test_lnL_thread_invariant(golden):
    fx, tree, codons = golden
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    a = O.Problem(tree, z, fpatt, pi, nthreads=1).neg_lnL(x)
    b = O.Problem(tree, z, fpatt, pi, nthreads=3).neg_lnL(x)
    assert a == b


def test_transformed_p_matches_untransformed():
    from tests.conftest import load_golden
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi)
    x = np.array(fx["x"])
    nb = tree.nbranch
    p0, p1 = x[nb + 1], x[nb + 2]
    xt = x.copy()
    xt[nb + 1] = np.log(p0 / (1 - p0 - p1))
    xt[nb + 2] = np.log(p1 / (1 - p0 - p1))
    assert abs(pb.neg_lnL(x, True) - pb.neg_lnL(xt, False)) < 1e-9
