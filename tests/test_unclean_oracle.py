"""The oracle on alignments with gaps and ambiguous codons (codeml's
cleandata = 0), pinned to the reference codeml's output.

The u* fixtures (tests/golden/make_unclean_golden.py) keep the data exactly
as codeml encoded it (ambiguity ids from 61 up, nChara / CharaMap, pi to
full precision) and codeml's lnL and per-pattern log f at fixed x.  The
oracle's restatement of the unclean tip (ConditionalPNode codeml.c:3438-3445)
must reproduce them to print precision."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import load_unclean, unclean_names


@pytest.mark.parametrize("name", unclean_names())
def test_oracle_matches_codeml_on_unclean_data(name):
    fx, tree, z, fpatt, pi, amb = load_unclean(name)
    assert z.max() >= 61
    pb = O.Problem(tree, z, fpatt, pi, ambiguity=amb)
    v, fhK, lnf, nsc = pb.neg_lnL(np.array(fx["x"]), True, True)
    assert abs(-v - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(v)
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))


def test_unclean_codes_cover_their_resolutions():
    """Every ambiguity id stands for 1..61 sense codons; an id's sum of tip
    probabilities is the sum over those codons (all codons for a gap)."""
    for name in unclean_names():
        fx, tree, z, fpatt, pi, amb = load_unclean(name)
        nch, cmap = amb
        used = np.unique(z[z >= 61])
        assert np.all((nch[used] >= 1) & (nch[used] <= 61))
        for c in used:
            assert len(set(cmap[c, :nch[c]])) == nch[c] and cmap[c, :nch[c]].max() < 61
        assert 61 in nch[used]            # a gap or NNN: every sense codon
