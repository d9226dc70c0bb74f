"""Host-side checks of gb_create_unclean (no GPU needed): the library
rejects ambiguity codes that stand for nothing or for a non-sense codon, and
codon ids >= 61 without the tables, before it touches a device."""
import numpy as np
import pytest

from cucodeml_gb300 import _lib, api
from tests.conftest import load_unclean, unclean_names


def test_unclean_validation_on_host():
    fx, tree, z, fpatt, pi, amb = load_unclean(unclean_names()[0])
    with pytest.raises(_lib.GBError) as e:
        api.Likelihood(tree, z, fpatt, pi)
    assert e.value.code == -1 and "gb_create_unclean" in str(e.value)
    nch, cmap = amb[0].copy(), amb[1].copy()
    c = int(z.max())
    cmap[c, 0] = 61
    with pytest.raises(_lib.GBError) as e:
        api.Likelihood(tree, z, fpatt, pi, ambiguity=(nch, cmap))
    assert e.value.code == -1
    with pytest.raises(_lib.GBError) as e:
        api.Likelihood(tree, z, fpatt, pi, precision="fast", ambiguity=amb)
    assert e.value.code == -1
