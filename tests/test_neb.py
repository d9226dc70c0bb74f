"""Naive empirical Bayes (NEB) site-class posteriors: the oracle against the
per-site posteriors the reference codeml prints to rst (lfunNSsites_rate
codeml.c:5079-5129; golden fixtures, 5 decimals), for models A and B."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import golden_names, load_golden, model_b_names
from tests.test_beb_oracle import site_patterns


@pytest.mark.parametrize("name", golden_names() + model_b_names())
def test_oracle_neb_matches_codeml(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi, nthreads=2, model_b=fx.get("model") == "B")
    post = pb.neb(np.array(fx["x"]))
    site = post[:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(fx["neb_site_post_5dp"]))) <= 5.01e-6
    assert np.allclose(post.sum(axis=0), 1.0, atol=1e-13)
