import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def golden_names():
    """Fixed-parameter model-A fixtures (codeml lnL and per-pattern log f at given x)."""
    return sorted(f[:-5] for f in os.listdir(GOLDEN)
                  if f.endswith(".json") and not f.startswith(("mle_", "mb", "ms", "mc", "u")))


def unclean_names():
    """Fixed-parameter model-A fixtures with gaps and ambiguous codons (cleandata = 0)."""
    return sorted(f[:-5] for f in os.listdir(GOLDEN) if f.startswith("u") and f.endswith(".json"))


def load_unclean(name):
    """(fixture, tree, z, fpatt, pi, (nchara[256], charamap[256, 64])) with the
    data as codeml encoded it."""
    from cucodeml_gb300.tree import parse_newick

    with open(os.path.join(GOLDEN, name + ".json")) as f:
        fx = json.load(f)
    tree = parse_newick(fx["newick"], fx["names"])
    enc = fx["enc"]
    z = np.array(enc["z"], dtype=np.uint8)
    nch = np.zeros(256, dtype=np.uint8)
    cmap = np.zeros((256, 64), dtype=np.uint8)
    for c, (n, row) in enumerate(zip(enc["nchara"], enc["charamap"])):
        nch[c] = n
        cmap[c, :n] = row
    return (fx, tree, z, np.array(enc["fpatt"], dtype=np.float64), np.array(enc["pi"], dtype=np.float64),
            (nch, cmap))


def site_model_names():
    """Fixed-parameter fixtures under the site models M2a / M1a (no branch labels)."""
    return sorted(f[:-5] for f in os.listdir(GOLDEN) if f.startswith("ms") and f.endswith(".json"))


def as_model_a(fx, tree):
    """A site-model fixture as the branch-site model A evaluation that equals
    it: every branch labelled foreground, so site classes 2a and 2b both carry
    w2 on every branch and together weigh 1 - p0 - p1 (M2a); M1a is that with
    p1 = 1 - p0 (no w2 class; w2 then carries no weight and is set to 1).
    M3 with three classes (free w0, w1, w2) is model B on that tree, with x
    unchanged (model B's layout); M7 / M8 have no model-A form (x returned
    as is; see site_model_classes).  Returns (tree with labels, x)."""
    import copy

    t = copy.deepcopy(tree)
    t.label[:] = 1
    t.label[t.root] = 0
    x = np.array(fx["x"], dtype=np.float64)
    nb = tree.nbranch
    if fx["model"] == "M1a":
        kappa, p0, w0 = x[nb:nb + 3]
        x = np.concatenate([x[:nb], [kappa, p0, 1.0 - p0, w0, 1.0]])
    return t, x


def clade_names():
    """Fixed-parameter fixtures under clade model C (two branch types)."""
    return sorted(f[:-5] for f in os.listdir(GOLDEN) if f.startswith("mcC") and f.endswith(".json"))


def clade_d_names():
    """Fixed-parameter fixtures under clade model D (two branch types, w1 free)."""
    return sorted(f[:-5] for f in os.listdir(GOLDEN) if f.startswith("mcD") and f.endswith(".json"))


def site_model_classes(fx, tree):
    """(omegas, proportions) of a site-model fixture's classes at its x:
    M2a / M1a / M3 directly, M7 / M8 by the discretised beta (ten categories
    at their medians, DiscreteNSsites codeml.c:2728-2770)."""
    from oracle import oracle as O

    x = np.array(fx["x"], dtype=np.float64)
    nb = tree.nbranch
    m = fx["model"]
    if m == "M7":
        return O.beta_classes(x[nb + 1], x[nb + 2])
    if m == "M8":
        p0, p, q, ws = x[nb + 1:nb + 5]
        om, pr = O.beta_classes(p, q)
        return np.append(om, ws), np.append(pr * p0, 1 - p0)
    if m == "M1a":
        p0, w0 = x[nb + 1:nb + 3]
        return np.array([w0, 1.0]), np.array([p0, 1 - p0])
    if m == "M2a":
        p0, p1, w0, w2 = x[nb + 1:nb + 5]
        return np.array([w0, 1.0, w2]), np.array([p0, p1, 1 - p0 - p1])
    p0, p1, w0, w1, w2 = x[nb + 1:nb + 6]          # M3, three classes
    return np.array([w0, w1, w2]), np.array([p0, p1, 1 - p0 - p1])


def model_b_names():
    """Fixed-parameter fixtures under branch-site model B (w1 free)."""
    return sorted(f[:-5] for f in os.listdir(GOLDEN) if f.startswith("mb") and f.endswith(".json"))


def mle_names():
    """Maximum-likelihood fixtures (codeml's optimised alternative and null)."""
    return sorted(f[:-5] for f in os.listdir(GOLDEN) if f.startswith("mle_") and f.endswith(".json"))


def load_golden(name):
    """Fixture dict plus parsed tree and codon matrix [ns, ncodon]."""
    from cucodeml_gb300 import codon
    from cucodeml_gb300.tree import parse_newick

    with open(os.path.join(GOLDEN, name + ".json")) as f:
        fx = json.load(f)
    tree = parse_newick(fx["newick"], fx["names"])
    lut = {codon.codon_string(i): i for i in range(61)}
    codons = np.array([[lut[c] for c in row.split()] for row in fx["codons"]], dtype=np.int64)
    return fx, tree, codons


@pytest.fixture(params=golden_names())
def golden(request):
    return load_golden(request.param)
