"""FP64 drop-in parity on the GPU, through the C ABI, against the oracle and
the reference codeml's golden outputs.

Bars: lnL within 1e-9 relative of codeml (the drop-in's contract) and of the
oracle; with identical U, V, Root the GPU and the oracle differ only by
summation order, so per-pattern log f must agree to 1e-11 absolute.
"""
import numpy as np
import pytest

from cucodeml_gb300 import api
from cucodeml_gb300.simulate import simulate
from oracle import oracle as O
from tests.conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu


def node_blength(tree, x):
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = np.asarray(x)[: tree.nbranch]
    return bl


@pytest.fixture(scope="module")
def cases():
    out = {}
    for name in golden_names():
        fx, tree, codons = load_golden(name)
        z, fpatt, pi = O.patterns(codons)
        out[name] = (fx, tree, z, fpatt, pi)
    return out


@pytest.mark.parametrize("name", golden_names())
def test_eval_uvr_matches_oracle(cases, name):
    fx, tree, z, fpatt, pi = cases[name]
    x = np.array(fx["x"])
    pb = O.Problem(tree, z, fpatt, pi)
    U, V, R, qf, fk = pb.set_params(x)
    v, fhK, lnf, nsc = pb.neg_lnL(x, True, True)
    lk = api.Likelihood(tree, z, fpatt, pi)
    r = lk.neg_lnL_uvr(U, V, R, qf, fk, node_blength(tree, x))
    assert lk.nscale == nsc
    assert abs(r.neg_lnL - v) <= 1e-12 * abs(v)
    assert np.max(np.abs(r.lnf - lnf)) <= 1e-11
    if nsc:
        assert np.max(np.abs(r.fhK - fhK)) <= 1e-10
    else:
        assert np.max(np.abs(r.fhK - fhK) / np.abs(fhK)) <= 1e-11
    lk.close()


@pytest.mark.parametrize("name", golden_names())
def test_eval_matches_codeml(cases, name):
    fx, tree, z, fpatt, pi = cases[name]
    x = np.array(fx["x"])
    nb = tree.nbranch
    lk = api.Likelihood(tree, z, fpatt, pi)
    r = lk.evaluate(node_blength(tree, x), x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2],
                    want_site=True)
    assert abs(-r.neg_lnL - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    assert abs(-r.neg_lnL - fx["codeml_lnL"]) <= 5.1e-7 + 1e-12 * abs(r.neg_lnL)
    # per pattern: print rounding (5e-11) plus the conditioning of P(t) = U e^{Lt} V
    # under a different eigensolver (small multi-change entries carry ~1e-16 absolute noise)
    ref = np.array(fx["lnf"])
    assert np.all(np.abs(r.lnf - ref) <= 5.1e-11 + 2e-11 * np.abs(ref))
    lk.close()


def test_repeat_is_deterministic(cases):
    fx, tree, z, fpatt, pi = cases["c24x400_s3"]
    x = np.array(fx["x"])
    nb = tree.nbranch
    lk = api.Likelihood(tree, z, fpatt, pi)
    args = (node_blength(tree, x), x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2])
    a = [lk.evaluate(*args).neg_lnL for _ in range(3)]
    assert a[0] == a[1] == a[2]
    lk.close()


def test_scaling_everywhere_is_invariant(cases):
    """Scaling every internal node must not change lnL (exact power of the
    scale factors is carried in fhK)."""
    fx, tree, z, fpatt, pi = cases["c8x300_s1"]
    x = np.array(fx["x"])
    nb = tree.nbranch
    args = (node_blength(tree, x), x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2])
    a = api.Likelihood(tree, z, fpatt, pi).evaluate(*args).neg_lnL
    sc = np.zeros(tree.nnode, dtype=np.int8)
    sc[tree.ns:] = 1
    sc[tree.root] = 0
    lk = api.Likelihood(tree, z, fpatt, pi, node_scale=sc)
    assert lk.nscale == tree.nnode - tree.ns - 1
    b = lk.evaluate(*args).neg_lnL
    assert abs(a - b) <= 1e-11 * abs(a)


def test_64x5000_matches_oracle():
    aln = simulate(64, 5000, seed=11)
    z, fpatt, pi = O.patterns(aln.codons)
    tree = aln.tree
    x = np.concatenate([tree.x_branch_lengths(), [2.0, 0.5, 0.3, 0.3, 3.0]])
    pb = O.Problem(tree, z, fpatt, pi)
    v = pb.neg_lnL(x)
    lk = api.Likelihood(tree, z, fpatt, pi)
    nb = tree.nbranch
    r = lk.evaluate(node_blength(tree, x), 2.0, 0.3, 3.0, 0.5, 0.3)
    assert lk.nscale > 0
    assert abs(r.neg_lnL - v) <= 1e-9 * abs(v)


@pytest.mark.parametrize("name", golden_names())
def test_neb_matches_oracle_and_codeml(cases, name):
    """gb_neb: the mixture's class posteriors of one FP64 evaluation against
    the oracle (1e-9: per-class log f may differ by 2e-11 |log f| between the
    two eigensolvers, as the per-pattern bar above allows) and
    codeml's printed NEB posteriors (5 decimals)."""
    from tests.test_beb_oracle import site_patterns
    fx, tree, z, fpatt, pi = cases[name]
    x = np.array(fx["x"])
    ref = O.Problem(tree, z, fpatt, pi).neb(x)
    lk = api.Likelihood(tree, z, fpatt, pi)
    post, f = lk.neb_x(x)
    assert np.max(np.abs(post - ref)) <= 1e-9
    _, _, codons = load_golden(name)
    site = post[:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(fx["neb_site_post_5dp"]))) <= 5.01e-6
    assert abs(-f - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    lk.close()
