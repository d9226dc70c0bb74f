"""The checkpointed FP64 adjoint (gb_tune GB_TUNE_CHECKPOINT = 1): the
conditional likelihoods stay at every internal node, the edge messages of
one tree level at a time are recomputed during the reverse sweep.  It must
give the non-checkpointed lnL and gradient bit for bit (same arithmetic in
the same order) in less device memory."""
import numpy as np
import pytest

from cucodeml_gb300 import _lib, api
from cucodeml_gb300.simulate import simulate
from oracle import oracle as O
from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def grad_vec(r):
    g = r.grad
    return np.concatenate([g["blength"], [g["kappa"], g["omega0"], g["omega2"], g["p0"], g["p1"]]])


def run(tree, z, fpatt, pi, args, checkpoint):
    import torch
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64", tuning={"checkpoint": checkpoint})
    r = lk.evaluate(*args, grad=True)
    r2 = lk.evaluate(*args, grad=True)
    torch.cuda.synchronize()
    used = free0 - torch.cuda.mem_get_info()[0]
    lk.close()
    return r, r2, used


@pytest.mark.parametrize("case", ["c24x400_s3", "c40x200_s4", "64x5000"])
def test_checkpointed_adjoint_is_bit_identical(case):
    if case == "64x5000":
        aln = simulate(64, 5000, seed=2024)
        z, fpatt, pi = api.patterns(aln.codons)
        tree = aln.tree
        args = (tree.branch, 2.0, 0.3, 3.0, 0.5, 0.3)
    else:
        fx, tree, codons = load_golden(case)
        z, fpatt, pi = O.patterns(codons)
        x = np.array(fx["x"])
        nb = tree.nbranch
        bl = np.zeros(tree.nnode)
        bl[tree.branch_nodes()] = x[:nb]
        args = (bl, x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2])
    a, a2, mem_a = run(tree, z, fpatt, pi, args, 0)
    b, b2, mem_b = run(tree, z, fpatt, pi, args, 1)
    print(f"{case}: device memory {mem_a / 2**20:.1f} MiB -> {mem_b / 2**20:.1f} MiB with checkpointing "
          f"({mem_b / max(mem_a, 1):.2f}); ms {a2.ms_device:.2f} -> {b2.ms_device:.2f}")
    assert a.neg_lnL == b.neg_lnL and a2.neg_lnL == b2.neg_lnL
    assert np.array_equal(grad_vec(a), grad_vec(b)) and np.array_equal(grad_vec(a2), grad_vec(b2))
    if case == "64x5000":
        assert mem_b < 0.7 * mem_a


def test_checkpoint_knob_needs_fp64_and_a_fresh_handle():
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    with pytest.raises(_lib.GBError):
        api.Likelihood(tree, z, fpatt, pi, precision="fast", tuning={"checkpoint": 1})
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64")
    x = np.array(fx["x"])
    lk.dfun_x(x, True)
    assert lk._L.gb_tune(lk._h, 6, 1) == -6
    lk.close()
