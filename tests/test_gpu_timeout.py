"""The bounded-wait error path of the persistent split-precision kernels.

gb_fault_inject makes every cross-CTA flag wait expect a value that no task
writes (a flag that nothing sets) with a 200 ms limit: the evaluation must
come back with GB_ERR_TIMEOUT in bounded time, with every CTA having freed
its tensor memory (a later evaluation and a new handle allocate it again),
and the same handle must give the same results as before once the hook is
off.  Nothing here faults, traps or hangs the GPU: the waits give up by
themselves and the kernels return."""
import time

import numpy as np
import pytest

from cucodeml_gb300 import _lib, api
from oracle import oracle as O
from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def grad_vec(r):
    g = r.grad
    return np.concatenate([g["blength"], [g["kappa"], g["omega0"], g["omega2"], g["p0"], g["p1"]]])


def test_withheld_flag_times_out_and_handle_recovers():
    fx, tree, codons = load_golden("c24x400_s3")
    z, fpatt, pi = O.patterns(codons)
    x = np.array(fx["x"])
    nb = tree.nbranch
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[:nb]
    args = (bl, x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2])
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fast")
    L = lk._L
    r0 = lk.evaluate(*args, grad=True)
    _lib.check(L.gb_fault_inject(lk._h, 200, 1))
    for _ in range(2):
        t0 = time.time()
        with pytest.raises(_lib.GBError) as e:
            lk.evaluate(*args, grad=True)
        dt = time.time() - t0
        assert e.value.code == -5, e.value
        assert dt < 30, dt
        print(f"withheld flags: GB_ERR_TIMEOUT after {dt:.2f} s")
    _lib.check(L.gb_fault_inject(lk._h, 0, 0))
    r1 = lk.evaluate(*args, grad=True)
    assert r1.neg_lnL == r0.neg_lnL
    assert np.array_equal(grad_vec(r1), grad_vec(r0))
    lk2 = api.Likelihood(tree, z, fpatt, pi, precision="fast")
    r2 = lk2.evaluate(*args, grad=True)
    assert r2.neg_lnL == r0.neg_lnL
    lk2.close()
    lk.close()


def test_fault_inject_needs_persistent_kernels():
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64")
    assert lk._L.gb_fault_inject(lk._h, 200, 1) == -6
    lk.close()
