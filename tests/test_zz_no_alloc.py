"""gb_lnL_noalloc: the lnL entry point for callers that cannot allocate GPU
memory (their device memory belongs to another allocator, or they cannot
afford the device-wide synchronisation of cudaMalloc/cudaFree).  It must give
the same lnL and per-class fhK as the regular entry point gb_eval_uvr on the
same inputs, on two calls in a row (the second call reuses the static scratch
array the first one left behind).

This file is collected last so that a run stopping at the first failure has
already run every other test.  The test allocates its own device buffers
with torch: the caller owns inputs and outputs, the library allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

from cucodeml_gb300 import _lib, api
from oracle import oracle as O
from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def test_noalloc_matches_gb_eval_uvr_on_two_calls():
    import torch
    fx, tree, codons = load_golden("c24x400_s3")      # 24 taxa: node scaling is exercised
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi)
    x = np.array(fx["x"])
    U, V, R, qf, fk = pb.set_params(x)
    lk = api.Likelihood(tree, z, fpatt, pi)
    assert lk.nscale > 0
    L = _lib.load()
    dev = torch.device("cuda", 0)
    d_z = torch.from_numpy(np.ascontiguousarray(z)).to(dev)
    d_fp = torch.from_numpy(fpatt).to(dev)
    d_pi = torch.from_numpy(pi).to(dev)
    model = np.concatenate([U.ravel(), V.ravel(), R.ravel(), qf, fk])
    assert model.size == 6 * 61 * 61 + 3 * 61 + 2 + 4
    d_model = torch.from_numpy(model).to(dev)
    d_out = torch.zeros(1, dtype=torch.float64, device=dev)
    d_fhK = torch.zeros(4 * len(fpatt), dtype=torch.float64, device=dev)
    father = np.ascontiguousarray(tree.father, dtype=np.int32)
    label = np.ascontiguousarray(tree.label, dtype=np.int32)
    ip = C.POINTER(C.c_int)
    bl0 = np.zeros(tree.nnode)
    bl0[tree.branch_nodes()] = x[: tree.nbranch]
    torch.cuda.synchronize()
    for call, scale in enumerate((1.0, 1.3)):
        bl = bl0 * scale
        ref = lk.neg_lnL_uvr(U, V, R, qf, fk, bl)
        d_bl = torch.from_numpy(bl).to(dev)
        torch.cuda.synchronize()
        rc = L.gb_lnL_noalloc(tree.ns, tree.nnode, tree.root, father.ctypes.data_as(ip),
                              label.ctypes.data_as(ip), None, len(fpatt), d_z.data_ptr(),
                              d_fp.data_ptr(), d_pi.data_ptr(), d_model.data_ptr(), d_bl.data_ptr(),
                              d_out.data_ptr(), d_fhK.data_ptr(), None)
        _lib.check(rc)
        got = float(d_out.cpu()[0])
        fhK = d_fhK.cpu().numpy().reshape(4, -1)
        assert abs(got - ref.neg_lnL) <= 1e-12 * abs(ref.neg_lnL), (call, got, ref.neg_lnL)
        assert np.max(np.abs(fhK - ref.fhK)) <= 1e-10, call
    lk.close()


def test_noalloc_rejects_too_large_problem():
    import torch
    from cucodeml_gb300.simulate import simulate
    aln = simulate(64, 3000, seed=5)
    z, fpatt, pi = O.patterns(aln.codons)
    tree = aln.tree
    L = _lib.load()
    dev = torch.device("cuda", 0)
    bufs = [torch.zeros(max(n, 1), dtype=torch.float64, device=dev)
            for n in (z.size, len(fpatt), 61, 6 * 61 * 61 + 3 * 61 + 6, tree.nnode, 1)]
    father = np.ascontiguousarray(tree.father, dtype=np.int32)
    label = np.ascontiguousarray(tree.label, dtype=np.int32)
    ip = C.POINTER(C.c_int)
    rc = L.gb_lnL_noalloc(tree.ns, tree.nnode, tree.root, father.ctypes.data_as(ip),
                          label.ctypes.data_as(ip), None, len(fpatt), *[b.data_ptr() for b in bufs],
                          None, None)
    assert rc == -1
    assert "GB_NOALLOC_SCRATCH_BYTES" in L.gb_last_error().decode()


def test_noalloc_rejects_bad_codon_ids_before_pruning():
    """A codon id of 61 (an ambiguity code, or any stray byte) would index
    past a 61-row transition matrix: the entry point must catch it on the
    device before any pruning kernel reads it, return GB_ERR_ARG, leave the
    caller's output alone, and serve the next good call normally."""
    import torch
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi)
    x = np.array(fx["x"])
    U, V, R, qf, fk = pb.set_params(x)
    L = _lib.load()
    dev = torch.device("cuda", 0)
    model = torch.from_numpy(np.concatenate([U.ravel(), V.ravel(), R.ravel(), qf, fk])).to(dev)
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = x[: tree.nbranch]
    d_bl = torch.from_numpy(bl).to(dev)
    d_fp = torch.from_numpy(fpatt).to(dev)
    d_pi = torch.from_numpy(pi).to(dev)
    father = np.ascontiguousarray(tree.father, dtype=np.int32)
    label = np.ascontiguousarray(tree.label, dtype=np.int32)
    ip = C.POINTER(C.c_int)
    for bad_id in (61, 255):
        zb = np.ascontiguousarray(z).copy()
        zb[tree.ns // 2, len(fpatt) // 3] = bad_id
        d_z = torch.from_numpy(zb).to(dev)
        d_out = torch.full((1,), 12345.0, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = L.gb_lnL_noalloc(tree.ns, tree.nnode, tree.root, father.ctypes.data_as(ip),
                              label.ctypes.data_as(ip), None, len(fpatt), d_z.data_ptr(),
                              d_fp.data_ptr(), d_pi.data_ptr(), model.data_ptr(), d_bl.data_ptr(),
                              d_out.data_ptr(), None, None)
        assert rc == -1, rc
        assert "0..60" in L.gb_last_error().decode()
        assert float(d_out.cpu()[0]) == 12345.0
    d_z = torch.from_numpy(np.ascontiguousarray(z)).to(dev)
    rc = L.gb_lnL_noalloc(tree.ns, tree.nnode, tree.root, father.ctypes.data_as(ip),
                          label.ctypes.data_as(ip), None, len(fpatt), d_z.data_ptr(),
                          d_fp.data_ptr(), d_pi.data_ptr(), model.data_ptr(), d_bl.data_ptr(),
                          d_out.data_ptr(), None, None)
    _lib.check(rc)
    ref = pb.neg_lnL(x)
    assert abs(float(d_out.cpu()[0]) - ref) <= 1e-12 * abs(ref)
