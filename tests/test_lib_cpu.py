"""CPU-side checks of the C-ABI library (no GPU): it loads, exports every
symbol include/*.h declares, and its host-only parts (pattern compression,
model set-up, argument validation) agree with the oracle and golden fixtures."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from cucodeml_gb300 import _lib, api, codon
from cucodeml_gb300.tree import parse_newick
from oracle import oracle as O
from tests.conftest import ROOT, golden_names, load_golden


def header_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        if "extern \"C\"" not in text and f != "gbcodeml.h":
            continue
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gb_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_header_symbols():
    L = _lib.load()
    names = header_functions()
    assert "gb_create" in names and "gb_eval" in names
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(_lib.SIGNATURES)
    assert L.gb_version().decode().startswith("gbcodeml")


@pytest.mark.parametrize("name", golden_names())
def test_library_patterns_match_codeml(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = api.patterns(codons)
    got = [" ".join(codon.codon_string(int(c)) for c in z[:, h]) for h in range(z.shape[1])]
    assert got == fx["patterns"]
    assert np.array_equal(fpatt, np.array(fx["fpatt"]))
    z2, fp2, pi2 = O.patterns(codons)
    assert np.array_equal(z, z2) and np.array_equal(pi, pi2)


def test_patterns_rejects_bad_codons():
    with pytest.raises(_lib.GBError):
        api.patterns(np.array([[0, 61], [1, 2], [3, 4]]))


@pytest.mark.parametrize("name", ["c8x300_s1", "c40x200_s4"])
def test_model_setup_matches_oracle(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = O.patterns(codons)
    pb = O.Problem(tree, z, fpatt, pi)
    x = np.array(fx["x"])
    nb = tree.nbranch
    U, V, R, qf, fk = api.model_setup(pi, x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2])
    Uo, Vo, Ro, qfo, fko = pb.set_params(x)
    assert np.allclose(qf, qfo, rtol=1e-14, atol=0)
    assert np.allclose(fk, fko, rtol=1e-14, atol=0)
    for w in range(3):
        for t in (0.01, 0.3, 2.0):
            P1 = U[w] @ np.diag(np.exp(t * R[w])) @ V[w]
            P2 = Uo[w] @ np.diag(np.exp(t * Ro[w])) @ Vo[w]
            assert np.abs(P1 - P2).max() < 1e-12
        assert np.abs(U[w] @ V[w] - np.eye(61)).max() < 1e-12


def test_model_setup_rejects_bad_params():
    pi = np.full(61, 1 / 61)
    with pytest.raises(_lib.GBError) as e:
        api.model_setup(pi, 2.0, 0.3, 3.0, 0.0, 0.0)
    assert e.value.code == -4


def _problem(tree, z, fpatt, pi, father=None):
    return dict(tree=tree, z=z, fpatt=fpatt, pi=pi)


def test_create_validates_before_device():
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    bad = parse_newick(fx["newick"], fx["names"])
    bad.label = bad.label.copy()
    bad.label[0] = 2                       # labels must be 0/1
    with pytest.raises(_lib.GBError) as e:
        api.Likelihood(bad, z, fpatt, pi)
    assert e.value.code == -1
    zb = z.copy()
    zb[0, 0] = 70                          # only clean data (sense codons)
    with pytest.raises(_lib.GBError) as e:
        api.Likelihood(tree, zb, fpatt, pi)
    assert e.value.code == -1


def test_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    with pytest.raises(_lib.GBError) as e:
        api.Likelihood(tree, z, fpatt, pi)
    assert e.value.code in (-7, -2)


def test_beta_classes_match_the_inverse_incomplete_beta():
    """gb_beta_classes (M7 / M8's discretised beta, DiscreteNSsites
    codeml.c:2728-2770) against the oracle's scipy-based quantiles over the
    range codeml allows for p and q (0.005 .. 99): 3e-11 relative (the
    extreme corners reach quantiles of 1e-263; 1e-12 inside [0.05, 99])."""
    from cucodeml_gb300 import api
    from oracle import oracle as O
    grid = [0.005, 0.01, 0.05, 0.1, 0.3, 0.5, 0.9, 1.0, 1.5, 2.0, 5.0, 20.0, 99.0]
    for p in grid:
        for q in grid:
            om, pr = api.beta_classes(p, q)
            ref, rpr = O.beta_classes(p, q)
            tol = 1e-12 if min(p, q) >= 0.05 else 3e-11
            assert np.all(np.abs(om - ref) <= tol * ref), (p, q)
            assert np.all(pr == rpr)
            assert np.all(np.diff(om) >= -4 * np.finfo(float).eps)        # ascending, to rounding near 1


def test_beta_classes_reject_bad_parameters():
    from cucodeml_gb300 import _lib, api
    for p, q in ((0.0, 1.0), (1.0, -2.0), (float("nan"), 1.0), (1.0, float("inf"))):
        with pytest.raises(Exception):
            api.beta_classes(p, q)
    L = _lib.load()
    assert L.gb_beta_classes(1.0, 1.0, 0, None, None) == -1          # GB_ERR_ARG


def _null_args(argtypes):
    """Arguments for one call: null pointers and arrays of null pointers,
    1 for integers and 1.0 for doubles."""
    out = []
    for t in argtypes:
        if t in (C.c_int, C.c_double):
            out.append(t(1))
        elif isinstance(t, type) and issubclass(t, C.Array):
            out.append(t())
        else:
            out.append(None)
    return out


# entries whose first argument is a gb_handle * or gb_batch *
HANDLE_ENTRIES = sorted(n for n, (_, a) in _lib.SIGNATURES.items()
                        if a and a[0] is C.c_void_p and n != "gb_lnL_noalloc")


def test_handle_entries_reject_a_null_handle():
    """Every entry taking a handle or batch returns an error code (and, where
    it sets one, a reason) for a null one before any device work, so a caller
    that lost its handle gets a status, not a crash."""
    L = _lib.load()
    assert len(HANDLE_ENTRIES) >= 30
    for name in HANDLE_ENTRIES:
        rc = getattr(L, name)(*_null_args(_lib.SIGNATURES[name][1]))
        assert rc < 0, name
        if name not in ("gb_nscale", "gb_batch_size"):
            assert L.gb_last_error().decode(), name


def _raw_problem(tree, z, fpatt, pi, keep):
    """A gb_problem over numpy copies (kept alive in `keep`)."""
    ip, ub = C.POINTER(C.c_int), C.POINTER(C.c_ubyte)
    father = np.ascontiguousarray(tree.father, dtype=np.int32)
    label = np.ascontiguousarray(tree.label, dtype=np.int32)
    z = np.ascontiguousarray(z, dtype=np.uint8)
    fpatt = np.ascontiguousarray(fpatt, dtype=np.float64)
    pi = np.ascontiguousarray(pi, dtype=np.float64)
    keep += [father, label, z, fpatt, pi]
    dp = C.POINTER(C.c_double)
    prob = _lib.Problem(tree.ns, tree.nnode, tree.root, father.ctypes.data_as(ip), label.ctypes.data_as(ip),
                        len(fpatt), z.ctypes.data_as(ub), fpatt.ctypes.data_as(dp), pi.ctypes.data_as(dp),
                        None, _lib.GB_PREC_FP64, 0)
    return prob, father, label, z, fpatt, pi


def _internal_pair(tree):
    """Two internal nodes other than the root, the second a son of the first."""
    for n in range(tree.ns, tree.nnode):
        f = int(tree.father[n])
        if n != tree.root and f != tree.root and f >= tree.ns:
            return f, n
    raise AssertionError("tree too small")


def _one_son(fa, t):
    """Move a son of internal node n to another internal node m outside its
    subtree, both with two sons and neither the root: n is left with one."""
    sons = {a: [s for s in range(t.nnode) if s != t.root and fa[s] == a] for a in range(t.ns, t.nnode)}
    for n in range(t.ns, t.nnode):
        if n == t.root or len(sons[n]) != 2:
            continue
        s = sons[n][0]
        below = {s}
        for v in range(t.nnode):           # nodes in the subtree of s
            a = v
            while a != t.root and a not in below:
                a = int(fa[a])
            if a in below:
                below.add(v)
        for m in range(t.ns, t.nnode):
            if m not in (n, t.root) and m not in below and len(sons[m]) == 2:
                fa[s] = m
                return
    raise AssertionError("tree too small")


# case -> (how the problem is spoiled, the reason gb_last_error gives)
BAD_PROBLEMS = {
    "root has a father": (lambda p, fa, la, z, fp, pi, t: fa.__setitem__(t.root, t.ns), "root must be"),
    "root is a tip": (lambda p, fa, la, z, fp, pi, t: setattr(p, "root", 0), "root must be"),
    "father out of range": (lambda p, fa, la, z, fp, pi, t: fa.__setitem__(0, t.nnode + 5), "father out of range"),
    "father is a tip": (lambda p, fa, la, z, fp, pi, t: fa.__setitem__(1, 0), "father out of range or a tip"),
    "four sons": (lambda p, fa, la, z, fp, pi, t: fa.__setitem__(_internal_pair(t)[1], t.root), "more than 3 sons"),
    "label 2": (lambda p, fa, la, z, fp, pi, t: la.__setitem__(0, 2), "labels must be 0 or 1"),
    "internal node with one son": (lambda p, fa, la, z, fp, pi, t: _one_son(fa, t), "< 2 sons"),
    "cycle off the root": (lambda p, fa, la, z, fp, pi, t: fa.__setitem__(_internal_pair(t)[0], _internal_pair(t)[1]),
                           "not connected"),
    "no patterns": (lambda p, fa, la, z, fp, pi, t: setattr(p, "npatt", 0), "sizes too small"),
    "null z": (lambda p, fa, la, z, fp, pi, t: setattr(p, "z", None), "missing arrays"),
    "two taxa": (lambda p, fa, la, z, fp, pi, t: setattr(p, "ns", 2), "sizes too small"),
    "codon id 61": (lambda p, fa, la, z, fp, pi, t: z.__setitem__((0, 0), 61), "codon id >= 61"),
    "pi zero": (lambda p, fa, la, z, fp, pi, t: pi.__setitem__(5, 0.0), "pi must be positive"),
    "negative count": (lambda p, fa, la, z, fp, pi, t: fp.__setitem__(0, -1.0), "fpatt must be >= 0"),
    "NaN count": (lambda p, fa, la, z, fp, pi, t: fp.__setitem__(1, float("nan")), "fpatt must be >= 0"),
}


@pytest.mark.parametrize("case", sorted(BAD_PROBLEMS))
def test_create_rejects_malformed_problems_on_the_host(case):
    """gb_create checks the tree (one father per node, the root's -1, 2-3
    sons at internal nodes, tips 0..ns-1, connected), the branch labels, the
    codon ids, pi and the pattern counts before it looks for a device:
    GB_ERR_ARG with a reason, here without a GPU as on a GPU machine."""
    L = _lib.load()
    fx, tree, codons = load_golden("c8x300_s1")
    z, fpatt, pi = O.patterns(codons)
    keep = []
    prob, fa, la, zz, fp, pp = _raw_problem(tree, z, fpatt, pi, keep)
    h = C.c_void_p()
    spoil, reason = BAD_PROBLEMS[case]
    spoil(prob, fa, la, zz, fp, pp, tree)
    rc = L.gb_create(C.byref(prob), C.byref(h))
    assert rc == -1, (case, rc, L.gb_last_error())
    assert reason in L.gb_last_error().decode() and not h.value
