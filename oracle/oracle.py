"""ctypes wrapper of the C oracle (oracle.c) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module.  It restates codeml's branch-site model A likelihood on
the CPU (see oracle.c for the reference routine behind each function) and is
the checker for the CUDA library, never the thing measured or shipped.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


class _Problem(C.Structure):
    _fields_ = [
        ("ns", C.c_int), ("nnode", C.c_int), ("root", C.c_int), ("npatt", C.c_int),
        ("nson", C.POINTER(C.c_int)), ("sons", C.POINTER(C.c_int)),
        ("label", C.POINTER(C.c_int)), ("bnode", C.POINTER(C.c_int)),
        ("z", C.POINTER(C.c_ubyte)), ("fpatt", C.POINTER(C.c_double)),
        ("pi", C.POINTER(C.c_double)), ("nthreads", C.c_int), ("model_b", C.c_int),
        ("amb", C.POINTER(C.c_ubyte)),
    ]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        L.oracle_lnL.restype = C.c_double
        L.oracle_lnL.argtypes = [C.POINTER(_Problem), dp, C.c_int, dp, dp, C.POINTER(C.c_int)]
        L.oracle_patterns.restype = C.c_int
        L.oracle_patterns.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_ubyte), dp, dp]
        L.oracle_set_params.restype = C.c_int
        L.oracle_set_params.argtypes = [C.POINTER(_Problem), dp, C.c_int, dp, dp, dp, dp, dp]
        L.oracle_gradientB.restype = C.c_int
        L.oracle_gradientB.argtypes = [C.POINTER(_Problem), dp, C.c_int, C.c_int, C.c_int, dp]
        L.oracle_build_q.restype = C.c_double
        L.oracle_build_q.argtypes = [dp, C.c_double, C.c_double, dp]
        L.oracle_pmat.restype = None
        L.oracle_pmat.argtypes = [dp, C.c_double, dp, dp, dp]
        L.oracle_max_threads.restype = C.c_int
        L.oracle_beb_clade.restype = C.c_int
        L.oracle_beb_clade.argtypes = [C.POINTER(_Problem), dp, dp, dp, dp, dp, dp]
        L.oracle_fhK_uvr.restype = C.c_int
        L.oracle_fhK_uvr.argtypes = [C.POINTER(_Problem), dp, dp, dp, dp, dp, dp]
        L.oracle_beb.restype = C.c_int
        L.oracle_beb.argtypes = [C.POINTER(_Problem), dp, C.c_int, dp, dp, dp, dp, dp, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def patterns(codons: np.ndarray):
    """codons [ns, ncodon] (0..60) -> (z [ns, npatt] uint8, fpatt [npatt], pi [61])."""
    codons = np.ascontiguousarray(codons, dtype=np.int32)
    ns, nc = codons.shape
    z = np.zeros(ns * nc, dtype=np.uint8)
    fp = np.zeros(nc)
    pi = np.zeros(61)
    npatt = C.c_int(0)
    rc = lib().oracle_patterns(ns, nc, codons.ctypes.data_as(C.POINTER(C.c_int)), C.byref(npatt),
                               z.ctypes.data_as(C.POINTER(C.c_ubyte)), _dp(fp), _dp(pi))
    if rc:
        raise ValueError(f"oracle_patterns failed rc={rc}")
    n = npatt.value
    return z[: ns * n].reshape(ns, n).copy(), fp[:n].copy(), pi


class Problem:
    """A tree + compressed patterns + codon frequencies, held for the C oracle."""

    def __init__(self, tree, z: np.ndarray, fpatt: np.ndarray, pi: np.ndarray, nthreads: int = 0,
                 model_b: bool = False, ambiguity=None):
        """ambiguity: None (clean data), or codeml's (nChara[256], CharaMap[256][64])
        for tip codes z >= 61."""
        self.tree = tree
        nn = tree.nnode
        self.nson = np.array([len(tree.sons[i]) for i in range(nn)], dtype=np.int32)
        sons = np.full((nn, 3), -1, dtype=np.int32)
        for i in range(nn):
            for k, s in enumerate(tree.sons[i]):
                sons[i, k] = s
        self.sons = sons.reshape(-1).copy()
        self.label = np.ascontiguousarray(tree.label, dtype=np.int32)
        self.bnode = np.ascontiguousarray(tree.branch_nodes(), dtype=np.int32)
        self.z = np.ascontiguousarray(z, dtype=np.uint8)
        self.fpatt = np.ascontiguousarray(fpatt, dtype=np.float64)
        self.pi = np.ascontiguousarray(pi, dtype=np.float64)
        self.npatt = int(self.fpatt.shape[0])
        self.np = tree.nbranch + 5 + int(model_b)
        ip = C.POINTER(C.c_int)
        self._s = _Problem(tree.ns, nn, tree.root, self.npatt,
                           self.nson.ctypes.data_as(ip), self.sons.ctypes.data_as(ip),
                           self.label.ctypes.data_as(ip), self.bnode.ctypes.data_as(ip),
                           self.z.ctypes.data_as(C.POINTER(C.c_ubyte)), _dp(self.fpatt),
                           _dp(self.pi), int(nthreads), int(model_b), None)
        if ambiguity is not None:
            nch, cmap = ambiguity
            self.amb = np.concatenate([np.asarray(nch, dtype=np.uint8).reshape(256),
                                       np.asarray(cmap, dtype=np.uint8).reshape(256 * 64)])
            self._s.amb = self.amb.ctypes.data_as(C.POINTER(C.c_ubyte))

    def set_threads(self, n: int) -> None:
        self._s.nthreads = int(n)

    def neg_lnL(self, x, lastround: bool = True, want_fhK: bool = False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        fhK = np.zeros(4 * self.npatt) if want_fhK else None
        lnf = np.zeros(self.npatt) if want_fhK else None
        nsc = C.c_int(0)
        v = lib().oracle_lnL(C.byref(self._s), _dp(x), int(lastround),
                             _dp(fhK) if fhK is not None else None,
                             _dp(lnf) if lnf is not None else None, C.byref(nsc))
        if want_fhK:
            return v, fhK.reshape(4, self.npatt), lnf, nsc.value
        return v

    def set_params(self, x, lastround: bool = True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        U = np.zeros((3, 61, 61)); V = np.zeros((3, 61, 61)); R = np.zeros((3, 61))
        qf = np.zeros(2); fk = np.zeros(4)
        rc = lib().oracle_set_params(C.byref(self._s), _dp(x), int(lastround), _dp(U), _dp(V),
                                     _dp(R), _dp(qf), _dp(fk))
        if rc:
            raise ValueError("parameter error")
        return U, V, R, qf, fk

    def gradientB(self, x, lastround: bool = True, central: bool = True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        g = np.zeros(len(x))
        lib().oracle_gradientB(C.byref(self._s), _dp(x), len(x), int(lastround), int(central), _dp(g))
        return g


    def beb(self, x, lastround: bool = True, want_lnfw: bool = True):
        """Bayes empirical Bayes of model A at x (oracle.c oracle_beb): a dict
        with lnfw [121, npatt], post [4, npatt], grid [4, 10], p0p1 [100] and
        lnfX, S1, S2."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        lnfw = np.zeros(121 * self.npatt) if want_lnfw else None
        post = np.zeros(4 * self.npatt)
        grid = np.zeros(40)
        p0p1 = np.zeros(100)
        fx = np.zeros(3)
        wmean = np.zeros(self.npatt)
        wsd = np.zeros(self.npatt)
        rc = lib().oracle_beb(C.byref(self._s), _dp(x), int(lastround),
                              _dp(lnfw) if lnfw is not None else None, _dp(post), _dp(grid),
                              _dp(p0p1), _dp(fx), _dp(wmean), _dp(wsd))
        if rc:
            raise ValueError("parameter error")
        return {"lnfw": lnfw.reshape(121, self.npatt) if lnfw is not None else None,
                "post": post.reshape(4, self.npatt), "grid": grid.reshape(4, 10), "p0p1": p0p1,
                "lnfX": fx[0], "S1": fx[1], "S2": fx[2], "wmean": wmean, "wsd": wsd}


    def beb_clade(self, x, want_lnfw: bool = True):
        """Bayes empirical Bayes under clade model C with two branch types
        (oracle.c oracle_beb_clade): lnfw [111, npatt], post [3, npatt],
        grid [5, 10], p0p1 [100], lnfX, S1, S2."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        lnfw = np.zeros(111 * self.npatt) if want_lnfw else None
        post = np.zeros(3 * self.npatt)
        grid = np.zeros(50)
        p0p1 = np.zeros(100)
        fx = np.zeros(3)
        lib().oracle_beb_clade(C.byref(self._s), _dp(x), _dp(lnfw) if lnfw is not None else None, _dp(post),
                               _dp(grid), _dp(p0p1), _dp(fx))
        return {"lnfw": lnfw.reshape(111, self.npatt) if lnfw is not None else None,
                "post": post.reshape(3, self.npatt), "grid": grid.reshape(5, 10), "p0p1": p0p1,
                "lnfX": fx[0], "S1": fx[1], "S2": fx[2]}

    def beb_clade_d(self, x):
        """Bayes empirical Bayes under clade model D with two branch types
        (lfunNSsites_ACD codeml.c:6617-6826 with modelACD = mD; grid and sets
        get_grid_para_like_ACD 6419-6530), in numpy over this oracle's
        pruning.  x = [branch lengths, kappa, p0, p1, w0, w1, w2, w3] (p0,
        p1 untransformed).  Sets: 10 w0 values in (0, 0.5) and 10 w1 values
        in (0.5, 1.5) on every branch, then (w2_i background, w3_j
        foreground) for w2, w3 in (0, 3), set 20 + 10 i + j; P from each
        omega's unscaled Q with the MLE's Qfactors applied to t.  Grid: 100
        ternary (p0, p1) triangles x w0 x w1 x w2 x w3 (10^6 points, uniform).
        Returns lnfw [120, npatt], post [3, npatt], grid rows w0, w1, w2, w3
        [4, 10], p0p1 [100], lnfX (as codeml prints it), S1."""
        x = np.asarray(x, dtype=np.float64)
        nb = self.tree.nbranch
        kappa, p0, p1, w0, w1, w2, w3 = x[nb:nb + 7]
        p2 = 1.0 - p0 - p1
        qf = np.array([1.0 / build_q(self.pi, kappa, p0 * w0 + p1 * w1 + p2 * w)[1] for w in (w2, w3)])
        sq = np.sqrt(self.pi)

        def eig(w):      # eigenQREV's symmetrisation, solved by LAPACK (numpy)
            Q = build_q(self.pi, kappa, w)[0]
            lam, E = np.linalg.eigh(sq[:, None] * Q / sq[None, :])
            return E / sq[:, None], E.T * sq[None, :], lam

        def classes(wa, wc):     # fhK of model A's classes with slots (wa, 1, wc) as log f
            e = [eig(wa), eig(1.0), eig(wc)]
            fh, nsc = self.fhK_uvr(np.stack([q[0] for q in e]), np.stack([q[1] for q in e]),
                                   np.stack([q[2] for q in e]), qf, x[:nb])
            return fh if nsc else np.log(np.where(fh <= 0, 1e-300, fh))

        g0 = 0.5 * (np.arange(10) + 0.5) / 10
        g1 = 0.5 + (np.arange(10) + 0.5) / 10
        g2 = 3.0 * (np.arange(10) + 0.5) / 10
        lnfw = np.empty((120, self.npatt))
        for i in range(10):
            lnfw[i] = classes(g0[i], 1.0)[0]
            lnfw[10 + i] = classes(g1[i], 1.0)[0]
            for j in range(10):
                lnfw[20 + 10 * i + j] = classes(g2[i], g2[j])[2]
        m = lnfw.max(axis=0)
        F = np.exp(lnfw - m)
        S1 = float(m @ self.fpatt)
        t = np.arange(100)
        ix = np.floor(np.sqrt(t)).astype(int)
        iy = t - ix * ix
        pa = (1 + (iy // 2) * 3 + (iy % 2)) / 30.0          # GetIndexTernary tools.c:4441-4461
        pb = (1 + (9 - ix) * 3 + (iy % 2)) / 30.0
        P3 = np.stack([pa, pb, 1 - pa - pb], axis=1)
        F0, F1, F2 = F[0:10], F[10:20], F[20:120]
        lnfXs = np.empty((100, 10, 10, 100))
        for a in range(100):
            for i0 in range(10):
                for i1 in range(10):
                    fh = P3[a, 0] * F0[i0] + P3[a, 1] * F1[i1] + P3[a, 2] * F2
                    lnfXs[a, i0, i1] = np.where(fh < 1e-300, 0.0, np.log(np.maximum(fh, 1e-300))) @ self.fpatt
        M = lnfXs.max()
        lfX = M + np.log(np.exp(lnfXs - M).sum())
        w = np.exp(lnfXs - lfX)
        post = np.zeros((3, self.npatt))
        for a in range(100):
            for i0 in range(10):
                for i1 in range(10):
                    fh = P3[a, 0] * F0[i0] + P3[a, 1] * F1[i1] + P3[a, 2] * F2
                    wk = w[a, i0, i1][:, None] / fh
                    post[0] += P3[a, 0] * F0[i0] * wk.sum(axis=0)
                    post[1] += P3[a, 1] * F1[i1] * wk.sum(axis=0)
                    post[2] += P3[a, 2] * (F2 * wk).sum(axis=0)
        w6 = w.reshape(100, 10, 10, 10, 10)
        grid = np.stack([w6.sum(axis=(0, 2, 3, 4)), w6.sum(axis=(0, 1, 3, 4)), w6.sum(axis=(0, 1, 2, 4)),
                         w6.sum(axis=(0, 1, 2, 3))])
        return {"lnfw": lnfw, "post": post, "grid": grid, "p0p1": w.sum(axis=(1, 2, 3)),
                "lnfX": float(lfX + S1 - 6 * np.log(10.0)), "S1": S1}

    def fhK_uvr(self, U, V, R, qf, xb):
        """Per-class fhK (4, npatt) from given eigen slots, Qfactors and branch
        lengths by branch index (oracle.c oracle_fhK_uvr); also nscale."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        R = np.ascontiguousarray(R, dtype=np.float64)
        qf = np.ascontiguousarray(qf, dtype=np.float64)
        xb = np.ascontiguousarray(xb, dtype=np.float64)
        fhK = np.zeros(4 * self.npatt)
        nsc = lib().oracle_fhK_uvr(C.byref(self._s), _dp(U), _dp(V), _dp(R), _dp(qf), _dp(xb), _dp(fhK))
        return fhK.reshape(4, self.npatt), nsc

    def clade_c(self, x):
        """Clade model C (codeml model = 3, NSsites = 2, two branch types) at x =
        [branch lengths, kappa, p0, p1, w0, w2 (background), w3 (foreground)]:
        classes w0 and w1 = 1 on every branch and (w2, w3) by branch type,
        Qfactor_NS_branch[b] = 1 / meanrate(Q(kappa, p0 w0 + p1 + p2 w_{2+b}))
        (SetParametersNSsites codeml.c:2437-2446, 2522-2539).  Classes 0 and 1
        are model A's with slots (w0, 1, -), the third is model A's class 2a
        with slots (w2, -, w3).  Clade model D (NSsites = 3, a Problem made
        with model_b=True): the same with w1 free, x ending p0, p1, w0, w1,
        w2, w3.  Returns (-lnL, fhK [3, npatt], lnf)."""
        x = np.asarray(x, dtype=np.float64)
        nb = self.tree.nbranch
        if self._s.model_b:
            # clade model D (NSsites = 3): w1 free as well, x ends p0, p1, w0, w1, w2, w3
            kappa, p0, p1, w0, w1, w2, w3 = x[nb:nb + 7]
            mid = [w0, w1]
        else:
            kappa, p0, p1, w0, w2, w3 = x[nb:nb + 6]
            w1, mid = 1.0, [w0]
        p2 = 1.0 - p0 - p1
        Ua, Va, Ra, _, _ = self.set_params(np.concatenate([x[:nb], [kappa, p0, p1], mid, [w2]]))
        U3, V3, R3, _, _ = self.set_params(np.concatenate([x[:nb], [kappa, p0, p1], mid, [w3]]))
        qf = np.array([1.0 / build_q(self.pi, kappa, p0 * w0 + p1 * w1 + p2 * w)[1] for w in (w2, w3)])
        fa, nsc = self.fhK_uvr(Ua, Va, Ra, qf, x[:nb])
        Ub = np.stack([Ua[2], Ua[1], U3[2]])
        Vb = np.stack([Va[2], Va[1], V3[2]])
        Rb = np.stack([Ra[2], Ra[1], R3[2]])
        fb, _ = self.fhK_uvr(Ub, Vb, Rb, qf, x[:nb])
        fhK = np.stack([fa[0], fa[1], fb[0 + 2]])
        fk = np.array([p0, p1, p2])
        if nsc:
            t = fhK.max(axis=0)
            lnf = t + np.log((fk[:, None] * np.exp(fhK - t)).sum(axis=0))
        else:
            s = (fk[:, None] * fhK).sum(axis=0)
            lnf = np.log(np.where(s <= 0, 1e-300, s))
        return -float((lnf * self.fpatt).sum()), fhK, lnf

    def site_classes(self, xb, kappa, omegas, props):
        """A site model with K classes (codeml model = 0): class k has omega
        omegas[k] on every branch and weight props[k]; Qfactor_NS =
        1 / meanrate(Q(kappa, sum props omegas)) (SetParametersNSsites
        codeml.c:2466-2487).  Needs every branch labelled foreground: each
        oracle_fhK_uvr call then yields three classes (slots 0, 1 and 2).
        Returns (-lnL, fhK [K, npatt], lnf)."""
        om = np.asarray(omegas, dtype=np.float64)
        pr = np.asarray(props, dtype=np.float64)
        qns = 1.0 / build_q(self.pi, kappa, float(pr @ om))[1]
        eig = Problem(self.tree, self.z, self.fpatt, self.pi, nthreads=1, model_b=True)
        rows = []
        for c in range(0, len(om), 3):
            w = list(om[c:c + 3]) + [1.0] * (3 - len(om[c:c + 3]))
            U, V, R, _, _ = eig.set_params(np.concatenate([xb, [kappa, 0.3, 0.3], w]))
            f, nsc = self.fhK_uvr(U, V, R, [qns, qns], xb)
            rows += [f[0], f[1], f[2]][: len(om[c:c + 3])]
        fhK = np.stack(rows)
        if nsc:
            t = fhK.max(axis=0)
            lnf = t + np.log((pr[:, None] * np.exp(fhK - t)).sum(axis=0))
        else:
            sm = (pr[:, None] * fhK).sum(axis=0)
            lnf = np.log(np.where(sm <= 0, 1e-300, sm))
        return -float((lnf * self.fpatt).sum()), fhK, lnf

    def neb(self, x, lastround: bool = True):
        """NEB posteriors of the four site classes at x (lfunNSsites_rate
        codeml.c:5079-5129): freqK_c f_c(h) normalised over c, from fhK (log
        values shifted by their maximum when nodes are scaled)."""
        v, fhK, lnf, nscale = self.neg_lnL(x, lastround=lastround, want_fhK=True)
        fk = self.set_params(x, lastround)[4]
        if nscale:
            f = np.exp(fhK - fhK.max(axis=0))
        else:
            f = fhK
        q = fk[:, None] * f
        return q / q.sum(axis=0)

    def opg_se(self, x, small_diff: float = 1e-6):
        """codeml's standard errors (getSE = 1): HessianSKT2004
        (treesub.c:6979-7048) -- per-pattern scores by central differences of
        log f_h with step 2 small_diff (|x_i| + 1) at untransformed p0, p1,
        H = -sum_h fpatt_h d_h d_h^T, g from the same lnL differences -- then
        SE_i = sqrt([(-H)^-1]_ii), -1 where that is not positive
        (codeml.c:754-783).  Returns (g, H, se)."""
        x = np.asarray(x, dtype=np.float64)
        n = len(x)
        eh = 2 * small_diff * (np.abs(x) + 1)
        lnL = np.zeros((2, n))
        lnf = np.zeros((2, n, self.npatt))
        for bf in range(2):
            for i in range(n):
                x1 = x.copy()
                x1[i] = x[i] - eh[i] if bf == 0 else x[i] + eh[i]
                v, _, f, _ = self.neg_lnL(x1, lastround=True, want_fhK=True)
                lnL[bf, i] = -v
                lnf[bf, i] = f
        g = (lnL[1] - lnL[0]) / (eh * 2)
        d = (lnf[1] - lnf[0]) / (eh * 2)[:, None]
        H = -(d * self.fpatt[None, :]) @ d.T
        H = 0.5 * (H + H.T)           # the matrix product is symmetric only up to its summation order
        V = np.linalg.inv(-H)
        dg = np.diag(V)
        se = np.where(dg > 0, np.sqrt(np.abs(dg)), -1.0)
        return g, H, se


def beta_classes(p, q, K=10):
    """M7's discrete beta: K equal-probability categories at their medians,
    QuantileBeta((2j + 1) / (2K), p, q) (DiscreteNSsites codeml.c:2746-2752);
    the inverse incomplete beta from scipy."""
    from scipy.special import betaincinv
    return np.array([betaincinv(p, q, (2 * j + 1) / (2.0 * K)) for j in range(K)]), np.full(K, 1.0 / K)


def build_q(pi, kappa, omega):
    Q = np.zeros((61, 61))
    pi = np.ascontiguousarray(pi, dtype=np.float64)
    mr = lib().oracle_build_q(_dp(pi), float(kappa), float(omega), _dp(Q))
    return Q, mr


def max_threads() -> int:
    return int(lib().oracle_max_threads())
