"""Python host mirror of the library's C ABI, shaped like codeml's interface.

`Likelihood` is one gb_handle: one tree + compressed alignment on one GPU.
Its methods mirror the reference's calls on the model-A hot path:

* `neg_lnL_uvr(...)`   codeml's CUDA_lfundG / CUDA_fx_r from host U, V, Root,
                       Qfactor and class proportions (treesub.c:7397-7450,
                       7554-7595); returns -lnL, com.fhK and per-pattern log f.
* `evaluate(...)`      -lnL (and optionally its analytic gradient) from the
                       natural parameters.
* `dfun_x(x, ...)`     ming2's dfun hook over codeml's x vector
                       (tools.c:6361-6363).

All work runs in libgbcodeml.so; nothing here computes likelihoods.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .tree import Tree

_dp = C.POINTER(C.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def patterns(codons: np.ndarray):
    """Codon alignment [ns, ncodon] (sense codon ids) -> (z [ns, npatt], fpatt, pi)."""
    L = _lib.load()
    codons = np.ascontiguousarray(codons, dtype=np.int32)
    ns, nc = codons.shape
    z = np.zeros(ns * nc, dtype=np.uint8)
    fp = np.zeros(nc)
    pi = np.zeros(61)
    npatt = C.c_int(0)
    _lib.check(L.gb_patterns(ns, nc, codons.ctypes.data_as(C.POINTER(C.c_int)), C.byref(npatt),
                             z.ctypes.data_as(C.POINTER(C.c_ubyte)), _ptr(fp), _ptr(pi)))
    n = npatt.value
    return z[: ns * n].reshape(ns, n).copy(), fp[:n].copy(), pi


def ng86(z: np.ndarray, fpatt: np.ndarray):
    """Pairwise Nei-Gojobori (1986) distances (gb_ng86): dict of dS, dN, dN/dS
    (-1 where not applicable, as codeml prints them) and codeml's distance,
    each [ns, ns]."""
    L = _lib.load()
    z = np.ascontiguousarray(z, dtype=np.uint8)
    fp = np.ascontiguousarray(fpatt, dtype=np.float64)
    ns, npatt = z.shape
    dS = np.zeros((ns, ns)); dN = np.zeros((ns, ns)); dist = np.zeros((ns, ns))
    _lib.check(L.gb_ng86(ns, npatt, z.ctypes.data_as(C.POINTER(C.c_ubyte)), _ptr(fp), _ptr(dS), _ptr(dN),
                         _ptr(dist)))
    w = np.where((dS > 0) & (dN > 0), dN / np.where(dS > 0, dS, 1.0), -1.0)
    np.fill_diagonal(w, 0.0)
    return {"dS": dS, "dN": dN, "dN_dS": w, "dist": dist}


def _ternary_classes():
    """(p0, p1, p2) at the centroids of the 100 ternary triangles (GetIndexTernary tools.c:4441-4461)."""
    t = np.arange(100)
    ix = np.floor(np.sqrt(t)).astype(int)
    iy = t - ix * ix
    a = (1 + (iy // 2) * 3 + (iy % 2)) / 30.0
    b = (1 + (9 - ix) * 3 + (iy % 2)) / 30.0
    return np.stack([a, b, 1 - a - b], axis=1)


def model_setup(pi, kappa, omega0, omega2, p0, p1):
    """(U [3,61,61], V [3,61,61], Root [3,61], qf [2], freqK [4]) computed by the library's host code."""
    L = _lib.load()
    pi = np.ascontiguousarray(pi, dtype=np.float64)
    U = np.zeros((3, 61, 61)); V = np.zeros((3, 61, 61)); R = np.zeros((3, 61))
    qf = np.zeros(2); fk = np.zeros(4)
    _lib.check(L.gb_model_setup(_ptr(pi), kappa, omega0, omega2, p0, p1, _ptr(U), _ptr(V), _ptr(R),
                                _ptr(qf), _ptr(fk)))
    return U, V, R, qf, fk


def beta_classes(p, q, K: int = 10):
    """(omegas [K], proportions [K]) of codeml's discretised beta under M7 /
    M8: K equal-probability categories at their medians (DiscreteNSsites
    codeml.c:2728-2770), from the library's host code."""
    L = _lib.load()
    om = np.zeros(K)
    pr = np.zeros(K)
    _lib.check(L.gb_beta_classes(float(p), float(q), int(K), _ptr(om), _ptr(pr)))
    return om, pr


@dataclass
class EvalResult:
    neg_lnL: float
    fhK: np.ndarray | None = None
    lnf: np.ndarray | None = None
    grad: dict | None = None
    ms_device: float = 0.0
    ms_host: float = 0.0
    kernels: int = 0
    h2d_bytes: float = 0.0
    d2h_bytes: float = 0.0


class Likelihood:
    def __init__(self, tree: Tree, z: np.ndarray, fpatt: np.ndarray, pi: np.ndarray,
                 precision: str = "fp64", device: int = 0, node_scale=None, tuning: dict | None = None,
                 ambiguity=None):
        """ambiguity: None for clean data, or codeml's (nChara[256],
        CharaMap[256][64]) for tip codes z >= 61 (gaps and ambiguous codons,
        cleandata = 0; FP64 only, gb_create_unclean)."""
        self._L = _lib.load()
        self.tree = tree
        self.ns, self.nnode = tree.ns, tree.nnode
        self.npatt = int(len(fpatt))
        self._father = np.ascontiguousarray(tree.father, dtype=np.int32)
        self._label = np.ascontiguousarray(tree.label, dtype=np.int32)
        self._z = np.ascontiguousarray(z, dtype=np.uint8)
        self._fpatt = np.ascontiguousarray(fpatt, dtype=np.float64)
        self._pi = np.ascontiguousarray(pi, dtype=np.float64)
        self._scale = None
        if node_scale is not None:
            self._scale = np.ascontiguousarray(node_scale, dtype=np.int8).tobytes()
        prec = precision if isinstance(precision, int) else \
            {"fp64": _lib.GB_PREC_FP64, "fast": _lib.GB_PREC_FAST}[precision]
        self._fp64 = prec == _lib.GB_PREC_FP64
        self.last_ms = 0.0
        ip = C.POINTER(C.c_int)
        self._prob = _lib.Problem(self.ns, self.nnode, tree.root, self._father.ctypes.data_as(ip),
                                  self._label.ctypes.data_as(ip), self.npatt,
                                  self._z.ctypes.data_as(C.POINTER(C.c_ubyte)), _ptr(self._fpatt),
                                  _ptr(self._pi), self._scale, prec, device)
        h = C.c_void_p()
        if ambiguity is None:
            _lib.check(self._L.gb_create(C.byref(self._prob), C.byref(h)))
        else:
            self._nch = np.ascontiguousarray(np.asarray(ambiguity[0]).reshape(256), dtype=np.uint8)
            self._cmap = np.ascontiguousarray(np.asarray(ambiguity[1]).reshape(256 * 64), dtype=np.uint8)
            ub = C.POINTER(C.c_ubyte)
            _lib.check(self._L.gb_create_unclean(C.byref(self._prob), self._nch.ctypes.data_as(ub),
                                                 self._cmap.ctypes.data_as(ub), C.byref(h)))
        self._h = h
        for knob, value in (tuning or {}).items():
            _lib.check(self._L.gb_tune(self._h, _lib.TUNE[knob], int(value)))
        self.bnode = np.ascontiguousarray(tree.branch_nodes(), dtype=np.int32)

    @property
    def nscale(self) -> int:
        return int(self._L.gb_nscale(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.gb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def neg_lnL_uvr(self, U, V, Root, qfactor, freqK, blength, want_site=True) -> EvalResult:
        U = [np.ascontiguousarray(u, dtype=np.float64) for u in U]
        V = [np.ascontiguousarray(v, dtype=np.float64) for v in V]
        R = [np.ascontiguousarray(r, dtype=np.float64) for r in Root]
        qf = np.ascontiguousarray(qfactor, dtype=np.float64)
        fk = np.ascontiguousarray(freqK, dtype=np.float64)
        bl = np.ascontiguousarray(blength, dtype=np.float64)
        f = C.c_double(0)
        fhK = np.zeros((4, self.npatt)) if want_site else None
        lnf = np.zeros(self.npatt) if want_site else None
        st = _lib.Stats()
        arr3 = _dp * 3
        _lib.check(self._L.gb_eval_uvr(self._h, arr3(*[_ptr(u) for u in U]), arr3(*[_ptr(v) for v in V]),
                                       arr3(*[_ptr(r) for r in R]), _ptr(qf), _ptr(fk), _ptr(bl),
                                       C.byref(f), _ptr(fhK) if want_site else None,
                                       _ptr(lnf) if want_site else None, C.byref(st)))
        return EvalResult(f.value, fhK, lnf, None, st.ms_device, st.ms_host, st.kernels)

    def clade(self, blength, kappa, p0, p1, w0, w2, w3, w1: float = 1.0, grad: bool = False):
        """Clade model C (w1 = 1) or D (w1 free) with two branch types from
        its parameters (gb_eval_clade: the library's eigen solutions and
        Qfactors; w2 on branch type 0, w3 on type 1).  FP64 handles.
        Returns (-lnL, fhK [3, npatt], lnf), with grad a fourth item: the
        gradient of -lnL as a dict (blength in node order, kappa, p0, p1, w0,
        w1, w2, w3)."""
        bl = np.ascontiguousarray(blength, dtype=np.float64)
        om = np.ascontiguousarray([w0, w1, w2, w3], dtype=np.float64)
        f = C.c_double(0)
        fhK = np.zeros((3, self.npatt))
        lnf = np.zeros(self.npatt)
        g = np.zeros(self.nnode + 7) if grad else None
        st = _lib.Stats()
        _lib.check(self._L.gb_eval_clade(self._h, _ptr(bl), float(kappa), float(p0), float(p1), _ptr(om),
                                         C.byref(f), _ptr(g) if grad else None, _ptr(fhK), _ptr(lnf), C.byref(st)))
        self.last_ms = st.ms_device
        if not grad:
            return f.value, fhK, lnf
        nn = self.nnode
        names = ("kappa", "p0", "p1", "omega0", "omega1", "omega2", "omega3")
        gd = {"blength": g[:nn].copy(), **{k: float(g[nn + i]) for i, k in enumerate(names)}}
        return f.value, fhK, lnf, gd

    def neb_clade(self, blength, kappa, p0, p1, w0, w2, w3, w1: float = 1.0):
        """codeml's NEB site-class posteriors under clade model C / D
        (gb_neb_clade): (post [3, npatt], -lnL)."""
        bl = np.ascontiguousarray(blength, dtype=np.float64)
        om = np.ascontiguousarray([w0, w1, w2, w3], dtype=np.float64)
        post = np.zeros((3, self.npatt))
        f = C.c_double(0)
        _lib.check(self._L.gb_neb_clade(self._h, _ptr(bl), float(kappa), float(p0), float(p1), _ptr(om),
                                        _ptr(post), C.byref(f)))
        return post, f.value

    def dfun_clade_x(self, x, lastround: bool = True, model_d: bool = False):
        """(-lnL, gradient) of a clade model in codeml's x space (gb_dfun_clade_x:
        branch lengths, kappa, p0, p1, w0, [w1 under clade D], w2, w3)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        dx = np.zeros_like(x)
        f = C.c_double(0)
        bn = np.ascontiguousarray(self.bnode, dtype=np.int32)
        _lib.check(self._L.gb_dfun_clade_x(self._h, bn.ctypes.data_as(C.POINTER(C.c_int)), int(lastround),
                                           int(model_d), _ptr(x), len(x), C.byref(f), _ptr(dx)))
        return f.value, dx

    def m7(self, blength, kappa, p, q, K: int = 10):
        """Site model M7 (beta, K categories) on a tree with every branch
        labelled foreground: (-lnL, fhK [K, npatt], lnf)."""
        om, pr = beta_classes(p, q, K)
        return self.site_model(blength, kappa, om, pr)

    def m8(self, blength, kappa, p0, p, q, ws, K: int = 10):
        """Site model M8 (beta with weight p0, K categories, and omega_s with
        1 - p0) on a tree with every branch labelled foreground: (-lnL, fhK
        [K + 1, npatt], lnf)."""
        om, pr = beta_classes(p, q, K)
        return self.site_model(blength, kappa, np.append(om, ws), np.append(pr * p0, 1 - p0))

    def site_model(self, blength, kappa, omegas, props):
        """A site model with K classes (codeml model = 0: M1a, M2a, M3, M7,
        M8, ...): class k has omegas[k] on every branch and weight props[k],
        Qfactor_NS = 1 / meanrate(Q(kappa, sum props omegas))
        (SetParametersNSsites codeml.c:2466-2487).  The handle's tree must
        have every branch labelled foreground: each gb_eval_uvr call then
        prunes three classes (eigen slots 0, 1, 2), so K classes take
        ceil(K / 3) calls; the mixture follows codeml's lfundG.  Eigen
        solutions from the library's host code.  Returns (-lnL, fhK [K,
        npatt], lnf)."""
        lab = np.asarray(self.tree.label).copy()
        lab[self.tree.root] = 1
        if not np.all(lab == 1):
            raise ValueError("site_model needs every branch labelled foreground")
        om = np.asarray(omegas, dtype=np.float64)
        pr = np.asarray(props, dtype=np.float64)
        U, V, R, _, _ = model_setup(self._pi, kappa, float(pr @ om), 1.0, 0.5, 0.3)
        mr = -float(np.sum(self._pi * np.einsum("im,m,mi->i", U[0], R[0], V[0])))
        qf = np.array([1.0 / mr, 1.0 / mr])
        eig = [model_setup(self._pi, kappa, float(w), 1.0, 0.5, 0.3) for w in om]
        fk4 = np.full(4, 0.25)
        rows = []
        for c in range(0, len(om), 3):
            grp = list(range(c, min(c + 3, len(om))))
            sl = grp + [grp[-1]] * (3 - len(grp))
            r = self.neg_lnL_uvr([eig[k][0][0] for k in sl], [eig[k][1][0] for k in sl],
                                 [eig[k][2][0] for k in sl], qf, fk4, blength)
            rows += [r.fhK[0], r.fhK[1], r.fhK[2]][: len(grp)]
        fhK = np.stack(rows)
        if self.nscale:
            t = fhK.max(axis=0)
            lnf = t + np.log((pr[:, None] * np.exp(fhK - t)).sum(axis=0))
        else:
            sm = (pr[:, None] * fhK).sum(axis=0)
            lnf = np.log(np.where(sm <= 0, 1e-300, sm))
        return -float((lnf * self._fpatt).sum()), fhK, lnf

    def site_classes_x(self, x, model: str):
        """(blength in node order, kappa, omegas, props) of a site model at
        codeml's x (branch lengths in codeml's branch order, then M1a: kappa,
        p0, w0; M2a: kappa, p0, p1, w0, w2; M3 (three classes): kappa, p0,
        p1, w0, w1, w2; M7: kappa, p, q; M8: kappa, p0, p, q, ws)."""
        x = np.asarray(x, dtype=np.float64)
        nb = self.nnode - 1
        bl = np.zeros(self.nnode)
        bl[self.bnode] = x[:nb]
        k, r = x[nb], x[nb + 1:]
        if model == "M1a":
            om, pr = np.array([r[1], 1.0]), np.array([r[0], 1 - r[0]])
        elif model == "M2a":
            om, pr = np.array([r[2], 1.0, r[3]]), np.array([r[0], r[1], 1 - r[0] - r[1]])
        elif model == "M3":
            om, pr = np.array(r[2:5]), np.array([r[0], r[1], 1 - r[0] - r[1]])
        elif model == "M7":
            om, pr = beta_classes(r[0], r[1])
        elif model == "M8":
            om, pr = beta_classes(r[1], r[2])
            om, pr = np.append(om, r[3]), np.append(pr * r[0], 1 - r[0])
        else:
            raise ValueError("site model: M1a, M2a, M3, M7 or M8")
        return bl, k, om, pr

    def se_opg_site(self, x, model: str, small_diff: float = 1e-6) -> dict:
        """codeml's standard errors (getSE = 1, HessianSKT2004 treesub.c:
        6979-7048) under a site model at codeml's x (site_classes_x; the
        proportions untransformed): per-pattern scores from central
        differences of log f_h, step 2 small_diff (|x_i| + 1), over 2 n
        site_model evaluations on the device; H = -sum_h fpatt_h s_h s_h^T,
        SE_i = sqrt([(-H)^-1]_ii) (-1 where not positive).  Needs the
        all-foreground tree of site_model."""
        x = np.asarray(x, dtype=np.float64)
        n = len(x)
        nb = self.nnode - 1
        eh = 2 * small_diff * (np.abs(x) + 1)
        D = np.zeros((n, self.npatt))
        lnL = np.zeros((2, n))
        for i in range(n):
            for bf, sgn in enumerate((-1.0, 1.0)):
                x1 = x.copy()
                x1[i] += sgn * eh[i]
                if i < nb:
                    x1[i] = max(x1[i], 0.0)        # a length moved below zero acts as zero
                f, _, lnf = self.site_model(*self.site_classes_x(x1, model))
                lnL[bf, i] = -f
                D[i] += sgn * lnf / (2 * eh[i])
        H = -(D * self._fpatt[None, :]) @ D.T
        H = 0.5 * (H + H.T)
        g = (lnL[1] - lnL[0]) / (2 * eh)
        try:
            V = np.linalg.inv(-H)
            dg = np.diag(V)
            se = np.where(dg > 0, np.sqrt(np.abs(dg)), -1.0)
        except np.linalg.LinAlgError:
            se = np.full(n, -1.0)
        return {"g": g, "H": H, "se": se}

    def site_neb(self, fhK, props):
        """codeml's NEB posteriors of a site model's classes (lfunNSsites_rate
        codeml.c:5079-5129: props_k f_k normalised over k, from site_model's
        fhK; log values shifted by their maximum when nodes are scaled):
        [K, npatt]."""
        fhK = np.asarray(fhK, dtype=np.float64)
        pr = np.asarray(props, dtype=np.float64)
        f = np.exp(fhK - fhK.max(axis=0)) if self.nscale else fhK
        q = pr[:, None] * f
        return q / q.sum(axis=0)

    def clade_uvr(self, U, V, Root, qfactor, freqK, blength, two_calls: bool = False):
        """Clade models C / D with two branch types from the host's eigen
        solutions of (w0, w1, w2 background, w3 foreground) -- codeml's
        _UU/_VV/_Root[0..3] and Qfactor_NS_branch -- and the three class
        weights.  FP64 handles: one gb_eval_clade_uvr call (three classes at
        every internal node).  Split-precision handles, or two_calls: two
        gb_eval_uvr calls (classes 0 and 1 are model A's with slots (w0, w1,
        -), the third is model A's class 2a with slots (w2, w1, w3)), then
        codeml's mixture of the three classes (lfundG treesub.c:7342-7394).
        Returns (-lnL, fhK [3, npatt], lnf) and keeps the call's device time
        in self.last_ms."""
        if self._fp64 and not two_calls:
            arr4 = _dp * 4
            U = [np.ascontiguousarray(u, dtype=np.float64) for u in U]
            V = [np.ascontiguousarray(v, dtype=np.float64) for v in V]
            R = [np.ascontiguousarray(r, dtype=np.float64) for r in Root]
            qf = np.ascontiguousarray(qfactor, dtype=np.float64)
            fk = np.ascontiguousarray(np.asarray(freqK, dtype=np.float64)[:3])
            bl = np.ascontiguousarray(blength, dtype=np.float64)
            f = C.c_double(0)
            fhK = np.zeros((3, self.npatt))
            lnf = np.zeros(self.npatt)
            st = _lib.Stats()
            _lib.check(self._L.gb_eval_clade_uvr(self._h, arr4(*[_ptr(u) for u in U]), arr4(*[_ptr(v) for v in V]),
                                                 arr4(*[_ptr(r) for r in R]), _ptr(qf), _ptr(fk), _ptr(bl),
                                                 C.byref(f), _ptr(fhK), _ptr(lnf), C.byref(st)))
            self.last_ms = st.ms_device
            return f.value, fhK, lnf
        fk4 = np.full(4, 0.25)           # the calls' own mixture is not used
        a = self.neg_lnL_uvr(U[:3], V[:3], Root[:3], qfactor, fk4, blength)
        b = self.neg_lnL_uvr([U[2], U[1], U[3]], [V[2], V[1], V[3]], [Root[2], Root[1], Root[3]],
                             qfactor, fk4, blength)
        self.last_ms = a.ms_device + b.ms_device
        fhK = np.stack([a.fhK[0], a.fhK[1], b.fhK[2]])
        fk = np.asarray(freqK, dtype=np.float64)[:3]
        if self.nscale:
            t = fhK.max(axis=0)
            lnf = t + np.log((fk[:, None] * np.exp(fhK - t)).sum(axis=0))
        else:
            sm = (fk[:, None] * fhK).sum(axis=0)
            lnf = np.log(np.where(sm <= 0, 1e-300, sm))
        return -float((lnf * self._fpatt).sum()), fhK, lnf

    def evaluate(self, blength, kappa, omega0, omega2, p0, p1, grad: bool = False,
                 want_site: bool = False, omega1: float | None = None) -> EvalResult:
        """-lnL (and gradient) of branch-site model A, or with omega1 given of
        model B (w1 free, gb_eval_b; the gradient then has "omega1" too)."""
        bl = np.ascontiguousarray(blength, dtype=np.float64)
        prm = _lib.Params(_ptr(bl), kappa, omega0, omega2, p0, p1)
        f = C.c_double(0)
        st = _lib.Stats()
        g = None
        dbl = None
        if grad:
            dbl = np.zeros(self.nnode)
            g = _lib.Grad(_ptr(dbl), 0, 0, 0, 0, 0)
        fhK = np.zeros((4, self.npatt)) if want_site else None
        lnf = np.zeros(self.npatt) if want_site else None
        dw1 = C.c_double(0)
        if omega1 is None:
            _lib.check(self._L.gb_eval(self._h, C.byref(prm), C.byref(f), C.byref(g) if grad else None,
                                       _ptr(fhK) if want_site else None, _ptr(lnf) if want_site else None,
                                       C.byref(st)))
        else:
            _lib.check(self._L.gb_eval_b(self._h, C.byref(prm), float(omega1), C.byref(f),
                                         C.byref(g) if grad else None, C.byref(dw1),
                                         _ptr(fhK) if want_site else None, _ptr(lnf) if want_site else None,
                                         C.byref(st)))
        gd = None
        if grad:
            gd = {"blength": dbl, "kappa": g.d_kappa, "omega0": g.d_omega0, "omega2": g.d_omega2,
                  "p0": g.d_p0, "p1": g.d_p1}
            if omega1 is not None:
                gd["omega1"] = dw1.value
        return EvalResult(f.value, fhK, lnf, gd, st.ms_device, st.ms_host, st.kernels,
                          st.h2d_bytes, st.d2h_bytes)

    def replay(self, iters: int, with_grad: bool) -> float:
        """Device ms for `iters` re-runs of the last evaluation with inputs resident."""
        ms = C.c_double(0)
        _lib.check(self._L.gb_replay(self._h, int(iters), int(with_grad), C.byref(ms)))
        return ms.value

    def profile(self, iters: int, with_grad: bool) -> dict:
        """Per kernel class: (device ms summed over iters, launches)."""
        ms = np.zeros(len(_lib.KCLASS))
        n = np.zeros(len(_lib.KCLASS), dtype=np.int32)
        _lib.check(self._L.gb_profile(self._h, int(iters), int(with_grad), _ptr(ms),
                                      n.ctypes.data_as(C.POINTER(C.c_int))))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(_lib.KCLASS)}

    def task_trace(self, kernel: int) -> np.ndarray:
        """[ntask, 12] uint64 trace of the last evaluation's persistent kernel
        (0 pruning, 1 adjoint propagation, 2 dlnL/dP): gene, item, tile, edge
        (adjoint: child edge of a split item, -1 as two's complement for a whole item),
        claim ns, dependencies-met ns, four phase stamps (0 if absent), end ns, SM.  Needs GBCODEML_TRACE=1 in
        the environment before the first evaluation of this handle."""
        n = self._L.gb_task_trace(self._h, int(kernel), None, 0)
        if n < 0:
            _lib.check(n)
        out = np.zeros((n, 12), dtype=np.uint64)
        r = self._L.gb_task_trace(self._h, int(kernel), out.ctypes.data_as(C.POINTER(C.c_ulonglong)), n)
        if r < 0:
            _lib.check(r)
        return out

    def evaluate_x(self, x, lastround: bool = True, grad: bool = False) -> EvalResult:
        """-lnL (and gradient in node order) from codeml's x vector."""
        x = np.asarray(x, dtype=np.float64)
        nb = self.nnode - 1
        bl = np.zeros(self.nnode)
        bl[self.bnode] = x[:nb]
        kappa, w0, w2 = x[nb], x[nb + 3], x[nb + 4]
        if lastround:
            p0, p1 = x[nb + 1], x[nb + 2]
        else:
            e = np.exp(x[nb + 1:nb + 3])
            p0, p1 = e / (1 + e.sum())
        return self.evaluate(bl, kappa, w0, w2, p0, p1, grad=grad)

    def beb(self, blength, kappa, omega0, omega2, p0, p1, want_lnfw: bool = False) -> dict:
        """Bayes empirical Bayes site analysis of model A at these (MLE)
        parameters (gb_beb; codeml's lfunNSsites_ACD, codeml.c:6617-6826).
        Needs an FP64 handle.  Returns post [4, npatt] (classes 0, 1, 2a, 2b),
        grid [4, 10] (rows p0, p1 = -1, w0, w2), p0p1 [100], lnfX, S1, S2,
        lnfw [121, npatt] when asked for, and the call's device / host ms."""
        bl = np.ascontiguousarray(blength, dtype=np.float64)
        prm = _lib.Params(_ptr(bl), kappa, omega0, omega2, p0, p1)
        lnfw = np.zeros((121, self.npatt)) if want_lnfw else None
        post = np.zeros((4, self.npatt))
        grid = np.zeros((4, 10))
        p0p1 = np.zeros(100)
        fx = np.zeros(3)
        st = _lib.Stats()
        _lib.check(self._L.gb_beb(self._h, C.byref(prm), _ptr(lnfw) if want_lnfw else None, _ptr(post),
                                  _ptr(grid), _ptr(p0p1), _ptr(fx), C.byref(st)))
        return {"post": post, "grid": grid, "p0p1": p0p1, "lnfX": float(fx[0]), "S1": float(fx[1]),
                "S2": float(fx[2]), "lnfw": lnfw, "ms_device": st.ms_device, "ms_host": st.ms_host,
                "kernels": st.kernels}

    def neb_x(self, x, lastround: bool = True):
        """(post [4, npatt], -lnL): the NEB posteriors of the four site classes
        at codeml's x (gb_neb; FP64 handle)."""
        x = np.asarray(x, dtype=np.float64)
        nb = self.nnode - 1
        bl = np.zeros(self.nnode)
        bl[self.bnode] = x[:nb]
        kappa, w0, w2 = x[nb], x[nb + 3], x[nb + 4]
        if lastround:
            p0, p1 = x[nb + 1], x[nb + 2]
        else:
            e = np.exp(x[nb + 1:nb + 3])
            p0, p1 = e / (1 + e.sum())
        bl = np.ascontiguousarray(bl)
        prm = _lib.Params(_ptr(bl), kappa, w0, w2, p0, p1)
        post = np.zeros((4, self.npatt))
        f = C.c_double(0)
        _lib.check(self._L.gb_neb(self._h, C.byref(prm), _ptr(post), C.byref(f)))
        return post, f.value

    def beb_qf(self, blength, kappa, qfactor, want_lnfw: bool = False) -> dict:
        """beb() with the branch Qfactors given (gb_beb_qf): model B, or a
        caller holding codeml's Qfactor_NS_branch.  Also returns wmean / wsd,
        the posterior mean and SD of each pattern's w."""
        bl = np.ascontiguousarray(blength, dtype=np.float64)
        qf = np.ascontiguousarray(qfactor, dtype=np.float64)
        lnfw = np.zeros((121, self.npatt)) if want_lnfw else None
        post = np.zeros((4, self.npatt))
        grid = np.zeros((4, 10))
        p0p1 = np.zeros(100)
        fx = np.zeros(3)
        st = _lib.Stats()
        wmean = np.zeros(self.npatt)
        wsd = np.zeros(self.npatt)
        _lib.check(self._L.gb_beb_qf(self._h, _ptr(bl), float(kappa), _ptr(qf),
                                     _ptr(lnfw) if want_lnfw else None, _ptr(post), _ptr(grid), _ptr(p0p1),
                                     _ptr(fx), _ptr(wmean), _ptr(wsd), C.byref(st)))
        return {"post": post, "grid": grid, "p0p1": p0p1, "lnfX": float(fx[0]), "S1": float(fx[1]),
                "S2": float(fx[2]), "lnfw": lnfw, "wmean": wmean, "wsd": wsd, "ms_device": st.ms_device,
                "ms_host": st.ms_host, "kernels": st.kernels}

    def beb_tables(self, blength, kappa, qfactor, w_slot0, w_slot2):
        """The 121 log f(x_h | w) tables with other omega grids (gb_beb_tables)."""
        bl = np.ascontiguousarray(blength, dtype=np.float64)
        qf = np.ascontiguousarray(qfactor, dtype=np.float64)
        g0 = np.ascontiguousarray(w_slot0, dtype=np.float64)
        g2 = np.ascontiguousarray(w_slot2, dtype=np.float64)
        lnfw = np.zeros((121, self.npatt))
        st = _lib.Stats()
        _lib.check(self._L.gb_beb_tables(self._h, _ptr(bl), float(kappa), _ptr(qf), _ptr(g0), _ptr(g2),
                                         _ptr(lnfw), C.byref(st)))
        return lnfw

    def beb_clade(self, lnfw, model_d: bool = False) -> dict:
        """The grid integral of codeml's BEB under clade model C (111 log f
        tables) or D (model_d: 120 tables) on the device (gb_beb_clade):
        post [3, npatt], grid [4, 10] (rows w0, w1 (-1 under C), w2, w3), p0p1
        [100], lnfX as codeml prints it, S1, S2, ms_device."""
        L = np.ascontiguousarray(lnfw, dtype=np.float64)
        assert L.shape == ((120 if model_d else 111), self.npatt)
        post = np.zeros((3, self.npatt))
        grid = np.zeros((4, 10))
        p0p1 = np.zeros(100)
        fx = np.zeros(3)
        st = _lib.Stats()
        _lib.check(self._L.gb_beb_clade(self._h, int(bool(model_d)), _ptr(L), _ptr(post), _ptr(grid), _ptr(p0p1),
                                        _ptr(fx), C.byref(st)))
        return {"post": post, "grid": grid, "p0p1": p0p1, "lnfX": float(fx[0]), "S1": float(fx[1]),
                "S2": float(fx[2]), "ms_device": st.ms_device}

    def beb_clade_c(self, blength, kappa, qfactor) -> dict:
        """codeml's BEB under clade model C with two branch types at the MLE
        (Qfactors qfactor of the two branch types; gb_beb_clade_bl): the 111
        omega sets from two gb_beb_tables calls (w0 grid in (0, 1); then the
        (0, 3) grids of w2 and w3 in eigen slots 0 and 2) and the 10^5-point
        grid integral, all on the device."""
        return self._beb_clade_bl(blength, kappa, qfactor, False)

    def _beb_clade_bl(self, blength, kappa, qfactor, model_d):
        bl = np.ascontiguousarray(blength, dtype=np.float64)
        qf = np.ascontiguousarray(qfactor, dtype=np.float64)
        post = np.zeros((3, self.npatt))
        grid = np.zeros((4, 10))
        p0p1 = np.zeros(100)
        fx = np.zeros(3)
        st = _lib.Stats()
        _lib.check(self._L.gb_beb_clade_bl(self._h, int(bool(model_d)), _ptr(bl), float(kappa), _ptr(qf),
                                           _ptr(post), _ptr(grid), _ptr(p0p1), _ptr(fx), C.byref(st)))
        return {"post": post, "grid": grid, "p0p1": p0p1, "lnfX": float(fx[0]), "S1": float(fx[1]),
                "S2": float(fx[2]), "ms_device": st.ms_device}

    def beb_clade_d(self, blength, kappa, qfactor) -> dict:
        """codeml's BEB under clade model D with two branch types at the MLE:
        120 omega sets (w0 in (0, 0.5), w1 in (0.5, 1.5) on every branch; w2, w3
        in (0, 3) by branch type; get_grid_para_like_ACD codeml.c:6457-6473)
        from three gb_beb_tables calls, and the 10^6-point grid integral, on
        the device."""
        return self._beb_clade_bl(blength, kappa, qfactor, True)

    def beb_x(self, x, lastround: bool = True, want_lnfw: bool = False) -> dict:
        """beb() from codeml's x vector."""
        x = np.asarray(x, dtype=np.float64)
        nb = self.nnode - 1
        bl = np.zeros(self.nnode)
        bl[self.bnode] = x[:nb]
        kappa, w0, w2 = x[nb], x[nb + 3], x[nb + 4]
        if lastround:
            p0, p1 = x[nb + 1], x[nb + 2]
        else:
            e = np.exp(x[nb + 1:nb + 3])
            p0, p1 = e / (1 + e.sum())
        return self.beb(bl, kappa, w0, w2, p0, p1, want_lnfw=want_lnfw)

    def se_opg(self, x, small_diff: float = 1e-6) -> dict:
        """codeml's standard errors (getSE = 1, HessianSKT2004) at codeml's x
        with untransformed p0, p1 (gb_se_opg; FP64 handle): g = dlnL/dx,
        H (codeml's, before negation) and se."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = len(x)
        g = np.zeros(n)
        H = np.zeros((n, n))
        se = np.zeros(n)
        st = _lib.Stats()
        _lib.check(self._L.gb_se_opg(self._h, self.bnode.ctypes.data_as(C.POINTER(C.c_int)), _ptr(x), n,
                                     float(small_diff), _ptr(g), _ptr(H), _ptr(se), C.byref(st)))
        return {"g": g, "H": H, "se": se, "ms_device": st.ms_device, "ms_host": st.ms_host,
                "kernels": st.kernels}

    def se_opg_clade(self, x, model_d: bool = False, small_diff: float = 1e-6) -> dict:
        """codeml's standard errors under clade model C / D at codeml's x
        (untransformed p0, p1; gb_se_opg_clade): g, H (before negation), se."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = len(x)
        g = np.zeros(n)
        H = np.zeros((n, n))
        se = np.zeros(n)
        _lib.check(self._L.gb_se_opg_clade(self._h, self.bnode.ctypes.data_as(C.POINTER(C.c_int)), int(model_d),
                                           _ptr(x), n, float(small_diff), _ptr(g), _ptr(H), _ptr(se)))
        return {"g": g, "H": H, "se": se}

    def hessian_x(self, x, lastround: bool = True, rel_step: float = 0.0):
        """(H, se): the Hessian of -lnL over codeml's x by central differences
        of the analytic gradient (gb_hessian_x) and the SEs from its inverse."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = len(x)
        H = np.zeros((n, n))
        se = np.zeros(n)
        _lib.check(self._L.gb_hessian_x(self._h, self.bnode.ctypes.data_as(C.POINTER(C.c_int)),
                                        int(lastround), _ptr(x), n, float(rel_step), _ptr(H), _ptr(se)))
        return H, se

    def dfun_x(self, x, lastround: bool = True):
        """(f, dx) as ming2's dfun hook: f = -lnL, dx = d(-lnL)/dx in codeml's x space."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = C.c_double(0)
        dx = np.zeros(len(x))
        _lib.check(self._L.gb_dfun_x(self._h, self.bnode.ctypes.data_as(C.POINTER(C.c_int)),
                                     int(lastround), _ptr(x), len(x), C.byref(f), _ptr(dx)))
        return f.value, dx


class Batch:
    """Many independent alignments evaluated together (gb_batch_*): one CUDA
    graph launch per evaluation (split precision: one persistent launch per
    phase over all genes; FP64: each gene an independent branch)."""

    def __init__(self, genes, precision: str = "fast", device: int = 0, tuning: dict | None = None):
        """genes: list of (tree, z, fpatt, pi)."""
        self._L = _lib.load()
        prec = precision if isinstance(precision, int) else \
            {"fp64": _lib.GB_PREC_FP64, "fast": _lib.GB_PREC_FAST}[precision]
        ip = C.POINTER(C.c_int)
        self._keep = []
        probs = (_lib.Problem * len(genes))()
        self.trees = []
        for i, (tree, z, fpatt, pi) in enumerate(genes):
            father = np.ascontiguousarray(tree.father, dtype=np.int32)
            label = np.ascontiguousarray(tree.label, dtype=np.int32)
            z = np.ascontiguousarray(z, dtype=np.uint8)
            fpatt = np.ascontiguousarray(fpatt, dtype=np.float64)
            pi = np.ascontiguousarray(pi, dtype=np.float64)
            self._keep += [father, label, z, fpatt, pi]
            probs[i] = _lib.Problem(tree.ns, tree.nnode, tree.root, father.ctypes.data_as(ip),
                                    label.ctypes.data_as(ip), len(fpatt),
                                    z.ctypes.data_as(C.POINTER(C.c_ubyte)), _ptr(fpatt), _ptr(pi), None,
                                    prec, device)
            self.trees.append(tree)
        h = C.c_void_p()
        _lib.check(self._L.gb_batch_create(len(genes), probs, C.byref(h)))
        self._h = h
        for knob, value in (tuning or {}).items():
            _lib.check(self._L.gb_batch_tune(self._h, _lib.TUNE[knob], int(value)))
        self.n = len(genes)

    def close(self):
        if getattr(self, "_h", None):
            self._L.gb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def evaluate(self, params, grad: bool = False):
        """params: list of dicts (blength, kappa, omega0, omega2, p0, p1) per gene,
        each with omega1 as well for branch-site model B (gb_batch_submit_b;
        its gradient then has "omega1").  Returns (neg_lnL [n], grads list or
        None, EvalResult stats)."""
        if any("omega1" in p for p in params):
            self.submit(params, grad)
            return self.collect()
        n = self.n
        pr = (_lib.Params * n)()
        keep = []
        for i, p in enumerate(params):
            bl = np.ascontiguousarray(p["blength"], dtype=np.float64)
            keep.append(bl)
            pr[i] = _lib.Params(_ptr(bl), p["kappa"], p["omega0"], p["omega2"], p["p0"], p["p1"])
        out = np.zeros(n)
        gr = None
        dbl = []
        if grad:
            gr = (_lib.Grad * n)()
            for i in range(n):
                d = np.zeros(self.trees[i].nnode)
                dbl.append(d)
                gr[i] = _lib.Grad(_ptr(d), 0, 0, 0, 0, 0)
        st = _lib.Stats()
        _lib.check(self._L.gb_batch_eval(self._h, pr, _ptr(out), gr, C.byref(st)))
        grads = None
        if grad:
            grads = [{"blength": dbl[i], "kappa": gr[i].d_kappa, "omega0": gr[i].d_omega0,
                      "omega2": gr[i].d_omega2, "p0": gr[i].d_p0, "p1": gr[i].d_p1} for i in range(n)]
        return out, grads, EvalResult(float(out.sum()), None, None, None, st.ms_device, st.ms_host,
                                      st.kernels, st.h2d_bytes, st.d2h_bytes)

    def submit(self, params, grad: bool = False, after: "Batch | None" = None) -> None:
        """Host set-up and graph launch of one evaluation without waiting
        (gb_batch_submit); after: another batch whose submitted evaluation the
        device runs first.  collect() returns the results."""
        n = self.n
        pr = (_lib.Params * n)()
        self._keep_bl = []
        for i, p in enumerate(params):
            bl = np.ascontiguousarray(p["blength"], dtype=np.float64)
            self._keep_bl.append(bl)
            pr[i] = _lib.Params(_ptr(bl), p["kappa"], p["omega0"], p["omega2"], p["p0"], p["p1"])
        self._pending_grad = bool(grad)
        self._pending_b = any("omega1" in p for p in params)
        ah = after._h if after is not None else None
        if self._pending_b:
            self._omega1 = np.ascontiguousarray([p.get("omega1", 1.0) for p in params], dtype=np.float64)
            _lib.check(self._L.gb_batch_submit_b(self._h, pr, _ptr(self._omega1), int(grad), ah))
        else:
            _lib.check(self._L.gb_batch_submit(self._h, pr, int(grad), ah))

    def collect(self):
        """(neg_lnL [n], grads or None, EvalResult stats) of the submitted evaluation."""
        n = self.n
        out = np.zeros(n)
        gr, dbl = None, []
        if self._pending_grad:
            gr = (_lib.Grad * n)()
            for i in range(n):
                d = np.zeros(self.trees[i].nnode)
                dbl.append(d)
                gr[i] = _lib.Grad(_ptr(d), 0, 0, 0, 0, 0)
        st = _lib.Stats()
        _lib.check(self._L.gb_batch_collect(self._h, _ptr(out), gr, C.byref(st)))
        grads = None
        if gr is not None:
            grads = [{"blength": dbl[i], "kappa": gr[i].d_kappa, "omega0": gr[i].d_omega0,
                      "omega2": gr[i].d_omega2, "p0": gr[i].d_p0, "p1": gr[i].d_p1} for i in range(n)]
            if getattr(self, "_pending_b", False):
                dw1 = np.zeros(n)
                _lib.check(self._L.gb_batch_omega1_grad(self._h, _ptr(dw1)))
                for i in range(n):
                    grads[i]["omega1"] = float(dw1[i])
        return out, grads, EvalResult(float(out.sum()), None, None, None, st.ms_device, st.ms_host,
                                      st.kernels, st.h2d_bytes, st.d2h_bytes)

    def replay(self, iters: int, with_grad: bool) -> float:
        ms = C.c_double(0)
        _lib.check(self._L.gb_batch_replay(self._h, int(iters), int(with_grad), C.byref(ms)))
        return ms.value


class PipelinedBatch:
    """The genes of a batch in two halves (two gb_batch objects), evaluated
    alternately with gb_batch_submit / gb_batch_collect: while the device runs
    one half's graph, the host sets up the other half (eigen solutions, chain
    rule), so a stream of evaluations runs at the device's rate.  evaluate()
    has Batch.evaluate's results; evaluate_many() pipelines a sequence of
    parameter sets (independent evaluations, e.g. many starting points)."""

    def __init__(self, genes, precision: str = "fast", device: int = 0, tuning: dict | None = None):
        self.n = len(genes)
        self.cut = (self.n + 1) // 2
        self.half = [Batch(genes[:self.cut], precision, device, tuning),
                     Batch(genes[self.cut:], precision, device, tuning)]

    def close(self):
        for b in self.half:
            b.close()

    def evaluate_many(self, param_sets, grad: bool = False):
        """[(neg_lnL [n], grads or None)] for each parameter set, pipelined."""
        A, B = self.half
        out = []
        prev_b = None
        for prm in param_sets:
            A.submit(prm[:self.cut], grad, after=B if prev_b is not None else None)
            if prev_b is not None:
                fb, gb_, _ = B.collect()
                out[-1] = (np.concatenate([out[-1][0], fb]), (out[-1][1] + gb_) if grad else None)
            B.submit(prm[self.cut:], grad, after=A)
            fa, ga, _ = A.collect()
            out.append((fa, ga if grad else None))
            prev_b = True
        if prev_b is not None:
            fb, gb_, _ = B.collect()
            out[-1] = (np.concatenate([out[-1][0], fb]), (out[-1][1] + gb_) if grad else None)
        return out

    def evaluate(self, params, grad: bool = False):
        return self.evaluate_many([params], grad)[0]

    def task_trace(self, kernel: int) -> np.ndarray:
        """As Likelihood.task_trace, for the batch's persistent kernels."""
        n = self._L.gb_batch_task_trace(self._h, int(kernel), None, 0)
        if n < 0:
            _lib.check(n)
        out = np.zeros((n, 12), dtype=np.uint64)
        r = self._L.gb_batch_task_trace(self._h, int(kernel), out.ctypes.data_as(C.POINTER(C.c_ulonglong)), n)
        if r < 0:
            _lib.check(r)
        return out
