"""Maximum-likelihood fits of branch-site model A and its null, and the
likelihood-ratio test, driven by the GPU likelihood and its adjoint gradient.

codeml fits both models with ming2 (tools.c:6361-6546), a bounded BFGS whose
gradient comes from finite differences (gradientB, tools.c:6326-6350: forward
differences with step Small_Diff (|x_i| + 1), central ones near the optimum),
because Forestry passes no gradient hook (codeml.c:688).  Here the objective
and gradient come from one call, Likelihood.dfun_x (gb_dfun_x: -lnL and its
adjoint gradient in codeml's x space, p0 and p1 transformed as in f_and_x),
and the minimiser is scipy's bounded L-BFGS-B on codeml's own bounds
(SetxBound, codeml.c:1786-1846):
    branch lengths [4e-6, 50], kappa [1e-4, 999], transformed p's [-99, 99],
    w0 [1e-6, 1], w2 [1, 999] (alternative only; the null fixes w2 = 1).
gradient="fd" replaces the adjoint by codeml's finite differences (one
likelihood evaluation per parameter) for comparison.

    python -m cucodeml_gb300.optimize --taxa 256 --codons 20000 --precision fast
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import api

TB = (4e-6, 50.0)
KAPPA_B = (1e-4, 999.0)
P_B = (-99.0, 99.0)
W0_B = (1e-6, 1.0)
W2_B = (1.0, 999.0)


def bounds(nbranch: int, fix_omega2: bool):
    b = [TB] * nbranch + [KAPPA_B, P_B, P_B, W0_B]
    if not fix_omega2:
        b.append(W2_B)
    return b


def initial_x(tree, kappa=2.0, p0=0.6, p1=0.3, omega0=0.5, omega2=1.5, blength=0.1, fix_omega2=False):
    """Start point in codeml's x space (branch lengths by branch index, kappa,
    log(p0/p2), log(p1/p2), w0[, w2])."""
    p2 = 1.0 - p0 - p1
    x = [blength] * tree.nbranch + [kappa, np.log(p0 / p2), np.log(p1 / p2), omega0]
    if not fix_omega2:
        x.append(omega2)
    return np.array(x, dtype=np.float64)


def fd_gradient(lk, x, f0, step=1e-6):
    """codeml's forward differences (gradientB with xmark = 0 away from the
    optimum): g_i = (f(x + eh e_i) - f0) / eh, eh = step (|x_i| + 1)."""
    g = np.empty_like(x)
    for i in range(len(x)):
        eh = step * (abs(x[i]) + 1.0)
        x1 = x.copy()
        x1[i] += eh
        g[i] = (lk.evaluate_x(x1, lastround=False).neg_lnL - f0) / eh
    return g


def fit(lk, x0, fix_omega2: bool = False, gradient: str = "adjoint", gtol: float = 1e-6,
        maxiter: int = 5000) -> dict:
    """Minimise -lnL over codeml's x (w2 = 1 appended when fix_omega2)."""
    from scipy.optimize import minimize

    nb = lk.nnode - 1
    nev = {"f": 0, "g": 0}
    # the objective is minimised as f - f(x0): same gradient, but L-BFGS-B's
    # relative-reduction test then measures progress against the improvement
    # itself instead of |lnL| (~1e6 for large alignments, where it would stop
    # with lnL still moving in the 5th decimal)
    base = {"f0": None}

    def full(x):
        return np.append(x, 1.0) if fix_omega2 else x

    def fun(x):
        nev["f"] += 1
        if gradient == "adjoint":
            nev["g"] += 1
            f, dx = lk.dfun_x(full(x), lastround=False)
            g = dx[:-1] if fix_omega2 else dx
        else:
            f = lk.evaluate_x(full(x), lastround=False).neg_lnL
            nev["g"] += len(x)
            g = fd_gradient(_Fixed(lk, fix_omega2), x, f)
        if base["f0"] is None:
            base["f0"] = f
        return f - base["f0"], g

    t0 = time.perf_counter()
    res = minimize(fun, x0, jac=True, method="L-BFGS-B", bounds=bounds(nb, fix_omega2),
                   options={"maxiter": maxiter, "maxfun": 4 * maxiter, "gtol": gtol, "ftol": 1e-15,
                            "maxcor": 20})
    secs = time.perf_counter() - t0
    res.fun = float(res.fun) + base["f0"]
    x = full(res.x)
    e = np.exp(x[nb + 1:nb + 3])
    p0, p1 = e / (1.0 + e.sum())
    return {"lnL": float(-res.fun), "x": x.tolist(), "nit": int(res.nit), "calls": nev["f"],
            "lnL_evals": nev["f"] + (nev["g"] if gradient == "fd" else 0),
            "gradients": nev["g"] if gradient == "adjoint" else nev["f"], "seconds": secs,
            "converged": bool(res.success), "message": str(res.message),
            "kappa": float(x[nb]), "p0": float(p0), "p1": float(p1), "omega0": float(x[nb + 3]),
            "omega2": float(x[nb + 4]), "max_abs_projected_grad": _pgrad(res, bounds(nb, fix_omega2))}


class _Fixed:
    """evaluate_x with w2 = 1 appended (null model) for the finite differences."""

    def __init__(self, lk, fix):
        self.lk, self.fix = lk, fix

    def evaluate_x(self, x, lastround=False):
        return self.lk.evaluate_x(np.append(x, 1.0) if self.fix else x, lastround=lastround)


def _pgrad(res, b):
    g = np.asarray(res.jac, dtype=np.float64)
    x = res.x
    lo = np.array([v[0] for v in b])
    hi = np.array([v[1] for v in b])
    pg = np.where((x <= lo) & (g > 0), 0.0, np.where((x >= hi) & (g < 0), 0.0, g))
    return float(np.max(np.abs(pg)))


def lrt(lnl_alt: float, lnl_null: float) -> dict:
    """2 (lnL_alt - lnL_null); p-values against chi2_1 and against the 50:50
    mixture of 0 and chi2_1 (w2 = 1 lies on the boundary)."""
    from scipy.stats import chi2
    s = max(0.0, 2.0 * (lnl_alt - lnl_null))
    return {"LRT": s, "p_chi2_1": float(chi2.sf(s, 1)), "p_mixture": float(0.5 * chi2.sf(s, 1))}


def alt_null(tree, z, fpatt, pi, precision: str = "fast", gradient: str = "adjoint", x0_alt=None,
             gtol: float = 1e-6, x0_null=None) -> dict:
    """Fit the alternative (w2 free) and the null (w2 = 1) from the same start
    (or from x0_alt / x0_null, e.g. another precision's maxima)."""
    lk = api.Likelihood(tree, z, fpatt, pi, precision=precision)
    try:
        xa = initial_x(tree) if x0_alt is None else np.asarray(x0_alt, dtype=np.float64)
        xn = xa[:-1] if x0_null is None else np.asarray(x0_null, dtype=np.float64)[:len(xa) - 1]
        alt = fit(lk, xa, False, gradient, gtol)
        null = fit(lk, xn, True, gradient, gtol)
        # the null maximum is feasible for the alternative (w2 = 1): restart the
        # alternative there if it ended lower (a local optimum)
        if alt["lnL"] < null["lnL"]:
            alt2 = fit(lk, np.asarray(null["x"]), False, gradient, gtol)
            alt2["restarted_from_null"] = True
            if alt2["lnL"] > alt["lnL"]:
                alt = alt2
        return {"precision": precision, "gradient": gradient, "alt": alt, "null": null,
                **lrt(alt["lnL"], null["lnL"])}
    finally:
        lk.close()


def natural_x(x):
    """codeml's x with transformed p0, p1 (f_and_x) -> the same with p0, p1 themselves."""
    x = np.array(x, dtype=np.float64)
    e = np.exp(x[-4:-2])
    x[-4:-2] = e / (1.0 + e.sum())
    return x


def site_analysis(tree, codons, z, fpatt, pi, x_alt, cutoff: float = 0.5) -> dict:
    """What codeml reports after the alternative fit, at its maximum x_alt
    (codeml's x, transformed p0, p1): standard errors (getSE = 1,
    gb_se_opg), NEB and BEB posteriors of the site classes (gb_neb, gb_beb),
    and the sites whose BEB probability of w > 1 (classes 2a + 2b) exceeds
    cutoff, with codeml's * (> 0.95) and ** (> 0.99) marks.  FP64 handle."""
    xn = natural_x(x_alt)
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64")
    try:
        t0 = time.perf_counter()
        se = lk.se_opg(xn)
        neb, _ = lk.neb_x(xn)
        beb = lk.beb_x(xn)
        secs = time.perf_counter() - t0
    finally:
        lk.close()
    key = {tuple(z[:, h]): h for h in range(z.shape[1])}
    pose = np.array([key[tuple(codons[:, i])] for i in range(codons.shape[1])])
    pos = []
    for i, h in enumerate(pose):
        pr = float(beb["post"][2, h] + beb["post"][3, h])
        if pr > cutoff:
            pos.append({"site": i + 1, "prob": pr, "mark": "**" if pr > 0.99 else ("*" if pr > 0.95 else "")})
    return {"x": xn.tolist(), "se": se["se"].tolist(), "lnfX": beb["lnfX"],
            "beb_grid_w0": beb["grid"][2].tolist(), "beb_grid_w2": beb["grid"][3].tolist(),
            "positive_sites_beb": pos,
            "neb_positive_sites": int(np.sum((neb[2] + neb[3])[pose] > cutoff)), "seconds": secs}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--taxa", type=int, default=256)
    ap.add_argument("--codons", type=int, default=20000)
    ap.add_argument("--seed", type=int, default=2025)
    ap.add_argument("--precision", nargs="+", default=["fast", "fp64"])
    ap.add_argument("--gradient", default="adjoint", choices=["adjoint", "fd"])
    ap.add_argument("--gtol", type=float, default=1e-6)
    ap.add_argument("--polish", action="store_true",
                    help="after each non-FP64 fit, continue with the FP64 path from its maxima")
    ap.add_argument("--out", default=None, help="write the JSON result here as well")
    ap.add_argument("--sites", action="store_true",
                    help="after the fits: standard errors, NEB and BEB at the alternative's maximum "
                         "(first precision listed)")
    ap.add_argument("--fd-sample", type=int, default=24,
                    help="lnL evaluations timed per precision to cost codeml's finite-difference "
                         "gradient (np evaluations) and a finite-difference-driven fit")
    a = ap.parse_args(argv)
    from .simulate import simulate
    t0 = time.perf_counter()
    aln = simulate(a.taxa, a.codons, seed=a.seed)
    z, fp, pi = api.patterns(aln.codons)
    out = {"workload": f"{a.taxa} taxa x {a.codons} codons, seeded model-A simulation (seed {a.seed})",
           "patterns": int(len(fp)), "setup_seconds": time.perf_counter() - t0, "fits": []}
    for prec in a.precision:
        r = alt_null(aln.tree, z, fp, pi, precision=prec, gradient=a.gradient, gtol=a.gtol)
        if a.polish and prec != "fp64":
            # continue with the FP64 path from this precision's maxima
            p = alt_null(aln.tree, z, fp, pi, precision="fp64", gradient=a.gradient, gtol=a.gtol,
                         x0_alt=r["alt"]["x"], x0_null=r["null"]["x"])
            r["fp64_polish"] = {m: {k2: p[m][k2] for k2 in ("lnL", "calls", "seconds", "omega2", "converged")}
                                for m in ("alt", "null")}
            r["fp64_polish"]["LRT"] = p["LRT"]
        if a.fd_sample > 0:
            # finite differences cost np lnL evaluations per gradient: time a sample
            lk = api.Likelihood(aln.tree, z, fp, pi, precision=prec)
            x = np.asarray(r["alt"]["x"])
            lk.evaluate_x(x, lastround=False)
            t1 = time.perf_counter()
            for i in range(a.fd_sample):
                x1 = x.copy()
                x1[i % len(x)] += 1e-6 * (abs(x1[i % len(x)]) + 1.0)
                lk.evaluate_x(x1, lastround=False)
            per = (time.perf_counter() - t1) / a.fd_sample
            lk.close()
            npar = len(x)
            calls = r["alt"]["calls"] + r["null"]["calls"]
            r["fd_estimate"] = {"lnL_eval_seconds": per, "fd_gradient_seconds": per * npar,
                                "fd_driven_fits_seconds_if_same_calls": per * (npar + 1) * calls,
                                "adjoint_fits_seconds": r["alt"]["seconds"] + r["null"]["seconds"],
                                "note": "estimate: sampled lnL evaluation time x (np + 1) per call, "
                                        "calls as in the adjoint-driven fits"}
        out["fits"].append(r)
    if a.sites:
        out["sites"] = site_analysis(aln.tree, aln.codons, z, fp, pi, out["fits"][0]["alt"]["x"])
    if len(out["fits"]) > 1:
        # each optimum re-evaluated with the FP64 path
        lk = api.Likelihood(aln.tree, z, fp, pi, precision="fp64")
        for r in out["fits"]:
            for m in ("alt", "null"):
                r[m]["lnL_fp64_at_x"] = -lk.evaluate_x(np.asarray(r[m]["x"]), lastround=False).neg_lnL
        lk.close()
        f0 = out["fits"][0]
        out["max_abs_dlnL_between_paths"] = max(abs(r[m]["lnL"] - f0[m]["lnL"]) for r in out["fits"]
                                                for m in ("alt", "null"))
    s = json.dumps(out, default=float)
    print(s)
    if a.out:
        with open(a.out, "w") as f:
            f.write(s + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
