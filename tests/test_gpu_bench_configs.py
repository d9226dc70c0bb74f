"""Parity at the benchmark's own workloads, against the oracle.

* 64 taxa x 5000 codons, seed 2024, the bench parameters (the headline
  workload): FP64 drop-in and split precision against the oracle, lnL and
  per-pattern log f; the FP64 adjoint gradient (all 130 entries) against
  central finite differences with h = 1e-6 and a five-point stencil of the
  FP64 lnL, twelve entries against a five-point stencil of the oracle, and
  all against codeml's own numerical gradient (gradientB, central, restated
  in the oracle); the split-precision gradient and the FP64 gradient with
  the checkpointed adjoint (GB_TUNE_CHECKPOINT) against the same.
* The batched workload's shape (taxa U{12..48}, codons log-uniform in
  [100, 3000], per-gene kappa, w0, w2): 32 genes through one batch, every
  gene's lnL against the oracle and, for eight of them, the gradient against
  a five-point stencil of the oracle.

Bars (written into each assertion): FP64 lnL 1e-11 relative, per-pattern
log f 1e-11 + 2e-11 |log f| (the two eigensolvers differ by 1e-11 relative
per pattern here, measured on the CPU); split precision |dlnL| <= 1e-6 and
per-pattern |d log f| <= 1e-8; gradients 1e-5 relative to max(1, |g|) plus,
for the h = 1e-6 difference, its own rounding error 4 eps |f| / h.
"""
import numpy as np
import pytest

from cucodeml_gb300 import api
from cucodeml_gb300.simulate import simulate, simulate_batch
from oracle import oracle as O

pytestmark = pytest.mark.gpu

BENCH = (2.0, 0.5, 0.3, 0.3, 3.0)       # kappa, p0, p1, w0, w2 (codeml's x order)


def x_grad(tree, r):
    """The library's gradient (node order, natural parameters) in codeml's x order."""
    g = r.grad
    return np.concatenate([g["blength"][tree.branch_nodes()], [g["kappa"], g["p0"], g["p1"], g["omega0"],
                                                                g["omega2"]]])


def node_blength(tree, x):
    bl = np.zeros(tree.nnode)
    bl[tree.branch_nodes()] = np.asarray(x)[: tree.nbranch]
    return bl


def natural(tree, x):
    nb = tree.nbranch
    return (node_blength(tree, x), x[nb], x[nb + 3], x[nb + 4], x[nb + 1], x[nb + 2])


@pytest.fixture(scope="module")
def bench_case():
    aln = simulate(64, 5000, seed=2024)
    z, fpatt, pi = O.patterns(aln.codons)
    tree = aln.tree
    x = np.concatenate([tree.x_branch_lengths(), BENCH])
    pb = O.Problem(tree, z, fpatt, pi, nthreads=O.max_threads())
    v, fhK, lnf, nsc = pb.neg_lnL(x, True, True)
    return tree, z, fpatt, pi, x, pb, v, lnf


@pytest.mark.parametrize("precision", ["fp64", "fast"])
def test_lnL_and_site_logf_vs_oracle_64x5000(bench_case, precision):
    tree, z, fpatt, pi, x, pb, v, lnf = bench_case
    lk = api.Likelihood(tree, z, fpatt, pi, precision=precision)
    r = lk.evaluate(*natural(tree, x), want_site=True)
    d = abs(r.neg_lnL - v)
    dl = np.abs(r.lnf - lnf)
    print(f"64x5000 {precision}: -lnL {r.neg_lnL:.9f} oracle {v:.9f} |dlnL| {d:.3e} "
          f"max |dlogf| {dl.max():.3e}")
    if precision == "fp64":
        assert d <= 1e-11 * abs(v)
        assert np.all(dl <= 1e-11 + 2e-11 * np.abs(lnf))
    else:
        assert d <= 1e-6
        assert dl.max() <= 1e-8
    lk.close()


@pytest.fixture(scope="module")
def bench_gradients(bench_case):
    tree, z, fpatt, pi, x, pb, v, lnf = bench_case
    out = {}
    for name, precision, tuning in (("fp64", "fp64", None), ("fast", "fast", None),
                                    ("fp64 checkpointed", "fp64", {"checkpoint": 1})):
        lk = api.Likelihood(tree, z, fpatt, pi, precision=precision, tuning=tuning)
        lk.evaluate(*natural(tree, x), grad=True)
        out[name] = x_grad(tree, lk.evaluate(*natural(tree, x), grad=True))
        lk.close()
    assert np.array_equal(out["fp64"], out["fp64 checkpointed"])
    return out


def five_point(f, x, i):
    """Five-point derivative of f along x_i, step 1e-4 (|x_i| + 0.05): truncation O(h^4)."""
    e = 1e-4 * (abs(x[i]) + 0.05)
    fs = []
    for k in (-2, -1, 1, 2):
        xk = x.copy()
        xk[i] += k * e
        fs.append(f(xk))
    return (fs[0] - 8 * fs[1] + 8 * fs[2] - fs[3]) / (12 * e)


@pytest.fixture(scope="module")
def bench_fd(bench_case):
    """Derivatives of the FP64 drop-in's lnL (itself equal to the oracle's to
    1e-11 relative, test above) along all 130 coordinates: central
    differences with h = 1e-6 and a five-point stencil."""
    tree, z, fpatt, pi, x, pb, v, lnf = bench_case
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64")

    def f_gpu(xx):
        return lk.evaluate(*natural(tree, xx)).neg_lnL

    h = 1e-6
    n = len(x)
    c6, f5 = np.zeros(n), np.zeros(n)
    for i in range(n):
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        c6[i] = (f_gpu(xp) - f_gpu(xm)) / (2 * h)
        f5[i] = five_point(f_gpu, x, i)
    lk.close()
    return c6, f5


def test_gradient_vs_central_differences_h1e6_64x5000(bench_case, bench_gradients, bench_fd):
    """All 130 entries against central differences with h = 1e-6 (bar: 1e-5
    relative plus the difference's own rounding error 4 eps |f| / h) and
    against the five-point stencil (1e-5 relative)."""
    tree, z, fpatt, pi, x, pb, v, lnf = bench_case
    c6, f5 = bench_fd
    h = 1e-6
    eps = np.finfo(float).eps
    tol = 1e-5 * np.maximum(1.0, np.abs(c6)) + 4 * eps * abs(v) / h
    for prec, g in bench_gradients.items():
        err = np.abs(g - c6)
        i = int(np.argmax(err / tol))
        print(f"{prec}: max |g - fd_h1e-6| / tol = {(err / tol).max():.3f} at {i} (g {g[i]:.6f} fd {c6[i]:.6f})")
        assert np.all(err <= tol), (prec, i, g[i], c6[i])
        e5 = np.abs(g - f5) / np.maximum(1.0, np.abs(f5))
        print(f"{prec}: max rel err vs five-point stencil {e5.max():.3e}")
        assert e5.max() <= 1e-5


def test_gradient_vs_oracle_differences_64x5000(bench_case, bench_gradients):
    """Twelve entries (the five model parameters, the foreground branch and six
    others) against a five-point stencil of the oracle's own lnL."""
    tree, z, fpatt, pi, x, pb, v, lnf = bench_case
    fg = int(tree.label[tree.branch_nodes()].argmax())
    sub = sorted({fg, 0, 17, 40, 77, 101, tree.nbranch - 1} | set(range(tree.nbranch, len(x))))
    ref = {i: five_point(pb.neg_lnL, x, i) for i in sub}
    for prec, g in bench_gradients.items():
        for i, r in ref.items():
            assert abs(g[i] - r) <= 1e-5 * max(1.0, abs(r)), (prec, i, g[i], r)


def test_gradient_vs_codeml_gradientB_64x5000(bench_case, bench_gradients, bench_fd):
    """codeml's own numerical gradient (gradientB, central: step
    (1e-6 (|x| + 1))^0.67, tools.c:6326-6350, restated in the oracle): the
    analytic gradient is no farther from it than the accurate five-point
    derivative is (gradientB's step error, large on the shortest branches),
    plus 1e-5 relative."""
    tree, z, fpatt, pi, x, pb, v, lnf = bench_case
    gB = pb.gradientB(x, True, central=True)
    c6, f5 = bench_fd
    own = np.abs(f5 - gB)
    for prec, g in bench_gradients.items():
        dev = np.abs(g - gB)
        print(f"{prec}: max rel deviation from codeml's gradientB {(dev / np.maximum(1.0, np.abs(gB))).max():.3e} "
              f"(gradientB's own {(own / np.maximum(1.0, np.abs(gB))).max():.3e})")
        assert np.all(dev <= own + 1e-5 * np.maximum(1.0, np.abs(gB)))


def test_batch_shaped_workload_vs_oracle():
    """32 genes of the batched workload's distribution through one split-
    precision batch: each gene's lnL against the oracle (|dlnL| <= 1e-6), and
    for every fourth gene the whole gradient against a five-point stencil of
    the oracle (step 1e-4 (|x| + 0.05); relative error <= 1e-5 of max(1, |g|))."""
    alns = simulate_batch(32, seed=31, taxa=(12, 48), codons=(100, 3000))
    genes, prm, probs = [], [], []
    for a in alns:
        z, fp, pi = O.patterns(a.codons)
        genes.append((a.tree, z, fp, pi))
        m = a.model
        prm.append({"blength": a.tree.branch, "kappa": m.kappa, "omega0": m.omega0, "omega2": m.omega2,
                    "p0": m.p0, "p1": m.p1})
        probs.append(O.Problem(a.tree, z, fp, pi, nthreads=O.max_threads()))
    b = api.Batch(genes, precision="fast")
    f, g, st = b.evaluate(prm, grad=True)
    f, g, st = b.evaluate(prm, grad=True)
    b.close()
    worst_l, worst_g = 0.0, 0.0
    for i, (a, pb) in enumerate(zip(alns, probs)):
        t = a.tree
        m = a.model
        x = np.concatenate([a.tree.branch[t.branch_nodes()], [m.kappa, m.p0, m.p1, m.omega0, m.omega2]])
        v = pb.neg_lnL(x)
        worst_l = max(worst_l, abs(f[i] - v))
        assert abs(f[i] - v) <= 1e-6, (i, f[i], v)
        if i % 4:
            continue
        gx = np.concatenate([g[i]["blength"][t.branch_nodes()],
                             [g[i]["kappa"], g[i]["p0"], g[i]["p1"], g[i]["omega0"], g[i]["omega2"]]])
        fd = np.array([five_point(pb.neg_lnL, x, k) for k in range(len(x))])
        err = np.abs(gx - fd) / np.maximum(1.0, np.abs(fd))
        worst_g = max(worst_g, err.max())
        assert err.max() <= 1e-5, (i, int(np.argmax(err)))
    print(f"32 genes ({sum(len(q[2]) for q in genes)} patterns): max |dlnL| {worst_l:.3e}, "
          f"max gradient rel err {worst_g:.3e} (8 genes)")
