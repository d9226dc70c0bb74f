"""Seeded simulator of codon alignments under branch-site model A.

Generates synthetic inputs with the shapes of the branch-site model A
workloads: a uniform random unrooted binary tree, branch lengths ~Exp(0.1),
one random foreground branch, F3x4 codon frequencies from per-position
Dirichlet(5,5,5,5) base frequencies, GY94 rate matrices, and the four
model-A site classes (0: w0 everywhere, 1: w=1 everywhere, 2a: w0 background
and w2 foreground, 2b: w=1 background and w2 foreground) with proportions
p0, p1, (1-p0-p1)p0/(p0+p1), (1-p0-p1)p1/(p0+p1) (codeml.c:2488-2495).
Branch lengths are in codeml's units: the rate matrix of a branch is scaled
by 1/(mean rate of the site-class mixture on that branch type)
(Qfactor_NS_branch, codeml.c:2497-2512).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import codon
from .tree import Tree, random_tree


@dataclass
class ModelA:
    kappa: float = 2.0
    omega0: float = 0.3
    omega2: float = 3.0
    p0: float = 0.5
    p1: float = 0.3

    def freqK(self) -> np.ndarray:
        p0, p1 = self.p0, self.p1
        t = p0 + p1
        return np.array([p0, p1, (1 - t) * p0 / t, (1 - t) * p1 / t])

    def omegas(self) -> np.ndarray:
        return np.array([self.omega0, 1.0, self.omega2])

    def qfactors(self, pi: np.ndarray) -> np.ndarray:
        p0, p1 = self.p0, self.p1
        t = p0 + p1
        w_bg = (p0 * self.omega0 + p1 * 1.0) / t
        w_fg = p0 * self.omega0 + p1 * 1.0 + (1 - t) * self.omega2
        out = []
        for w in (w_bg, w_fg):
            _, mr = codon.gy94_q(pi, self.kappa, w)
            out.append(1.0 / mr)
        return np.array(out)


@dataclass
class Alignment:
    tree: Tree
    codons: np.ndarray           # [ns, ncodon] sense-codon index 0..60
    classes: np.ndarray          # [ncodon] true site class (0..3)
    pi_true: np.ndarray          # [61] generating codon frequencies
    model: ModelA

    @property
    def ns(self) -> int:
        return self.codons.shape[0]

    @property
    def ncodon(self) -> int:
        return self.codons.shape[1]

    def sequences(self) -> list:
        """Nucleotide strings, one per species."""
        lut = np.array([codon.codon_string(i) for i in range(61)])
        return ["".join(lut[row]) for row in self.codons]


def f3x4_pi(base_freqs: np.ndarray) -> np.ndarray:
    """pi_c proportional to f1[b0] f2[b1] f3[b2] over the 61 sense codons (F3x4)."""
    pi = np.empty(61)
    for i, ic in enumerate(codon.SENSE64):
        b = codon.codon_bases(int(ic))
        pi[i] = base_freqs[0, b[0]] * base_freqs[1, b[1]] * base_freqs[2, b[2]]
    return pi / pi.sum()


def eigen_q(pi: np.ndarray, kappa: float, omega: float):
    """(U, lam, V) with Q = U diag(lam) V for the unscaled GY94 Q."""
    Q, _ = codon.gy94_q(pi, kappa, omega)
    s = np.sqrt(pi)
    A = (s[:, None] * Q) / s[None, :]
    A = 0.5 * (A + A.T)
    lam, R = np.linalg.eigh(A)
    return R / s[:, None], lam, R.T * s[None, :]


def transition_matrix(pi: np.ndarray, kappa: float, omega: float, t: float, eig=None) -> np.ndarray:
    """P(t) = exp(Q t) for the unscaled GY94 Q, via the symmetric eigenproblem."""
    U, lam, V = eig if eig is not None else eigen_q(pi, kappa, omega)
    return np.clip((U * np.exp(lam * t)[None, :]) @ V, 0.0, None)


def simulate(ns: int, ncodon: int, seed: int, model: ModelA | None = None,
             mean_blen: float = 0.1, dirichlet_alpha: float = 5.0) -> Alignment:
    rng = np.random.default_rng(seed)
    model = model or ModelA()
    tree = random_tree(ns, rng, mean_blen)
    base = rng.dirichlet([dirichlet_alpha] * 4, size=3)
    pi = f3x4_pi(base)
    qf = model.qfactors(pi)
    w = model.omegas()
    fk = model.freqK()
    classes = rng.choice(4, size=ncodon, p=fk / fk.sum())
    states = np.full((tree.nnode, ncodon), -1, dtype=np.int64)
    states[tree.root] = rng.choice(61, size=ncodon, p=pi)
    # class -> omega index on background / foreground branches (Set_UVR_BranchSite)
    bg_w = [0, 1, 0, 1]
    fg_w = [0, 1, 2, 2]
    eig = [eigen_q(pi, model.kappa, w[i]) for i in range(3)]
    stack = [tree.root]
    while stack:
        a = stack.pop()
        for c in tree.sons[a]:
            lab = int(tree.label[c])
            tt = float(tree.branch[c]) * qf[lab]
            for k in range(4):
                idx = np.nonzero(classes == k)[0]
                if len(idx) == 0:
                    continue
                wi = fg_w[k] if lab else bg_w[k]
                P = transition_matrix(pi, model.kappa, w[wi], tt, eig[wi])
                cdf = np.cumsum(P, axis=1)
                cdf /= cdf[:, -1:]
                u = rng.random(len(idx))
                par = states[a, idx]
                states[c, idx] = np.minimum((u[:, None] > cdf[par]).sum(axis=1), 60)
            stack.append(c)
    return Alignment(tree=tree, codons=states[:ns].copy(), classes=classes,
                     pi_true=pi, model=model)


def write_phylip(path: str, aln: Alignment) -> None:
    seqs = aln.sequences()
    with open(path, "w") as f:
        f.write(f"{aln.ns} {3 * aln.ncodon}\n")
        for nm, s in zip(aln.tree.names, seqs):
            f.write(f"{nm}    {s}\n")


def simulate_batch(ngene: int, seed: int, taxa=(12, 48), codons=(100, 3000)):
    """Independent alignments for the batched workload: taxa ~ U{12..48},
    codons log-uniform in [100, 3000], and per gene kappa ~ LogN(ln 2, 0.3),
    w0 ~ U(0.05, 0.8), w2 ~ U(1, 8) (p0 = 0.5, p1 = 0.3)."""
    rng = np.random.default_rng(seed)
    out = []
    for g in range(ngene):
        ns = int(rng.integers(taxa[0], taxa[1] + 1))
        nc = int(round(np.exp(rng.uniform(np.log(codons[0]), np.log(codons[1])))))
        m = ModelA(kappa=float(np.exp(rng.normal(np.log(2.0), 0.3))), omega0=float(rng.uniform(0.05, 0.8)),
                   omega2=float(rng.uniform(1.0, 8.0)), p0=0.5, p1=0.3)
        out.append(simulate(ns, nc, seed=int(rng.integers(1 << 31)), model=m))
    return out
