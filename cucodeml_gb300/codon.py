"""Universal genetic code and codon indexing used by codeml's codon models.

Codons are indexed 0..63 in TCAG order (index = 16*b0 + 4*b1 + b2 with
T=0, C=1, A=2, G=3).  The 61 sense codons are renumbered 0..60 in the same
order with the three stop codons (TAA, TAG, TGA) removed; codeml calls these
maps FROM61 / FROM64 (codeml.c, `GeneticCode[0]`, treesub.c:1108-1133 uses
FROM64 to encode a codon site).
"""
from __future__ import annotations

import numpy as np

BASES = "TCAG"
# Standard (universal) code, amino acid letter per codon in TCAG order; '*' = stop.
AA64 = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG"

SENSE64 = np.array([i for i in range(64) if AA64[i] != "*"], dtype=np.int64)  # FROM61
FROM64 = np.full(64, -1, dtype=np.int64)
FROM64[SENSE64] = np.arange(61)
NCODE = 61


def codon_bases(ic64: int) -> tuple[int, int, int]:
    return ic64 // 16, (ic64 // 4) % 4, ic64 % 4


def codon_string(ic61: int) -> str:
    b = codon_bases(int(SENSE64[ic61]))
    return "".join(BASES[x] for x in b)


def gy94_structure() -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Return (single, transition, nonsyn) 61x61 boolean masks.

    single[i,j]: codons i and j differ at exactly one position (the only
    non-zero rates of the GY94 matrix built by eigenQcodon, codeml.c:3144-3180).
    transition[i,j]: that difference is T<->C or A<->G (codeml.c:3166-3167).
    nonsyn[i,j]: the two codons code for different amino acids (codeml.c:3172-3174).
    """
    single = np.zeros((61, 61), dtype=bool)
    ts = np.zeros((61, 61), dtype=bool)
    ns = np.zeros((61, 61), dtype=bool)
    for i in range(61):
        a = codon_bases(int(SENSE64[i]))
        for j in range(61):
            if i == j:
                continue
            b = codon_bases(int(SENSE64[j]))
            diff = [k for k in range(3) if a[k] != b[k]]
            if len(diff) != 1:
                continue
            single[i, j] = True
            s = a[diff[0]] + b[diff[0]]
            ts[i, j] = s in (1, 5)
            ns[i, j] = AA64[SENSE64[i]] != AA64[SENSE64[j]]
    return single, ts, ns


def gy94_q(pi: np.ndarray, kappa: float, omega: float) -> tuple[np.ndarray, float]:
    """GY94 rate matrix Q and its mean rate (eigenQcodon mode 0, codeml.c:3144-3185)."""
    single, ts, ns = _STRUCT
    q = np.where(single, 1.0, 0.0)
    q = np.where(ts, q * kappa, q)
    q = np.where(ns, q * omega, q)
    Q = q * pi[None, :]
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    mr = float(-(pi * np.diag(Q)).sum())
    return Q, mr


_STRUCT = gy94_structure()
