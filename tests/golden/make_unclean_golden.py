"""Golden fixtures for alignments with gaps and ambiguous codons (cleandata = 0).

Test infrastructure.  Needs the staged reference sources (`make -C oracle
stage`) to build oracle/_ref/codeml and oracle/_ref/codeml_timed; the
fixtures it writes (tests/golden/u*.json) are committed.

A seeded model-A alignment is simulated and, in a seeded fraction of the
cells, one to three nucleotides of the codon are replaced by an IUPAC
ambiguity (N, R, Y) or a gap; the true codon stays among the resolutions, so
every ambiguous codon stands for at least one sense codon.  With cleandata =
0 codeml keeps those sites: EncodeSeqs (treesub.c:1075-1143) gives every
distinct ambiguous codon an id from 61 up, SetMapAmbiguity
(treesub.c:1146-1200) lists the sense codons it stands for (nChara,
CharaMap), and the pruning sums the transition probabilities over them
(ConditionalPNode codeml.c:3438-3445; cuda-codeml.cu:166-204 on the GPU).

Per case, two codeml runs on the same files:
  * at fixed x (in.codeml starts with -1, RateAncestor = -1): lnL (6 dp) and
    per-pattern log f (10 dp), as make_golden.py;
  * the CPU build linked with oracle/ref_harness.c in its "dump" mode: the
    data as codeml encoded it (z with the ambiguity ids, fpatt, pi to full
    precision, nChara / CharaMap), in the pattern order of the lnf file.

    python tests/golden/make_unclean_golden.py
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from cucodeml_gb300.simulate import ModelA, simulate  # noqa: E402
from oracle import refcodeml as R  # noqa: E402
from tests.golden.make_golden import CTL  # noqa: E402

# name, ns, ncodon, seed, fraction of ambiguous cells, (kappa, p0, p1, w0, w2)
CASES = [
    ("u8x300_s31", 8, 300, 31, 0.06, (2.0, 0.5, 0.3, 0.3, 3.0)),
    ("u24x400_s32", 24, 400, 32, 0.04, (2.2, 0.45, 0.35, 0.2, 4.0)),
]

IUPAC = {"A": "RN-", "G": "RN-", "C": "YN-", "T": "YN-"}


def blur(rows, frac, rng):
    """Replace 1-3 nucleotides of a fraction of the codons by an ambiguity
    that keeps the true base among its resolutions (or by a gap)."""
    out = []
    for row in rows:
        r = list(row)
        for c in range(len(r) // 3):
            if rng.random() >= frac:
                continue
            if rng.random() < 0.3:
                r[3 * c:3 * c + 3] = "---"
                continue
            for k in rng.choice(3, size=int(rng.integers(1, 4)), replace=False):
                choices = IUPAC[r[3 * c + k]]
                r[3 * c + k] = choices[int(rng.integers(len(choices)))]
        out.append("".join(r))
    return out


def run_case(name, ns, ncodon, seed, frac, params):
    aln = simulate(ns, ncodon, seed=seed, model=ModelA())
    tree = aln.tree
    rows = blur(R.alignment_rows(aln), frac, np.random.default_rng(seed + 1000))
    x = np.concatenate([tree.x_branch_lengths(), list(params)])
    ctl = CTL.replace("cleandata = 1", "cleandata = 0")
    with tempfile.TemporaryDirectory() as d:
        R.write_case(d, tree.names, rows, tree.to_newick(), ctl=ctl)
        with open(os.path.join(d, "in.codeml"), "w") as f:
            f.write("-1 " + " ".join(repr(float(v)) for v in x) + "\n")
        subprocess.run([R.binary("codeml"), "codeml.ctl"], cwd=d, check=True, capture_output=True, text=True)
        out = open(os.path.join(d, "out.txt")).read()
        lnf_lines = open(os.path.join(d, "lnf")).read().splitlines()
    with tempfile.TemporaryDirectory() as d:
        R.write_case(d, tree.names, rows, tree.to_newick(), x, ctl=ctl)
        enc = R.run(R.binary("codeml_timed"), d, "dump", timeout=600)
    m = re.search(r"lnL\(ntime:\s*(\d+)\s+np:\s*(\d+)\):\s*(-?\d+\.\d+)", out)
    fp, lnf, pats = [], [], []
    for ln in lnf_lines:
        parts = ln.split()
        if len(parts) > 5 and parts[0].isdigit() and re.match(r"^-?\d", parts[2]):
            if int(parts[0]) == 1:
                fp, lnf, pats = [], [], []
            fp.append(float(parts[1]))
            lnf.append(float(parts[2]))
            pats.append(" ".join(p for p in parts[5:] if not p.startswith("(")))
    assert enc["cleandata"] == 0 and len(enc["fpatt"]) == len(lnf) and enc["fpatt"] == fp
    return {
        "name": name, "ns": ns, "ncodon": ncodon, "seed": seed,
        "names": tree.names, "newick": tree.to_newick(digits=17), "seqs": rows,
        "x": [float(v) for v in x], "lastround": 1,
        "codeml_lnL": float(m.group(3)), "codeml_np": int(m.group(2)),
        "lnf": lnf, "fpatt": fp, "patterns": pats,
        "enc": {k: enc[k] for k in ("z", "fpatt", "pi", "nchara", "charamap")},
    }


def main():
    oracle = os.path.join(ROOT, "oracle")
    subprocess.check_call(["make", "-s", "-C", oracle, "stage"])
    subprocess.check_call(["make", "-s", "-C", oracle, os.path.join(oracle, "_ref", "codeml"),
                           os.path.join(oracle, "_ref", "codeml_timed")])
    outdir = os.path.dirname(os.path.abspath(__file__))
    for case in CASES:
        fx = run_case(*case)
        with open(os.path.join(outdir, fx["name"] + ".json"), "w") as f:
            json.dump(fx, f, separators=(",", ":"))
        namb = len(fx["enc"]["nchara"]) - 61
        print(fx["name"], "npatt", len(fx["lnf"]), "ambiguous codes", namb, "lnL", fx["codeml_lnL"])


if __name__ == "__main__":
    main()
