"""Golden maximum-likelihood fixtures from the reference codeml's own optimiser.

Test infrastructure.  Needs the reference sources (GBCODEML_REFERENCE, or
the staged copy of `make -C oracle stage`) to build oracle/_ref/codeml via
`make -C oracle ref`; the
fixtures it writes (tests/golden/mle_*.json) are committed.

For each case a seeded model-A alignment is simulated and codeml optimises,
from its own initial values, the branch-site model A alternative (model = 2,
NSsites = 2, w2 free, w2 >= 1) and the null (fix_omega = 1, omega = 1) with
ming2 and finite-difference gradients (method = 0, Forestry codeml.c:676-697).
The fixture keeps the alignment and tree and, per model, codeml's maximised
lnL (out file, 6 dp), np and the wall time of the codeml run.

    python tests/golden/make_mle_golden.py
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from cucodeml_gb300 import codon  # noqa: E402
from cucodeml_gb300.simulate import ModelA, simulate, write_phylip  # noqa: E402

CTL = """\
      seqfile = seq.phy
     treefile = tree.nwk
      outfile = out.txt
        noisy = 0
      verbose = 0
      runmode = 0
      seqtype = 1
    CodonFreq = 2
        clock = 0
       aaDist = 0
        model = 2
      NSsites = 2
        icode = 0
        Mgene = 0
    fix_kappa = 0
        kappa = 2
    fix_omega = {fix}
        omega = {omega}
    fix_alpha = 1
        alpha = 0
       Malpha = 0
        ncatG = 4
        getSE = 0
 RateAncestor = 0
   Small_Diff = 1e-6
    cleandata = 1
  fix_blength = 0
       method = 0
"""

# name, taxa, codons, seed, simulation model, mean branch length: one case with
# little foreground signal (LRT ~ 0) and two with strong signal
CASES = [
    ("mle_c8x300_s1", 8, 300, 1, ModelA(), 0.1),
    ("mle_c10x500_s11", 10, 500, 11, ModelA(kappa=2.0, omega0=0.2, omega2=8.0, p0=0.4, p1=0.2), 0.3),
    ("mle_c16x400_s12", 16, 400, 12, ModelA(kappa=2.5, omega0=0.15, omega2=6.0, p0=0.45, p1=0.2), 0.25),
]


def run_model(codeml, d, fix, omega):
    with open(os.path.join(d, "codeml.ctl"), "w") as f:
        f.write(CTL.format(fix=fix, omega=omega))
    t0 = time.perf_counter()
    subprocess.run([codeml, "codeml.ctl"], cwd=d, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    secs = time.perf_counter() - t0
    out = open(os.path.join(d, "out.txt")).read()
    m = re.search(r"lnL\(ntime:\s*(\d+)\s+np:\s*(\d+)\):\s*(-?\d+\.\d+)", out)
    return {"lnL": float(m.group(3)), "np": int(m.group(2)), "seconds": secs}


def run_case(codeml, name, ns, ncodon, seed, model, mean_blen):
    aln = simulate(ns, ncodon, seed=seed, model=model, mean_blen=mean_blen)
    tree = aln.tree
    with tempfile.TemporaryDirectory() as d:
        write_phylip(os.path.join(d, "seq.phy"), aln)
        with open(os.path.join(d, "tree.nwk"), "w") as f:
            f.write(f"{ns} 1\n{tree.to_newick(lengths=False)}\n")
        alt = run_model(codeml, d, 0, 1.5)
        null = run_model(codeml, d, 1, 1)
    lut = [codon.codon_string(i) for i in range(61)]
    return {
        "name": name, "ns": ns, "ncodon": ncodon, "seed": seed, "mean_blen": mean_blen,
        "names": tree.names, "newick": tree.to_newick(digits=17),
        "codons": [" ".join(lut[c] for c in row) for row in aln.codons],
        "alt": alt, "null": null, "codeml_LRT": 2.0 * (alt["lnL"] - null["lnL"]),
    }


def main():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    codeml = os.path.join(ROOT, "oracle", "_ref", "codeml")
    outdir = os.path.dirname(os.path.abspath(__file__))
    for case in CASES:
        fx = run_case(codeml, *case)
        with open(os.path.join(outdir, fx["name"] + ".json"), "w") as f:
            json.dump(fx, f, separators=(",", ":"))
        print(fx["name"], "alt", fx["alt"], "null", fx["null"], "LRT", fx["codeml_LRT"])


if __name__ == "__main__":
    main()
