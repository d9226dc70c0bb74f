"""Run the reference codeml builds of oracle/Makefile (test infrastructure).

The binaries are codeml itself (oracle/_ref/codeml_timed: the CPU build;
oracle/_ref/cucodeml: the reference GPU build, cuda-codeml.cu for sm_103a;
oracle/_ref/codeml_gb: codeml.c over this library's drop-in adapter), each
linked with oracle/ref_harness.c, which takes over codeml's call of ming2
(codeml.c:683-692) when GBREF_MODE is set: "time" times lnL + forward-
difference gradient steps of codeml's own objective (lfundG or CUDA_lfundG,
gradientB tools.c:6326-6350), "eval" compares the objective with codeml's
CPU lfundG at the same x.  This module writes the control, sequence, tree and
in.codeml files for an alignment, runs a binary and parses its "GBREF" line.

Only tests, smoke() and bench.py's CPU baseline / reference arm use it.
"""
from __future__ import annotations

import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

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
    fix_omega = 0
        omega = 1
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


def binary(name: str) -> str:
    """Path of a built reference binary; raises if oracle/Makefile has not built it."""
    p = os.path.join(REF_DIR, name)
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} not built (make -C oracle stage {name})")
    return p


def write_case(d: str, names, codon_rows, newick: str, x=None, ctl: str = CTL) -> None:
    """codeml input files in directory d.  codon_rows: per taxon a string of
    nucleotides (3 per codon); newick with #1 on the foreground branch; x
    (optional) codeml's initial values written to in.codeml (not fixed: the
    run reaches ming2)."""
    ns = len(names)
    with open(os.path.join(d, "seq.phy"), "w") as f:
        f.write(f"{ns} {len(codon_rows[0])}\n")
        for nm, row in zip(names, codon_rows):
            f.write(f"{nm}    {row}\n")
    with open(os.path.join(d, "tree.nwk"), "w") as f:
        f.write(f"{ns} 1\n{newick}\n")
    if x is not None:
        with open(os.path.join(d, "in.codeml"), "w") as f:
            f.write(" ".join(repr(float(v)) for v in x) + "\n")
    with open(os.path.join(d, "codeml.ctl"), "w") as f:
        f.write(ctl)


def alignment_rows(aln, cols=None):
    """Nucleotide rows of a simulated alignment (optionally a column subset of codons)."""
    from cucodeml_gb300 import codon
    lut = [codon.codon_string(i) for i in range(61)]
    c = aln.codons if cols is None else aln.codons[:, cols]
    return ["".join(lut[k] for k in row) for row in c]


def parse(stdout: str) -> dict:
    for ln in stdout.splitlines():
        if ln.startswith("GBREF "):
            return json.loads(ln[6:])
    raise RuntimeError("no GBREF line in codeml's output:\n" + stdout[-3000:])


def run(exe: str, d: str, mode: str, steps: int = 1, warmup: int = 0, timeout: float = 3600,
        env: dict | None = None) -> dict:
    e = dict(os.environ, GBREF_MODE=mode, GBREF_STEPS=str(steps), GBREF_WARMUP=str(warmup))
    if env:
        e.update(env)
    r = subprocess.run([exe, "codeml.ctl"], cwd=d, capture_output=True, text=True, timeout=timeout, env=e)
    if r.returncode != 0:
        raise RuntimeError(f"{os.path.basename(exe)} exited {r.returncode}:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    return parse(r.stdout)


def time_steps(exe: str, names, rows, newick, x, steps: int, warmup: int, env=None) -> dict:
    with tempfile.TemporaryDirectory() as d:
        write_case(d, names, rows, newick, x)
        return run(exe, d, "time", steps, warmup, env=env)


def sample_columns(ncodon: int, nsample: int, part: int, seed: int = 0) -> np.ndarray:
    """Codon columns of the part-th of several disjoint random samples."""
    perm = np.random.default_rng(seed).permutation(ncodon)
    return np.sort(perm[part * nsample:(part + 1) * nsample])
