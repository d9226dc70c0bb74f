"""Generate golden fixtures by running the reference codeml (CPU build).

Test infrastructure.  Needs the reference sources (GBCODEML_REFERENCE, or
the staged copy of `make -C oracle stage`) to build oracle/_ref/codeml via
`make -C oracle ref`; the
fixtures it writes (tests/golden/*.json) are committed, so tests never need
the reference at run time.

For each case a seeded model-A alignment is simulated, written as PHYLIP +
Newick (#1 on the foreground branch), and codeml is run at FIXED parameters:
in.codeml starts with -1, so codeml evaluates lnL once at x with p0, p1
untransformed (readx treesub.c:3927, Forestry codeml.c:646-673) and, with
RateAncestor = -1, writes per-pattern log f to file `lnf` together with the
pattern's codons and count (print_lnf_site treesub.c:7332-7340).  The
fixture keeps: the codon alignment, tree, x, codeml's lnL (out file, 6 dp),
per-pattern log f (10 dp), pattern codons and counts (pattern order), and the
F3x4 codon frequencies (out file, 8 dp).

With fix_omega = 0 codeml then runs its Bayes empirical Bayes analysis
(lfunNSsites_rate codeml.c:5215 -> lfunNSsites_ACD 6617-6826) at the same x;
the fixture also keeps its per-site posteriors of the four site classes (rst,
5 dp), the posterior on the w0 / w2 grid and on the p0-p1 triangles (out
file, 3 dp) and the printed log f(X) with its scale terms S1, S2 (stdout, 6
dp).  The fixtures also keep the naive empirical Bayes (NEB) per-site
posteriors codeml prints first (lfunNSsites_rate codeml.c:5079-5129; rst, 5
dp).  Every fixture also keeps the Nei-Gojobori (1986) pairwise dN/dS, dN,
dS table codeml prints before the fit (DistanceMatNG86 treesub.c:2270-2366;
out file, 4 dp).

A second run of the same case with getSE = 1 gives codeml's standard errors
("SEs for parameters", out file, 6 dp): HessianSKT2004 (treesub.c:6979-7048)
approximates the Hessian by the outer products of per-pattern score vectors
from central differences of log f_h (step 2 Small_Diff (|x_i| + 1)), and the
SEs are the square roots of the diagonal of its negated inverse
(codeml.c:754-783).

codeml runs the same BEB for model B (lfunNSsites_ACD treats model = 2 as
model A's grid, w1 = 1 in class 1, with model B's Qfactors), kept for the
mb* fixtures too.
The mcC* fixtures are clade model C (model = 3, NSsites = 2; branch types
#1 and background; x ends p0, p1, w0, w2, w3): lnL, log f, NG86 and codeml's
clade-C BEB (three classes; grid w0, w2, w3).  The mcD* fixtures are clade
model D (model = 3, NSsites = 3, ncatG = 3; x ends p0, p1, w0, w1, w2, w3):
lnL, log f, NG86 and codeml's clade-D BEB (three classes; grid w0, w1, w2,
w3: 10^6 points).
The ms* fixtures are site models M2a and M1a (model = 0, no branch labels;
x ends p0, p1, w0, w2 for M2a, p0, w0 for M1a, p0, p1, w0, w1, w2 for M3
with three classes, p, q for M7, p0, p, q, ws for M8 with ten beta
categories): lnL, log f, NG86, and for M2a codeml's BEB (three classes).
The mb_* fixtures are the same evaluation under branch-site model B
(NSsites = 3, ncatG = 3: w1 free; x ends w0, w1, w2), lnL and log f only.

    python tests/golden/make_golden.py [name prefix]
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

from cucodeml_gb300 import codon  # noqa: E402
from cucodeml_gb300.simulate import ModelA, simulate, write_phylip  # noqa: E402

CTL = """\
      seqfile = seq.phy
     treefile = tree.nwk
      outfile = out.txt
        noisy = 0
      verbose = 1
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
 RateAncestor = -1
   Small_Diff = 1e-6
    cleandata = 1
  fix_blength = 0
       method = 0
"""

# name, ns, ncodon, seed, simulation model, evaluation params (kappa,p0,p1,w0,w2), blen scale
CASES = [
    ("c8x300_s1", 8, 300, 1, ModelA(), (2.0, 0.5, 0.3, 0.3, 3.0), 1.0),
    ("c8x300_s2", 8, 300, 2, ModelA(kappa=1.5, omega0=0.1, omega2=5.0, p0=0.6, p1=0.25),
     (1.7, 0.55, 0.3, 0.15, 4.0), 1.3),
    ("c5x120_s5", 5, 120, 5, ModelA(), (2.5, 0.4, 0.4, 0.5, 2.0), 0.7),
    ("c24x400_s3", 24, 400, 3, ModelA(), (2.0, 0.5, 0.3, 0.3, 3.0), 1.0),
    ("c40x200_s4", 40, 200, 4, ModelA(kappa=3.0, omega0=0.2, omega2=6.0, p0=0.45, p1=0.35),
     (2.8, 0.45, 0.35, 0.25, 5.5), 1.0),
    ("c12x150_s6_long", 12, 150, 6, ModelA(), (2.0, 0.5, 0.3, 0.3, 3.0), 6.0),
]

# branch-site model B (NSsites = 3, ncatG = 3: w1 free): evaluation params
# (kappa, p0, p1, w0, w1, w2); lnL, lnf and patterns only
CASES_B = [
    ("mb8x300_s7", 8, 300, 7, ModelA(), (2.0, 0.5, 0.3, 0.2, 0.8, 3.0), 1.0),
    ("mb24x400_s8", 24, 400, 8, ModelA(kappa=2.5, omega0=0.1, omega2=4.0),
     (2.4, 0.45, 0.35, 0.1, 1.6, 4.0), 1.0),
]


# site models without branch labels (model = 0): M2a (NSsites = 2, x ends p0,
# p1, w0, w2) and M1a (NSsites = 1, x ends p0, w0); lnL, lnf, patterns, NG86
CASES_SITE = [
    ("msM2a8x300_s9", 8, 300, 9, ModelA(), (2.0, 0.6, 0.3, 0.2, 2.5), 1.0, "M2a"),
    ("msM2a24x400_s10", 24, 400, 10, ModelA(omega2=4.0), (2.2, 0.5, 0.35, 0.15, 3.5), 1.0, "M2a"),
    ("msM1a12x300_s11", 12, 300, 11, ModelA(), (2.0, 0.7, 0.25), 1.0, "M1a"),
    ("msM3k3x8x300_s14", 8, 300, 14, ModelA(), (2.0, 0.5, 0.3, 0.1, 0.6, 2.5), 1.0, "M3"),
    ("msM7x8x300_s15", 8, 300, 15, ModelA(), (2.0, 0.4, 1.3), 1.0, "M7"),
    ("msM8x24x400_s16", 24, 400, 16, ModelA(), (2.2, 0.85, 0.5, 1.5, 3.0), 1.0, "M8"),
]


# clade model C (model = 3, NSsites = 2, two branch types: #1 and the rest):
# evaluation params (kappa, p0, p1, w0, w2 background, w3 foreground)
CASES_CLADE = [
    ("mcC8x300_s12", 8, 300, 12, ModelA(), (2.0, 0.5, 0.3, 0.2, 0.8, 3.0), 1.0),
    ("mcC24x400_s13", 24, 400, 13, ModelA(kappa=2.5, omega2=4.0), (2.4, 0.45, 0.35, 0.1, 1.5, 4.0), 1.0),
]


def run_case(codeml: str, name, ns, ncodon, seed, model, params, bscale, model_b=False, site_model=None,
             clade=False, clade_d=False):
    aln = simulate(ns, ncodon, seed=seed, model=model)
    tree = aln.tree
    if site_model:
        tree.label[:] = 0          # site models: no foreground branch in the tree file
    xb = tree.x_branch_lengths() * bscale
    if name.startswith("c5x120"):
        xb[2] = 0.0          # internal branch with t = 0: P = I (PMatUVRoot, t < 1e-100)
        xb[1] = 0.01         # short tip branch (P entries of order t^3 stay well-conditioned)
    x = np.concatenate([xb, list(params)])
    with tempfile.TemporaryDirectory() as d:
        write_phylip(os.path.join(d, "seq.phy"), aln)
        with open(os.path.join(d, "tree.nwk"), "w") as f:
            f.write(f"{ns} 1\n{tree.to_newick()}\n")
        with open(os.path.join(d, "in.codeml"), "w") as f:
            f.write("-1 " + " ".join(repr(float(v)) for v in x) + "\n")
        ctl = CTL.replace("NSsites = 2", "NSsites = 3").replace("ncatG = 4", "ncatG = 3") if model_b else CTL
        if site_model:
            ctl = CTL.replace("model = 2", "model = 0").replace(
                "NSsites = 2", "NSsites = " + {"M1a": "1", "M2a": "2", "M3": "3", "M7": "7", "M8": "8"}[site_model])
            if site_model == "M3":
                ctl = ctl.replace("ncatG = 4", "ncatG = 3")
            if site_model in ("M7", "M8"):
                ctl = ctl.replace("ncatG = 4", "ncatG = 10")
        if clade:
            ctl = CTL.replace("model = 2", "model = 3")
        if clade_d:
            ctl = ctl.replace("NSsites = 2", "NSsites = 3").replace("ncatG = 4", "ncatG = 3")
        with open(os.path.join(d, "codeml.ctl"), "w") as f:
            f.write(ctl)
        r = subprocess.run([codeml, "codeml.ctl"], cwd=d, check=True, capture_output=True, text=True)
        out = open(os.path.join(d, "out.txt")).read()
        lnf_lines = open(os.path.join(d, "lnf")).read().splitlines()
        rst = open(os.path.join(d, "rst")).read()
        # a second run with getSE = 1 for codeml's standard errors
        with open(os.path.join(d, "codeml.ctl"), "w") as f:
            f.write(ctl.replace("getSE = 0", "getSE = 1"))
        subprocess.run([codeml, "codeml.ctl"], cwd=d, check=True, capture_output=True, text=True)
        out_se = open(os.path.join(d, "out.txt")).read()
    if clade:
        k = out_se.index("SEs for parameters:")
        se = {"se_6dp": [float(v) for v in out_se[k:].splitlines()[1].split()], "small_diff": 1e-6}
    if clade_d:       # clade-D BEB: grid w0 in (0, 0.5), w1 in (0.5, 1.5), w2, w3 in (0, 3)
        extra = {"model": "D", "ng86_4dp": parse_ng86(out, ns), "beb": parse_beb(out, rst, r.stdout, ncls=3),
                 "neb_site_post_5dp": parse_site_post(rst, "Naive", ncls=3), **se}
    elif clade:
        extra = {"model": "C", "ng86_4dp": parse_ng86(out, ns), "beb": parse_beb(out, rst, r.stdout, ncls=3),
                 "neb_site_post_5dp": parse_site_post(rst, "Naive", ncls=3), **se}
    elif site_model:
        ncat = {"M1a": 2, "M2a": 3, "M3": 3, "M7": 10, "M8": 11}[site_model]
        extra = {"model": site_model, "ng86_4dp": parse_ng86(out, ns),
                 "neb_site_post_5dp": parse_site_post(rst, "Naive", ncls=ncat)}
        if site_model == "M2a":       # BEB of M2a (lfunNSsites_M2M8 codeml.c:6190-6415): 3 classes
            extra["beb"] = parse_beb(out, rst, r.stdout, ncls=3)
            extra["beb"]["site_wmean_sd_3dp"] = parse_site_meanw(rst)
        if site_model:                    # codeml's getSE = 1 SEs
            k = out_se.index("SEs for parameters:")
            extra["se_6dp"] = [float(v) for v in out_se[k:].splitlines()[1].split()]
            extra["small_diff"] = 1e-6
    elif model_b:
        k = out_se.index("SEs for parameters:")
        extra = {"model": "B", "ng86_4dp": parse_ng86(out, ns), "neb_site_post_5dp": parse_site_post(rst, "Naive"),
                 "beb": parse_beb(out, rst, r.stdout),
                 "se_6dp": [float(v) for v in out_se[k:].splitlines()[1].split()], "small_diff": 1e-6}
    else:
        k = out_se.index("SEs for parameters:")
        extra = {"beb": parse_beb(out, rst, r.stdout), "ng86_4dp": parse_ng86(out, ns),
                 "neb_site_post_5dp": parse_site_post(rst, "Naive"),
                 "se_6dp": [float(v) for v in out_se[k:].splitlines()[1].split()], "small_diff": 1e-6}
    m = re.search(r"lnL\(ntime:\s*(\d+)\s+np:\s*(\d+)\):\s*(-?\d+\.\d+)", out)
    lnL = float(m.group(3))
    i0 = out.index("Codon frequencies under model")
    vals = [float(v) for v in out[i0:].split("\n", 1)[1].split()[:64]]
    pi8 = [vals[k] for k in codon.SENSE64]
    pats, fp, lnf = [], [], []
    for ln in lnf_lines:
        parts = ln.split()
        if len(parts) > 5 and parts[0].isdigit() and re.match(r"^-?\d", parts[2]):
            if int(parts[0]) == 1:       # codeml writes one block per lfundG call: keep the last
                pats, fp, lnf = [], [], []
            fp.append(float(parts[1]))
            lnf.append(float(parts[2]))
            pats.append([p for p in parts[5:] if not p.startswith("(")])
    lut = [codon.codon_string(i) for i in range(61)]
    return {
        "name": name, "ns": ns, "ncodon": ncodon, "seed": seed,
        "names": tree.names, "newick": tree.to_newick(digits=17),
        "codons": [" ".join(lut[c] for c in row) for row in aln.codons],
        "x": [float(v) for v in x], "lastround": 1,
        "codeml_lnL": lnL, "codeml_np": int(m.group(2)),
        "lnf": lnf, "fpatt": fp, "patterns": [" ".join(p) for p in pats], "pi_8dp": pi8,
        **extra,
    }


def parse_ng86(out: str, ns: int) -> dict:
    """codeml's Nei-Gojobori (1986) table (DistanceMatNG86 treesub.c:2270-2366,
    printed before the fit): for each pair j < i, dN/dS, dN and dS (4 dp; -1
    where NG86 does not apply)."""
    i0 = out.index("Nei & Gojobori 1986. dN/dS (dN, dS)")
    i1 = out.index("TREE #", i0)
    rows = [ln for ln in out[i0:i1].splitlines()[4:] if ln.strip()]
    assert len(rows) == ns
    w, dn, ds = [], [], []
    for i, ln in enumerate(rows):
        vals = re.findall(r"(-?\d+\.\d+) ?\((-?\d+\.\d+) (-?\d+\.\d+)\)", ln)
        assert len(vals) == i
        for a, b, c in vals:
            w.append(float(a)); dn.append(float(b)); ds.append(float(c))
    return {"dN_dS": w, "dN": dn, "dS": ds}


def parse_site_post(rst: str, which: str, ncls: int = 4) -> list:
    """Per-site posteriors of the four site classes from codeml's rst
    (PrintProbNSsites codeml.c:4975-5030): the "Naive Empirical Bayes (NEB)"
    or the "Bayes Empirical Bayes (BEB)" block, 5 dp."""
    head = {"Naive": "Naive Empirical Bayes (NEB) probabilities",
            "Bayes": "Bayes Empirical Bayes (BEB) probabilities"}[which]
    i0 = rst.index(head)
    site = []
    for ln in rst[i0:].splitlines()[3:]:
        parts = ln.split()
        if len(parts) < ncls + 3 or not parts[0].isdigit():
            break
        site.append([float(v) for v in parts[2:2 + ncls]])
    return site


def parse_site_meanw(rst: str) -> list:
    """The BEB block's per-site posterior mean and SD of w ("x +- y", 3 dp)
    that codeml prints for the site models (PrintProbNSsites codeml.c:5000-5016)."""
    i0 = rst.index("Bayes Empirical Bayes (BEB) probabilities")
    out = []
    for ln in rst[i0:].splitlines()[3:]:
        m = re.search(r"\)\s+(-?\d+\.\d+)\s+\+-\s+(-?\d+\.\d+)", ln)
        if not ln.split() or not ln.split()[0].isdigit() or not m:
            break
        out.append([float(m.group(1)), float(m.group(2))])
    return out


def parse_beb(out: str, rst: str, stdout: str, ncls: int = 4) -> dict:
    """codeml's BEB results: per-site class posteriors (rst), grid posteriors
    (out) and log f(X), S1, S2 (stdout)."""
    site = parse_site_post(rst, "Bayes", ncls)
    j0 = out.index("Posterior on the grid")
    rows = {}
    for ln in out[j0:].splitlines()[1:7]:
        parts = ln.split()
        if parts and parts[0] in ("w0:", "w1:", "w2:", "w3:"):
            rows[parts[0][:2]] = [float(v) for v in parts[1:]]
    k0 = out.index("Posterior for p0-p1")
    k1 = out.index("sum of density on p0-p1")
    p0p1 = [float(v) for v in out[k0:k1].split("\n", 1)[1].split()]
    m = re.search(r"log\(fX\) =\s*(-?\d+\.\d+)\s+S =\s*(-?\d+\.\d+)\s+(-?\d+\.\d+)",
                  stdout.replace("\r", "\n"))
    extra = {"w3_post_3dp": rows["w3"]} if "w3" in rows else {}
    if "w1" in rows:
        extra["w1_post_3dp"] = rows["w1"]
    return {**extra, "site_post_5dp": site, "w0_post_3dp": rows["w0"], "w2_post_3dp": rows["w2"],
            "p0p1_post_3dp": p0p1, "lnfX_6dp": float(m.group(1)), "S1_6dp": float(m.group(2)),
            "S2_6dp": float(m.group(3))}


# clade model D (model = 3, NSsites = 3, ncatG = 3: w1 free as well):
# evaluation params (kappa, p0, p1, w0, w1, w2 background, w3 foreground)
CASES_CLADE_D = [
    ("mcD8x300_s17", 8, 300, 17, ModelA(), (2.0, 0.5, 0.3, 0.1, 0.7, 1.5, 3.5), 1.0),
    ("mcD24x400_s18", 24, 400, 18, ModelA(kappa=2.5, omega2=4.0), (2.4, 0.45, 0.35, 0.15, 0.9, 2.0, 4.5), 1.0),
]


def main(only: str | None = None):
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    codeml = os.path.join(ROOT, "oracle", "_ref", "codeml")
    outdir = os.path.dirname(os.path.abspath(__file__))
    for case in (CASES + [c + (True,) for c in CASES_B] + [c[:7] + (False, c[7]) for c in CASES_SITE]
                 + [c + (False, None, True) for c in CASES_CLADE]
                 + [c + (False, None, True, True) for c in CASES_CLADE_D]):
        if only and not case[0].startswith(only):
            continue
        fx = run_case(codeml, *case)
        with open(os.path.join(outdir, fx["name"] + ".json"), "w") as f:
            json.dump(fx, f, separators=(",", ":"))
        print(fx["name"], "npatt", len(fx["lnf"]), "lnL", fx["codeml_lnL"])


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
