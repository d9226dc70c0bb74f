"""The drop-in boundary as codeml sees it.

The reference codeml.c, built with -DCUDA from the staged reference sources
(oracle/Makefile `dropin`), is linked against libgbcodeml.so through
codeml_adapter.c in place of cuda-codeml.o, together with oracle/ref_harness.c,
which wraps codeml's call of ming2 (codeml.c:683-692).  Inside one codeml
process, after codeml has read the data, compressed the patterns and called
CUDA_Init:

* `eval`: codeml's CUDA objective CUDA_lfundG (treesub.c:7397-7450, whose
  CUDA_fx_r calls the adapter's CUDA_ScheduleConditionalPNode per class) must
  equal codeml's own CPU lfundG at the same x within 1e-9 relative, for
  branch-site models A and B and clade models C and D; the adapter's GB_dfun
  must equal codeml's central-difference gradient (gradientB with
  AlwaysCenter, tools.c:6326-6350) within its step error.
* `sites`: the adapter's GB_BEB and GB_HessianSKT2004 inside codeml at the
  fixture's x must give the BEB and the SEs the reference codeml printed.
* `dfun` / unchanged: codeml's whole model-A fit, ming2 driven by GB_dfun
  (the one-argument change at codeml.c:688) or by its own finite differences
  of CUDA_lfundG, must reach the maximum codeml's CPU build reached
  (tests/golden/mle_*).

Without a GPU the run must get through CUDA_Init's marshalling and stop at
the device check with the library's status.  The tests need the staged
reference sources (oracle/_ref/src, `make -C oracle stage`)."""
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import refcodeml as R
from tests.conftest import (ROOT, clade_d_names, clade_names, golden_names, load_golden, mle_names, model_b_names,
                            unclean_names)

SRC = os.path.join(ROOT, "oracle", "_ref", "src")


def dropin_binary():
    if not os.path.isfile(os.path.join(SRC, "codeml.c")):
        pytest.skip("reference sources not staged (make -C oracle stage)")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"])
    return R.binary("codeml_gb")


def fixture_case(d, fx, x=None, ctl=R.CTL):
    rows = fx["seqs"] if "seqs" in fx else [row.replace(" ", "") for row in fx["codons"]]
    R.write_case(d, fx["names"], rows, fx["newick"], fx["x"] if x is None else x, ctl)


def load_fixture(name):
    import json
    with open(os.path.join(ROOT, "tests", "golden", name + ".json")) as f:
        return json.load(f)


def ctl_for(name):
    if name.startswith("u"):
        return R.CTL.replace("cleandata = 1", "cleandata = 0")
    if name.startswith("mb"):
        return R.CTL.replace("NSsites = 2", "NSsites = 3").replace("ncatG = 4", "ncatG = 3")
    if name.startswith("mcD"):
        return R.CTL.replace("model = 2", "model = 3").replace("NSsites = 2", "NSsites = 3").replace(
            "ncatG = 4", "ncatG = 3")
    if name.startswith("mc"):
        return R.CTL.replace("model = 2", "model = 3")
    return R.CTL


def test_dropin_links_and_stops_at_device_check_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the GPU tests below run the drop-in")
    exe = dropin_binary()
    fx, _, _ = load_golden("c24x400_s3")
    with tempfile.TemporaryDirectory() as d:
        fixture_case(d, fx)
        r = subprocess.run([exe, "codeml.ctl"], cwd=d, capture_output=True, text=True, timeout=300)
    assert r.returncode != 0
    assert "gbcodeml: gb_create failed (-7)" in r.stderr, r.stderr[-2000:]


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names() + unclean_names() + model_b_names() + clade_names()
                         + clade_d_names())
def test_dropin_objective_matches_codeml_cpu(name):
    exe = dropin_binary()
    fx = load_fixture(name)
    model_a = name.startswith(("c", "u", "mb", "mc"))      # GB_dfun: models A, B and clade models C, D
    with tempfile.TemporaryDirectory() as d:
        fixture_case(d, fx, ctl=ctl_for(name))
        r = R.run(exe, d, "eval", env={"GBREF_DFUN": "1" if model_a else "0"}, timeout=900)
    print(f"{name}: GPU {r['f_fun']:.10f} codeml CPU {r['f_cpu']:.10f}")
    assert abs(r["f_fun"] - r["f_cpu"]) <= 1e-9 * abs(r["f_cpu"])
    if model_a:
        ga, gc, g5 = (np.array(r[k]) for k in ("grad_dfun", "grad_cpu_central", "grad_cpu_5pt"))
        assert abs(r["f_dfun"] - r["f_cpu"]) <= 1e-9 * abs(r["f_cpu"])
        # against a five-point stencil of codeml's own lnL (truncation O(h^4))
        err5 = np.abs(ga - g5) / (1.0 + np.abs(g5))
        # codeml's gradientB (central, step (1e-6 (|x| + 1))^0.67) is as far
        # from the analytic gradient as from that stencil: its own step error
        errB = np.abs(ga - gc) - np.abs(g5 - gc)
        print(f"{name}: gradient vs codeml 5-point {err5.max():.2e}; vs gradientB "
              f"{(np.abs(ga - gc) / (1 + np.abs(gc))).max():.2e} (gradientB's own error "
              f"{(np.abs(g5 - gc) / (1 + np.abs(gc))).max():.2e})")
        # a branch closer to t = 0 than the stencil's reach (c5x120_s5 has a
        # zero-length branch) is differentiated one-sidedly by codeml's lnL
        # (PMatUVRoot: t < 1e-100 gives the identity): no stencil there
        x = np.array(r["x"])
        nb = len(fx["names"]) * 2 - 3
        inside = np.ones(len(x), dtype=bool)
        inside[:nb] = x[:nb] > 2e-4 * (np.abs(x[:nb]) + 0.05)
        assert err5[inside].max() <= 1e-5
        assert np.all(errB[inside] <= 1e-5 * (1.0 + np.abs(gc[inside])))


def codeml_fit_lnL(exe, fx, mode):
    with tempfile.TemporaryDirectory() as d:
        rows = [row.replace(" ", "") for row in fx["codons"]]
        R.write_case(d, fx["names"], rows, fx["newick"])
        env = dict(os.environ)
        env.pop("GBREF_MODE", None)
        if mode:
            env["GBREF_MODE"] = mode
        r = subprocess.run([exe, "codeml.ctl"], cwd=d, capture_output=True, text=True, timeout=1800, env=env)
        assert r.returncode == 0, r.stderr[-2000:]
        out = open(os.path.join(d, "out.txt")).read()
    m = re.search(r"lnL\(ntime:\s*\d+\s+np:\s*\d+\):\s*(-?\d+\.\d+)", out)
    return float(m.group(1))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["dfun", None])
def test_dropin_fit_reaches_codeml_maximum(mode):
    exe = dropin_binary()
    fx, _, _ = load_golden(mle_names()[0])
    lnL = codeml_fit_lnL(exe, fx, mode)
    print(f"codeml over the GPU drop-in ({mode or 'finite differences'}): lnL {lnL:.6f}, "
          f"codeml CPU {fx['alt']['lnL']:.6f}")
    assert lnL >= fx["alt"]["lnL"] - 1e-5
    assert lnL - fx["alt"]["lnL"] <= 2e-3


def test_codeml_itself_rejects_branch_site_models_on_partitioned_data():
    """codeml has no branch-site (or any model != 0) analysis of data with
    several genes: it stops at codeml.c:357 ("NSbranchsites with ngene.")
    before any likelihood, so the drop-in's CUDA_Init never sees ngene > 1
    under model A.  Checked with the reference codeml (CPU build)."""
    if not os.path.isfile(os.path.join(SRC, "codeml.c")):
        pytest.skip("reference sources not staged (make -C oracle stage)")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    fx, _, _ = load_golden("c8x300_s1")
    rows = [row.replace(" ", "") for row in fx["codons"]]
    with tempfile.TemporaryDirectory() as d:
        R.write_case(d, fx["names"], rows, fx["newick"], ctl=R.CTL)
        with open(os.path.join(d, "seq.phy"), "w") as f:
            f.write(f"{fx['ns']} {3 * fx['ncodon']} G\nG 2 100 {fx['ncodon'] - 100}\n")
            for nm, row in zip(fx["names"], rows):
                f.write(f"{nm}    {row}\n")
        r = subprocess.run([R.binary("codeml"), "codeml.ctl"], cwd=d, capture_output=True, text=True,
                           timeout=300)
    assert r.returncode != 0
    assert "NSbranchsites with ngene" in r.stdout + r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in golden_names() if not n.startswith("c5x120")] + model_b_names())
def test_dropin_beb_and_se_inside_codeml(name):
    """The adapter's GB_BEB and GB_HessianSKT2004 inside codeml (harness mode
    `sites`, at the fixture's x as final values): the BEB arrays codeml
    prints from (lfunNSsites_ACD's postSite, the w0 / w2 grid posteriors,
    postp0p1, log f(X); codeml.c:6697-6775) and the SEs from codeml's own
    arithmetic after HessianSKT2004 (codeml.c:764-782), against what the
    reference codeml printed for the same x (rst / out, print precision).
    Not c5x120_s5: its zero-length branch is an initial value below codeml's
    lower bound, which codeml moves to the bound before ming2 (the fixture's
    own run fixed x with in.codeml's -1, where no bound applies)."""
    from tests.test_beb_oracle import site_patterns
    exe = dropin_binary()
    fx, tree, codons = load_golden(name)
    with tempfile.TemporaryDirectory() as d:
        fixture_case(d, fx, ctl=ctl_for(name))
        r = R.run(exe, d, "sites", timeout=900)
    from oracle import oracle as O
    z, fpatt, pi = O.patterns(codons)
    assert r["npatt"] == len(fpatt)
    assert abs(-r["f"] - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    b = fx["beb"]
    post = np.array(r["post"]).reshape(4, -1)
    site = post[:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(b["site_post_5dp"]))) <= 5.01e-6
    grid = np.array(r["grid"])
    assert np.max(np.abs(grid[20:30] - b["w0_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(grid[30:40] - b["w2_post_3dp"])) <= 5.01e-4
    assert np.max(np.abs(np.array(r["p0p1"]) - b["p0p1_post_3dp"])) <= 5.01e-4
    assert abs(r["lnfX"][0] - b["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(b["lnfX_6dp"])
    ref = np.array(fx["se_6dp"])
    se = np.array(r["se"])
    print(f"{name}: SE max rel diff {np.max(np.abs(se - ref) / np.abs(ref)):.1e}")
    assert np.all(np.abs(se - ref) <= 5.01e-7 + 1e-4 * np.abs(ref))


@pytest.mark.gpu
@pytest.mark.parametrize("name", clade_names() + clade_d_names())
def test_dropin_clade_beb_inside_codeml(name):
    """The adapter's GB_BEB and GB_HessianSKT2004 under clade models C and D
    inside codeml (harness mode `sites`): the three-class site posteriors, the
    w0 / (w1) / w2 / w3 rows of lfunNSsites_ACD's postpara, postp0p1, log f(X)
    and the SEs against what the reference codeml printed for the same x."""
    from tests.test_beb_oracle import site_patterns
    exe = dropin_binary()
    fx, tree, codons = load_golden(name)
    with tempfile.TemporaryDirectory() as d:
        fixture_case(d, fx, ctl=ctl_for(name))
        r = R.run(exe, d, "sites", timeout=900)
    from oracle import oracle as O
    z, fpatt, pi = O.patterns(codons)
    assert r["ncls"] == 3
    assert abs(-r["f"] - fx["codeml_lnL"]) / abs(fx["codeml_lnL"]) <= 1e-9
    b = fx["beb"]
    post = np.array(r["post"]).reshape(3, -1)
    site = post[:, site_patterns(z, codons)].T
    assert np.max(np.abs(site - np.array(b["site_post_5dp"]))) <= 5.01e-6
    grid = np.array(r["grid"]).reshape(-1, 10)
    assert np.all(grid[:2] == -1.0)
    rows = ["w0_post_3dp"] + (["w1_post_3dp"] if name.startswith("mcD") else []) + ["w2_post_3dp", "w3_post_3dp"]
    for i, key in enumerate(rows):
        assert np.max(np.abs(grid[2 + i] - b[key])) <= 5.01e-4, key
    assert np.max(np.abs(np.array(r["p0p1"]) - b["p0p1_post_3dp"])) <= 5.01e-4
    assert abs(r["lnfX"][0] - b["lnfX_6dp"]) <= 5.01e-7 + 1e-12 * abs(b["lnfX_6dp"])
    ref = np.array(fx["se_6dp"])
    assert np.all(np.abs(np.array(r["se"]) - ref) <= 5.01e-7 + 1e-4 * np.abs(ref))
