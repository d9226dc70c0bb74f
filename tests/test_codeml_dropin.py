"""The drop-in boundary as codeml sees it: codeml.c (unmodified, built with
-DCUDA) linked against libgbcodeml.so through codeml_adapter.c instead of
cuda-codeml.o.  Needs the reference sources, so it runs only where they are;
without a GPU the run must get through CUDA_Init's marshalling of codeml's
globals (tree, patterns, scale nodes all accepted by gb_create's checks) and
stop at the device check with the library's status, not crash."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from tests.conftest import ROOT, load_golden

REF = "/root/reference"


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_dropin_codeml_links_and_marshals():
    import torch
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"])
    exe = os.path.join(ROOT, "oracle", "_ref", "codeml_gb")
    from cucodeml_gb300.simulate import write_phylip
    from tests.golden.make_golden import CTL
    fx, tree, codons = load_golden("c24x400_s3")
    with tempfile.TemporaryDirectory() as d:
        from cucodeml_gb300 import codon
        with open(os.path.join(d, "seq.phy"), "w") as f:
            f.write(f"{fx['ns']} {3 * fx['ncodon']}\n")
            for nm, row in zip(fx["names"], fx["codons"]):
                f.write(f"{nm}    {row.replace(' ', '')}\n")
        with open(os.path.join(d, "tree.nwk"), "w") as f:
            f.write(f"{fx['ns']} 1\n{fx['newick']}\n")
        with open(os.path.join(d, "codeml.ctl"), "w") as f:
            f.write(CTL.replace("RateAncestor = -1", "RateAncestor = 0"))
        r = subprocess.run([exe, "codeml.ctl"], cwd=d, capture_output=True, text=True, timeout=300)
    if torch.cuda.is_available():
        pytest.skip("GPU present: the drop-in would run the optimisation")
    assert r.returncode != 0
    assert "gbcodeml: gb_create failed (-7)" in r.stderr, r.stderr[-2000:]
