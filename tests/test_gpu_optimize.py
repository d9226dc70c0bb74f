"""Alternative vs null fits driven by the GPU adjoint gradient against the
reference codeml's own optimiser (ming2 with finite-difference gradients,
golden fixtures made by tests/golden/make_mle_golden.py).

codeml prints lnL to 6 decimals and stops ming2 at its own tolerance, so each
maximum here must be at least codeml's (-1e-5) and within 2e-3 of it; the
split-precision and FP64 fits must agree within 1e-6 (lnL) and the LRT with
codeml's within 4e-3."""
import numpy as np
import pytest

from cucodeml_gb300 import api, optimize
from tests.conftest import load_golden, mle_names

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", mle_names())
def test_alt_null_matches_codeml(name):
    fx, tree, codons = load_golden(name)
    z, fpatt, pi = api.patterns(codons)
    res = {p: optimize.alt_null(tree, z, fpatt, pi, precision=p) for p in ("fp64", "fast")}
    for p, r in res.items():
        print(f"{name} {p}: alt {r['alt']['lnL']:.6f} ({r['alt']['calls']} calls, w2 {r['alt']['omega2']:.3f}) "
              f"null {r['null']['lnL']:.6f} ({r['null']['calls']} calls) LRT {r['LRT']:.4f} "
              f"| codeml alt {fx['alt']['lnL']:.6f} null {fx['null']['lnL']:.6f} LRT {fx['codeml_LRT']:.4f}")
        for m in ("alt", "null"):
            assert r[m]["lnL"] >= fx[m]["lnL"] - 1e-5, (p, m)
            assert r[m]["lnL"] - fx[m]["lnL"] <= 2e-3, (p, m)
        assert abs(r["LRT"] - fx["codeml_LRT"]) <= 4e-3
    for m in ("alt", "null"):
        assert abs(res["fast"][m]["lnL"] - res["fp64"][m]["lnL"]) <= 1e-6, m


def test_fd_and_adjoint_reach_the_same_maximum():
    """codeml's finite-difference gradient and the adjoint drive the same
    optimiser to the same maximum (smallest fixture)."""
    fx, tree, codons = load_golden(mle_names()[0])
    z, fpatt, pi = api.patterns(codons)
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64")
    x0 = optimize.initial_x(tree)
    a = optimize.fit(lk, x0, gradient="adjoint")
    f = optimize.fit(lk, x0, gradient="fd", gtol=1e-5)
    lk.close()
    print(f"adjoint {a['lnL']:.8f} in {a['calls']} calls; fd {f['lnL']:.8f} in {f['lnL_evals']} lnL evaluations")
    assert abs(a["lnL"] - f["lnL"]) <= 1e-5
    assert a["lnL"] >= f["lnL"] - 1e-7
