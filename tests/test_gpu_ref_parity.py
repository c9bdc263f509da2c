"""The FP64 and mixed engines, through the C ABI, against runs of the reference's own
time loop (tests/golden/ref_fixtures.npz: smaiso-wcomp.cpp run as 2 or 4 MPI ranks
through oracle/_ref; see tests/golden/ref_cases.py and make_ref_fixtures.py).

The FP64 engine must meet the FP64 parity bar (1e-10 relative L2 per field, vector
components against the whole vector) at every dump step, including the 500-step 64^3
flat-interface configuration, and reproduce the reference's diagnostics at every
50-step diagnostic step; the mixed engine stays within its FP32-transform error.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import ref_cases  # noqa: E402

from smaiso_wcomp_gb300 import abi  # noqa: E402
from smaiso_wcomp_gb300.engine import Engine  # noqa: E402

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-5   # psi and rho, relative L2 (the mixed engine's bar against FP64)
NPZ = os.path.join(HERE, "golden", "ref_fixtures.npz")


@pytest.fixture(scope="module")
def npz():
    return np.load(NPZ)


def _checkpoints(fx):
    """Steps at which the engine stops: every dump step and every diagnostic step."""
    stops = set(fx.spec["dumps"]) | {int(s) for s in fx.diag[:, 0]}
    return sorted(stops)


@pytest.mark.parametrize("case", list(ref_cases.CASES))
def test_fp64_engine_matches_reference_run(lib, npz, case):
    fx = ref_cases.Fixture(npz, case)
    p = abi.default_params(*fx.shape, ref_ranks=fx.spec["ranks"])
    with Engine(p) as e:
        e.set_state(fx.psi0, None)   # rho = 0, as the reference starts (REF:1053)
        for stop in _checkpoints(fx):
            e.step(stop - e.nloop)
            if stop in fx.spec["dumps"]:
                errs = fx.errors(stop, e.field)
                bad = {f: v for f, v in errs.items() if not v <= FP64_TOL}
                assert not bad, (case, stop, bad)
                for f in ("psi", "rho", "psiq", "mu"):
                    n = fx.norm(stop, f)
                    assert abs(np.linalg.norm(e.field(f)) - n) <= FP64_TOL * n, (case, stop, f)
            rows = fx.diag[fx.diag[:, 0] == stop]
            if len(rows):
                d = e.diagnostics()
                _, l1, sum_a, sum_b, mass, energy = rows[0]
                assert d["step"] == stop and d["nonfinite"] == 0
                for k, want in (("l1", l1), ("sum_abs_psi", sum_b), ("mass", mass), ("energy", energy)):
                    assert abs(d[k] - want) <= FP64_TOL * abs(want), (case, stop, k, d[k], want)


@pytest.mark.parametrize("case", ["s64_p4", "flat64_p2"])
def test_mixed_engine_against_reference_run(lib, npz, case):
    fx = ref_cases.Fixture(npz, case)
    p = abi.default_params(*fx.shape, ref_ranks=fx.spec["ranks"], precision=abi.SWC_PREC_MIXED)
    with Engine(p) as e:
        e.set_state(fx.psi0, None)
        for stop in sorted(fx.spec["dumps"]):
            e.step(stop - e.nloop)
            errs = fx.errors(stop, e.field)
            assert errs["psi"] <= MIXED_TOL and errs["rho"] <= MIXED_TOL, (case, stop, errs)
            assert max(errs[c] for c in ("vx", "vy", "vz")) <= 1e-3, (case, stop, errs)
            rows = fx.diag[fx.diag[:, 0] == stop]
            if len(rows):
                mass = rows[0][4]
                assert abs(e.diagnostics()["mass"] - mass) <= 1e-7 * abs(mass)
