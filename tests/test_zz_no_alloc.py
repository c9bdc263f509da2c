"""swc_diagnostics_noalloc: the diagnostic reduction for callers that cannot allocate
device memory (its scratch is a fixed array inside libswc.so).

It must give the same sums as swc_diagnostics -- the context's reduction, whose
scratch is allocated with cudaMalloc -- on the same fields, call after call. This
file is collected last so a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

from smaiso_wcomp_gb300 import abi, ic
from smaiso_wcomp_gb300.engine import Engine

pytestmark = pytest.mark.gpu
TOL = 1e-10   # the FP64 parity tolerance of the other GPU tests


def noalloc(lib, p, e, stream=None):
    ptrs = [ctypes.c_void_p(e.device_ptr(f)[0]) for f in ("psi", "psi_old", "rho", "lpsi", "amp")]
    d = abi.SwcDiag()
    rc = lib.swc_diagnostics_noalloc(ctypes.byref(p), *ptrs, ctypes.c_void_p(stream), ctypes.byref(d))
    assert rc == abi.SWC_OK, lib.swc_last_error()
    return d.as_dict()


@pytest.mark.parametrize("shape,steps", [((32, 32, 32), 12), ((256, 128, 128), 3)])
def test_noalloc_matches_context_diagnostics(lib, shape, steps):
    p = abi.default_params(*shape, rho_0=0.8, divv_switch=4)
    psi, rho = ic.undulated_interface(p)
    with Engine(p, lib=lib) as e:
        e.set_state(psi, rho)
        e.step(steps)
        for name in ("psi", "psi_old", "rho", "lpsi", "amp"):
            assert e.device_ptr(name)[1] == 8
        ref = e.diagnostics()
        first = noalloc(lib, p, e)
        second = noalloc(lib, p, e)
    for got in (first, second):
        for k in ("l1", "mass", "energy", "sum_abs_dpsi", "sum_abs_psi", "sum_rho", "sum_energy"):
            assert abs(got[k] - ref[k]) <= TOL * abs(ref[k]), (k, got[k], ref[k])
        assert got["nonfinite"] == 0
    assert first == second


def test_noalloc_on_a_caller_stream(lib):
    """On a stream the caller created (not the legacy default stream), twice in a row."""
    torch = pytest.importorskip("torch")
    p = abi.default_params(64, 32, 32, rho_0=0.8, divv_switch=2)
    psi, rho = ic.undulated_interface(p)
    s = torch.cuda.Stream()
    with Engine(p, lib=lib) as e:
        e.set_state(psi, rho)
        e.step(5)
        ref = e.diagnostics()
        got = [noalloc(lib, p, e, s.cuda_stream) for _ in range(2)]
    for g in got:
        for k in ("l1", "mass", "energy", "sum_rho"):
            assert abs(g[k] - ref[k]) <= TOL * abs(ref[k]), (k, g[k], ref[k])
    assert got[0] == got[1]


def test_noalloc_counts_nonfinite_values(lib):
    """A NaN in the initial psi spreads through the step; the non-finite count of the
    allocation-free reduction equals the context's."""
    p = abi.default_params(16, 16, 32, rho_0=0.8, divv_switch=2)
    psi, rho = ic.undulated_interface(p)
    psi = psi.copy()
    psi[3, 4, 5] = np.nan
    with Engine(p, lib=lib) as e:
        e.set_state(psi, rho)
        assert e.step(2, check=False) == abi.SWC_ERR_NONFINITE
        ref = e.diagnostics()
        got = noalloc(lib, p, e)
    assert ref["nonfinite"] > 0
    assert got["nonfinite"] == ref["nonfinite"]


def test_noalloc_rejects_grids_beyond_its_scratch(lib):
    p = abi.default_params(1024, 1024, 512)   # 2^29 points > SWC_NOALLOC_MAX_POINTS
    d = abi.SwcDiag()
    rc = lib.swc_diagnostics_noalloc(ctypes.byref(p), *([ctypes.c_void_p(16)] * 5), None, ctypes.byref(d))
    assert rc == abi.SWC_ERR_BAD_PARAM
    assert b"exceed" in lib.swc_last_error()
