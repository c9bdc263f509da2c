"""Initial conditions generated on the device (swc_ic_generate, swc_set_state_ic)
against the host generators (smaiso_wcomp_gb300/ic.py), the oracle's restatement of
the reference's band and focal-conic loops (REF:575-707), and a run of the
reference's own code from its own initial state."""
import ctypes
import os
import sys

import numpy as np
import pytest

from smaiso_wcomp_gb300 import abi, ic
from smaiso_wcomp_gb300.engine import Engine, default_ic

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import ref_cases  # noqa: E402

pytestmark = pytest.mark.gpu


def generate(lib, p, kind, with_rho=True, **fields):
    torch = pytest.importorskip("torch")
    spec = default_ic(p, kind, lib=lib, **fields)
    psi = torch.empty((p.nx, p.ny, p.nz), dtype=torch.float64, device="cuda")
    rho = torch.empty_like(psi) if with_rho else None
    s = torch.cuda.current_stream()
    rc = lib.swc_ic_generate(ctypes.byref(p), ctypes.byref(spec), ctypes.c_void_p(psi.data_ptr()),
                             ctypes.c_void_p(rho.data_ptr() if with_rho else None), ctypes.c_void_p(s.cuda_stream))
    assert rc == abi.SWC_OK, lib.swc_last_error()
    torch.cuda.synchronize()
    return psi.cpu().numpy(), (rho.cpu().numpy() if with_rho else None)


SHAPES = [(32, 32, 32), (64, 16, 32), (16, 32, 128)]


@pytest.mark.parametrize("shape", SHAPES)
def test_uniform_noise_is_bit_exact(lib, shape):
    """The counter-based uniform noise (SplitMix64 of seed ^ index) is integer hashing:
    with a vanishing smooth part the device field is the host noise bit for bit."""
    p = abi.default_params(*shape)
    psi, _ = generate(lib, p, abi.SWC_IC_FLAT, amp=1e-300, noise=1e-4)
    assert np.array_equal(psi, ic.uniform_noise(shape, 1001, 1e-4))


@pytest.mark.parametrize("shape", SHAPES)
def test_workload_states_match_host_generators(lib, shape):
    p = abi.default_params(*shape, rho_0=0.8)
    cases = [
        (abi.SWC_IC_FLAT, ic.flat_interface(p)),
        (abi.SWC_IC_UNDULATED, ic.undulated_interface(p)),
        (abi.SWC_IC_DISLOCATIONS, ic.dislocations(p)),
    ]
    for kind, (hpsi, hrho) in cases:
        psi, rho = generate(lib, p, kind)
        # the dislocation phase sums 16 atan2 terms of up to ~pi each before the cosine
        tol = 1e-13 if kind == abi.SWC_IC_DISLOCATIONS else 1e-14
        assert np.linalg.norm(psi - hpsi) <= tol * np.linalg.norm(hpsi), kind
        assert np.linalg.norm(rho - hrho) <= 1e-14 * np.linalg.norm(hrho), kind


@pytest.mark.parametrize("shape", [(32, 32, 32), (64, 64, 64), (32, 64, 64)])
def test_reference_states_match_the_oracle(lib, oracle_mod, shape):
    """The reference's band (with and without its layer perturbation phi) and its two
    commented-out focal-conic states, against the oracle's restatement of those loops."""
    p = abi.default_params(*shape)
    ae = 3.0 * p.nz / 8
    cases = [
        (abi.SWC_IC_BAND, {}, dict()),
        (abi.SWC_IC_BAND, dict(phi=3.0, qi=0.3), dict(phi=3.0, qi=0.3)),
        (abi.SWC_IC_FOCAL_CONIC, {}, dict(ae=ae)),
        (abi.SWC_IC_FOCAL_CONICS, dict(gap=2.0), dict(ae=ae, gap=2.0)),
    ]
    for kind, fields, oargs in cases:
        psi, rho = generate(lib, p, kind, **fields)
        ref = oracle_mod.reference_ic(p, kind, **oargs)
        assert np.count_nonzero(ref) > 0
        assert np.array_equal(psi != 0, ref != 0), kind
        assert np.max(np.abs(psi - ref)) <= 1e-15, (kind, np.max(np.abs(psi - ref)))
        assert not np.any(rho), kind   # the reference zero-fills rho (REF:1053)


def test_set_state_ic_band_matches_reference_run(lib):
    """The reference's own initial state generated on the device, then 100 steps: the
    fields of the reference's run from that state (fixture band_p2) to the FP64 bar."""
    fx = ref_cases.Fixture(np.load(os.path.join(HERE, "golden", "ref_fixtures.npz")), "band_p2")
    p = abi.default_params(*fx.shape, ref_ranks=fx.spec["ranks"])
    with Engine(p) as e:
        e.set_state_ic(abi.SWC_IC_BAND)
        for stop in sorted(fx.spec["dumps"]):
            e.step(stop - e.nloop)
            errs = fx.errors(stop, e.field)
            bad = {f: v for f, v in errs.items() if not v <= 1e-10}
            assert not bad, (stop, bad)


@pytest.mark.parametrize("prec", [abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED])
def test_set_state_ic_matches_host_state(lib, prec):
    """swc_set_state_ic and swc_set_state from the host generator's arrays start the same
    run. The device and the host evaluate the initial formula separately, so the two FP64
    states differ in their last bits; the FP64 engine keeps them that close (1e-12 after
    3 steps). The mixed engine narrows FP64 values to FP32 every step, and where two values
    that differ in their last bits round to neighbouring FP32 numbers the runs part at
    FP32 rounding (2.5e-8 in psi after 3 steps here): it is held to 1e-6. Two runs from the
    same start are bit for bit equal in both engines."""
    p = abi.default_params(64, 32, 64, rho_0=0.8, divv_switch=2, precision=prec)
    hpsi, hrho = ic.undulated_interface(p)
    tol = 1e-12 if prec == abi.SWC_PREC_FP64 else 1e-6
    with Engine(p) as a, Engine(p) as b, Engine(p) as c:
        a.set_state(hpsi, hrho)
        b.set_state_ic(abi.SWC_IC_UNDULATED)
        c.set_state_ic(abi.SWC_IC_UNDULATED)
        a.step(3)
        b.step(3)
        c.step(3)
        for f in ("psi", "rho", "psiq", "amp"):
            x, y = a.field(f), b.field(f)
            assert np.linalg.norm(x - y) <= tol * np.linalg.norm(x), f
            assert np.array_equal(y, c.field(f)), f


def test_bad_initial_condition_is_rejected(lib):
    from smaiso_wcomp_gb300.engine import SwcError
    p = abi.default_params(16)
    with Engine(p) as e:
        with pytest.raises(SwcError) as ex:
            e.set_state_ic(abi.SWC_IC_FOCAL_CONIC, ae=0.0)
        assert ex.value.status == abi.SWC_ERR_BAD_PARAM
        with pytest.raises(SwcError):
            e.set_state_ic(abi.SWC_IC_FLAT, xi=0.0)
