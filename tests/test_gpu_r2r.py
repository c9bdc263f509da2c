"""GPU r2r plans (swc_r2r_*) against the golden vectors and the oracle."""
import os

import numpy as np
import pytest

from smaiso_wcomp_gb300 import abi
from smaiso_wcomp_gb300.engine import R2RPlan

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "r2r_golden.npz"))
PLANS = {"CT": (0, 0, 0), "iCT": (1, 1, 1), "STx": (2, 0, 0), "iSTx": (3, 1, 1),
         "STy": (0, 2, 0), "iSTy": (1, 3, 1), "STz": (0, 0, 2), "iSTz": (1, 1, 3)}
TOL = {abi.SWC_PREC_FP64: 1e-14, abi.SWC_PREC_MIXED: 3e-6}


@pytest.mark.parametrize("prec", [abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED])
@pytest.mark.parametrize("plan", list(PLANS))
def test_plans_golden(lib, plan, prec):
    a = GOLD["a3"]
    got = R2RPlan(a.shape, PLANS[plan], prec, lib=lib)(a)
    ref = GOLD[f"plan_{plan}"]
    assert np.max(np.abs(got - ref)) <= TOL[prec] * np.max(np.abs(ref))


@pytest.mark.parametrize("prec", [abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED])
@pytest.mark.parametrize("n", [4, 8, 16, 32, 64, 128, 256, 512, 1024])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_every_length_and_axis(lib, oracle_mod, n, axis, prec):
    shape = [4, 4, 4]
    shape[axis] = n
    a = np.random.default_rng(n + axis).standard_normal(shape)
    eps = 2.2e-16 if prec == abi.SWC_PREC_FP64 else 1.2e-7
    for kinds in [(0, 0, 0), (1, 1, 1), (2, 2, 2), (3, 3, 3), (2, 1, 0), (3, 0, 1)]:
        ref = oracle_mod.r2r3d(a, kinds)
        got = R2RPlan(shape, kinds, prec, lib=lib)(a)
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= 40 * eps * np.log2(8 * n), (kinds, err)


@pytest.mark.parametrize("n", [64, 128, 256, 512])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_fp32_two_line_pass(lib, oracle_mod, n, axis):
    """FP32 compile-time lengths on every axis and kind, against the oracle, with nz = 64
    and 512 lines so every axis takes the TMA-fed two-lines-per-thread pass."""
    shape = [8, 8, 64] if axis != 2 else [8, 64, n]
    shape[axis] = n
    a = np.random.default_rng(100 * n + axis).standard_normal(shape)
    for kinds in [(0, 0, 0), (1, 1, 1), (2, 2, 2), (3, 3, 3), (2, 1, 0), (3, 0, 1), (1, 2, 3)]:
        ref = oracle_mod.r2r3d(a, kinds)
        got = R2RPlan(shape, kinds, abi.SWC_PREC_MIXED, lib=lib)(a)
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= 40 * 1.2e-7 * np.log2(8 * n), (kinds, err)


def test_misaligned_device_buffer_is_rejected(lib):
    torch = pytest.importorskip("torch")
    from smaiso_wcomp_gb300.engine import SwcError
    t = torch.zeros(8 * 8 * 64 + 4, dtype=torch.float32, device="cuda")
    plan = R2RPlan((8, 8, 64), (0, 0, 0), abi.SWC_PREC_MIXED, lib=lib)
    with pytest.raises(SwcError):
        plan.execute_device(t.data_ptr() + 4, torch.cuda.current_stream().cuda_stream)
    with pytest.raises(SwcError):
        plan.execute_axis(2, t.data_ptr() + 4, torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("prec", [abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED])
def test_round_trip_256(lib, prec):
    """Size-independent property at the benchmark size: DCT-III^3(DCT-II^3 x) = (2n)^3 x,
    DST-III(DST-II) on x likewise."""
    n = 256
    x = np.random.default_rng(7).standard_normal((n, n, n))
    for f, b in (((0, 0, 0), (1, 1, 1)), ((2, 0, 0), (3, 1, 1)), ((0, 2, 2), (1, 3, 3))):
        y = R2RPlan(x.shape, b, prec, lib=lib)(R2RPlan(x.shape, f, prec, lib=lib)(x))
        err = np.linalg.norm(y / (8.0 * n ** 3) - x) / np.linalg.norm(x)
        assert err <= (1e-14 if prec == abi.SWC_PREC_FP64 else 2e-6), err


@pytest.mark.parametrize("plan", ["CT", "iCT", "STx", "iSTy", "STz", "iSTz"])
def test_fp64_plan_256_against_oracle(lib, oracle_mod, plan):
    """FP64 plans at the benchmark size (compile-time 256-point passes on every axis)
    against the oracle's transform of the same array, element by element."""
    n = 256
    x = np.random.default_rng(31).standard_normal((n, n, n))
    ref = oracle_mod.r2r3d(x, PLANS[plan])
    got = R2RPlan(x.shape, PLANS[plan], abi.SWC_PREC_FP64, lib=lib)(x)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-14
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_execute_on_device_buffer(lib):
    """swc_r2r_execute on caller-owned device memory (the in-place fftw_execute analogue)."""
    torch = pytest.importorskip("torch")
    a = np.random.default_rng(3).standard_normal((16, 32, 64))
    t = torch.from_numpy(a).cuda()
    plan = R2RPlan(a.shape, (2, 0, 1), abi.SWC_PREC_FP64, lib=lib)
    plan.execute_device(t.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    np.testing.assert_allclose(t.cpu().numpy(), plan(a), rtol=0, atol=1e-12 * np.abs(plan(a)).max())


@pytest.mark.parametrize("shape", [(256, 64, 64), (64, 64, 256)])
def test_tma_wait_that_runs_out_reports_status_and_recovers(lib, oracle_mod, shape):
    """The TMA-fed pass's bounded wait: a wait that expects 16 bytes more than its copy
    delivers runs out after 4096 polls, the CTA sets the status flag and returns, the host
    reads SWC_ERR_CUDA; the context stays usable and the next run is correct. Every axis
    takes the TMA-fed pass; in the second shape the z pass is the 256-point one whose
    tile arrives as 32 line copies (row staging)."""
    from smaiso_wcomp_gb300.engine import SwcError
    a = np.random.default_rng(11).standard_normal(shape)
    plan = R2RPlan(shape, (0, 0, 0), abi.SWC_PREC_MIXED, lib=lib)
    plan.set_wait_test(16, 4096)
    with pytest.raises(SwcError) as ei:
        plan(a)
    assert "did not complete" in str(ei.value)
    plan.set_wait_test(0, 1 << 22)
    ref = oracle_mod.r2r3d(a, (0, 0, 0))
    got = plan(a)
    assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(np.abs(ref))
