"""Discrete adjoint (swc_backward) against central finite differences of the FP64
forward through the C ABI, and a torch.autograd.gradcheck over the thin shim."""
import numpy as np
import pytest

from smaiso_wcomp_gb300 import abi, ic, schedule
from smaiso_wcomp_gb300.engine import Engine

pytestmark = pytest.mark.gpu
COEFFS = ("alpha", "beta", "gamma", "nu", "rho_0")


def loss(e, wp, wr):
    return float(np.sum(wp * e.field("psi")) + np.sum(wr * e.field("rho")))


def run(p, psi0, rho0, nsteps, wp, wr):
    with Engine(p) as e:
        e.set_state(psi0, rho0)
        for _ in range(nsteps):
            e.step(1)
        return loss(e, wp, wr)


CASES = [  # shape, divv_switch, steps, checkpoint interval (-1: binomial): relax + normal phase
    ((16, 16, 32), 3, 6, 2),
    ((16, 8, 16), 2, 5, 4),
    ((8, 16, 16), 0, 3, 1),
    ((16, 16, 16), 2, 7, -1),
]


@pytest.mark.parametrize("shape,ds,nsteps,ckpt", CASES)
def test_adjoint_matches_finite_differences(lib, shape, ds, nsteps, ckpt):
    rng = np.random.default_rng(7)
    p = abi.default_params(*shape, rho_0=0.8, divv_switch=ds, adjoint_ckpt=ckpt, ref_ranks=2)
    psi0, rho0 = ic.undulated_interface(p, sigma=1e-2)
    wp = rng.standard_normal(shape)
    wr = rng.standard_normal(shape)
    with Engine(p) as e:
        e.set_state(psi0, rho0)
        e.step(nsteps)
        L0 = loss(e, wp, wr)
        g = e.backward(dpsi=wp, drho=wr, want_psi0=True, want_rho0=True)
        # the state at step T is restored
        assert abs(loss(e, wp, wr) - L0) <= 1e-14 * abs(L0)
    assert g["steps"] == nsteps
    # directional derivative along psi0 and rho0
    for key, base in (("psi0", psi0), ("rho0", rho0)):
        d = rng.standard_normal(shape)
        h = 1e-5
        args_p = (psi0 + h * d, rho0) if key == "psi0" else (psi0, rho0 + h * d)
        args_m = (psi0 - h * d, rho0) if key == "psi0" else (psi0, rho0 - h * d)
        fd = (run(p, *args_p, nsteps, wp, wr) - run(p, *args_m, nsteps, wp, wr)) / (2 * h)
        ad = float(np.sum(g[key] * d))
        assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-12 * abs(L0)), (key, ad, fd)
    # coefficients: 4th-order central difference, h = 1e-3 relative (truncation O(h^4),
    # rounding ~1e-13 |L| / h): accurate to well below the 1e-6 bar for small gradients
    errs = {}
    for name in COEFFS:
        v = getattr(p, name)
        h = 1e-3 * max(abs(v), 1e-3)

        def L_at(x):
            q = abi.SwcParams.from_buffer_copy(p)
            setattr(q, name, x)
            return run(q, psi0, rho0, nsteps, wp, wr)

        fd = (8 * (L_at(v + h) - L_at(v - h)) - (L_at(v + 2 * h) - L_at(v - 2 * h))) / (12 * h)
        errs[name] = (g[name], fd, abs(g[name] - fd) / max(abs(fd), 1e-9))
    bad = {k: e for k, e in errs.items() if not e[2] <= 1e-6}
    assert not bad, bad


def energy_loss(e, wp, lam):
    return float(np.sum(wp * e.field("psi"))) + lam * e.diagnostics()["energy"]


@pytest.mark.parametrize("ckpt", [2, -1])
def test_energy_term_adjoint_matches_finite_differences(lib, ckpt):
    """swc_backward_energy: L = sum(w psi(T)) + lambda E(T), E(T) the free-energy
    diagnostic of the last step (its stale dfDlapPsi and the step's filtered amplitude),
    against 4th-order central differences of the FP64 forward: directional derivatives
    along psi0 and rho0 and the five coefficient gradients within 1e-6. A second call
    returns the same gradients (the last step's dfDlapPsi and amplitude are put back)."""
    shape, ds, nsteps, lam = (16, 16, 16), 2, 5, 0.7
    rng = np.random.default_rng(11)
    p = abi.default_params(*shape, rho_0=0.8, divv_switch=ds, adjoint_ckpt=ckpt, ref_ranks=2)
    psi0, rho0 = ic.undulated_interface(p, sigma=1e-2)
    wp = rng.standard_normal(shape)

    def L_run(q, a, b):
        with Engine(q) as e:
            e.set_state(a, b)
            e.step(nsteps)
            return energy_loss(e, wp, lam)

    with Engine(p) as e:
        e.set_state(psi0, rho0)
        e.step(nsteps)
        L0 = energy_loss(e, wp, lam)
        g = e.backward(dpsi=wp, want_psi0=True, want_rho0=True, energy_lambda=lam)
        g2 = e.backward(dpsi=wp, want_psi0=True, want_rho0=True, energy_lambda=lam)
        g0 = e.backward(dpsi=wp, want_psi0=True, want_rho0=True)
    for key in ("psi0", "rho0"):
        assert np.array_equal(g[key], g2[key]), key
        assert not np.allclose(g[key], g0[key]), key   # the energy term contributes
    # 4th-order differences: truncation O(h^4), FP64 roundoff about 1e-14 |L| / h, the
    # floor under the 1e-6 bar. psi0 (L strongly nonlinear in it) at h = 1e-4; rho0 at
    # h = 1e-3: its directional derivative is ~5e-6 |L| (the relax phase resets rho, REF:1371)
    for key, h in (("psi0", 1e-4), ("rho0", 1e-3)):
        d = rng.standard_normal(shape)
        at = lambda t: L_run(p, psi0 + t * d, rho0) if key == "psi0" else L_run(p, psi0, rho0 + t * d)  # noqa: E731
        fd = (8 * (at(h) - at(-h)) - (at(2 * h) - at(-2 * h))) / (12 * h)
        ad = float(np.sum(g[key] * d))
        assert abs(ad - fd) <= 1e-6 * abs(fd) + 1e-14 * abs(L0) / h, (key, ad, fd)
    errs = {}
    for name in COEFFS:
        v = getattr(p, name)
        h = 1e-3 * max(abs(v), 1e-3)

        def L_at(x):
            q = abi.SwcParams.from_buffer_copy(p)
            setattr(q, name, x)
            return L_run(q, psi0, rho0)

        fd = (8 * (L_at(v + h) - L_at(v - h)) - (L_at(v + 2 * h) - L_at(v - 2 * h))) / (12 * h)
        errs[name] = (g[name], fd, abs(g[name] - fd) / max(abs(fd), 1e-9))
        assert g2[name] == g[name], name
    bad = {k: v for k, v in errs.items() if not v[2] <= 1e-6}
    assert not bad, bad


def test_backward_needs_checkpoints_and_fp64(lib):
    from smaiso_wcomp_gb300.engine import SwcError
    with Engine(abi.default_params(8)) as e:
        e.set_state(np.zeros((8, 8, 8)))
        e.step(1)
        with pytest.raises(SwcError):
            e.backward(dpsi=np.zeros((8, 8, 8)))


def test_torch_gradcheck_through_the_shim(lib):
    torch = pytest.importorskip("torch")
    from smaiso_wcomp_gb300.autograd import StepFunction
    base = abi.default_params(8, 8, 8, rho_0=0.8, divv_switch=1)
    psi0, rho0 = ic.undulated_interface(base, sigma=1e-2)
    x = torch.tensor(psi0, dtype=torch.float64, requires_grad=True)
    c = torch.tensor([base.alpha, base.beta, base.gamma, base.nu, base.rho_0], dtype=torch.float64,
                     requires_grad=True)
    f = lambda x, c: StepFunction.apply(x, c, base, 2, rho0, 1)  # noqa: E731
    assert torch.autograd.gradcheck(f, (x, c), eps=1e-6, atol=1e-7, rtol=1e-5, fast_mode=True)


@pytest.mark.parametrize("snapshots", [0, 1, 2, 4, 12])
def test_binomial_schedule_matches_segments(lib, snapshots):
    """Binomial checkpointing (adjoint_ckpt = -1) with 0, 1, 2, 4 and 12 snapshot slots
    reverses the same trajectory as the fixed-interval schedule: the same gradients
    (the recompute is deterministic, snapshots after step 0 recompute psi from psiq),
    at the optimal binomial cost (smaiso_wcomp_gb300.schedule) plus one taped rerun per
    step."""
    shape, ds, nsteps = (16, 16, 32), 4, 13
    rng = np.random.default_rng(3)
    wp, wr = rng.standard_normal(shape), rng.standard_normal(shape)
    grads = {}
    for ckpt in (3, -1):
        p = abi.default_params(*shape, rho_0=0.8, divv_switch=ds, adjoint_ckpt=ckpt, ref_ranks=2,
                               adjoint_snapshots=snapshots if ckpt < 0 else 0)
        psi0, rho0 = ic.undulated_interface(p, sigma=1e-2)
        with Engine(p) as e:
            e.set_state(psi0, rho0)
            e.step(nsteps)
            grads[ckpt] = e.backward(dpsi=wp, drho=wr, want_psi0=True, want_rho0=True)
    a, b = grads[-1], grads[3]
    s = min(snapshots, nsteps - 1) if snapshots > 0 else nsteps - 1
    assert a["snapshots"] == s
    assert a["forward_steps"] == schedule.forward_steps(nsteps, s)
    assert a["forward_steps"] == schedule.optimal_advances(nsteps, s) + nsteps
    assert b["forward_steps"] == nsteps
    for key in ("psi0", "rho0"):
        assert np.linalg.norm(a[key] - b[key]) <= 1e-12 * np.linalg.norm(b[key]), key
    for name in COEFFS:
        assert abs(a[name] - b[name]) <= 1e-12 * max(abs(b[name]), 1e-30), name


def test_binomial_cap_too_small_is_rejected(lib):
    from smaiso_wcomp_gb300.engine import SwcError
    p = abi.default_params(16, 16, 16, adjoint_ckpt=-1, adjoint_cap_gb=1e-6)
    with Engine(p) as e:
        e.set_state(np.zeros((16, 16, 16)))
        e.step(3)
        with pytest.raises(SwcError):
            e.backward(dpsi=np.ones((16, 16, 16)))


@pytest.mark.parametrize("shape", [(32, 32, 32), (64, 64, 64)])
def test_fp32_adjoint_of_the_mixed_engine(lib, shape):
    """The mixed engine's FP32 adjoint (same kernels, T = float, on the mixed trajectory)
    agrees with the FP64 adjoint of the FP64 engine to FP32 accuracy, and its binomial
    schedule returns its fixed-interval gradients. 32-point lines run the runtime-length
    passes, 64-point lines the TMA-fed FP32 passes (and the FP64 engine its fixed-length
    ones), each with its own transposed derivative pass."""
    ds, nsteps = 3, 10
    rng = np.random.default_rng(5)
    wp, wr = rng.standard_normal(shape), rng.standard_normal(shape)
    g = {}
    for prec, ckpt in ((abi.SWC_PREC_FP64, 5), (abi.SWC_PREC_MIXED, 5), (abi.SWC_PREC_MIXED, -1)):
        p = abi.default_params(*shape, rho_0=0.8, divv_switch=ds, adjoint_ckpt=ckpt, ref_ranks=2, precision=prec)
        psi0, rho0 = ic.undulated_interface(p, sigma=1e-2)
        with Engine(p) as e:
            e.set_state(psi0, rho0)
            e.step(nsteps)
            g[(prec, ckpt)] = e.backward(dpsi=wp, drho=wr, want_psi0=True, want_rho0=True)
    ref, f32, f32b = g[(abi.SWC_PREC_FP64, 5)], g[(abi.SWC_PREC_MIXED, 5)], g[(abi.SWC_PREC_MIXED, -1)]
    for key in ("psi0", "rho0"):
        assert np.linalg.norm(f32[key] - ref[key]) <= 1e-4 * np.linalg.norm(ref[key]), key
        assert np.array_equal(f32b[key], f32[key]), key
    for name in COEFFS:
        assert abs(f32[name] - ref[name]) <= 1e-3 * abs(ref[name]) + 1e-6, (name, f32[name], ref[name])
        assert f32b[name] == f32[name], name
