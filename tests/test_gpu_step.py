"""GPU time step through the C ABI against the FP64 oracle on the same seeded inputs."""
import os

import numpy as np
import pytest

from smaiso_wcomp_gb300 import abi, ic
from smaiso_wcomp_gb300.engine import Engine, SwcError

pytestmark = pytest.mark.gpu

FIELDS = ["psi", "rho", "amp", "divv", "vx", "vy", "vz", "vsolx", "vsoly", "vsolz", "energy", "psiq",
          "psiq_old", "nlq", "frho", "lpsi", "mu", "gpsix", "gpsiy", "gpsiz", "grhox", "grhoy", "grhoz",
          "psi_old"]
FP64_TOL = 1e-10   # relative L2 per field (the FP64 parity bar)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a)


def run_pair(O, p, psi, rho, schedule):
    o = O.Oracle(p)
    o.set_state(psi, rho)
    e = Engine(p)
    e.set_state(psi, rho)
    for n in schedule:
        assert o.step(n) == 0
        e.step(n)
    return o, e


CASES = [
    ((16, 16, 32), dict(rho_0=0.9, divv_switch=3, ref_ranks=2), "flat", [2, 3, 4]),
    ((32, 16, 8), dict(rho_0=0.8, divv_switch=2, ref_ranks=4), "undulated", [5, 5]),
    ((8, 32, 16), dict(rho_0=0.01, divv_switch=50, ref_ranks=2, nu=0.5), "band", [4]),
    ((16, 16, 16), dict(rho_0=0.5, divv_switch=0, load=1, ref_ranks=8, dt=0.002), "undulated", [3, 1]),
]


@pytest.mark.parametrize("shape,kw,gen,schedule", CASES)
def test_fp64_step_parity(lib, oracle_mod, shape, kw, gen, schedule):
    p = abi.default_params(*shape, **kw)
    psi, rho = {"flat": ic.flat_interface, "undulated": ic.undulated_interface,
                "band": ic.reference_band}[gen](p)
    if gen == "band":
        rho = None  # the reference's own start: rho = 0 (REF:1053)
    o, e = run_pair(oracle_mod, p, psi, rho, schedule)
    errs = {f: rel(e.field(f), o.field(f)) for f in FIELDS}
    # Components of vector fields are measured against the norm of the whole vector:
    # in (nearly) layered states the x and y components and v_sol are cancellations
    # (rounding noise of both codes), so a per-component relative error is meaningless.
    vectors = {"gpsi": ["gpsix", "gpsiy", "gpsiz"], "grho": ["grhox", "grhoy", "grhoz"],
               "v": ["vx", "vy", "vz", "vsolx", "vsoly", "vsolz"]}
    for comps in vectors.values():
        scale = np.sqrt(sum(np.linalg.norm(o.field(c)) ** 2 for c in comps[:3]))
        for c in comps:
            errs[c] = np.linalg.norm(e.field(c) - o.field(c)) / max(scale, 1e-300)
    bad = {f: v for f, v in errs.items() if not v <= FP64_TOL}
    assert not bad, bad
    do, de = o.diagnostics(), e.diagnostics()
    for k in ("l1", "mass", "energy", "sum_abs_psi"):
        assert abs(de[k] - do[k]) <= FP64_TOL * abs(do[k]) + 1e-300, (k, de[k], do[k])
    assert de["step"] == do["step"] == sum(schedule)


# Every compile-time FP64 line length (64, 128, 256, 512) on every axis: the first
# pass of a 3D transform runs along z (where the fused loaders LdAmp, LdLpsi,
# LdRelaxLap, LdRhoL, LdNl sit), the last along x (StNlUpdate), and the derivative
# passes (LdOffset on rho) along each axis in turn.
PRODUCTION_SHAPES = [(128, 64, 64), (256, 32, 32), (32, 256, 32), (32, 32, 256), (512, 16, 16),
                     (16, 512, 16), (16, 16, 512), (32, 128, 128)]


@pytest.mark.parametrize("shape", PRODUCTION_SHAPES)
def test_fp64_production_lengths(lib, oracle_mod, shape):
    """FP64 engine against the oracle where its compile-time passes and fused
    loaders/stores run: relax steps 1-2 and normal steps 3-4 (divv_switch = 2), all
    24 fields and the diagnostics to the FP64 parity bar."""
    p = abi.default_params(*shape, rho_0=0.8, divv_switch=2)
    psi, rho = ic.undulated_interface(p)
    o, e = run_pair(oracle_mod, p, psi, rho, [1, 3])
    errs = {f: rel(e.field(f), o.field(f)) for f in FIELDS}
    vectors = {"gpsi": ["gpsix", "gpsiy", "gpsiz"], "grho": ["grhox", "grhoy", "grhoz"],
               "v": ["vx", "vy", "vz", "vsolx", "vsoly", "vsolz"]}
    for comps in vectors.values():
        scale = np.sqrt(sum(np.linalg.norm(o.field(c)) ** 2 for c in comps[:3]))
        for c in comps:
            errs[c] = np.linalg.norm(e.field(c) - o.field(c)) / max(scale, 1e-300)
    bad = {f: v for f, v in errs.items() if not v <= FP64_TOL}
    assert not bad, bad
    do, de = o.diagnostics(), e.diagnostics()
    for k in ("l1", "mass", "energy"):
        assert abs(de[k] - do[k]) <= FP64_TOL * abs(do[k]), (k, de[k], do[k])
    e.close()
    o.close()


@pytest.mark.parametrize("shape,nsteps", [((32, 32, 32), 60), ((64, 64, 64), 30), ((128, 64, 64), 16)])
def test_mixed_step_accuracy(lib, oracle_mod, shape, nsteps):
    """Mixed engine against the FP64 oracle; 64 and 128 point lines run the FP32
    two-lines-per-thread pass, 32 point lines the runtime-length one."""
    p = abi.default_params(*shape, rho_0=0.8, divv_switch=10)
    psi, rho = ic.undulated_interface(p)
    o = oracle_mod.Oracle(p)
    o.set_state(psi, rho)
    o.step(nsteps)
    pm = abi.default_params(*shape, rho_0=0.8, divv_switch=10, precision=abi.SWC_PREC_MIXED)
    with Engine(pm) as e:
        e.set_state(psi, rho)
        e.step(nsteps)
        for f in ("psi", "rho"):
            assert rel(e.field(f), o.field(f)) <= 1e-5, f
        for f in ("vx", "vy", "vz"):
            assert rel(e.field(f), o.field(f)) <= 1e-3, f
        # mass: FP64 sums of an FP64 density advanced with FP32 sources
        assert abs(e.diagnostics()["mass"] - o.diagnostics()["mass"]) <= 1e-7 * abs(o.diagnostics()["mass"])


@pytest.mark.parametrize("shape", [(64, 64, 64), (256, 32, 32), (32, 256, 32), (32, 32, 256)])
def test_mixed_gradients_one_step(lib, oracle_mod, shape):
    """The FP32 derivative passes (DCT-II, shifted multiply, DST-III in one pass; lines
    of 64 and 256 points, each axis) and the filter pass of the amplitude (DCT-II,
    Gaussian, DCT-III along x) against the FP64 oracle after one step."""
    p = abi.default_params(*shape, rho_0=0.8, divv_switch=10)
    psi, rho = ic.undulated_interface(p)
    o = oracle_mod.Oracle(p)
    o.set_state(psi, rho)
    o.step(1)
    pm = abi.default_params(*shape, rho_0=0.8, divv_switch=10, precision=abi.SWC_PREC_MIXED)
    with Engine(pm) as e:
        e.set_state(psi, rho)
        e.step(1)
        for vec in (("gpsix", "gpsiy", "gpsiz"), ("grhox", "grhoy", "grhoz")):
            scale = np.sqrt(sum(np.linalg.norm(o.field(c)) ** 2 for c in vec))
            for c in vec:
                assert np.linalg.norm(e.field(c) - o.field(c)) <= 1e-5 * scale, c
        assert rel(e.field("amp"), o.field("amp")) <= 1e-5


def test_zero_state_fixed_point(lib):
    p = abi.default_params(16, rho_0=0.3, divv_switch=2)
    with Engine(p) as e:
        e.set_state(np.zeros((16, 16, 16)), np.full((16, 16, 16), 0.3))
        e.step(5)
        assert np.max(np.abs(e.field("psi"))) == 0.0
        np.testing.assert_allclose(e.field("rho"), 0.3, rtol=0, atol=1e-15)


@pytest.mark.parametrize("prec", [abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED])
@pytest.mark.parametrize("nsave", [3, 4])
def test_checkpoint_continuation_is_bitwise(lib, tmp_path, prec, nsave):
    """Save after nsave steps, continue, and continue a loaded copy: every field equal
    bit for bit. After an odd number of steps the mixed engine's psiq / psiq_old and
    Nl / Nl_old buffers have exchanged roles, while the loaded engine starts with the
    first assignment."""
    p = abi.default_params(16, 16, 16, rho_0=0.8, divv_switch=3, precision=prec)
    psi, rho = ic.undulated_interface(p)
    path = os.path.join(tmp_path, "state.swc")
    with Engine(p) as e:
        e.set_state(psi, rho)
        e.step(nsave)
        e.save(path)
        e.step(5)
        a = {f: e.field(f) for f in ("psi", "rho", "psiq", "psiq_old", "nlq")}
    with Engine(p) as e2:
        e2.load(path)
        assert e2.nloop == nsave
        e2.step(5)
        for f, v in a.items():
            assert np.array_equal(e2.field(f), v), f


def _pinned(shape):
    import torch
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


@pytest.mark.parametrize("prec", [abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED])
def test_field_async_matches_sync_read(lib, prec):
    """swc_get_field_async after every step returns that step's field: distinct host
    buffers (pinned and pageable) and then two alternating pinned buffers, checked
    after swc_get_field_wait."""
    p = abi.default_params(32, 16, 16, rho_0=0.8, divv_switch=2, precision=prec)
    psi, rho = ic.undulated_interface(p)
    with Engine(p) as e:
        e.set_state(psi, rho)
        bufs = [_pinned(e.shape) if s % 2 == 0 else np.empty(e.shape) for s in range(6)]
        refs = []
        for s in range(6):
            e.step(1)
            e.field_async("psi" if s != 3 else "rho", bufs[s])
            refs.append(e.field("psi" if s != 3 else "rho"))
        e.field_wait()
        for s in range(6):
            assert np.array_equal(bufs[s], refs[s]), s
        alt = [_pinned(e.shape), _pinned(e.shape)]
        refs = []
        for s in range(5):
            e.step(1)
            refs.append(e.field("psi"))
            e.field_async("psi", alt[s & 1])
        e.field_wait()
        assert np.array_equal(alt[0], refs[4])
        assert np.array_equal(alt[1], refs[3])
        assert not np.array_equal(refs[3], refs[4])


@pytest.mark.parametrize("prec", [abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED])
def test_step_async_matches_step(lib, prec):
    """swc_step_async + swc_sync give the fields and diagnostics of swc_step; a field
    read after swc_step_async waits for the steps; swc_sync reports a non-finite state."""
    p = abi.default_params(16, 32, 16, rho_0=0.8, divv_switch=3, precision=prec, diag_interval=4)
    psi, rho = ic.undulated_interface(p)
    with Engine(p) as a, Engine(p) as b:
        a.set_state(psi, rho)
        b.set_state(psi, rho)
        b.prepare()
        for _ in range(9):
            a.step(1)
            b.step_async(1)
        assert np.array_equal(b.field("psi"), a.field("psi"))
        b.sync()
        assert b.diagnostics() == a.diagnostics() and b.diagnostics()["step"] == 8
        for f in ("psi", "rho", "vx", "vsoly", "psiq"):
            assert np.array_equal(a.field(f), b.field(f)), f
        bad = psi.copy()
        bad[3, 4, 5] = np.nan
        b.set_state(bad, rho)
        b.step_async(4)
        with pytest.raises(SwcError) as ex:
            b.sync()
        assert ex.value.status == abi.SWC_ERR_NONFINITE


def test_nonfinite_detected(lib):
    p = abi.default_params(8)
    psi = np.zeros((8, 8, 8))
    psi[1, 2, 3] = np.nan
    with Engine(p) as e:
        e.set_state(psi)
        with pytest.raises(SwcError) as ex:
            e.step(2)
        assert ex.value.status == abi.SWC_ERR_NONFINITE


def test_step_before_state_is_rejected(lib):
    with Engine(abi.default_params(8)) as e:
        with pytest.raises(SwcError) as ex:
            e.step(1)
        assert ex.value.status == abi.SWC_ERR_STATE


def test_watchdog_returns_timeout_and_context_recovers(lib):
    p = abi.default_params(128, rho_0=0.8, watchdog_s=1e-6)
    psi, rho = ic.flat_interface(p)
    with Engine(p) as e:
        e.set_state(psi, rho)
        rc = e.step(3, check=False)
        assert rc == abi.SWC_ERR_TIMEOUT
        # the queued steps still complete; the context stays usable
        psi_after = e.field("psi")
        assert np.all(np.isfinite(psi_after))
        assert e.nloop == 3


def test_full_size_fp64_vs_mixed_256(lib):
    """At 256^3, with both engines alive in one process (each on its own non-blocking
    stream): a few steps stay finite and agree (mixed within 1e-5 on psi)."""
    engines = {}
    for prec in (abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED):
        engines[prec] = Engine(abi.default_params(256, rho_0=0.8, divv_switch=3, precision=prec))
    p = engines[0].p
    psi, rho = ic.undulated_interface(p)
    out = {}
    for prec, e in engines.items():
        e.set_state(psi, rho)
        e.step(5)
        out[prec] = (e.field("psi"), e.diagnostics())
    for e in engines.values():
        e.close()
    assert out[0][1]["nonfinite"] == 0 and out[1][1]["nonfinite"] == 0
    assert rel(out[1][0], out[0][0]) <= 1e-5


def test_dislocations_512x512x256_mixed_vs_fp64(lib):
    """The 512x512x256 layer-dislocation workload (16 seeded edge dislocations below a
    flat interface): both engines run 8 steps from the same state; the mixed engine's
    psi, rho and v stay within the FP32-transform error of the FP64 engine."""
    p64 = abi.default_params(512, 512, 256, rho_0=0.8)
    psi, rho = ic.dislocations(p64)
    out = {}
    for prec in (abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED):
        with Engine(abi.default_params(512, 512, 256, rho_0=0.8, precision=prec)) as e:
            e.set_state(psi, rho)
            e.step(8)
            assert e.diagnostics()["nonfinite"] == 0
            out[prec] = {f: e.field(f) for f in ("psi", "rho", "vx", "vy", "vz")}
    a, b = out[abi.SWC_PREC_MIXED], out[abi.SWC_PREC_FP64]
    assert rel(a["psi"], b["psi"]) <= 1e-5
    assert rel(a["rho"], b["rho"]) <= 1e-6
    vn = np.sqrt(sum(np.linalg.norm(b[c]) ** 2 for c in ("vx", "vy", "vz")))
    dv = np.sqrt(sum(np.linalg.norm(a[c] - b[c]) ** 2 for c in ("vx", "vy", "vz")))
    assert dv <= 1e-3 * vn


@pytest.mark.parametrize("prec", [abi.SWC_PREC_FP64, abi.SWC_PREC_MIXED])
def test_diag_interval_cadence(lib, prec):
    """diag_interval = 3: diagnostics at nLoop % 3 == 0 only, equal to those of a run that
    ends its swc_step call on the same step; every field of the current step is still
    readable (v_sol included), the energy density only at diagnostic steps."""
    p = abi.default_params(16, 16, 32, rho_0=0.8, divv_switch=2, precision=prec)
    psi, rho = ic.undulated_interface(p)
    q = abi.default_params(16, 16, 32, rho_0=0.8, divv_switch=2, precision=prec, diag_interval=3)
    with Engine(p) as a, Engine(q) as b:
        a.set_state(psi, rho)
        b.set_state(psi, rho)
        a.step(6)
        for _ in range(6):
            b.step(1)
        da, db = a.diagnostics(), b.diagnostics()
        assert db["step"] == 6 and da == db
        assert np.array_equal(a.field("energy"), b.field("energy"))
        a.step(1)
        b.step(1)
        assert b.diagnostics() == db  # step 7 ran no diagnostics
        for f in ("psi", "rho", "vx", "vsolx", "vsolz", "divv", "psiq"):
            assert np.array_equal(a.field(f), b.field(f)), f
        with pytest.raises(SwcError) as ex:
            b.field("energy")
        assert ex.value.status == abi.SWC_ERR_STATE
        a.step(2)
        b.step(2)
        assert b.diagnostics()["step"] == 9 and a.diagnostics() == b.diagnostics()
