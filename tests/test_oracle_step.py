"""Analytic properties of the FP64 oracle's time step (the reference has no tests
or fixtures for its loop, so these pin the restatement instead)."""
import numpy as np

from smaiso_wcomp_gb300 import abi, ic


def make(O, shape=(8, 8, 16), **kw):
    p = abi.default_params(*shape, **kw)
    return p, O.Oracle(p)


def test_zero_state_is_a_fixed_point(oracle_mod):
    p, o = make(oracle_mod, rho_0=0.3, divv_switch=3)
    psi = np.zeros((8, 8, 16))
    rho = np.full_like(psi, 0.3)
    o.set_state(psi, rho)
    assert o.step(6) == 0
    assert np.max(np.abs(o.field("psi"))) == 0.0
    np.testing.assert_allclose(o.field("rho"), 0.3, rtol=0, atol=1e-15)
    for f in ("vx", "vy", "vz", "divv", "amp"):
        assert np.max(np.abs(o.field(f))) < 1e-15


def test_single_cosine_mode_derivatives(oracle_mod):
    """psi = a cos(pi m (k+1/2)/nz) is DCT mode m: its gradient is the sine mode m-1
    with wavenumber Vs[m-1] = pi m / Lz (REF:1218), and dfDlapPsi = alpha (q0^2 - q^2) psi."""
    p, o = make(oracle_mod, shape=(4, 4, 32))
    d = abi.derived(p)
    m, a = 5, 0.3
    k = np.arange(32)
    psi = np.broadcast_to(a * np.cos(np.pi * m * (k + 0.5) / 32), (4, 4, 32)).copy()
    o.set_state(psi)
    o.step(1)
    q = np.pi * m / d["lz"]
    gz = o.field("gpsiz")[0, 0]
    np.testing.assert_allclose(gz, -a * q * np.sin(np.pi * m * (k + 0.5) / 32), atol=1e-13)
    assert np.max(np.abs(o.field("gpsix"))) < 1e-14 and np.max(np.abs(o.field("gpsiy"))) < 1e-14
    np.testing.assert_allclose(o.field("lpsi")[0, 0], p.alpha * (p.q0 ** 2 - q * q) * psi[0, 0], atol=1e-13)


def test_layered_state_stays_one_dimensional(oracle_mod):
    """psi(z), rho(z) stay x,y independent; the flow is then purely irrotational
    (v_x = v_y = 0 and v_sol = 0 up to rounding)."""
    p, o = make(oracle_mod, shape=(8, 8, 32), rho_0=0.9, divv_switch=2)
    psi, rho = ic.flat_interface(p, noise=0.0)
    o.set_state(psi, rho)
    assert o.step(5) == 0
    for f in ("psi", "rho", "amp", "vz", "divv"):
        a = o.field(f)
        assert np.max(np.abs(a - a[:1, :1, :])) <= 1e-12 * max(1.0, np.max(np.abs(a)))
    vz = np.max(np.abs(o.field("vz")))
    assert vz > 0
    for f in ("vx", "vy", "vsolx", "vsoly", "vsolz"):
        assert np.max(np.abs(o.field(f))) <= 1e-12 * max(vz, 1e-30) + 1e-300


def test_relax_phase_resets_density(oracle_mod):
    """REF:1371-1374: while nLoop <= divvSwitch, rho = rho_0 + kp A before the AB2 update."""
    p, o = make(oracle_mod, shape=(8, 8, 16), rho_0=0.5, divv_switch=10)
    psi, rho = ic.flat_interface(p, rho_i=0.2, rho_s=0.2, noise=1e-3)
    o.set_state(psi, rho)
    o.step(3)
    d = abi.derived(p)
    # rho after the step = rho_0 + kp A + dt * (AB2 source); the source is small
    np.testing.assert_allclose(o.field("rho"), p.rho_0 + d["kp"] * o.field("amp"), atol=5e-3 * p.dt * 1e3)


def test_rank_count_quirk_is_modelled(oracle_mod):
    """REF:1780-1804 vs REF:1932: the v_z filter at k = 0 depends on whether the x slab
    starts a rank's block, so the reference's result depends on its rank count."""
    outs = []
    for ranks in (2, 4):
        p = abi.default_params(8, 8, 16, rho_0=0.5, divv_switch=0, ref_ranks=ranks)
        o = oracle_mod.Oracle(p)
        psi, rho = ic.undulated_interface(p, sigma=1e-2)
        o.set_state(psi, rho)
        o.step(1)
        outs.append(o.field("vz"))
    diff = np.max(np.abs(outs[0] - outs[1]))
    assert 0 < diff < 1e-2 * np.max(np.abs(outs[0]))


def test_diagnostics_definitions(oracle_mod):
    """L1, mass and energy follow REF:2214-2258 on the returned fields."""
    p, o = make(oracle_mod, shape=(8, 8, 16), rho_0=0.8, divv_switch=1)
    psi, rho = ic.flat_interface(p)
    o.set_state(psi, rho)
    o.step(3)
    d = o.diagnostics()
    der = abi.derived(p)
    psin, psio, r = o.field("psi"), o.field("psi_old"), o.field("rho")
    l1 = np.sum(np.abs(psin - psio)) / (p.dt * np.sum(np.abs(psin)))
    assert abs(d["l1"] - l1) <= 1e-12 * l1
    assert abs(d["mass"] - r.sum() * der["dx"] ** 3) <= 1e-12 * abs(d["mass"])
    assert d["step"] == 3 and d["nonfinite"] == 0
