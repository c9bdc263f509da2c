"""CPU-only checks: host logic, the IC generators, and that libswc.so loads and
exports every entry point include/swc.h declares (no compute calls here)."""
import os
import re

import numpy as np
import pytest

from smaiso_wcomp_gb300 import abi, ic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "swc.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+char\*|int|void)\s+(swc_\w+)\s*\(", text, re.M)))


def test_header_matches_export_list():
    assert header_functions() == sorted(abi.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name


def test_default_params_match_c(lib):
    import ctypes
    c = abi.SwcParams()
    assert lib.swc_default_params(ctypes.byref(c), 64, 32, 16) == 0
    py = abi.default_params(64, 32, 16)
    for name, _ in abi.SwcParams._fields_:
        assert getattr(c, name) == getattr(py, name), name


def test_derived_match_c(lib):
    import ctypes
    p = abi.default_params(32, rho_0=0.8, ep=-0.002, beta=1.5)
    d = abi.SwcDerived()
    assert lib.swc_derive(ctypes.byref(p), ctypes.byref(d)) == 0
    py = abi.derived(p)
    for k, v in py.items():
        assert getattr(d, k) == pytest.approx(v, rel=1e-15), k
    # reference values (REF:250-254): Amp = sqrt((6 + sqrt(36 - 0.08))/5)
    assert abi.derived(abi.default_params(8))["amp"] == pytest.approx(np.sqrt((6 + np.sqrt(36 - 0.04)) / 5))


def test_bad_params_rejected_before_device(lib):
    import ctypes
    h = ctypes.c_void_p()
    for bad in (dict(nz=12), dict(ref_ranks=3), dict(dt=0.0), dict(nu=-1.0), dict(precision=7),
                dict(diag_interval=-1), dict(adjoint_ckpt=-2)):
        p = abi.default_params(16)
        for k, v in bad.items():
            setattr(p, k, v)
        assert lib.swc_create(ctypes.byref(p), ctypes.byref(h)) == abi.SWC_ERR_BAD_PARAM
        assert len(lib.swc_last_error()) > 0


def test_strerror_covers_codes(lib):
    for code in range(0, -9, -1):
        assert lib.swc_strerror(code) not in (b"", b"unknown status")


def _splitmix_py(x):
    m = (1 << 64) - 1
    z = (x + 0x9E3779B97F4A7C15) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    return z ^ (z >> 31)


def test_splitmix64_matches_scalar_definition():
    xs = np.array([0, 1, 2, 12345, 2 ** 63 + 7, 2 ** 64 - 1], dtype=np.uint64)
    got = ic.splitmix64(xs)
    for x, g in zip(xs, got):
        assert int(g) == _splitmix_py(int(x))


def test_noise_is_counter_based_and_bounded():
    a = ic.uniform_noise((4, 5, 6), 1001, 1e-4)
    b = ic.uniform_noise((4, 5, 6), 1001, 1e-4)
    assert np.array_equal(a, b) and np.max(np.abs(a)) <= 1e-4
    # any sub-block is reproducible from its global indices alone
    flat = ic.uniform_noise((120,), 1001, 1e-4)
    assert np.array_equal(flat, a.ravel())
    g = ic.gaussian_noise((64, 64, 64), 1002, 1.0)
    assert abs(g.mean()) < 5e-3 and abs(g.std() - 1.0) < 5e-3


@pytest.mark.parametrize("gen", [ic.flat_interface, ic.undulated_interface, ic.dislocations, ic.reference_band])
def test_ic_shapes(gen):
    p = abi.default_params(16, 8, 32, rho_0=0.8)
    psi, rho = gen(p)
    assert psi.shape == rho.shape == (16, 8, 32)
    assert np.all(np.isfinite(psi)) and np.all(np.isfinite(rho))
