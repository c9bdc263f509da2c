"""ctypes wrapper of the FP64 CPU oracle (oracle/swc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker. The product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libswc_oracle.so")

import sys  # noqa: E402

sys.path.insert(0, os.path.dirname(HERE))
from smaiso_wcomp_gb300.abi import (  # noqa: E402
    FIELD_ID, SwcDiag, SwcParams, as_dptr, SWC_OK)

_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(
            os.path.join(HERE, "swc_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        vp = ctypes.c_void_p
        dp = P(ctypes.c_double)
        L.swco_create.argtypes = [P(SwcParams), P(vp)]
        L.swco_destroy.argtypes = [vp]
        L.swco_destroy.restype = None
        L.swco_set_state.argtypes = [vp, dp, dp]
        L.swco_step.argtypes = [vp, ctypes.c_int]
        L.swco_diagnostics.argtypes = [vp, P(SwcDiag)]
        L.swco_get_field.argtypes = [vp, ctypes.c_int, dp]
        L.swco_get_step.argtypes = [vp]
        L.swco_get_step.restype = ctypes.c_long
        L.swco_r2r1d.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int]
        L.swco_r2r3d.argtypes = [ctypes.c_int] * 6 + [dp, dp, ctypes.c_int]
        L.swco_set_threads.argtypes = [ctypes.c_int]
        L.swco_reference_ic.argtypes = [P(SwcParams), ctypes.c_int] + [ctypes.c_double] * 5 + [dp]
        _lib = L
    return _lib


def set_threads(n):
    return lib().swco_set_threads(int(n))


def reference_ic(p, kind, amp=0.0, phi=0.0, qi=0.0625, ae=0.0, gap=0.0):
    """psi of the reference's band (REF:575-590) and focal-conic (REF:594-707) states."""
    out = np.empty((p.nx, p.ny, p.nz))
    rc = lib().swco_reference_ic(ctypes.byref(p), int(kind), amp, phi, qi, ae, gap, as_dptr(out))
    assert rc == SWC_OK, rc
    return out


def r2r1d(x, kind, direct=False):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    rc = lib().swco_r2r1d(x.size, kind, as_dptr(x), as_dptr(out), int(direct))
    assert rc == SWC_OK, rc
    return out


def r2r3d(a, kinds, direct=False):
    a = np.ascontiguousarray(a, dtype=np.float64)
    out = np.empty_like(a)
    nx, ny, nz = a.shape
    rc = lib().swco_r2r3d(nx, ny, nz, kinds[0], kinds[1], kinds[2], as_dptr(a), as_dptr(out),
                          int(direct))
    assert rc == SWC_OK, rc
    return out


class Oracle:
    """Same call sequence as the C ABI: create / set_state / step / diagnostics / get_field."""

    def __init__(self, params):
        self.p = params
        self.shape = (params.nx, params.ny, params.nz)
        self._h = ctypes.c_void_p()
        rc = lib().swco_create(ctypes.byref(params), ctypes.byref(self._h))
        if rc != SWC_OK:
            raise ValueError(f"swco_create failed: {rc}")

    def close(self):
        if self._h:
            lib().swco_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, psi, rho=None):
        psi = np.ascontiguousarray(psi, dtype=np.float64).reshape(self.shape)
        r = None if rho is None else as_dptr(np.ascontiguousarray(rho, dtype=np.float64))
        self._keep = (psi, rho)
        rc = lib().swco_set_state(self._h, as_dptr(psi), r)
        assert rc == SWC_OK, rc

    def step(self, n):
        return lib().swco_step(self._h, int(n))

    def diagnostics(self):
        d = SwcDiag()
        assert lib().swco_diagnostics(self._h, ctypes.byref(d)) == SWC_OK
        return d.as_dict()

    def field(self, name):
        out = np.empty(self.shape, dtype=np.float64)
        rc = lib().swco_get_field(self._h, FIELD_ID[name], as_dptr(out))
        assert rc == SWC_OK, rc
        return out

    @property
    def nloop(self):
        return lib().swco_get_step(self._h)
