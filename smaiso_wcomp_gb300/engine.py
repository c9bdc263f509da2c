"""Python host mirror of the C ABI (include/swc.h): the time loop and r2r plans.

Every call goes through libswc.so (the sm_103a CUDA library); a failing status
raises SwcError carrying swc_last_error(). There is no CPU fallback.
"""
import ctypes

import numpy as np

from . import abi


class SwcError(RuntimeError):
    def __init__(self, status, where, msg=""):
        self.status = status
        super().__init__(f"{where}: status {status} ({msg})")


def _check(lib, rc, where):
    if rc != abi.SWC_OK:
        raise SwcError(rc, where, lib.swc_last_error().decode(errors="replace"))


class Engine:
    """One simulation context: swc_create / swc_set_state / swc_step / ... / swc_destroy."""

    def __init__(self, params, lib=None):
        self.lib = lib or abi.load_library()
        self.p = params
        self.shape = (params.nx, params.ny, params.nz)
        self._h = ctypes.c_void_p()
        _check(self.lib, self.lib.swc_create(ctypes.byref(params), ctypes.byref(self._h)), "swc_create")

    def close(self):
        if self._h:
            self.lib.swc_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, psi, rho=None):
        psi = np.ascontiguousarray(psi, dtype=np.float64).reshape(self.shape)
        rp = None
        if rho is not None:
            rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(self.shape)
            rp = abi.as_dptr(rho)
        _check(self.lib, self.lib.swc_set_state(self._h, abi.as_dptr(psi), rp), "swc_set_state")

    def set_state_ic(self, kind, **fields):
        """swc_set_state_ic: the initial state generated on the device (swc_default_ic of
        `kind`, with the given swc_ic fields overridden)."""
        ic = default_ic(self.p, kind, lib=self.lib, **fields)
        _check(self.lib, self.lib.swc_set_state_ic(self._h, ctypes.byref(ic)), "swc_set_state_ic")
        return ic

    def step(self, n=1, check=True):
        rc = self.lib.swc_step(self._h, int(n))
        if check:
            _check(self.lib, rc, "swc_step")
        return rc

    def step_async(self, n=1):
        """swc_step_async: enqueue n steps and return; sync() collects their status."""
        _check(self.lib, self.lib.swc_step_async(self._h, int(n)), "swc_step_async")

    def prepare(self):
        """swc_prepare: capture every step variant's CUDA graph now."""
        _check(self.lib, self.lib.swc_prepare(self._h), "swc_prepare")

    def sync(self):
        _check(self.lib, self.lib.swc_sync(self._h), "swc_sync")

    def diagnostics(self):
        d = abi.SwcDiag()
        _check(self.lib, self.lib.swc_diagnostics(self._h, ctypes.byref(d)), "swc_diagnostics")
        return d.as_dict()

    def field(self, name, out=None):
        if out is None:
            out = np.empty(self.shape, dtype=np.float64)
        _check(self.lib, self.lib.swc_get_field(self._h, abi.FIELD_ID[name], abi.as_dptr(out)),
               f"swc_get_field({name})")
        return out

    def field_async(self, name, out):
        """swc_get_field_async: queue the read of `name` into `out` (pinned for overlap);
        `out` is complete after field_wait() or after the next-but-one field_async."""
        _check(self.lib, self.lib.swc_get_field_async(self._h, abi.FIELD_ID[name], abi.as_dptr(out)),
               f"swc_get_field_async({name})")
        return out

    def field_wait(self):
        _check(self.lib, self.lib.swc_get_field_wait(self._h), "swc_get_field_wait")

    def device_ptr(self, name):
        ptr = ctypes.c_void_p()
        eb = ctypes.c_int()
        _check(self.lib, self.lib.swc_field_device_ptr(self._h, abi.FIELD_ID[name], ctypes.byref(ptr),
                                                       ctypes.byref(eb)), "swc_field_device_ptr")
        return ptr.value, eb.value

    @property
    def nloop(self):
        n = ctypes.c_int64()
        _check(self.lib, self.lib.swc_get_step(self._h, ctypes.byref(n)), "swc_get_step")
        return n.value

    def last_step_ms(self):
        ms = ctypes.c_double()
        _check(self.lib, self.lib.swc_last_step_ms(self._h, ctypes.byref(ms)), "swc_last_step_ms")
        return ms.value

    def last_step_launches(self):
        n = ctypes.c_int64()
        _check(self.lib, self.lib.swc_last_step_launches(self._h, ctypes.byref(n)), "swc_last_step_launches")
        return n.value

    def backward(self, dpsi=None, drho=None, want_psi0=True, want_rho0=False, energy_lambda=0.0):
        """swc_backward: gradients of a loss with dL/dpsi(T) = dpsi, dL/drho(T) = drho;
        energy_lambda != 0: swc_backward_energy, the loss plus energy_lambda times the
        free-energy diagnostic of the last step."""
        n = self.shape
        dp = None if dpsi is None else np.ascontiguousarray(dpsi, dtype=np.float64).reshape(n)
        dr = None if drho is None else np.ascontiguousarray(drho, dtype=np.float64).reshape(n)
        o_psi = np.empty(n) if want_psi0 else None
        o_rho = np.empty(n) if want_rho0 else None
        g = abi.SwcGrad()
        ptr = lambda a: None if a is None else abi.as_dptr(a)  # noqa: E731
        if energy_lambda:
            _check(self.lib, self.lib.swc_backward_energy(self._h, float(energy_lambda), ptr(dp), ptr(dr), ptr(o_psi),
                                                          ptr(o_rho), ctypes.byref(g)), "swc_backward_energy")
        else:
            _check(self.lib, self.lib.swc_backward(self._h, ptr(dp), ptr(dr), ptr(o_psi), ptr(o_rho),
                                                   ctypes.byref(g)), "swc_backward")
        out = g.as_dict()
        out["psi0"], out["rho0"] = o_psi, o_rho
        return out

    def save(self, path):
        _check(self.lib, self.lib.swc_save(self._h, str(path).encode()), "swc_save")

    def load(self, path):
        _check(self.lib, self.lib.swc_load(self._h, str(path).encode()), "swc_load")


def default_ic(params, kind, lib=None, **fields):
    """swc_default_ic of `kind` for the grid of `params`, with fields overridden."""
    lib = lib or abi.load_library()
    ic = abi.SwcIc()
    _check(lib, lib.swc_default_ic(ctypes.byref(params), int(kind), ctypes.byref(ic)), "swc_default_ic")
    for k, v in fields.items():
        if not hasattr(ic, k):
            raise AttributeError(f"swc_ic has no field {k}")
        setattr(ic, k, v)
    return ic


def device_fma_peak(precision, lib=None):
    """Measured dense FMA TFLOP/s of the current device (FMA = 2 flops)."""
    lib = lib or abi.load_library()
    t = ctypes.c_double()
    _check(lib, lib.swc_device_fma_peak(int(precision), ctypes.byref(t)), "swc_device_fma_peak")
    return t.value


class R2RPlan:
    """3D r2r transform with FFTW semantics (kinds SWC_REDFT10/01, SWC_RODFT10/01 per axis)."""

    def __init__(self, shape, kinds, precision=abi.SWC_PREC_FP64, lib=None):
        self.lib = lib or abi.load_library()
        self.shape = tuple(shape)
        self._h = ctypes.c_void_p()
        _check(self.lib, self.lib.swc_r2r_plan_create(*self.shape, *kinds, precision, ctypes.byref(self._h)),
               "swc_r2r_plan_create")

    def __call__(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape)
        out = np.empty_like(x)
        _check(self.lib, self.lib.swc_r2r_execute_host(self._h, abi.as_dptr(x), abi.as_dptr(out)),
               "swc_r2r_execute_host")
        return out

    def execute_device(self, dev_ptr, stream=None):
        _check(self.lib, self.lib.swc_r2r_execute(self._h, ctypes.c_void_p(dev_ptr), ctypes.c_void_p(stream)),
               "swc_r2r_execute")

    def set_wait_test(self, extra_tx_bytes, max_polls):
        _check(self.lib, self.lib.swc_r2r_plan_set_wait_test(self._h, int(extra_tx_bytes), int(max_polls)),
               "swc_r2r_plan_set_wait_test")

    def execute_axis(self, axis, dev_ptr, stream=None):
        _check(self.lib, self.lib.swc_r2r_execute_axis(self._h, int(axis), ctypes.c_void_p(dev_ptr),
                                                       ctypes.c_void_p(stream)), "swc_r2r_execute_axis")

    def close(self):
        if self._h:
            self.lib.swc_r2r_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
