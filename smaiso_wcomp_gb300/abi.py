"""ctypes mirror of include/swc.h and the loader of the CUDA library libswc.so.

The library is the product: there is no CPU fallback. `load_library()` raises if
the in-tree build (smaiso_wcomp_gb300/_build/libswc.so) is missing.
"""
import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libswc.so")

# status codes
SWC_OK = 0
SWC_ERR_BAD_PARAM = -1
SWC_ERR_OOM = -2
SWC_ERR_CUDA = -3
SWC_ERR_NONFINITE = -4
SWC_ERR_TIMEOUT = -5
SWC_ERR_STATE = -6
SWC_ERR_IO = -7
SWC_ERR_NO_DEVICE = -8

SWC_PREC_FP64 = 0
SWC_PREC_MIXED = 1

SWC_REDFT10, SWC_REDFT01, SWC_RODFT10, SWC_RODFT01 = 0, 1, 2, 3

# device initial conditions (swc_ic.kind)
SWC_IC_BAND, SWC_IC_FLAT, SWC_IC_UNDULATED, SWC_IC_DISLOCATIONS, SWC_IC_FOCAL_CONIC, SWC_IC_FOCAL_CONICS = range(6)

FIELDS = [
    "psi", "rho", "amp", "divv", "vx", "vy", "vz", "vsolx", "vsoly", "vsolz", "energy",
    "psiq", "psiq_old", "nlq", "frho", "lpsi", "mu", "gpsix", "gpsiy", "gpsiz",
    "grhox", "grhoy", "grhoz", "psi_old",
]
FIELD_ID = {name: i for i, name in enumerate(FIELDS)}

# Every symbol include/swc.h declares (checked by the CPU test suite).
EXPORTS = [
    "swc_abi_version", "swc_strerror", "swc_last_error", "swc_default_params", "swc_derive",
    "swc_create", "swc_destroy", "swc_set_state", "swc_set_state_ic", "swc_default_ic", "swc_ic_generate",
    "swc_step", "swc_step_async", "swc_sync",
    "swc_prepare", "swc_diagnostics",
    "swc_get_field", "swc_get_field_async", "swc_get_field_wait", "swc_field_device_ptr", "swc_get_step",
    "swc_last_step_ms",
    "swc_last_step_launches", "swc_device_fma_peak", "swc_diagnostics_noalloc",
    "swc_backward", "swc_backward_energy", "swc_save", "swc_load", "swc_r2r_plan_create", "swc_r2r_plan_destroy",
    "swc_r2r_execute", "swc_r2r_execute_axis", "swc_r2r_execute_host", "swc_r2r_plan_set_wait_test",
]


class SwcParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("nw", ctypes.c_int),
        ("dt", ctypes.c_double), ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
        ("gamma", ctypes.c_double), ("ep", ctypes.c_double), ("q0", ctypes.c_double),
        ("nu", ctypes.c_double), ("lambda_", ctypes.c_double), ("zeta", ctypes.c_double),
        ("rho_0", ctypes.c_double), ("divv_switch", ctypes.c_int), ("load", ctypes.c_int),
        ("ref_ranks", ctypes.c_int), ("precision", ctypes.c_int), ("device", ctypes.c_int),
        ("watchdog_s", ctypes.c_double), ("adjoint_ckpt", ctypes.c_int), ("adjoint_cap_gb", ctypes.c_double),
        ("adjoint_snapshots", ctypes.c_int), ("diag_interval", ctypes.c_int),
    ]


class SwcIc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int), ("ncores", ctypes.c_int), ("seed", ctypes.c_uint64),
        ("amp", ctypes.c_double), ("xi", ctypes.c_double), ("noise", ctypes.c_double),
        ("rho_s", ctypes.c_double), ("rho_i", ctypes.c_double), ("phi", ctypes.c_double),
        ("qi", ctypes.c_double), ("ae", ctypes.c_double), ("gap", ctypes.c_double),
    ]


class SwcDiag(ctypes.Structure):
    _fields_ = [
        ("l1", ctypes.c_double), ("mass", ctypes.c_double), ("energy", ctypes.c_double),
        ("sum_abs_dpsi", ctypes.c_double), ("sum_abs_psi", ctypes.c_double),
        ("sum_rho", ctypes.c_double), ("sum_energy", ctypes.c_double),
        ("step", ctypes.c_int64), ("nonfinite", ctypes.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class SwcGrad(ctypes.Structure):
    _fields_ = [("alpha", ctypes.c_double), ("beta", ctypes.c_double), ("gamma", ctypes.c_double),
                ("nu", ctypes.c_double), ("rho_0", ctypes.c_double), ("steps", ctypes.c_int64),
                ("forward_steps", ctypes.c_int64), ("snapshots", ctypes.c_int64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class SwcDerived(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("amp", "kp", "rho_s", "rho_m", "dx", "dy", "dz", "lx", "ly", "lz", "scale")]


def default_params(nx, ny=None, nz=None, **overrides):
    """Reference defaults (smaiso-wcomp.cpp:206-278) with nu = 1, ep = -0.001.

    Pure-Python restatement of swc_default_params so host logic can run without
    the CUDA library; tests check that both agree.
    """
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    p = SwcParams(nx=nx, ny=ny, nz=nz, nw=8, dt=0.001, alpha=1.0, beta=2.0, gamma=1.0,
                  ep=-0.001, q0=1.0, nu=1.0, lambda_=1.0, zeta=1.0, rho_0=0.01,
                  divv_switch=50, load=0, ref_ranks=2, precision=SWC_PREC_FP64, device=0,
                  watchdog_s=0.0, adjoint_ckpt=0, adjoint_cap_gb=0.0, adjoint_snapshots=0,
                  diag_interval=0)
    for k, v in overrides.items():
        setattr(p, "lambda_" if k == "lambda" else k, v)
    return p


def derived(p):
    """Derived constants exactly as smaiso-wcomp.cpp:250-272 computes them."""
    amp = np.sqrt((3 * p.beta + np.sqrt(9 * p.beta * p.beta + 40 * p.ep * p.gamma)) / 5)
    kp = (1 - p.rho_0) / amp
    rho_s = kp * amp + p.rho_0
    lx = p.nx * 2.0 * np.pi / (p.q0 * p.nw)
    ly = p.ny * 2.0 * np.pi / (p.q0 * p.nw)
    lz = p.nz * 2.0 * np.pi / (p.q0 * p.nw)
    return dict(amp=amp, kp=kp, rho_s=rho_s, rho_m=rho_s / 2, dx=lx / p.nx, dy=ly / p.ny,
                dz=lz / p.nz, lx=lx, ly=ly, lz=lz, scale=0.125 / (p.nx * p.ny * p.nz))


_lib = None


def load_library(path=None):
    """Load libswc.so (the CUDA product). Raises OSError if it is not built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError(f"libswc.so not built at {path}; run __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    dp = P(ctypes.c_double)
    sig = {
        "swc_abi_version": (ctypes.c_int, []),
        "swc_strerror": (ctypes.c_char_p, [ctypes.c_int]),
        "swc_last_error": (ctypes.c_char_p, []),
        "swc_default_params": (ctypes.c_int, [P(SwcParams), ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "swc_derive": (ctypes.c_int, [P(SwcParams), P(SwcDerived)]),
        "swc_create": (ctypes.c_int, [P(SwcParams), P(vp)]),
        "swc_destroy": (ctypes.c_int, [vp]),
        "swc_set_state": (ctypes.c_int, [vp, dp, dp]),
        "swc_set_state_ic": (ctypes.c_int, [vp, P(SwcIc)]),
        "swc_default_ic": (ctypes.c_int, [P(SwcParams), ctypes.c_int, P(SwcIc)]),
        "swc_ic_generate": (ctypes.c_int, [P(SwcParams), P(SwcIc), vp, vp, vp]),
        "swc_step": (ctypes.c_int, [vp, ctypes.c_int]),
        "swc_diagnostics": (ctypes.c_int, [vp, P(SwcDiag)]),
        "swc_get_field": (ctypes.c_int, [vp, ctypes.c_int, dp]),
        "swc_step_async": (ctypes.c_int, [vp, ctypes.c_int]),
        "swc_sync": (ctypes.c_int, [vp]),
        "swc_prepare": (ctypes.c_int, [vp]),
        "swc_get_field_async": (ctypes.c_int, [vp, ctypes.c_int, dp]),
        "swc_get_field_wait": (ctypes.c_int, [vp]),
        "swc_field_device_ptr": (ctypes.c_int, [vp, ctypes.c_int, P(vp), P(ctypes.c_int)]),
        "swc_get_step": (ctypes.c_int, [vp, P(ctypes.c_int64)]),
        "swc_last_step_ms": (ctypes.c_int, [vp, dp]),
        "swc_last_step_launches": (ctypes.c_int, [vp, P(ctypes.c_int64)]),
        "swc_device_fma_peak": (ctypes.c_int, [ctypes.c_int, dp]),
        "swc_diagnostics_noalloc": (ctypes.c_int, [P(SwcParams), vp, vp, vp, vp, vp, vp, P(SwcDiag)]),
        "swc_backward": (ctypes.c_int, [vp, dp, dp, dp, dp, P(SwcGrad)]),
        "swc_backward_energy": (ctypes.c_int, [vp, ctypes.c_double, dp, dp, dp, dp, P(SwcGrad)]),
        "swc_save": (ctypes.c_int, [vp, ctypes.c_char_p]),
        "swc_load": (ctypes.c_int, [vp, ctypes.c_char_p]),
        "swc_r2r_plan_create": (ctypes.c_int, [ctypes.c_int] * 7 + [P(vp)]),
        "swc_r2r_plan_destroy": (ctypes.c_int, [vp]),
        "swc_r2r_execute": (ctypes.c_int, [vp, vp, vp]),
        "swc_r2r_execute_axis": (ctypes.c_int, [vp, ctypes.c_int, vp, vp]),
        "swc_r2r_execute_host": (ctypes.c_int, [vp, dp, dp]),
        "swc_r2r_plan_set_wait_test": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib if path == LIB_PATH else _lib
    return lib


def as_dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
