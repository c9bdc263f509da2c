"""Runs the reference's own time loop (oracle/_ref/smaiso_wcomp_ref, built by
oracle/build_ref.sh from smaiso-wcomp.cpp and the MPI/FFTW-MPI stand-in in
oracle/refshim/) and reads back its fields and diagnostics.

TEST INFRASTRUCTURE ONLY: used by tests/golden/make_ref_fixtures.py to write the
fixtures that pin the oracle, and by the CPU tests that rebuild a small case when
the reference source is present. Never imported by the product.
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
REF_BIN = os.path.join(REF_DIR, "smaiso_wcomp_ref")
DEFAULT_SRC = "/root/reference/smaiso-wcomp.cpp"

FIELDS = [
    "psi", "rho", "amp", "divv", "vx", "vy", "vz", "vsolx", "vsoly", "vsolz", "energy",
    "psiq", "psiq_old", "nlq", "frho", "lpsi", "mu", "gpsix", "gpsiy", "gpsiz",
    "grhox", "grhoy", "grhoz", "psi_old",
]


def source_path():
    return os.environ.get("SWC_REFERENCE_SRC", DEFAULT_SRC)


def available():
    """True when the reference source can be read (it is not shipped with the repo)."""
    return os.path.isfile(source_path())


def build(force=False):
    """Compile oracle/_ref/smaiso_wcomp_ref from the reference source (build_ref.sh)."""
    deps = [os.path.join(HERE, f) for f in
            ("build_ref.sh", "swc_oracle.c", "refshim/refshim.cpp", "refshim/fftw3-mpi.h")]
    if (force or not os.path.exists(REF_BIN)
            or os.path.getmtime(REF_BIN) < max(os.path.getmtime(d) for d in deps)):
        subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), source_path(), REF_DIR],
                       check=True, stdout=subprocess.DEVNULL)
    return REF_BIN


def run(shape, ranks, steps, dump_steps, psi0=None, threads=None, timeout=1800):
    """Run the reference for `steps` steps on an nx x ny x nz grid as `ranks` MPI ranks
    (argv: nu = 1, ep_arg = 1, aE = 0, load = 0; dt, coefficients and the relax phase
    are the reference's own). psi0 (optional) replaces the reference's initial psi.

    Returns {"fields": {step: {name: array}}, "diag": [(step, l1, sumA, sumB, mass,
    energy), ...]}.
    """
    build()
    nx, ny, nz = shape
    work = tempfile.mkdtemp(prefix="swc_ref_", dir=REF_DIR)
    try:
        env = dict(os.environ)
        env.update(SWC_REF_NX=str(nx), SWC_REF_NY=str(ny), SWC_REF_NZ=str(nz),
                   SWC_REF_RANKS=str(ranks), SWC_REF_STEPS=str(steps), SWC_REF_DIR=work,
                   SWC_REF_DUMP=",".join(str(s) for s in dump_steps))
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        if psi0 is not None:
            path = os.path.join(work, "psi0.bin")
            np.ascontiguousarray(psi0, dtype=np.float64).reshape(shape).tofile(path)
            env["SWC_REF_PSI0"] = path
        res = subprocess.run([REF_BIN, "1", "1", "0", "0"], env=env, cwd=work,
                             stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                             timeout=timeout)
        if res.returncode != 0:
            raise RuntimeError(f"reference run failed ({res.returncode}): {res.stderr[-2000:]}")
        out = {"fields": {}, "diag": []}
        for s in dump_steps:
            out["fields"][s] = {
                f: np.fromfile(os.path.join(work, "dump", f"s{s}_{f}.bin"),
                               dtype=np.float64).reshape(shape)
                for f in FIELDS}
        diag_path = os.path.join(work, "dump", "diag.txt")
        if os.path.exists(diag_path):
            with open(diag_path) as fh:
                for line in fh:
                    v = line.split()
                    out["diag"].append((int(v[0]),) + tuple(float(x) for x in v[1:]))
        return out
    finally:
        shutil.rmtree(work, ignore_errors=True)
