"""The C++ host driver (swc_run: the reference's command line and output files)
against the oracle run with the same cadence and text layout."""
import os
import subprocess

import numpy as np
import pytest

from smaiso_wcomp_gb300 import abi, ic

pytestmark = pytest.mark.gpu
EXE = os.path.join(os.path.dirname(abi.LIB_PATH), "swc_run")


def read(path):
    with open(path) as f:
        return np.array([float(x) for x in f.read().split()])


def test_driver_outputs_match_oracle(lib, oracle_mod, tmp_path):
    nx, ny, nz, l1step, save = 16, 8, 32, 5, 2
    out = os.path.join(tmp_path, "box")
    cmd = [EXE, "--grid", str(nx), str(ny), str(nz), "--max-steps", "20", "--step-l1", str(l1step),
           "--step-save", str(save), "--divv-switch", "3", "--out", out, "1.5", "2", "0", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    p = abi.default_params(nx, ny, nz, nu=1.5, ep=-0.002, divv_switch=3)
    psi0, _ = ic.reference_band(p)
    o = oracle_mod.Oracle(p)
    o.set_state(psi0)          # rho = 0 as REF:1053
    exp = {k: [] for k in ("L1", "mass", "energy", "psiMid", "rho", "vz", "amp", "energyMid")}
    surf = np.zeros((nx, ny))
    der = abi.derived(p)
    for blk in range(4):
        o.step(l1step)
        d = o.diagnostics()
        exp["L1"].append(d["l1"]); exp["mass"].append(d["mass"]); exp["energy"].append(d["energy"])
        if (blk + 1) % save == 0:
            rho = o.field("rho")
            for i in range(nx):
                for j in range(ny):
                    ks = np.nonzero(rho[i, j] > der["rho_s"] - 0.15)[0]
                    if ks.size:
                        surf[i, j] = ks.max()
            exp["psiMid"].append(o.field("psi")[:, ny // 2, :].ravel())
            for f, name in (("rho", "rho"), ("vz", "vz"), ("amp", "amp"), ("energy", "energyMid")):
                exp[name].append(o.field(f)[:, ny // 2, :].ravel())
    for k in ("L1", "mass", "energy"):
        np.testing.assert_allclose(read(os.path.join(out, k + ".dat")), exp[k], rtol=2e-5)
    for k in ("psiMid", "rho", "vz", "amp", "energyMid"):
        got = read(os.path.join(out, k + ".dat"))
        want = np.concatenate(exp[k])
        scale = np.max(np.abs(want))
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-5 * scale)
    np.testing.assert_array_equal(read(os.path.join(out, "surfPsi.dat"))[-nx * ny:], surf.ravel())
    # psi<rank>.dat: one file per reproduced x slab (2 by default), i-major order
    parts = [read(os.path.join(out, f"psi{r}.dat")) for r in range(2)]
    np.testing.assert_allclose(np.concatenate(parts), o.field("psi").ravel(), rtol=1e-5,
                               atol=1e-5 * np.max(np.abs(o.field("psi"))))
    info = open(os.path.join(out, "info")).read()
    assert "Viscosity (nu): 1.5" in info and "epsilon: -0.002" in info
