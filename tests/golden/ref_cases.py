"""Cases of tests/golden/ref_fixtures.npz: runs of the reference's own time loop
(smaiso-wcomp.cpp through oracle/_ref, see oracle/build_ref.sh) that pin the oracle
and the FP64 engine.

Each case is a grid, an MPI rank count of the reference run, a step count (dt, the
coefficients and the 50-step relax phase are the reference's own: nu = 1,
ep = -0.001, rho_0 = 0.01, dt = 0.001) and an initial psi; rho starts at 0 as in
the reference (smaiso-wcomp.cpp:1053). The initial psi is rebuilt bit for bit on
any machine from the 1D profiles stored in the fixture and counter-based noise,
with IEEE additions and products only:
    psi0[i,j,k] = (P[k] + (X[i] * Y[j]) * Z[k]) + noise[i,j,k]
    noise = SplitMix64 uniform on [-a, a] (smaiso_wcomp_gb300.ic.uniform_noise)
"sep" cases carry a 3D perturbation at the interface (X, Y, Z); "flat" is the 64^3
flat-interface state (P only; a = 1e-4, seed 1001); "ref" is the reference's own
initial state (the band of smaiso-wcomp.cpp:575-590, no file read), rebuilt here by
smaiso_wcomp_gb300.ic.reference_band.

At each dump step the fixture holds, per field, its values at `sample` seeded
point indices (every point when sample is None) and the whole field's L2 norm.
"""
import numpy as np

CASES = {
    # name: shape, ranks, steps, {dump step: sample size or None}, ic, seed, noise
    "s16_p2": dict(shape=(16, 16, 16), ranks=2, steps=100, dumps={1: 1024, 100: None},
                   ic="sep", seed=2001, noise=1e-3),
    "s16_p4": dict(shape=(16, 16, 16), ranks=4, steps=100, dumps={100: 1024},
                   ic="sep", seed=2001, noise=1e-3),
    "s32x16x8_p4": dict(shape=(32, 16, 8), ranks=4, steps=100, dumps={100: 1024},
                        ic="sep", seed=2002, noise=1e-3),
    "s8x32x16_p2": dict(shape=(8, 32, 16), ranks=2, steps=100, dumps={100: 1024},
                        ic="sep", seed=2003, noise=1e-3),
    "s32_p2": dict(shape=(32, 32, 32), ranks=2, steps=100, dumps={100: 1024},
                   ic="sep", seed=2004, noise=1e-3),
    "s64_p4": dict(shape=(64, 64, 64), ranks=4, steps=100, dumps={100: 1024},
                   ic="sep", seed=2005, noise=1e-3),
    # BASELINE's 64^3 flat-interface configuration (A = 0.8, xi = 2, uniform noise
    # 1e-4, seed 1001) at the reference's dt = 0.001, 500 steps.
    "flat64_p2": dict(shape=(64, 64, 64), ranks=2, steps=500, dumps={100: 1024, 500: 1024},
                      ic="flat", seed=1001, noise=1e-4),
    # the reference's own band initial state, 16 x 16 x 64
    "band_p2": dict(shape=(16, 16, 64), ranks=2, steps=100, dumps={1: 1024, 100: 1024},
                    ic="ref", seed=2006, noise=0.0),
}

FIELDS = [
    "psi", "rho", "amp", "divv", "vx", "vy", "vz", "vsolx", "vsoly", "vsolz", "energy",
    "psiq", "psiq_old", "nlq", "frho", "lpsi", "mu", "gpsix", "gpsiy", "gpsiz",
    "grhox", "grhoy", "grhoz", "psi_old",
]

# Vector components are compared against the norm of the whole vector: in nearly
# layered states the x/y components and v_sol are small cancellations.
VECTORS = {"gpsi": ["gpsix", "gpsiy", "gpsiz"], "grho": ["grhox", "grhoy", "grhoz"],
           "v": ["vx", "vy", "vz", "vsolx", "vsoly", "vsolz"]}


def fields_at(step):
    """Fields meaningful at a dump step: the energy density is formed on the
    reference's diagnostic steps only (every 50th, smaiso-wcomp.cpp:2202)."""
    return [f for f in FIELDS if f != "energy" or step % 50 == 0]


def profiles(case, dx, dz):
    """1D profiles of the initial psi (computed once, stored in the fixture)."""
    c = CASES[case]
    nx, ny, nz = c["shape"]
    A, xi, q0 = 0.8, 2.0, 1.0
    z = np.arange(nz) * dz
    lz = nz * dz
    h = 0.5 * (1.0 + np.tanh((z - lz / 2) / xi))
    P = h * A * np.cos(q0 * z)
    if c["ic"] == "flat":
        return dict(P=P, X=np.zeros(nx), Y=np.zeros(ny), Z=np.zeros(nz))
    x = np.arange(nx) * dx
    y = np.arange(ny) * dx
    X = np.sin(2 * np.pi * x / (nx * dx))
    Y = np.cos(2 * np.pi * y / (ny * dx))
    Z = 0.3 * A * (1.0 / np.cosh((z - lz / 2) / xi)) ** 2 * np.sin(q0 * z)
    return dict(P=P, X=X, Y=Y, Z=Z)


def initial_psi(prof, shape, seed, noise):
    from smaiso_wcomp_gb300.ic import uniform_noise
    P, X, Y, Z = prof["P"], prof["X"], prof["Y"], prof["Z"]
    smooth = P[None, None, :] + (X[:, None, None] * Y[None, :, None]) * Z[None, None, :]
    return np.ascontiguousarray(smooth + uniform_noise(shape, seed, noise))


def sample_index(case, step, size):
    n = int(np.prod(CASES[case]["shape"]))
    if size is None:
        return np.arange(n, dtype=np.int64)
    rng = np.random.default_rng(CASES[case]["seed"] * 1000 + step)
    return np.sort(rng.choice(n, size, replace=False)).astype(np.int64)


class Fixture:
    """Reader of tests/golden/ref_fixtures.npz for one case."""

    def __init__(self, npz, case):
        self.case = case
        self.spec = CASES[case]
        self.shape = self.spec["shape"]
        self._z = npz
        if self.spec["ic"] == "ref":
            from smaiso_wcomp_gb300.abi import default_params
            from smaiso_wcomp_gb300.ic import reference_band
            self.psi0 = reference_band(default_params(*self.shape))[0]
        else:
            prof = {k: npz[f"{case}.{k}"] for k in "PXYZ"}
            self.psi0 = initial_psi(prof, self.shape, self.spec["seed"], self.spec["noise"])
        self.diag = npz[f"{case}.diag"]   # rows: step, L1, sumA, sumB, mass, energy

    def index(self, step):
        return sample_index(self.case, step, self.spec["dumps"][step])

    def values(self, step, field):
        return self._z[f"{self.case}.s{step}.{field}"]

    def norm(self, step, field):
        return float(self._z[f"{self.case}.s{step}.{field}.norm"])

    def errors(self, step, get_field):
        """Relative L2 error per field at the sampled points of `step` for fields
        given by get_field(name) -> full nx*ny*nz array (vector components against
        the whole vector's sampled norm)."""
        idx = self.index(step)
        names = fields_at(step)
        got = {f: np.asarray(get_field(f)).reshape(-1)[idx] for f in names}
        ref = {f: self.values(step, f) for f in names}
        errs = {}
        for f in names:
            nb = np.linalg.norm(ref[f])
            errs[f] = np.linalg.norm(got[f] - ref[f]) / nb if nb > 0 else np.linalg.norm(got[f])
        for comps in VECTORS.values():
            scale = np.sqrt(sum(np.linalg.norm(ref[c]) ** 2 for c in comps[:3]))
            for c in comps:
                errs[c] = np.linalg.norm(got[c] - ref[c]) / max(scale, 1e-300)
        return errs
