"""Generate tests/golden/r2r_golden.npz: known-answer vectors for the four r2r kinds.

FFTW (the reference's transform library, not vendored) defines REDFT10, REDFT01,
RODFT10 and RODFT01 by closed formulas; scipy.fft.dct/dst with type 2/3 and
norm=None implement the same formulas independently. Inputs are seeded
(numpy PCG64, seed 20240517). Run: python tests/golden/make_golden.py
"""
import os

import numpy as np
import scipy.fft as sf

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    rng = np.random.default_rng(20240517)
    out = {}
    for n in (4, 8, 12, 16, 32, 64, 128, 256, 512):
        x = rng.standard_normal(n)
        out[f"x_{n}"] = x
        out[f"redft10_{n}"] = sf.dct(x, type=2)
        out[f"redft01_{n}"] = sf.dct(x, type=3)
        out[f"rodft10_{n}"] = sf.dst(x, type=2)
        out[f"rodft01_{n}"] = sf.dst(x, type=3)
    # one 3D mixed-kind case per plan of the reference (REF:499-545)
    a = rng.standard_normal((4, 8, 16))
    out["a3"] = a
    plans = {"CT": (2, 2, 2), "iCT": (3, 3, 3), "STx": ("s2", 2, 2), "iSTx": ("s3", 3, 3),
             "STy": (2, "s2", 2), "iSTy": (3, "s3", 3), "STz": (2, 2, "s2"), "iSTz": (3, 3, "s3")}
    for name, kinds in plans.items():
        r = a.copy()
        for ax, k in enumerate(kinds):
            if isinstance(k, str):
                r = sf.dst(r, type=int(k[1]), axis=ax)
            else:
                r = sf.dct(r, type=k, axis=ax)
        out[f"plan_{name}"] = r
    np.savez_compressed(os.path.join(HERE, "r2r_golden.npz"), **out)


if __name__ == "__main__":
    main()
