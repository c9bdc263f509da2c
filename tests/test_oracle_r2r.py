"""The oracle's r2r transforms against the committed golden vectors (scipy.fft,
an independent implementation of FFTW's REDFT/RODFT definitions) and against the
defining O(N^2) sums."""
import os

import numpy as np
import pytest

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "r2r_golden.npz"))
KINDS = {"redft10": 0, "redft01": 1, "rodft10": 2, "rodft01": 3}
SIZES = (4, 8, 12, 16, 32, 64, 128, 256, 512)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("direct", [False, True])
def test_r2r1d_golden(oracle_mod, n, kind, direct):
    x = GOLD[f"x_{n}"]
    ref = GOLD[f"{kind}_{n}"]
    got = oracle_mod.r2r1d(x, KINDS[kind], direct=direct)
    tol = 1e-15 * n if (direct or n & (n - 1)) else 2e-15
    assert np.max(np.abs(got - ref)) <= tol * np.max(np.abs(ref))


PLANS = {"CT": (0, 0, 0), "iCT": (1, 1, 1), "STx": (2, 0, 0), "iSTx": (3, 1, 1),
         "STy": (0, 2, 0), "iSTy": (1, 3, 1), "STz": (0, 0, 2), "iSTz": (1, 1, 3)}


@pytest.mark.parametrize("plan", list(PLANS))
def test_r2r3d_plans_golden(oracle_mod, plan):
    a = GOLD["a3"]
    got = oracle_mod.r2r3d(a, PLANS[plan])
    ref = GOLD[f"plan_{plan}"]
    assert np.max(np.abs(got - ref)) <= 2e-15 * np.max(np.abs(ref))


@pytest.mark.parametrize("n", (8, 16, 64))
def test_forward_inverse_pairs(oracle_mod, n):
    """FFTW normalisation (REF:488-496): each forward/inverse pair multiplies by 2N."""
    x = np.random.default_rng(n).standard_normal(n)
    for f, b in ((0, 1), (2, 3)):
        y = oracle_mod.r2r1d(oracle_mod.r2r1d(x, f), b)
        np.testing.assert_allclose(y, 2 * n * x, rtol=0, atol=1e-13 * n)


def test_separable_gaussian_filter(oracle_mod):
    """The mixed engine's Gaussian amplitude filter as three one-axis filter passes (along
    z, y, x: DCT-II along the axis, that axis's factor, DCT-III; the scale 1/(8 N^3) in
    the last) equals the reference's 3D form DCT-III^3(scale g_x g_y g_z DCT-II^3 A)
    (REF:1271-1289): each DCT-III DCT-II pair along an axis gives 2n."""
    shape = (8, 4, 16)
    rng = np.random.default_rng(5)
    a = rng.standard_normal(shape)
    g = [np.exp(-1.57 ** 2 * 2 * (np.pi * np.arange(n) / (0.7 * n)) ** 2) for n in shape]
    scale = 0.125 / np.prod(shape)
    G = scale * g[0][:, None, None] * g[1][None, :, None] * g[2][None, None, :]
    ref = oracle_mod.r2r3d(G * oracle_mod.r2r3d(a, (0, 0, 0)), (1, 1, 1))

    def filt(x, axis, factor):
        y = np.apply_along_axis(lambda v: oracle_mod.r2r1d(v, 0), axis, x)
        sh = [1, 1, 1]
        sh[axis] = -1
        y = y * factor.reshape(sh)
        return np.apply_along_axis(lambda v: oracle_mod.r2r1d(v, 1), axis, y)

    out = filt(filt(filt(a, 2, g[2]), 1, g[1]), 0, scale * g[0])
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-13 * np.max(np.abs(ref)))
