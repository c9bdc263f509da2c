"""Seeded synthetic initial conditions for the benchmark workloads.

The reference's own initial condition (smaiso-wcomp.cpp:571-590: psi = Amp cos(q0 k dz)
in a 16-point band around Nz/2, rho = 0) is available as `reference_band`. The
workloads below are synthetic stand-ins with stated shapes, sizes and value
distributions; none comes from a dataset.

Noise is counter-based: value(index) = f(SplitMix64(seed XOR global linear index)),
so any process (or a device kernel) regenerates the same field without sharing
state. Uniform on [-a, a] from the top 53 bits; Gaussian by Box-Muller on the
pair of counters (2m, 2m+1).
"""
import numpy as np

from .abi import derived

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x):
    """SplitMix64 finaliser of a uint64 array (Steele, Lea, Flood 2014)."""
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed, index):
    """U[0,1) from the top 53 bits of SplitMix64(seed ^ index)."""
    z = splitmix64(np.uint64(seed) ^ np.asarray(index, dtype=np.uint64))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform_noise(shape, seed, a):
    n = int(np.prod(shape))
    return (2.0 * uniform01(seed, np.arange(n, dtype=np.uint64)) - 1.0).reshape(shape) * a


def gaussian_noise(shape, seed, sigma):
    n = int(np.prod(shape))
    m = (n + 1) // 2
    base = np.arange(m, dtype=np.uint64) * np.uint64(2)
    u1 = uniform01(seed, base)
    u2 = uniform01(seed, base + np.uint64(1))
    r = np.sqrt(-2.0 * np.log1p(-u1))          # 1-u1 in (0,1]
    g = np.empty(2 * m)
    g[0::2] = r * np.cos(2.0 * np.pi * u2)
    g[1::2] = r * np.sin(2.0 * np.pi * u2)
    return g[:n].reshape(shape) * sigma


def _coords(p):
    d = derived(p)
    x = np.arange(p.nx) * d["dx"]
    y = np.arange(p.ny) * d["dy"]
    z = np.arange(p.nz) * d["dz"]
    return d, x[:, None, None], y[None, :, None], z[None, None, :]


def reference_band(p):
    """smaiso-wcomp.cpp:571-590 with phi = 0: Amp cos(q0 k dz) for Nz/2-8 < k < Nz/2+8."""
    d = derived(p)
    psi = np.zeros((p.nx, p.ny, p.nz))
    k = np.arange(p.nz)
    band = (k > p.nz // 2 - 8) & (k < p.nz // 2 + 8)
    psi[:, :, band] = d["amp"] * np.cos(p.q0 * k[band] * d["dz"])
    return psi, np.zeros_like(psi)


def flat_interface(p, seed=1001, A=0.8, xi=2.0, rho_s=1.0, rho_i=0.9, noise=1e-4):
    """Flat smectic/isotropic interface at z0 = Lz/2, layers parallel to it:
    psi = 0.5 (1 + tanh((z - z0)/xi)) A cos(q0 z) + U(-noise, noise);
    rho = rho_i + (rho_s - rho_i) * 0.5 (1 + tanh((z - z0)/xi))."""
    d, x, y, z = _coords(p)
    h = 0.5 * (1.0 + np.tanh((z - d["lz"] / 2) / xi))
    shape = (p.nx, p.ny, p.nz)
    psi = np.broadcast_to(h * A * np.cos(p.q0 * z), shape) + uniform_noise(shape, seed, noise)
    rho = np.broadcast_to(rho_i + (rho_s - rho_i) * h, shape).copy()
    return np.ascontiguousarray(psi), rho


def undulated_interface(p, seed=1002, A=0.8, xi=2.0, ratio=0.8, sigma=1e-3):
    """Interface z0(x,y) = Lz/2 + 2 (2 pi/q0) sin(2 pi x/Lx) cos(2 pi y/Ly);
    density ratio rho_i/rho_s = ratio with rho_s = 1; Gaussian psi noise sigma."""
    d, x, y, z = _coords(p)
    z0 = d["lz"] / 2 + 2.0 * (2.0 * np.pi / p.q0) * np.sin(2 * np.pi * x / d["lx"]) * \
        np.cos(2 * np.pi * y / d["ly"])
    h = 0.5 * (1.0 + np.tanh((z - z0) / xi))
    shape = (p.nx, p.ny, p.nz)
    psi = h * A * np.cos(p.q0 * z) + gaussian_noise(shape, seed, sigma)
    rho = ratio + (1.0 - ratio) * h
    return np.ascontiguousarray(np.broadcast_to(psi, shape)), np.ascontiguousarray(
        np.broadcast_to(rho, shape))


def dislocations(p, seed=1003, A=0.8, ncores=16, xi=2.0):
    """Layer-dislocation state psi = A cos(q0 z + sum_k theta_k) below a flat
    interface at 3Lz/4, theta_k = atan2(z - z_k, x - x_k) (edge dislocations with
    cores at seeded positions in the lower half); rho = rho_s below, rho_0 above."""
    d, x, y, z = _coords(p)
    u = uniform01(seed, np.arange(2 * ncores, dtype=np.uint64))
    xk = u[0::2] * d["lx"]
    zk = (0.15 + 0.45 * u[1::2]) * d["lz"]
    theta = np.zeros((p.nx, 1, p.nz))
    for a, b in zip(xk, zk):
        theta += np.arctan2(z - b, x - a)
    h = 0.5 * (1.0 - np.tanh((z - 0.75 * d["lz"]) / xi))
    shape = (p.nx, p.ny, p.nz)
    psi = np.broadcast_to(h * A * np.cos(p.q0 * z + theta), shape)
    rho = np.broadcast_to(p.rho_0 + (1.0 - p.rho_0) * h, shape)
    return np.ascontiguousarray(psi), np.ascontiguousarray(rho)
