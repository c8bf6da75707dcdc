"""Seeded synthetic DUGKS states shared by the tests and tests/golden/make_golden.py.

The generator is defined here, not by a library distribution: splitmix64 of
(seed, cell, component) -> 53-bit uniform in [-1, 1).  States are
f_p = feq_p(rho, u) * (1 + eps * r_p) with rho = 1 + 0.02 r, u = umax * r'
per cell, so that both the equilibrium and the non-equilibrium parts of the
step are exercised.  Arrays are in dump order, shape (nz, ny, nx, 19).
"""
import numpy as np

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)

_M64 = (1 << 64) - 1


def splitmix64(z):
    z = (z + np.uint64(0x9E3779B97F4A7C15))
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform_sym(seed, n, stream):
    """n values in [-1, 1) from (seed, index, stream)."""
    with np.errstate(over="ignore"):
        idx = np.arange(n, dtype=np.uint64)
        base = np.uint64((seed * 0xD1B54A32D192ED03 + stream * 0x632BE59BD9B4E019) & _M64)
        z = splitmix64(base + idx * np.uint64(64))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def feq(rho, ux, uy, uz):
    """D3Q19 second-order equilibrium, last axis = population."""
    eu = 3.0 * (CX * ux[..., None] + CY * uy[..., None] + CZ * uz[..., None])
    uv = 3.0 * (ux * ux + uy * uy + uz * uz)[..., None]
    return W * rho[..., None] * (1.0 + eu + 0.5 * (eu * eu - uv))


def seeded_state(nx, ny, nz, seed=0, umax=0.05, eps=0.01):
    n = nx * ny * nz
    rho = 1.0 + 0.02 * uniform_sym(seed, n, 0)
    ux = umax * uniform_sym(seed, n, 1)
    uy = umax * uniform_sym(seed, n, 2)
    uz = umax * uniform_sym(seed, n, 3)
    f = feq(rho, ux, uy, uz)
    r = uniform_sym(seed, n * 19, 4).reshape(n, 19)
    f = f * (1.0 + eps * r)
    return np.ascontiguousarray(f.reshape(nz, ny, nx, 19))


def rel_err(a, b):
    """max |a-b| / max |b|"""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
