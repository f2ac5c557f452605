"""Seeded initial states of the benchmark workloads.

psi = sqrt(rho_WS) * (1 + 1e-3 * U(0,1)), rho_WS = rho0 / (1 + exp((r-R)/a)),
R = 2.22 N^(1/3) A, a = 1 A, rho0 = 0.0218 A^-3, noise drawn with
numpy.random.default_rng(seed) in x-fastest order, normalised to N atoms.
"""
import numpy as np


def grid_axes(nx, ny, nz, xmax, ymax, zmax):
    hx, hy, hz = 2 * abs(xmax) / nx, 2 * abs(ymax) / ny, 2 * abs(zmax) / nz
    return (-xmax + hx * np.arange(nx), -ymax + hy * np.arange(ny), -zmax + hz * np.arange(nz),
            hx * hy * hz)


def woods_saxon_psi(nx, ny, nz, xmax, ymax, zmax, n4, seed, rho0=0.0218, a=1.0,
                    center=(0.0, 0.0, 0.0), noise=1e-3):
    x, y, z, dv = grid_axes(nx, ny, nz, xmax, ymax, zmax)
    X, Y, Z = np.meshgrid(x - center[0], y - center[1], z - center[2], indexing="ij")
    r = np.sqrt(X * X + Y * Y + Z * Z)
    R = 2.22 * n4 ** (1.0 / 3.0)
    rho = rho0 / (1.0 + np.exp((r - R) / a))
    rng = np.random.default_rng(seed)
    u = rng.random(nx * ny * nz).reshape((nx, ny, nz), order="F")
    psi = np.sqrt(rho) * (1.0 + noise * u)
    psi *= np.sqrt(n4 / (np.sum(psi * psi) * dv))
    return np.asfortranarray(psi.astype(np.complex128))
