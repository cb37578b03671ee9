"""Synthetic initial data for the benchmark and test configurations.

All families are seeded, and all are evaluated on the velocity grid v of
the plan.  Index order is (i, j, k) -> k + N*(j + N*i), with i the x axis.
"""
from __future__ import annotations

import math

import numpy as np


def _mesh(v: np.ndarray):
    return v[:, None, None], v[None, :, None], v[None, None, :]


def trapezoid_mass(v: np.ndarray, f: np.ndarray) -> float:
    """Density with the trapezoid weights of getDensity
    (momentRoutines.c:58-69), unit mass."""
    N = v.size
    wt = np.ones(N)
    wt[0] = wt[-1] = 0.5
    dv = v[1] - v[0]
    w3 = wt[:, None, None] * wt[None, :, None] * wt[None, None, :] * dv ** 3
    return float((w3 * f.reshape(N, N, N)).sum())


def maxwellian(v, rho, u, T):
    """rho (2 pi T)^(-3/2) exp(-|v-u|^2 / (2T))."""
    vx, vy, vz = _mesh(v)
    return rho * (2 * np.pi * T) ** -1.5 * np.exp(
        -((vx - u[0]) ** 2 + (vy - u[1]) ** 2 + (vz - u[2]) ** 2) / (2 * T))


def two_maxwellian_batch(v: np.ndarray, B: int, seed: int) -> np.ndarray:
    """Discontinuous two-Maxwellian in v_x with +-5% seeded jitter on each
    parameter: density 1, temperature 1 for v_x < 0; density 1,
    temperature 2, drift 0.5 for v_x >= 0."""
    rng = np.random.default_rng(seed)
    N = v.size
    vx = v[:, None, None]
    out = np.empty((B, N ** 3))
    for b in range(B):
        j = rng.uniform(-0.05, 0.05, 5) + 1.0
        m1 = maxwellian(v, 1.0 * j[0], (0, 0, 0), 1.0 * j[1])
        m2 = maxwellian(v, 1.0 * j[2], (0.5 * j[4], 0, 0), 2.0 * j[3])
        out[b] = np.where(vx < 0, m1, m2).reshape(-1)
    return out


def maxwellian_mixture_batch(v: np.ndarray, B: int, seed: int) -> np.ndarray:
    """Mixtures of 2-3 Maxwellians with density U(0.2, 1), drift components
    U(-1, 1) and temperature U(0.5, 2), normalised to unit mass."""
    rng = np.random.default_rng(seed)
    N = v.size
    out = np.empty((B, N ** 3))
    for b in range(B):
        f = np.zeros((N, N, N))
        for _ in range(int(rng.integers(2, 4))):
            f += maxwellian(v, rng.uniform(0.2, 1.0), rng.uniform(-1, 1, 3),
                            rng.uniform(0.5, 2.0))
        out[b] = (f / trapezoid_mass(v, f)).reshape(-1)
    return out


def bkw(v: np.ndarray, K: float = 0.65) -> np.ndarray:
    """BKW-type data exp(-|v|^2/(2K)) / (2 (2 pi K)^1.5) ((5K-3)/K +
    (1-K)/K^2 |v|^2) (initializer.c:123-135 with Temp = 1)."""
    vx, vy, vz = _mesh(v)
    v2 = vx ** 2 + vy ** 2 + vz ** 2
    f = np.exp(-v2 / (2 * K)) / (2.0 * (2 * np.pi * K) ** 1.5) * ((5 * K - 3) / K +
                                                                (1 - K) * v2 / (K * K))
    return f.reshape(-1)


def mesh_1d(nX: int, order: int, length: float = 1.0):
    """Cell centres x and widths dx of nX uniform cells on [0, length] plus
    `order` ghost cells on each side (mesh_setup.c:59-160 for one zone on
    one rank; the right ghosts extend the grid uniformly)."""
    dx = length / nX
    x = (np.arange(nX + 2 * order) - order + 0.5) * dx
    return x, np.full(nX + 2 * order, dx)


# (rho_l, ux_l, T_l, rho_r, ux_r, T_r) of the reference's initial fields
# (initializer.c:297-351, Ma = 1 for case 0)
_IC = {
    0: (1.0, -math.sqrt(5.0 / 3.0), 1.0, 1.0, -math.sqrt(5.0 / 3.0), 1.0),
    2: (1.0, -1.0, 1.0, 1.0, -1.0, 2.0),
    3: (1.0, 0.0, 1.0, 1.0, 0.0, 1.5),
    5: (1.0, 0.0, 1.0, 1.0, 0.0, 1.0),
    6: (1.0, 1.2972, 1.0, 1.297, 1.0, 1.195),
}


def init_1d(v: np.ndarray, nX: int, order: int, ic: int, TWall: float = 1.0,
            mass: float = 1.0, KB: float = 1.0) -> np.ndarray:
    """Initial f[nX + 2 order][N^3] of the reference's Init_field cases
    (initializer.c:296-424): 0 (Ma = 1 shock), 1 (sudden heating), 2, 3 (heat
    transfer between walls), 5 (Poiseuille), 6 (the Mach-1.2 shock).  Ghost
    cells stay zero, as in the reference."""
    N = v.size
    vx, vy, vz = _mesh(v)
    out = np.zeros((nX + 2 * order, N ** 3))

    def gauss(rho, ux, T):
        return (rho * np.exp(-((vx - ux) ** 2 + vy ** 2 + vz ** 2) / T) /
                ((T * math.pi) * math.sqrt(T * math.pi))).reshape(-1)

    if ic == 1:
        T = TWall
        m = (1.0 / mass) * (0.5 * mass / (math.pi * KB * T)) ** 1.5 * np.exp(
            -(0.5 * mass / (KB * T)) * (vx ** 2 + vy ** 2 + vz ** 2))
        out[order:nX + order] = m.reshape(-1)
        return out
    rl, ul, tl, rr, ur, tr = _IC[ic]
    if ic == 0:  # the reference's case 0 uses no drift in f (initializer.c:361-373)
        ul = ur = 0.0
        Ma = 1.0
        rl = 4.0 * Ma * Ma / (Ma * Ma + 3.0)
        tl = (5.0 * Ma * Ma - 1.0) * (Ma * Ma + 3.0) / (16.0 * Ma * Ma)
    left, right = gauss(rl, ul, tl), gauss(rr, ur, tr)
    for l in range(order, nX + order):
        if ic in (0, 6):
            out[l] = left if l < nX // 2 else right
        elif ic == 2:
            out[l] = left
        elif ic == 3:
            out[l] = right
        else:
            out[l] = left
    return out


def moment_residual(v: np.ndarray, Q) -> dict:
    """Largest |mass|, |momentum| and |energy| moment of the rows of Q (B x
    N^3, numpy or torch) with the trapezoid weights of conserve.c, each over
    the largest of |Q| times the moment's natural scale (the check of the
    FP64 conservation projection)."""
    Q = np.asarray(Q.detach().cpu().numpy() if hasattr(Q, "detach") else Q, dtype=np.float64)
    N = v.size
    wt = np.ones(N)
    wt[0] = wt[-1] = 0.5
    dv = v[1] - v[0]
    w = (wt[:, None, None] * wt[None, :, None] * wt[None, None, :] * dv ** 3).reshape(-1)
    vx, vy, vz = (a.reshape(-1) for a in np.meshgrid(v, v, v, indexing="ij"))
    e = 0.5 * (vx ** 2 + vy ** 2 + vz ** 2)
    mom = np.stack([Q @ w, Q @ (w * vx), Q @ (w * vy), Q @ (w * vz), Q @ (w * e)], 1)
    scale = np.abs(Q).max(axis=1, keepdims=True) * np.array(
        [w.sum(), (w * np.abs(vx)).sum(), (w * np.abs(vy)).sum(), (w * np.abs(vz)).sum(),
         (w * e).sum()])[None, :]
    r = np.abs(mom) / np.maximum(scale, 1e-300)
    return {"mass": float(r[:, 0].max()), "momentum": float(r[:, 1:4].max()),
            "energy": float(r[:, 4].max())}
