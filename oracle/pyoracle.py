"""ctypes bindings for the CPU oracle (liboracle.so) and the CPU reference
build (_ref/libspectral_ref.so).

TEST INFRASTRUCTURE, NOT PRODUCT.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import this module.  They use it to check or
time the GPU library, never as a fallback for it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_dp = C.POINTER(C.c_double)


def build(quiet: bool = True) -> str:
    """Compile liboracle.so in place (gcc, a second or two)."""
    out = subprocess.run(["make", "-C", HERE, "liboracle.so"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(HERE, "liboracle.so")


def build_ref(ref_dir: str) -> bool:
    """Compile _ref/ from the reference sources in ref_dir, if they are
    present there."""
    if not ref_dir or not os.path.isdir(os.path.join(ref_dir, "src")):
        return False
    out = subprocess.run(["make", "-C", HERE, "ref", f"REF={ref_dir}"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)
    return True


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        i, d = C.c_int, C.c_double
        sigs = {
            "oracle_grid_0d": (None, [i, d, _dp, _dp]),
            "oracle_grid_1d": (None, [i, d, _dp, _dp]),
            "oracle_fft3d": (None, [i, d, _dp, _dp, _dp, _dp, i]),
            "oracle_compute_qhat": (None, [i, d, _dp, _dp, _dp, _dp, _dp, _dp,
                                           _dp, _dp, _dp, i]),
            "oracle_computeQ": (None, [i, d, _dp, _dp, _dp, _dp, _dp, _dp, i]),
            "oracle_computeQ_maxPreserve": (None, [i, d, _dp, _dp, _dp, _dp, _dp,
                                                   _dp, d, d, i]),
            "oracle_density": (d, [i, _dp, _dp, d]),
            "oracle_bulk_velocity": (None, [i, _dp, _dp, d, d, _dp]),
            "oracle_temperature": (d, [i, _dp, _dp, _dp, d, d, d]),
            "oracle_ghat_integral": (d, [d, d, d, d, d]),
            "oracle_gauss_legendre": (None, [i, _dp, _dp]),
            "oracle_weights_iso": (None, [i, _dp, d, d, d, d, d, d, i, i, _dp, i]),
            "oracle_weights_iso_closed": (None, [i, _dp, d, d, d, d, d, d, i, i, _dp, i]),
            "oracle_ghat_closed": (d, [d, d, d, d, d]),
            "oracle_weights_landau": (None, [i, _dp, d, d, i, i, _dp]),
            "oracle_ghat3l": (d, [d, d, d, d, d, d, d, d]),
            "oracle_graze_panels": (i, [d, d]),
            "oracle_ghat3_graze": (d, [d, d, d, d, d, d, d, d, d, i]),
            "oracle_ghat3_graze_pairs": (None, [i, _dp, d, d, d, i, _dp]),
            "oracle_run_0d": (None, [i, d, _dp, _dp, d, d, i, i, i, _dp, i]),
            "oracle_init_bkw": (None, [i, _dp, d, _dp]),
            "oracle_conserve_batch1": (None, [C.c_void_p, _dp, i]),
            "oracle_conservation_init": (i, [C.c_void_p, i, d, _dp, _dp, i]),
            "oracle_qhat_rows": (None, [i, _dp, i, i, _dp, _dp, _dp, i]),
            "oracle_mesh_uniform": (None, [i, d, i, _dp, _dp]),
            "oracle_init_1d": (None, [C.c_void_p, _dp, _dp]),
            "oracle_advect": (None, [C.c_void_p, _dp, _dp, _dp, _dp]),
            "oracle_run_1d": (None, [C.c_void_p, _dp, _dp, i, _dp, i]),
            "oracle_diffuse_bc": (None, [i, _dp, _dp, _dp, d, i, d, d]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


class Grid:
    """Velocity and Fourier grids of the reference (initializer.c:66-82 for
    0D, :256-266 for 1D)."""

    def __init__(self, N: int, L_v: float, kind: str = "0d"):
        self.N, self.L_v, self.kind = N, float(L_v), kind
        self.v = np.zeros(N)
        self.zeta = np.zeros(N)
        fn = lib().oracle_grid_0d if kind == "0d" else lib().oracle_grid_1d
        fn(N, self.L_v, _p(self.v), _p(self.zeta))
        self.n3 = N ** 3


def fft3d(g: Grid, x: np.ndarray, invert: int) -> np.ndarray:
    """fft3D (collisions.c:232-283) on a complex N^3 array."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128).reshape(-1))
    ai = a.view(np.float64)
    out = np.zeros(2 * g.n3)
    lib().oracle_fft3d(g.N, g.L_v, _p(g.v), _p(g.zeta), _p(ai), _p(out), invert)
    return out.view(np.complex128)


def compute_qhat(g: Grid, W: np.ndarray, f: np.ndarray, gg: np.ndarray,
                 nthreads: int = 0):
    """Returns (Q, fhat, ghat, qhat) of compute_Qhat (collisions.c:108-169)."""
    n3 = g.n3
    W = np.ascontiguousarray(W, dtype=np.float64).reshape(n3, n3)
    q = np.zeros(n3)
    fh, gh, qh = np.zeros(2 * n3), np.zeros(2 * n3), np.zeros(2 * n3)
    lib().oracle_compute_qhat(g.N, g.L_v, _p(g.v), _p(g.zeta), _p(W),
                              _p(np.ascontiguousarray(f, dtype=np.float64)),
                              _p(np.ascontiguousarray(gg, dtype=np.float64)),
                              _p(q), _p(fh), _p(gh), _p(qh), nthreads)
    return q, fh.view(np.complex128), gh.view(np.complex128), qh.view(np.complex128)


def computeQ(g: Grid, W, f, gg=None, nthreads: int = 0) -> np.ndarray:
    gg = f if gg is None else gg
    Q = np.zeros(g.n3)
    W = np.ascontiguousarray(W, dtype=np.float64)
    lib().oracle_computeQ(g.N, g.L_v, _p(g.v), _p(g.zeta), _p(W),
                          _p(np.ascontiguousarray(f, dtype=np.float64)),
                          _p(np.ascontiguousarray(gg, dtype=np.float64)),
                          _p(Q), nthreads)
    return Q


def computeQ_maxPreserve(g: Grid, W, f, gg=None, mass=1.0, KB=1.0,
                         nthreads: int = 0) -> np.ndarray:
    gg = f if gg is None else gg
    Q = np.zeros(g.n3)
    W = np.ascontiguousarray(W, dtype=np.float64)
    lib().oracle_computeQ_maxPreserve(
        g.N, g.L_v, _p(g.v), _p(g.zeta), _p(W),
        _p(np.ascontiguousarray(f, dtype=np.float64)),
        _p(np.ascontiguousarray(gg, dtype=np.float64)), _p(Q), mass, KB,
        nthreads)
    return Q


class _Cons(C.Structure):
    _fields_ = [("N", C.c_int), ("Ns", C.c_int), ("dv", C.c_double),
                ("v", C.c_void_p), ("mass", C.c_double * 4),
                ("CCt", (C.c_double * 8) * 8), ("pivot", C.c_int * 8)]


class Conservation:
    """initialize_conservation + conserveAllMoments (conserve.c) for one
    species."""

    def __init__(self, g: Grid, mass: float = 1.0):
        self._v = g.v  # keep alive: the struct points at it
        self.c = _Cons()
        m = np.array([mass])
        rc = lib().oracle_conservation_init(C.byref(self.c), g.N,
                                            float(g.v[1] - g.v[0]), _p(g.v),
                                            _p(m), 1)
        if rc != 0:
            raise ValueError("singular CC^T")
        self.n3 = g.n3

    def __call__(self, Q: np.ndarray) -> np.ndarray:
        Q = np.array(Q, dtype=np.float64, copy=True)
        B = Q.size // self.n3
        lib().oracle_conserve_batch1(C.byref(self.c), _p(Q.reshape(-1)), B)
        return Q


def moments(g: Grid, f: np.ndarray, mass: float = 1.0, KB: float = 1.0):
    """(rho, u[3], T) as momentRoutines.c computes them."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    L = lib()
    rho = L.oracle_density(g.N, _p(g.v), _p(f), mass)
    u = np.zeros(3)
    L.oracle_bulk_velocity(g.N, _p(g.v), _p(f), rho, mass, _p(u))
    T = L.oracle_temperature(g.N, _p(g.v), _p(f), _p(u), rho, mass, KB)
    return rho, u, T


def qhat_rows(g: Grid, W_rows: np.ndarray, row0: int, fhat: np.ndarray,
              ghat: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """compute_Qhat's convolution for zeta rows [row0, row0 + len(W_rows))."""
    W_rows = np.ascontiguousarray(W_rows, dtype=np.float64)
    nrows = W_rows.shape[0]
    fh = np.ascontiguousarray(fhat, dtype=np.complex128).view(np.float64)
    gh = np.ascontiguousarray(ghat, dtype=np.complex128).view(np.float64)
    out = np.zeros(2 * nrows)
    lib().oracle_qhat_rows(g.N, _p(W_rows), row0, nrows, _p(fh), _p(gh), _p(out), nthreads)
    return out.view(np.complex128)


def weights_iso(g: Grid, lam: float, rows=None, d_i=2.0, d_j=2.0, m_i=1.0,
                m_j=1.0, nthreads: int = 0, closed: bool = False) -> np.ndarray:
    """Rows of the isotropic weights (weights.c:265-281); default all.
    closed=True evaluates the radial integral in closed form (lambda 0, 1)."""
    n3 = g.n3
    r0, r1 = (0, n3) if rows is None else rows
    W = np.zeros((r1 - r0, n3))
    fn = lib().oracle_weights_iso_closed if closed else lib().oracle_weights_iso
    fn(g.N, _p(g.zeta), g.L_v, float(lam), d_i, d_j, m_i, m_j, r0, r1, _p(W), nthreads)
    return W


def weights_landau(N: int, zeta: np.ndarray, L_v: float, lam: float, rows=None) -> np.ndarray:
    """Rows of the Landau-kernel weights (aniso_weights.c:370-425); default all."""
    n3 = N ** 3
    r0, r1 = (0, n3) if rows is None else rows
    zeta = np.ascontiguousarray(zeta, dtype=np.float64)
    W = np.zeros((r1 - r0, n3))
    lib().oracle_weights_landau(N, _p(zeta), float(L_v), float(lam), r0, r1 - r0, _p(W))
    return W


def graze_unique(N: int, eta: np.ndarray):
    """Group the N^6 (zeta, xi) pairs of a weight table by the exact integer
    key (|2k|^2, 2k.2l, |2l|^2) of their offsets from the grid centre
    (2 k_a = 2 i_a - N), on which gHat3 depends alone (through |zeta|,
    xi.zeta and |xi|).  Returns (pairs [U][6] of one representative each,
    inverse [N^3 * N^3] index of each table entry into them)."""
    eta = np.asarray(eta, dtype=np.float64)
    k = 2 * np.arange(N) - N
    Kx = np.stack(np.meshgrid(k, k, k, indexing="ij"), -1).reshape(-1, 3)
    a = (Kx * Kx).sum(1)
    d = Kx @ Kx.T
    n3 = N ** 3
    key = (a[:, None].astype(np.int64) * (1 << 40) + (d.astype(np.int64) + (1 << 20)) * (1 << 20)
           + a[None, :].astype(np.int64)).reshape(-1)
    uniq, first, inverse = np.unique(key, return_index=True, return_inverse=True)
    z, x = first // n3, first % n3
    idx = np.stack(np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij"),
                   -1).reshape(-1, 3)
    pairs = np.concatenate([eta[idx[z]], eta[idx[x]]], 1)
    return np.ascontiguousarray(pairs), inverse.astype(np.int64)


def weights_graze(N: int, eta: np.ndarray, L_v: float, lam: float, glance: float,
                  pairs_only=None):
    """Grazing-collision weights of the stand-alone generator
    (MPIcollisionRoutines.c:154-274) on the grid eta: the whole table, or,
    with pairs_only = (pairs, npan), gHat3 of those pairs."""
    L = lib()
    if pairs_only is not None:
        pairs, npan = pairs_only
        pairs = np.ascontiguousarray(pairs, dtype=np.float64)
        out = np.zeros(pairs.shape[0])
        L.oracle_ghat3_graze_pairs(pairs.shape[0], _p(pairs), float(L_v), float(lam),
                                   float(glance), int(npan), _p(out))
        return out
    npan = L.oracle_graze_panels(float(np.abs(eta).max()), float(L_v))
    pairs, inverse = graze_unique(N, eta)
    vals = weights_graze(N, eta, L_v, lam, glance, (pairs, npan))
    return vals[inverse].reshape(N ** 3, N ** 3)


def gauss_legendre(n: int):
    x, w = np.zeros(n), np.zeros(n)
    lib().oracle_gauss_legendre(n, _p(x), _p(w))
    return x, w


def init_bkw(g: Grid, K: float = 0.0) -> np.ndarray:
    f = np.zeros(g.n3)
    lib().oracle_init_bkw(g.N, _p(g.v), float(K), _p(f))
    return f


def run_0d(N, L_v, W, f0, dt, Kn, nT, order, maxpreserve=True,
           nthreads: int = 0) -> np.ndarray:
    """0D time loop of boltz.c:186-250; returns the write_streams rows."""
    rows = np.zeros((nT + 1, 6 + N))
    f = np.array(f0, dtype=np.float64, copy=True)
    lib().oracle_run_0d(N, float(L_v), _p(np.ascontiguousarray(W, dtype=np.float64)),
                        _p(f), float(dt), float(Kn), nT, order,
                        1 if maxpreserve else 0, _p(rows), nthreads)
    return rows


class _P1D(C.Structure):
    _fields_ = [("N", C.c_int), ("nX", C.c_int), ("order", C.c_int), ("ic", C.c_int),
                ("L_v", C.c_double), ("dt", C.c_double), ("Kn", C.c_double),
                ("T0", C.c_double), ("T1", C.c_double), ("TWall", C.c_double),
                ("mass", C.c_double), ("KB", C.c_double),
                ("x", C.c_void_p), ("dx", C.c_void_p)]


class Run1D:
    """The 1D solver of boltz.c:254-394 on one rank: transport
    (transportroutines.c), walls (boundaryConditions.c), initial data
    (initializer.c:296-424), ComputeQ + conservation per cell."""

    def __init__(self, N, L_v, nX, order, ic, dt, Kn, length=1.0, T0=1.0, T1=2.0,
                 TWall=1.0, mass=1.0):
        self.N, self.nX, self.order = N, nX, order
        self.g = Grid(N, L_v, "1d")
        nc = nX + 2 * order
        self.x = np.zeros(nc)
        self.dx = np.zeros(nc)
        lib().oracle_mesh_uniform(nX, float(length), order, _p(self.x), _p(self.dx))
        self.p = _P1D(N, nX, order, ic, float(L_v), float(dt), float(Kn), T0, T1, TWall,
                      mass, 1.0 if mass == 1.0 else 1.380658e-23,
                      self.x.ctypes.data, self.dx.ctypes.data)
        self.n3 = N ** 3

    def init(self) -> np.ndarray:
        f = np.zeros((self.nX + 2 * self.order, self.n3))
        lib().oracle_init_1d(C.byref(self.p), _p(self.g.v), _p(f))
        return f

    def advect(self, f: np.ndarray) -> np.ndarray:
        fconv = np.zeros_like(f)
        scratch = np.zeros((self.nX + 6, self.n3))
        lib().oracle_advect(C.byref(self.p), _p(self.g.v), _p(f), _p(fconv), _p(scratch))
        return fconv

    def run(self, W, f, nT, nthreads=0) -> np.ndarray:
        rows = np.zeros((nT + 1, self.nX, 6))
        lib().oracle_run_1d(C.byref(self.p), _p(np.ascontiguousarray(W, dtype=np.float64)),
                            _p(f), nT, _p(rows), nthreads)
        return rows
