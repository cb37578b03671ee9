"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the reference checkout exists, naming it by argument or by the
SPECTRAL_REFERENCE_DIR environment variable:

    python tests/golden/make_golden.py REF_DIR

It builds oracle/_ref/libspectral_ref.so from the reference's own
collisions.c, conserve.c, momentRoutines.c and weights.c, compiled with the
project's stand-ins for FFTW, GSL and MPI (oracle/stubs).  It then calls the
reference functions through ctypes and writes:

  golden_w_n8.npz      every 8th row of the two shipped .wts fixtures
                       (tests/BKW8/target, tests/heat_transport/target), plus
                       full-array checksums;
  golden_q.npz         inputs and outputs of fft3D, ComputeQ,
                       ComputeQ_maxPreserve and conserveAllMoments for grids
                       N = 6, 7, 8 (both fixtures' settings) and 16;
  moments_BKW8.txt, moments_heat_transport.txt
                       copies of the reference's golden moment tables;
  golden_landau.npz    Landau-kernel weights from the reference's own
                       initialize_weights_AnIso (aniso_weights.c, glance = 0,
                       64-point Gauss-Legendre through the GSL stand-in) on
                       two small grids (python make_golden.py REF --landau
                       writes only this file).

For N other than 8, W comes from the oracle's quadrature (pinned to the .wts
fixtures).  Tests regenerate it the same way, or on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import pyoracle as po  # noqa: E402

_dp = C.POINTER(C.c_double)


class Species(C.Structure):
    """Layout of the reference's species struct (species.h:11-26)."""
    _fields_ = [("id", C.c_size_t), ("num_levels", C.c_size_t),
                ("lev_id", C.c_void_p), ("Rgas", C.c_double),
                ("mass", C.c_double), ("mm", C.c_double),
                ("d_ref", C.c_double), ("T_ref", C.c_double),
                ("mu_ref", C.c_double), ("omega", C.c_double),
                ("E0", C.c_double), ("Ei", C.c_void_p), ("gi", C.c_void_p),
                ("name", C.c_char * 80)]


def default_species() -> Species:
    """species.c:28-42 defaults."""
    s = Species()
    s.id, s.num_levels = 0, 0
    s.Rgas = s.mass = s.mm = 1.0
    s.d_ref = 2.0
    s.T_ref = s.mu_ref = 1.0
    s.E0 = 0.0
    s.name = b"default"
    return s


class RefLib:
    """The reference's collision module, one grid at a time (it keeps
    file-scope state, collisions.c:11-24)."""

    def __init__(self, path):
        self.L = C.CDLL(path)
        L = self.L
        L.initialize_coll.argtypes = [C.c_int, C.c_double, _dp, _dp]
        L.initialize_moments.argtypes = [C.c_int, _dp, C.POINTER(Species)]
        L.initialize_conservation.argtypes = [C.c_int, C.c_double, _dp,
                                              C.POINTER(Species), C.c_int]
        L.ComputeQ.argtypes = [_dp, _dp, _dp, C.POINTER(_dp)]
        L.ComputeQ_maxPreserve.argtypes = [_dp, _dp, _dp, C.POINTER(_dp)]
        L.conserveAllMoments.argtypes = [C.POINTER(_dp)]
        L.fft3D.argtypes = [_dp, _dp, C.c_int]

    def setup(self, g: po.Grid):
        self._keep = [g.v, g.zeta]
        self.sp = (Species * 1)(default_species())
        self.L.initialize_coll(g.N, g.L_v, po._p(g.v), po._p(g.zeta))
        self.L.initialize_moments(g.N, po._p(g.v), self.sp)
        self.L.initialize_conservation(g.N, float(g.v[1] - g.v[0]), po._p(g.v),
                                       self.sp, 1)
        self.n3 = g.n3

    def rows(self, W):
        W = np.ascontiguousarray(W, dtype=np.float64)
        self._W = W
        ptrs = (_dp * self.n3)()
        for i in range(self.n3):
            ptrs[i] = C.cast(W.ctypes.data + 8 * self.n3 * i, _dp)
        self._ptrs = ptrs
        return ptrs

    def computeQ(self, f, W, maxpreserve=False):
        f = np.ascontiguousarray(f, dtype=np.float64)
        Q = np.zeros(self.n3)
        fn = self.L.ComputeQ_maxPreserve if maxpreserve else self.L.ComputeQ
        fn(po._p(f), po._p(f), po._p(Q), self.rows(W))
        return Q

    def conserve(self, Q):
        Q = np.array(Q, dtype=np.float64, copy=True)
        arr = (_dp * 1)(po._p(Q))
        self.L.conserveAllMoments(arr)
        return Q

    def fft3d(self, x, invert):
        a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128)).view(np.float64)
        out = np.zeros_like(a)
        self.L.fft3D(po._p(a), po._p(out), invert)
        return out.view(np.complex128)


def heat_init(g: po.Grid, rho=1.0, T=1.5):
    """initializer.c:391-397 (Init_field 3)."""
    v = g.v
    vv = v[:, None, None] ** 2 + v[None, :, None] ** 2 + v[None, None, :] ** 2
    return (rho * np.exp(-vv / T) / ((T * np.pi) * np.sqrt(T * np.pi))).reshape(-1)


def two_maxwellian(g: po.Grid, rng, jitter=0.05):
    """A discontinuous two-Maxwellian in v_x, with seeded jitter."""
    v = g.v
    j = lambda x: x * (1 + jitter * rng.uniform(-1, 1))  # noqa: E731
    r1, t1, r2, t2, u2 = j(1.0), j(1.0), j(1.0), j(2.0), j(0.5)
    vx = v[:, None, None]
    vy = v[None, :, None]
    vz = v[None, None, :]
    m1 = r1 * (2 * np.pi * t1) ** -1.5 * np.exp(-(vx ** 2 + vy ** 2 + vz ** 2) / (2 * t1))
    m2 = r2 * (2 * np.pi * t2) ** -1.5 * np.exp(-((vx - u2) ** 2 + vy ** 2 + vz ** 2) / (2 * t2))
    f = np.where(vx < 0, m1, m2)
    return np.ascontiguousarray(f.reshape(-1))


def landau(ref_dir):
    """golden_landau.npz: the reference's initialize_weights_AnIso, run in a
    scratch directory (it writes Weights/N*_Aniso_*_Landau.wts there)."""
    import tempfile
    assert po.build_ref(ref_dir), "reference sources not found"
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libspectral_ref.so"))
    L.initialize_weights_AnIso.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_int,
                                           C.POINTER(_dp), C.c_double]
    out = {}
    cwd = os.getcwd()
    # g4 passes a non-zero glance: the reference then writes the *_glance*.wts
    # name, and its generator still takes the Landau branch.
    for name, N, L_v, lam, glance in (("n4", 4, 4.0, 0.0, 0.0), ("n5", 5, 3.0, 1.0, 0.0),
                                      ("g4", 4, 4.0, 0.0, 0.3)):
        g = po.Grid(N, L_v, "0d")
        rows = (_dp * g.n3)()
        with tempfile.TemporaryDirectory() as d:
            os.makedirs(os.path.join(d, "Weights"))
            os.chdir(d)
            try:
                L.initialize_weights_AnIso(N, po._p(g.zeta), L_v, lam, 1, rows, glance)
            finally:
                os.chdir(cwd)
            (fname,) = os.listdir(os.path.join(d, "Weights"))
        W = np.stack([np.ctypeslib.as_array(rows[i], shape=(g.n3,)).copy() for i in range(g.n3)])
        out[f"{name}_meta"] = np.array([N, L_v, lam, glance])
        out[f"{name}_file"] = np.array("Weights/" + fname)
        out[f"{name}_zeta"] = g.zeta.copy()
        out[f"{name}_W"] = W
        print("landau", name, W.shape, np.abs(W).max())
    np.savez_compressed(os.path.join(HERE, "golden_landau.npz"), **out)


def main(ref_dir):
    assert po.build_ref(ref_dir), "reference sources not found"
    po.build()
    ref = RefLib(os.path.join(ROOT, "oracle", "_ref", "libspectral_ref.so"))
    rng = np.random.default_rng(20261203)

    # ---- the shipped weight fixtures, subsampled
    wout = {}
    for tag, sub in (("bkw8", "BKW8/target/N8_isotropic_L_v5_lambda0.wts"),
                     ("heat", "heat_transport/target/N8_isotropic_L_v9_lambda1.wts")):
        W = np.fromfile(os.path.join(ref_dir, "tests", sub)).reshape(512, 512)
        wout[f"{tag}_rows"] = W[::8].copy()
        wout[f"{tag}_row_index"] = np.arange(0, 512, 8)
        wout[f"{tag}_sum"] = np.array(W.sum())
        wout[f"{tag}_sumsq"] = np.array((W * W).sum())
        wout[f"{tag}_abssum"] = np.array(np.abs(W).sum())
    np.savez_compressed(os.path.join(HERE, "golden_w_n8.npz"), **wout)

    cases = [
        # name, N, L_v, grid, lambda, weights source
        ("bkw8", 8, 5.0, "0d", 0.0, "BKW8/target/N8_isotropic_L_v5_lambda0.wts"),
        ("heat8", 8, 9.0, "1d", 1.0, "heat_transport/target/N8_isotropic_L_v9_lambda1.wts"),
        ("n6", 6, 4.0, "0d", 1.0, None),
        ("n7", 7, 4.5, "0d", 0.0, None),
        ("n16", 16, 5.0, "0d", 1.0, None),
    ]
    out = {}
    for name, N, L_v, kind, lam, wsrc in cases:
        g = po.Grid(N, L_v, kind)
        if wsrc:
            W = np.fromfile(os.path.join(ref_dir, "tests", wsrc)).reshape(g.n3, g.n3)
        else:
            W = po.weights_iso(g, lam)
        ref.setup(g)
        if name == "bkw8":
            f = po.init_bkw(g)
        elif name == "heat8":
            f = heat_init(g) * (1 + 0.02 * rng.uniform(-1, 1, g.n3))
        else:
            f = two_maxwellian(g, rng)
        fhat = ref.fft3d(f.astype(np.complex128), 0)
        finv = ref.fft3d(fhat, 1)
        Q = ref.computeQ(f, W)
        Qmp = ref.computeQ(f, W, maxpreserve=True)
        out[f"{name}_meta"] = np.array([N, L_v, 0 if kind == "0d" else 1, lam])
        out[f"{name}_f"] = f
        out[f"{name}_fhat"] = fhat
        out[f"{name}_finv"] = finv
        out[f"{name}_Q"] = Q
        out[f"{name}_Qc"] = ref.conserve(Q)
        out[f"{name}_Qmp"] = Qmp
        out[f"{name}_Qmpc"] = ref.conserve(Qmp)
        print(name, "done", np.abs(Q).max())
    np.savez_compressed(os.path.join(HERE, "golden_q.npz"), **out)

    for t in ("BKW8", "heat_transport"):
        shutil.copy(os.path.join(ref_dir, "tests", t, "target", f"moments_{t}.test.in"),
                    os.path.join(HERE, f"moments_{t}.txt"))


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = args[0] if args else os.environ.get("SPECTRAL_REFERENCE_DIR", "")
    if not ref:
        sys.exit("usage: make_golden.py REF_DIR (or set SPECTRAL_REFERENCE_DIR)")
    if "--landau" in sys.argv:
        landau(ref)
    else:
        main(ref)
        landau(ref)
