"""spectralbte_gb300 -- Python host mirror of the GB300 collision library.

The compute runs in libspectral_gb300.so (hand-written CUDA for sm_103a).
This module binds its C ABI (include/spectral_bte.h) with ctypes.

* ``ReferenceAPI`` mirrors the reference's collisions.h, conserve.h and
  weights.h entry points one for one: initialize_coll, ComputeQ,
  ComputeQ_maxPreserve, fft3D, initialize_conservation, conserveAllMoments,
  alloc_weights, initialize_weights and dealloc_weights.  Each takes numpy
  arrays.
* ``Plan`` wraps the batched device API.  f and Q stay in device memory,
  either torch CUDA tensors or raw device pointers.

There is no CPU fallback.  If the shared library is missing, or no GPU is
present, loading or calling it raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libspectral_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "spectral_bte.h")

FP64 = 0
FP32 = 1
MAXPRESERVE = 2
CONSERVE = 4
LEARNED = 8

_dp = C.POINTER(C.c_double)
_LIB: Optional[C.CDLL] = None


class SpectralError(RuntimeError):
    pass


class Species(C.Structure):
    """Layout of the reference's species struct (species.h:11-26)."""
    _fields_ = [("id", C.c_size_t), ("num_levels", C.c_size_t),
                ("lev_id", C.c_void_p), ("Rgas", C.c_double),
                ("mass", C.c_double), ("mm", C.c_double),
                ("d_ref", C.c_double), ("T_ref", C.c_double),
                ("mu_ref", C.c_double), ("omega", C.c_double),
                ("E0", C.c_double), ("Ei", C.c_void_p), ("gi", C.c_void_p),
                ("name", C.c_char * 80)]

    @classmethod
    def default(cls, mass: float = 1.0, d_ref: float = 2.0, name: bytes = b"default",
                sid: int = 0) -> "Species":
        """species.c:28-42 defaults."""
        s = cls()
        s.id, s.num_levels = sid, 0
        s.Rgas, s.mass, s.mm = 1.0, mass, 1.0
        s.d_ref, s.T_ref, s.mu_ref, s.E0 = d_ref, 1.0, 1.0, 0.0
        s.name = name
        return s


def grid_0d(N: int, L_v: float):
    """(v, zeta) of the homogeneous solver (initializer.c:66-82)."""
    dv = 2 * L_v / (N - 1)
    v = np.array([-L_v + i * dv for i in range(N)])
    deta = (2 * np.pi / N) / dv
    L_eta = 0.5 * N * deta if N % 2 == 0 else 0.5 * (N - 1) * deta
    zeta = np.array([-L_eta + i * deta for i in range(N)])
    return v, zeta


def grid_1d(N: int, L_v: float):
    """(v, zeta) of the inhomogeneous solver (initializer.c:256-266)."""
    dv = 2 * L_v / (N - 1)
    v = np.array([-L_v + i * dv for i in range(N)])
    L_eta = 0.5 * (N - 1) * np.pi / L_v
    deta = np.pi * (N - 1) / (N * L_v)
    zeta = np.array([-L_eta + i * deta for i in range(N)])
    return v, zeta


def build(force: bool = False) -> str:
    from . import builder as _b
    return _b.build(force=force)


def lib() -> C.CDLL:
    """Load libspectral_gb300.so; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise SpectralError(
            f"{LIB_PATH} is missing: build it with spectralbte_gb300.build() "
            "(there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    i, d, v, p = C.c_int, C.c_double, C.c_void_p, C.c_void_p
    pp = C.POINTER(C.c_void_p)
    sigs = {
        # reference ABI
        "initialize_coll": (None, [i, d, _dp, _dp]),
        "dealloc_coll": (None, []),
        "ComputeQ": (None, [_dp, _dp, _dp, C.POINTER(_dp)]),
        "ComputeQ_maxPreserve": (None, [_dp, _dp, _dp, C.POINTER(_dp)]),
        "fft3D": (None, [_dp, _dp, i]),
        "initialize_conservation": (None, [i, d, _dp, C.POINTER(Species), i]),
        "initialize_conservation_fast": (None, [i, d, _dp]),
        "dealloc_conservation": (None, []),
        "conserveAllMoments": (None, [C.POINTER(_dp)]),
        "solveWithCCt": (None, [i, _dp]),
        "alloc_weights": (None, [i, v, i]),
        "initialize_weights": (None, [i, _dp, d, d, i, i, C.POINTER(_dp), Species, Species]),
        "dealloc_weights": (None, [i, C.POINTER(_dp)]),
        "generate_conv_weights_iso": (None, [C.POINTER(_dp)]),
        "gHat3": (d, [d, d, d, d, d, d]),
        # batched API
        "spectral_last_error": (i, []),
        "spectral_last_error_message": (C.c_char_p, []),
        "spectral_version": (C.c_char_p, []),
        "spectral_kernel_launches": (C.c_longlong, []),
        "spectral_plan_create": (i, [pp, i, d, _dp, _dp, i]),
        "spectral_plan_destroy": (i, [v]),
        "spectral_plan_set_weights": (i, [v, v, i]),
        "spectral_plan_generate_weights_iso": (i, [v, d, d, d, d, d]),
        "spectral_plan_generate_weights_landau": (i, [v, d]),
        "spectral_plan_generate_weights_grazing": (i, [v, d, d]),
        "spectral_plan_generate_weights_closed": (i, [v, d, d, d, d, d, i]),
        "spectral_weights_generator": (i, [i, d, d, d, d]),
        "initialize_weights_AnIso": (None, [i, _dp, d, d, i, C.POINTER(_dp), d]),
        "spectral_plan_get_weights": (i, [v, _dp, C.c_longlong, C.c_longlong]),
        "spectral_plan_set_conservation": (i, [v, d]),
        "spectral_computeQ_device": (i, [v, v, v, i, i, v]),
        "spectral_computeQ_host": (i, [v, _dp, _dp, i, i]),
        "spectral_conserve_device": (i, [v, v, i, v]),
        "spectral_step_device": (i, [v, v, i, d, d, i, i, v]),
        "spectral_plan_set_tuning": (i, [v, i, i, i, i, i]),
        "spectral_plan_autotune": (i, [v, i, i, C.POINTER(C.c_int)]),
        "spectral_plan_set_symmetric": (i, [v, i]),
        "spectral_plan_inject_stall": (i, [v, i, C.c_longlong]),
        "spectral_plan_status": (i, [v, C.POINTER(C.c_uint)]),
        "spectral_plan_sync": (i, [v]),
        "spectral_plan_set_profiling": (i, [v, i]),
        "spectral_1d_setup": (i, [v, i, i, i, d, d, _dp, _dp, d, d, d, d]),
        "spectral_1d_step": (i, [v, v, i, v]),
        "spectral_1d_advect": (i, [v, v, v, v]),
        "spectral_graph_capture": (i, [v, i, v, i, d, d, i, i]),
        "spectral_graph_launch": (i, [v, v]),
        "spectral_group_computeQ": (i, [C.POINTER(C.c_void_p), i, C.POINTER(C.c_void_p),
                                        C.POINTER(C.c_void_p), C.POINTER(C.c_int), i, v]),
        "spectral_plan_conv_time": (i, [v, _dp, C.POINTER(C.c_int)]),
        # learned operator
        "spectral_fno_create": (i, [pp, i, i, i, i, i, i, i, C.c_ulonglong]),
        "spectral_fno_precision": (i, [v]),
        "spectral_fno_set_profiling": (i, [v, i]),
        "spectral_fno_kernel_time": (i, [v, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
        "spectral_fno_destroy": (i, [v]),
        "spectral_fno_num_params": (C.c_longlong, [v]),
        "spectral_fno_num_classes": (i, [v]),
        "spectral_fno_get_params": (i, [v, C.POINTER(C.c_float)]),
        "spectral_fno_set_params": (i, [v, C.POINTER(C.c_float)]),
        "spectral_fno_set_output_scale": (i, [v, C.c_float]),
        "spectral_fno_output_scale": (C.c_float, [v]),
        "spectral_fno_set_loss_floor": (i, [v, C.c_float]),
        "spectral_fno_set_loss_power": (i, [v, C.c_float]),
        "spectral_fno_set_equilibrium": (i, [v, i, _dp]),
        "spectral_fno_set_channel_mix_kernel": (i, [v, i]),
        "spectral_fno_set_readout_kernel": (i, [v, i]),
        "spectral_fno_set_axis_kernel": (i, [v, i]),
        "spectral_fno_status": (i, [v, C.POINTER(C.c_uint)]),
        "spectral_fno_equilibrium": (i, [v]),
        "spectral_plan_set_learned_floor": (i, [v, d]),
        "spectral_fno_predict": (i, [v, v, v, i, v]),
        "spectral_fno_loss_grad": (i, [v, v, v, i, _dp, C.POINTER(C.c_float)]),
        "spectral_fno_train_step": (i, [v, v, v, i, C.c_float, _dp, v]),
        "spectral_plan_set_learned": (i, [v, v, d, i]),
        "spectral_moments_device": (i, [v, v, i, v, v]),
        "spectral_plan_learned_stats": (i, [v, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                            C.POINTER(C.c_longlong), _dp]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def _check(rc: int, what: str):
    if rc != 0:
        msg = lib().spectral_last_error_message().decode(errors="replace")
        raise SpectralError(f"{what} failed ({rc}): {msg}")


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _legacy_check(what: str):
    rc = lib().spectral_last_error()
    if rc != 0:
        msg = lib().spectral_last_error_message().decode(errors="replace")
        raise SpectralError(f"{what}: {msg}")


def declared_symbols(header: str = HEADER) -> list[str]:
    """Function names declared in include/spectral_bte.h."""
    import re
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b([A-Za-z_]\w*)\s*\(", txt, flags=re.M)
    skip = {"if", "defined", "typedef", "struct"}
    return sorted({n for n in names if n not in skip})


# --------------------------------------------------------------------------
class ReferenceAPI:
    """One-for-one mirror of the reference's C entry points.

    Like the reference, the library keeps one collision grid, one set of
    conservation factors and per-table weights as module state.
    """

    def __init__(self):
        self.L = lib()
        self._keep = []
        self._tables = {}

    def reset_error(self):
        # spectral_last_error is sticky; reading it does not clear, so the
        # mirror compares before/after codes through fresh calls only.
        pass

    def initialize_coll(self, N: int, L_v: float, v: np.ndarray, zeta: np.ndarray):
        v = np.ascontiguousarray(v, dtype=np.float64)
        zeta = np.ascontiguousarray(zeta, dtype=np.float64)
        self._keep += [v, zeta]
        self.N, self.n3 = N, N ** 3
        self.L.initialize_coll(N, float(L_v), _p(v), _p(zeta))

    def dealloc_coll(self):
        self.L.dealloc_coll()

    def rows(self, W: np.ndarray):
        """A double** over the rows of a [N^3][N^3] array (kept alive)."""
        W = np.ascontiguousarray(W, dtype=np.float64)
        n3 = W.shape[0]
        ptrs = (_dp * n3)(*[C.cast(W.ctypes.data + 8 * n3 * r, _dp) for r in range(n3)])
        self._tables[C.addressof(ptrs)] = (W, ptrs)
        return ptrs

    def ComputeQ(self, f, g, W_rows) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float64)
        g = f if g is None else np.ascontiguousarray(g, dtype=np.float64)
        Q = np.zeros(self.n3)
        self.L.ComputeQ(_p(f), _p(g), _p(Q), W_rows)
        return Q

    def ComputeQ_maxPreserve(self, f, g, W_rows) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float64)
        g = f if g is None else np.ascontiguousarray(g, dtype=np.float64)
        Q = np.zeros(self.n3)
        self.L.ComputeQ_maxPreserve(_p(f), _p(g), _p(Q), W_rows)
        return Q

    def fft3D(self, x, invert: int) -> np.ndarray:
        a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128)).view(np.float64)
        out = np.zeros_like(a)
        self.L.fft3D(_p(a), _p(out), int(invert))
        return out.view(np.complex128)

    def initialize_conservation(self, N, h_v, v, masses=(1.0,)):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self._keep.append(v)
        sp = (Species * len(masses))(*[Species.default(mass=m) for m in masses])
        self._keep.append(sp)
        self.L.initialize_conservation(N, float(h_v), _p(v), sp, len(masses))

    def conserveAllMoments(self, Qs):
        """Qs: list of Ns*Ns arrays of N^3 (modified copies returned)."""
        arrs = [np.array(q, dtype=np.float64, copy=True) for q in Qs]
        ptrs = (_dp * len(arrs))(*[_p(a) for a in arrs])
        self.L.conserveAllMoments(ptrs)
        return arrs

    def alloc_weights(self, N, total_species=1):
        """weights.c:26-31; returns the double** table of each species pair."""
        out = C.c_void_p()
        self.L.alloc_weights(N, C.byref(out), total_species)
        tbl = C.cast(out, C.POINTER(C.POINTER(_dp)))  # double***
        self._keep.append(out)
        return [tbl[i] for i in range(total_species)]

    def initialize_weights(self, N, zeta, L_v, lam, weightFlag, isoFlag, table,
                           sp_i=None, sp_j=None):
        zeta = np.ascontiguousarray(zeta, dtype=np.float64)
        self._keep.append(zeta)
        sp_i = sp_i or Species.default()
        sp_j = sp_j or Species.default()
        self.L.initialize_weights(N, _p(zeta), float(L_v), float(lam), int(weightFlag),
                                  int(isoFlag), table, sp_i, sp_j)

    def table_to_numpy(self, table, N) -> np.ndarray:
        n3 = N ** 3
        W = np.empty((n3, n3))
        for r in range(n3):
            C.memmove(W[r].ctypes.data, table[r], 8 * n3)
        return W

    def initialize_weights_AnIso(self, N, zeta, L_v, lam, weightFlag, table, glance=0.0):
        """aniso_weights.c:37 (definition argument order)."""
        zeta = np.ascontiguousarray(zeta, dtype=np.float64)
        self._keep.append(zeta)
        self.L.initialize_weights_AnIso(N, _p(zeta), float(L_v), float(lam), int(weightFlag),
                                        table, float(glance))

    def dealloc_weights(self, N, table):
        self.L.dealloc_weights(N, table)


# --------------------------------------------------------------------------
def _ptr(x, itemsize: int = 8) -> int:
    """Device pointer of a torch CUDA tensor, or an int address."""
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise SpectralError("expected a CUDA tensor")
        if not x.is_contiguous() or x.dtype.itemsize != itemsize:
            raise SpectralError(f"expected a contiguous tensor of {itemsize}-byte floats")
        return x.data_ptr()
    raise SpectralError(f"cannot take a device pointer of {type(x)}")


def _stream(stream) -> Optional[int]:
    """The CUDA stream to launch on: the given handle, else torch's current
    stream, so the library's work is ordered with the caller's torch ops.
    None (NULL) is the CUDA default stream, which is torch's default."""
    if stream:
        return int(stream)
    try:
        import torch
        if torch.cuda.is_available():
            return int(torch.cuda.current_stream().cuda_stream) or None
    except Exception:
        pass
    return None


class Plan:
    """Batched device operator for one velocity grid (spectral_plan).

    Device calls run on the caller's stream (torch's current stream unless
    one is given) and are asynchronous like any CUDA launch.
    """

    def __init__(self, N: int, L_v: float, v: np.ndarray, zeta: np.ndarray,
                 max_batch: int = 1):
        self.L = lib()
        self.N, self.n3, self.L_v = N, N ** 3, float(L_v)
        self.v = np.ascontiguousarray(v, dtype=np.float64)
        self.zeta = np.ascontiguousarray(zeta, dtype=np.float64)
        h = C.c_void_p()
        _check(self.L.spectral_plan_create(C.byref(h), N, self.L_v, _p(self.v),
                                           _p(self.zeta), max_batch),
               "spectral_plan_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.spectral_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_weights(self, W):
        if isinstance(W, np.ndarray):
            W = np.ascontiguousarray(W, dtype=np.float64)
            _check(self.L.spectral_plan_set_weights(self.h, W.ctypes.data, 0), "set_weights")
        else:
            _check(self.L.spectral_plan_set_weights(self.h, _ptr(W), 1), "set_weights")

    def generate_weights_iso(self, lam: float, d_i=2.0, d_j=2.0, m_i=1.0, m_j=1.0):
        _check(self.L.spectral_plan_generate_weights_iso(self.h, float(lam), d_i, d_j, m_i, m_j),
               "generate_weights_iso")

    def generate_weights_closed(self, lam: float, fp64_table: bool = True, d_i=2.0, d_j=2.0,
                                m_i=1.0, m_j=1.0):
        """Isotropic weights from the closed-form radial integral (lambda 0, 1);
        fp64_table=False keeps only the row-pair FP32 table (FP32 calls only)."""
        _check(self.L.spectral_plan_generate_weights_closed(self.h, float(lam), d_i, d_j, m_i,
                                                            m_j, 1 if fp64_table else 0),
               "generate_weights_closed")

    def generate_weights_grazing(self, lam: float, glance: float):
        """Grazing-collision weights (gHat3 of the stand-alone generator)."""
        _check(self.L.spectral_plan_generate_weights_grazing(self.h, float(lam), float(glance)),
               "generate_weights_grazing")

    def generate_weights_landau(self, lam: float):
        """Landau-kernel weights (aniso_weights.c:370-425) on the device."""
        _check(self.L.spectral_plan_generate_weights_landau(self.h, float(lam)),
               "generate_weights_landau")

    def get_weights(self, row0: int = 0, nrows: Optional[int] = None) -> np.ndarray:
        nrows = self.n3 - row0 if nrows is None else nrows
        W = np.empty((nrows, self.n3))
        _check(self.L.spectral_plan_get_weights(self.h, _p(W), row0, nrows), "get_weights")
        return W

    def set_conservation(self, mass: float = 1.0):
        _check(self.L.spectral_plan_set_conservation(self.h, float(mass)), "set_conservation")

    def computeQ_device(self, f, Q, B: int, flags: int = FP64, stream: int = 0):
        _check(self.L.spectral_computeQ_device(self.h, _ptr(f), _ptr(Q), B, flags,
                                               _stream(stream)), "computeQ_device")

    def computeQ_host(self, f: np.ndarray, flags: int = FP64) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1, self.n3)
        Q = np.empty_like(f)
        _check(self.L.spectral_computeQ_host(self.h, _p(f), _p(Q), f.shape[0], flags),
               "computeQ_host")
        return Q

    def conserve_device(self, Q, B: int, stream: int = 0):
        _check(self.L.spectral_conserve_device(self.h, _ptr(Q), B, _stream(stream)),
               "conserve_device")

    def step_device(self, f, B: int, dt: float, Kn: float, order: int, flags: int = FP64,
                    stream: int = 0):
        _check(self.L.spectral_step_device(self.h, _ptr(f), B, float(dt), float(Kn), order,
                                           flags, _stream(stream)), "step_device")

    def set_tuning(self, bg: int, stages: int = 0, flush: int = 16, variant: int = 1,
                   zs: int = 0):
        _check(self.L.spectral_plan_set_tuning(self.h, variant, bg, zs, stages, flush),
               "set_tuning")

    def set_symmetric(self, on: bool):
        """Symmetric (row-pair) form of the FP32 convolution, variants 2, 3."""
        _check(self.L.spectral_plan_set_symmetric(self.h, int(bool(on))), "set_symmetric")

    def autotune(self, B: int, flags: int = FP32) -> tuple:
        """(variant, bg, zs, stages, flush) of the fastest FP32 shape."""
        out = (C.c_int * 5)()
        _check(self.L.spectral_plan_autotune(self.h, B, flags, out), "autotune")
        return tuple(out)

    def inject_stall(self, slot: int, limit_clocks: int):
        """Test hook: the next FP32 convolution launch skips the copies of
        pipeline slot `slot` in its first CTA, whose waits give up after
        limit_clocks (spectral_plan_inject_stall)."""
        _check(self.L.spectral_plan_inject_stall(self.h, int(slot), int(limit_clocks)),
               "inject_stall")

    def status(self) -> int:
        s = C.c_uint()
        _check(self.L.spectral_plan_status(self.h, C.byref(s)), "status")
        return s.value

    def sync(self):
        _check(self.L.spectral_plan_sync(self.h), "sync")

    def setup_1d(self, nX: int, order: int, ic: int, dt: float, Kn: float, x, dx,
                 T0: float = 1.0, T1: float = 2.0, TWall: float = 1.0, mass: float = 1.0):
        """1D-3V solver state: nX cells + 2*order ghosts (see spectral_1d_setup)."""
        self._x = np.ascontiguousarray(x, dtype=np.float64)
        self._dx = np.ascontiguousarray(dx, dtype=np.float64)
        _check(self.L.spectral_1d_setup(self.h, nX, order, ic, float(dt), float(Kn),
                                        _p(self._x), _p(self._dx), T0, T1, TWall, mass),
               "spectral_1d_setup")

    def step_1d(self, f, flags: int = FP64, stream: int = 0):
        _check(self.L.spectral_1d_step(self.h, _ptr(f), flags, _stream(stream)), "spectral_1d_step")

    def advect_1d(self, f, fconv, stream: int = 0):
        _check(self.L.spectral_1d_advect(self.h, _ptr(f), _ptr(fconv), _stream(stream)),
               "spectral_1d_advect")

    def capture(self, kind: int, f, B: int = 0, dt: float = 0.0, Kn: float = 1.0,
                order: int = 1, flags: int = FP64):
        """Capture one time step (kind 0: 0D step, 1: 1D step) as a CUDA graph."""
        _check(self.L.spectral_graph_capture(self.h, kind, _ptr(f), B, float(dt), float(Kn),
                                             order, flags), "spectral_graph_capture")

    def launch(self, stream: int = 0):
        _check(self.L.spectral_graph_launch(self.h, _stream(stream)), "spectral_graph_launch")

    def moments_device(self, f, B: int, out, stream: int = 0):
        """out[B][8] = rho, u_x, u_y, u_z, T, rho T, E+, E- of each instance."""
        _check(self.L.spectral_moments_device(self.h, _ptr(f), B, _ptr(out), _stream(stream)),
               "moments_device")

    def set_learned(self, net: Optional["FourierOperator"], tol: float = 1e-3,
                    check_every: int = 1):
        """Use net for computeQ with LEARNED, spot-checked against the plain
        FP32 operator every check_every calls (spectral_plan_set_learned)."""
        self._net = net
        _check(self.L.spectral_plan_set_learned(self.h, net.h if net else None, float(tol),
                                                int(check_every)), "set_learned")

    def set_learned_floor(self, eps: float):
        """Floor of the spot check's relative distance (spectral_plan_set_learned_floor)."""
        _check(self.L.spectral_plan_set_learned_floor(self.h, float(eps)), "set_learned_floor")

    def learned_stats(self) -> dict:
        c, k, fb = C.c_longlong(), C.c_longlong(), C.c_longlong()
        e = C.c_double()
        _check(self.L.spectral_plan_learned_stats(self.h, C.byref(c), C.byref(k), C.byref(fb),
                                                  C.byref(e)), "learned_stats")
        return {"calls": c.value, "checks": k.value, "fallbacks": fb.value,
                "last_err": e.value}

    def set_profiling(self, on: bool):
        _check(self.L.spectral_plan_set_profiling(self.h, 1 if on else 0), "set_profiling")

    def conv_time(self) -> tuple:
        """(summed convolution-kernel ms, launches) since the last query."""
        ms = C.c_double()
        n = C.c_int()
        _check(self.L.spectral_plan_conv_time(self.h, C.byref(ms), C.byref(n)), "conv_time")
        return ms.value, n.value


class FourierOperator:
    """The learned collision operator (spectral_fno): a Fourier neural
    operator on the lowest modes^3 Fourier modes, BF16 tensor-core GEMMs with
    FP32 accumulation, trained on the device by the library's own forward
    and backward kernels."""

    def __init__(self, N: int, width: int = 64, modes: int = 12, layers: int = 4,
                 hidden: int = 128, seed: int = 1, kind: int = 0, precision: int = 1):
        self.L = lib()
        self.N, self.n3 = N, N ** 3
        self.width, self.modes, self.layers, self.hidden = width, modes, layers, hidden
        self.kind, self.precision = kind, precision
        h = C.c_void_p()
        _check(self.L.spectral_fno_create(C.byref(h), N, width, modes, layers, hidden, kind,
                                          precision, int(seed)), "spectral_fno_create")
        self.h = h
        self.nparams = int(self.L.spectral_fno_num_params(h))
        self.nclasses = int(self.L.spectral_fno_num_classes(h))

    def close(self):
        if getattr(self, "h", None):
            self.L.spectral_fno_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.empty(self.nparams, dtype=np.float32)
        _check(self.L.spectral_fno_get_params(self.h, out.ctypes.data_as(C.POINTER(C.c_float))),
               "fno_get_params")
        return out

    def set_params(self, theta: np.ndarray):
        theta = np.ascontiguousarray(theta, dtype=np.float32)
        if theta.size != self.nparams:
            raise SpectralError(f"expected {self.nparams} parameters, got {theta.size}")
        _check(self.L.spectral_fno_set_params(self.h, theta.ctypes.data_as(C.POINTER(C.c_float))),
               "fno_set_params")

    @property
    def output_scale(self) -> float:
        return float(self.L.spectral_fno_output_scale(self.h))

    @output_scale.setter
    def output_scale(self, sigma: float):
        _check(self.L.spectral_fno_set_output_scale(self.h, float(sigma)), "fno_set_output_scale")

    def set_channel_mix_kernel(self, mode):
        """Inference channel mix: 1 (default), 2, 3 = shapes of the TMA
        warp-specialised kernel; 0 (or False) = the general GEMM."""
        _check(self.L.spectral_fno_set_channel_mix_kernel(self.h, int(mode)),
               "fno_set_channel_mix_kernel")

    def set_axis_kernel(self, tma: bool):
        """1: the TMA warp-specialised axis-k transforms in inference (default); 0: gemm_sa."""
        _check(self.L.spectral_fno_set_axis_kernel(self.h, 1 if tma else 0),
               "fno_set_axis_kernel")

    def set_readout_kernel(self, tma: bool):
        """1: the TMA warp-specialised readout in inference (default); 0: the general GEMM."""
        _check(self.L.spectral_fno_set_readout_kernel(self.h, 1 if tma else 0),
               "fno_set_readout_kernel")

    def status(self) -> int:
        s = C.c_uint()
        _check(self.L.spectral_fno_status(self.h, C.byref(s)), "fno_status")
        return s.value


    def set_profiling(self, on: bool):
        """Time every channel-mix launch with CUDA events on its stream."""
        _check(self.L.spectral_fno_set_profiling(self.h, 1 if on else 0), "fno_set_profiling")

    def kernel_time(self) -> tuple:
        """(total ms, launches) of the channel-mix launches timed so far."""
        ms, n = C.c_double(), C.c_int()
        _check(self.L.spectral_fno_kernel_time(self.h, C.byref(ms), C.byref(n)),
               "fno_kernel_time")
        return ms.value, n.value

    def set_loss_floor(self, eps: float):
        _check(self.L.spectral_fno_set_loss_floor(self.h, float(eps)), "fno_set_loss_floor")

    def set_loss_power(self, k: float):
        """Training loss mean_b e_b^k (spectral_fno_set_loss_power); k > 1
        weights the worst instances of each batch up."""
        _check(self.L.spectral_fno_set_loss_power(self.h, float(k)), "fno_set_loss_power")

    def set_equilibrium(self, on: bool, v=None):
        """Equilibrium-exact form Q(f) = P(f) - P(M_f) (spectral_fno_set_equilibrium);
        v: the N velocity nodes of the grid."""
        vv = None
        if on:
            vv = np.ascontiguousarray(v, dtype=np.float64)
            if vv.size != self.N:
                raise SpectralError(f"expected {self.N} velocity nodes, got {vv.size}")
            self._v = vv
        _check(self.L.spectral_fno_set_equilibrium(self.h, 1 if on else 0,
                                                   _p(vv) if on else None),
               "fno_set_equilibrium")

    @property
    def equilibrium(self) -> bool:
        return bool(self.L.spectral_fno_equilibrium(self.h) == 1)

    def predict(self, f, Q, B: int, stream: int = 0):
        """Network output (FP64 device) for f (FP64 device), no projection."""
        _check(self.L.spectral_fno_predict(self.h, _ptr(f), _ptr(Q), B, _stream(stream)),
               "fno_predict")

    def loss_grad(self, f32, Q32, B: int):
        """(loss, gradient) for FP32 device data; the gradient is a host array."""
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_double()
        _check(self.L.spectral_fno_loss_grad(self.h, _ptr(f32, 4), _ptr(Q32, 4), B,
                                             C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_float))),
               "fno_loss_grad")
        return loss.value, g

    def train_step(self, f32, Q32, B: int, lr: float, want_loss: bool = False,
                   stream: int = 0):
        loss = C.c_double()
        _check(self.L.spectral_fno_train_step(self.h, _ptr(f32, 4), _ptr(Q32, 4), B, float(lr),
                                              C.byref(loss) if want_loss else None,
                                              _stream(stream)), "fno_train_step")
        return loss.value if want_loss else None

    def save(self, path: str):
        extra = {}
        if self.equilibrium:
            extra["v"] = self._v
        np.savez(path, theta=self.get_params(), sigma=self.output_scale,
                 shape=np.array([self.N, self.width, self.modes, self.layers, self.hidden,
                                 self.kind, self.precision]),
                 equilibrium=np.array(int(self.equilibrium)), **extra)

    @classmethod
    def load(cls, path: str) -> "FourierOperator":
        d = np.load(path)
        shape = [int(x) for x in d["shape"]]
        N, width, modes, layers, hidden, kind = shape[:6]
        precision = shape[6] if len(shape) > 6 else 0   # BF16 before the precision field
        net = cls(N, width, modes, layers, hidden, kind=kind, precision=precision)
        net.set_params(d["theta"])
        net.output_scale = float(d["sigma"])
        if "equilibrium" in d.files and int(d["equilibrium"]) == 1:
            net.set_equilibrium(True, d["v"])
        return net


def group_computeQ(plans, fs, Qs, flags: int = FP32 | CONSERVE, stream: int = 0):
    """Q for several plans at once (spectral_group_computeQ); fs[i], Qs[i]
    are [B_i][N_i^3] device tensors of plan i."""
    n = len(plans)
    ph = (C.c_void_p * n)(*[p.h.value for p in plans])
    fp = (C.c_void_p * n)(*[_ptr(f) for f in fs])
    qp = (C.c_void_p * n)(*[_ptr(q) for q in Qs])
    bs = (C.c_int * n)(*[int(f.shape[0]) for f in fs])
    _check(lib().spectral_group_computeQ(ph, n, fp, qp, bs, flags, _stream(stream)),
           "spectral_group_computeQ")


def fp32_fma_rate() -> float:
    """Sustained FP32 FMA rate of the current GPU in TFLOP/s, measured by the
    benchmark's calibration library (libspectral_calib.so, a probe kernel of
    independent register FMA chains); the collision library does not
    contain it."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libspectral_calib.so")
    if not os.path.exists(path):
        raise SpectralError(f"calibration library missing: {path} (run the build)")
    cal = C.CDLL(path)
    cal.spectral_calib_fp32_fma_rate.restype = C.c_int
    cal.spectral_calib_fp32_fma_rate.argtypes = [_dp, C.c_void_p]
    out = C.c_double()
    rc = cal.spectral_calib_fp32_fma_rate(C.byref(out), _stream(0))
    if rc != 0:
        raise SpectralError(f"spectral_calib_fp32_fma_rate: CUDA error {rc}")
    return out.value


def kernel_launches() -> int:
    return int(lib().spectral_kernel_launches())
