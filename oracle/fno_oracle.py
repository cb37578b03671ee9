"""CPU restatement of the learned collision operator in FP64 numpy:
forward pass, loss and hand-derived gradients.

TEST INFRASTRUCTURE, NOT PRODUCT.  Only tests/ and bench.py import this
module, to check the GPU network (spectralbte_gb300/csrc/fno.cu) and its
gradients.  The network has no counterpart in the reference, so this file
is its oracle: the algorithm is restated here from its definition, and the
gradients are checked against central finite differences by the CPU tests.

With ``rounding=True`` every tensor that the GPU stores in BF16 between two
GEMMs (and every GEMM's small operand) is rounded to BF16 at the same place,
so the GPU and the oracle then differ only by FP32 accumulation order.
Shapes follow the GPU code: f is (B, N, N, N); activations (B, N, N, N, C);
the Fourier modes m in [-Km/2, Km/2) per axis sit at index m + Km/2.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
from scipy.special import erf

SQRT_HALF = 0.70710678118654752
INV_SQRT_2PI = 0.39894228040143268


def bf16(x):
    """Round to the nearest BF16 (ties to even) through float32; returns float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def cbf16(z):
    return bf16(z.real) + 1j * bf16(z.imag)


def fp16(x):
    """Round to the nearest IEEE half (ties to even, subnormals kept); returns float64."""
    return np.asarray(np.asarray(x, dtype=np.float32), dtype=np.float16).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x * SQRT_HALF))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x * SQRT_HALF)) + x * INV_SQRT_2PI * np.exp(-0.5 * x * x)


@dataclass
class Spec:
    N: int
    C: int
    Km: int
    L: int
    Hd: int
    kind: int = 0  # 0: GELU layers and readout; 1: linear layers, bilinear readout

    def pairs(self):
        """Left and right rows of each readout pair (kind 1): 16 (e/8) + e%8 and +8."""
        e = np.arange(self.Hd // 2)
        left = 16 * (e // 8) + e % 8
        return left, left + 8

    def classes(self):
        """Class index of each mode (a, b, c) by |m|^2, in increasing order."""
        m = np.arange(self.Km) - self.Km // 2
        r2 = m[:, None, None] ** 2 + m[None, :, None] ** 2 + m[None, None, :] ** 2
        vals = np.unique(r2)
        return np.searchsorted(vals, r2), len(vals)

    def layout(self):
        """Offsets of the flat parameter vector (the order of spectral_fno_get_params)."""
        C, Hd = self.C, self.Hd
        _, nc = self.classes()
        off, o = {}, 0

        def put(name, n):
            nonlocal o
            off[name] = (o, n)
            o += n
        put("P", C)
        put("bP", C)
        for l in range(self.L):
            put(f"W{l}", C * C)
            put(f"b{l}", C)
            put(f"R{l}", nc * C * C)
        put("Q1", Hd * C)
        put("c1", Hd)
        put("q2", Hd // 2 if self.kind == 1 else Hd)
        put("c2", 1)
        return off, o


def unpack(spec: Spec, theta: np.ndarray) -> dict:
    off, n = spec.layout()
    assert theta.size == n, (theta.size, n)
    _, nc = spec.classes()
    C, Hd = spec.C, spec.Hd
    nq = Hd // 2 if spec.kind == 1 else Hd
    shapes = {"P": (C,), "bP": (C,), "Q1": (Hd, C), "c1": (Hd,), "q2": (nq,), "c2": (1,)}
    for l in range(spec.L):
        shapes[f"W{l}"] = (C, C)
        shapes[f"b{l}"] = (C,)
        shapes[f"R{l}"] = (nc, C, C)
    return {k: np.asarray(theta[o:o + n], dtype=np.float64).reshape(shapes[k])
            for k, (o, n) in off.items()}


def pack(spec: Spec, d: dict) -> np.ndarray:
    off, n = spec.layout()
    out = np.zeros(n)
    for k, (o, m) in off.items():
        out[o:o + m] = d[k].reshape(-1)
    return out


def dft_mats(N: int, Km: int, scaled: bool = True):
    """F[m][n] = e^{-2 pi i m n / N} / N (without the 1/N when not scaled)
    and G[n][m] = e^{+2 pi i m n / N}, m = index - Km/2, with cos and sin
    rounded to float32 as the GPU holds them."""
    m = np.arange(Km) - Km // 2
    n = np.arange(N)
    r = np.mod(np.outer(m, n), N)
    th = 2.0 * np.pi * r / N
    c = np.float32(np.cos(th)).astype(np.float64)
    s = np.float32(np.sin(th)).astype(np.float64)
    d = N if scaled else 1
    cN = np.float32(np.cos(th) / d).astype(np.float64)
    sN = np.float32(np.sin(th) / d).astype(np.float64)
    F = cN - 1j * sN
    G = (c + 1j * s).T
    return F, G


class Net:
    """The network of fno.cu with parameters theta (flat, FP64 copy)."""

    def __init__(self, spec: Spec, theta: np.ndarray, sigma: float = 1.0,
                 rounding: bool = False, precision: int = 0):
        """precision 0: BF16 elements, 1: FP16 elements (the device's
        spectral_fno_create precision); used when rounding is on."""
        self.spec, self.sigma, self.rnd = spec, float(sigma), rounding
        self.q = fp16 if precision == 1 else bf16
        self.p = unpack(spec, theta)
        self.cls, self.ncls = spec.classes()
        F, G = dft_mats(spec.N, spec.Km)
        Fu, _ = dft_mats(spec.N, spec.Km, scaled=False)
        self.F, self.G, self.Fu = (self.rc(M) if rounding else M for M in (F, G, Fu))

    # rounding helpers
    def r(self, x):
        return self.q(x) if self.rnd else x

    def rc(self, z):
        return (self.q(z.real) + 1j * self.q(z.imag)) if self.rnd else z

    def mat(self, a):
        return self.q(a) if self.rnd else a

    # truncated transforms, axis by axis in the GPU's order (k, j, i).  The
    # backward pass keeps the 1/N of the first axis only (N^2 F3 h).
    def fwd_modes(self, h, bwd: bool = False):
        F, F23 = self.F, (self.Fu if bwd else self.F)
        t1 = self.rc(np.einsum("ak,bijkc->bijac", F, h))
        t2 = self.rc(np.einsum("aj,bijkc->biakc", F23, t1))
        return self.rc(np.einsum("ai,bijkc->bajkc", F23, t2))

    def inv_modes(self, y):
        """Real part of the inverse transform (FP64; the forward pass stores it as BF16)."""
        G = self.G
        u1 = self.rc(np.einsum("ia,bajkc->bijkc", G, y))
        u2 = self.rc(np.einsum("ja,biakc->bijkc", G, u1))
        return np.einsum("ka,bijac->bijkc", G, u2).real

    def mix(self, R, X, transpose=False):
        Rm = self.mat(R)[self.cls]  # (Km, Km, Km, C, C) = R[cls][d][c]
        eq = "xyzcd,bxyzc->bxyzd" if transpose else "xyzdc,bxyzc->bxyzd"
        out = np.einsum(eq, Rm, X.real) + 1j * np.einsum(eq, Rm, X.imag)
        return self.rc(out)

    def forward(self, f: np.ndarray):
        """y (B, N, N, N) and the cache for backward."""
        p, sp = self.p, self.spec
        f = np.asarray(f, dtype=np.float64).reshape(-1, sp.N, sp.N, sp.N)
        s = np.float32(f.reshape(f.shape[0], -1).max(axis=1)).astype(np.float64)
        s = np.where(s > 0, s, 1.0)
        x = f / s[:, None, None, None]
        h = self.r(p["P"] * x[..., None] + p["bP"])
        cache = {"x": x, "s": s, "h": [h], "z": [], "X": []}
        for l in range(sp.L):
            X = self.fwd_modes(h)
            Y = self.mix(p[f"R{l}"], X)
            S = self.r(self.inv_modes(Y))   # stored as BF16 on the device
            z = np.einsum("dc,bijkc->bijkd", self.mat(p[f"W{l}"]), h) + p[f"b{l}"] + S
            h = self.r(gelu(z) if (sp.kind == 0 and l < sp.L - 1) else z)
            cache["X"].append(X)
            cache["z"].append(z)
            cache["h"].append(h)
        u = np.einsum("ec,bijkc->bijke", self.mat(p["Q1"]), h) + p["c1"]
        if sp.kind == 1:
            lft, rgt = sp.pairs()
            y = (u[..., lft] * u[..., rgt]) @ p["q2"] + p["c2"][0]
        else:
            y = gelu(u) @ p["q2"] + p["c2"][0]
        cache["u"] = u
        return y, cache

    def predict(self, f):
        y, c = self.forward(f)
        return y * (c["s"] ** 2 * self.sigma)[:, None, None, None]

    def predict_eq(self, f, M):
        """Equilibrium-exact form: predict(f) - predict(M), M the Maxwellian
        of each f (fno.cu header)."""
        return self.predict(f) - self.predict(M)

    def loss_grad(self, f, Q, floor: float = 0.0, M=None, power: float = 1.0):
        """Mean over instances of e_b = |y - t|^2/(|t|^2 + floor mean_b |t_b|^2),
        t = Q / (s^2 sigma), and its gradient as a dict of arrays shaped like
        the parameters.  With M (the Maxwellian of each f) the equilibrium-
        exact form: y is replaced by y(f) - (s_M / s_f)^2 y(M), both halves
        run as one batch [f; M], and the M half receives the output gradient
        times -(s_M / s_f)^2.  With power k > 1 (plain form only) the loss is
        mean_b e_b^k, which weights each instance's gradient by
        w_b = k e_b^(k-1): the worst instances count for more.  As on the
        device, the returned gradient is that of the loss divided by mean_b
        w_b, the plain loss's gradient scale."""
        p, sp = self.p, self.spec
        B = f.shape[0]
        if M is None:
            y, c = self.forward(f)
            sf = c["s"]
        else:
            f = np.asarray(f, dtype=np.float64).reshape(B, sp.N, sp.N, sp.N)
            M = np.asarray(M, dtype=np.float64).reshape(B, sp.N, sp.N, sp.N)
            y2, c = self.forward(np.concatenate([f, M]))
            sf, sM = c["s"][:B], c["s"][B:]
            rho = (sM / sf) ** 2
            y = y2[:B] - rho[:, None, None, None] * y2[B:]
        t = np.asarray(Q, dtype=np.float64).reshape(y.shape) / \
            (sf ** 2 * self.sigma)[:, None, None, None]
        den = (t.reshape(B, -1) ** 2).sum(axis=1)
        den = den + floor * den.mean()
        r = y - t
        e = (r.reshape(B, -1) ** 2).sum(axis=1) / den
        # the device carries gradients times the loss scale gs = B mean(den) / 2
        gs = 0.5 * den.sum()
        if power == 1.0:
            loss = float(e.sum() / B)
            w = np.ones(B)
        else:
            if M is not None:
                raise ValueError("the power loss is for the plain form")
            loss = float((e ** power).sum() / B)
            w = power * e ** (power - 1.0)
            w = w / w.mean()
        dy = 2.0 * r / (den * B)[:, None, None, None] * (w * gs)[:, None, None, None]
        if M is not None:
            dy = np.concatenate([dy, -rho[:, None, None, None] * dy])
        return loss, self._backward(c, dy, gs)

    def _backward(self, c, dy, gs):
        """Parameter gradients (divided by the loss scale gs) of the cached
        forward pass c for the output gradient dy."""
        p, sp = self.p, self.spec
        g = {k: np.zeros_like(v) for k, v in p.items()}
        g["c2"][0] = dy.sum()
        u = c["u"]
        if sp.kind == 1:
            lft, rgt = sp.pairs()
            g["q2"] = np.einsum("bijk,bijke->e", dy, u[..., lft] * u[..., rgt])
            du = np.zeros_like(u)
            du[..., lft] = dy[..., None] * p["q2"] * u[..., rgt]
            du[..., rgt] = dy[..., None] * p["q2"] * u[..., lft]
        else:
            g["q2"] = np.einsum("bijk,bijke->e", dy, gelu(u))
            du = dy[..., None] * p["q2"] * gelu_grad(u)
        g["c1"] = du.sum(axis=(0, 1, 2, 3))
        du = self.r(du)
        hL = c["h"][sp.L]
        g["Q1"] = np.einsum("bijke,bijkc->ec", du, hL)
        dh = np.einsum("ec,bijke->bijkc", self.mat(p["Q1"]), du)
        for l in range(sp.L - 1, -1, -1):
            dz = dh * gelu_grad(c["z"][l]) if (sp.kind == 0 and l < sp.L - 1) else dh
            g[f"b{l}"] = dz.sum(axis=(0, 1, 2, 3))
            dz = self.r(dz)
            hl = c["h"][l]
            g[f"W{l}"] = np.einsum("bijkd,bijkc->dc", dz, hl)
            dh = np.einsum("dc,bijkd->bijkc", self.mat(p[f"W{l}"]), dz)
            # spectral path: GY = N^2 F3 dz (the backward transform keeps
            # one 1/N); the complex gradient of Y is N^3 F3 dz, so
            # dR = N sum Re(GY conj X), and dh += Re(G3 R^T GY) / N^2
            GY = self.fwd_modes(dz, bwd=True)
            X = c["X"][l]
            per_mode = np.einsum("bxyzd,bxyzc->xyzdc", GY.real, X.real) + \
                np.einsum("bxyzd,bxyzc->xyzdc", GY.imag, X.imag)
            dR = np.zeros_like(p[f"R{l}"])
            np.add.at(dR, self.cls, per_mode)
            g[f"R{l}"] = sp.N * dR
            GX = self.mix(p[f"R{l}"], GY, transpose=True)
            dh = dh + self.inv_modes(GX) / (sp.N * sp.N)
        x = c["x"]
        g["P"] = np.einsum("bijkc,bijk->c", dh, x)
        g["bP"] = dh.sum(axis=(0, 1, 2, 3))
        return {k: val / gs for k, val in g.items()}


def maxwellian_of(f: np.ndarray, v: np.ndarray) -> np.ndarray:
    """The Maxwellian with the density, bulk velocity and temperature of each
    f (B, N^3), with unit mass and Boltzmann constant and the trapezoid
    weights of momentRoutines.c:58-185 (getDensity, getBulkVelocity,
    getTemperature), as the device builds it for the equilibrium form."""
    v = np.asarray(v, dtype=np.float64)
    N = v.size
    f = np.asarray(f, dtype=np.float64).reshape(-1, N, N, N)
    wt = np.ones(N)
    wt[0] = wt[-1] = 0.5
    dv = v[1] - v[0]
    w = wt[:, None, None] * wt[None, :, None] * wt[None, None, :] * dv ** 3
    vx, vy, vz = v[:, None, None], v[None, :, None], v[None, None, :]
    out = np.empty_like(f)
    for b in range(f.shape[0]):
        fb = f[b]
        rho = (w * fb).sum()
        u = [(w * vx * fb).sum() / rho, (w * vy * fb).sum() / rho, (w * vz * fb).sum() / rho]
        d2 = (vx - u[0]) ** 2 + (vy - u[1]) ** 2 + (vz - u[2]) ** 2
        T = (w * d2 * fb).sum() / (3.0 * rho)
        out[b] = rho * (0.5 / (np.pi * T)) ** 1.5 * np.exp(-(0.5 / T) * d2)
    return out.reshape(f.shape[0], -1)
