"""CPU checks of the learned operator's oracle (oracle/fno_oracle.py).

* Its hand-derived gradients equal central finite differences of its own
  loss, FP64, every parameter of a small network.
* With every mode kept, the truncated transform pair is the identity, so the
  spectral layer with R = identity returns its input.
* BF16 rounding is round-to-nearest-even on known values.
* The parameter layout matches the library's count for the same shape.
"""
import numpy as np
import pytest

from oracle import fno_oracle as fo


def _small(rounding=False, seed=0, spec=None):
    spec = spec or fo.Spec(N=4, C=3, Km=2, L=2, Hd=4)
    _, n = spec.layout()
    rng = np.random.default_rng(seed)
    theta = rng.uniform(-0.6, 0.6, n)
    return spec, theta, fo.Net(spec, theta, sigma=0.7, rounding=rounding)


def _data(spec, B, seed):
    rng = np.random.default_rng(seed)
    N = spec.N
    f = rng.uniform(0.1, 1.0, (B, N, N, N))
    Q = rng.normal(size=(B, N, N, N))
    return f, Q


def test_gradients_match_finite_differences():
    spec, theta, net = _small()
    f, Q = _data(spec, 2, 1)
    loss, g = net.loss_grad(f, Q)
    ga = fo.pack(spec, g)
    eps = 1e-6
    gn = np.empty_like(theta)
    for i in range(theta.size):
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        lp, _ = fo.Net(spec, tp, sigma=0.7).loss_grad(f, Q)
        lm, _ = fo.Net(spec, tm, sigma=0.7).loss_grad(f, Q)
        gn[i] = (lp - lm) / (2 * eps)
    assert loss > 0
    err = np.abs(ga - gn).max() / np.abs(gn).max()
    assert err < 1e-6, err


def test_gradients_with_odd_modes_and_three_layers():
    spec = fo.Spec(N=6, C=2, Km=4, L=3, Hd=3)
    spec, theta, net = _small(spec=spec, seed=3)
    f, Q = _data(spec, 1, 2)
    _, g = net.loss_grad(f, Q)
    ga = fo.pack(spec, g)
    rng = np.random.default_rng(5)
    eps = 1e-6
    for i in rng.choice(theta.size, 40, replace=False):
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        lp, _ = fo.Net(spec, tp, sigma=0.7).loss_grad(f, Q)
        lm, _ = fo.Net(spec, tm, sigma=0.7).loss_grad(f, Q)
        gn = (lp - lm) / (2 * eps)
        assert abs(ga[i] - gn) <= 1e-6 * max(1.0, abs(gn)), (i, ga[i], gn)


def test_bilinear_gradients_and_homogeneity():
    spec = fo.Spec(N=4, C=3, Km=2, L=2, Hd=16, kind=1)
    spec, theta, net = _small(spec=spec, seed=7)
    f, Q = _data(spec, 2, 3)
    _, g = net.loss_grad(f, Q, floor=0.2)
    ga = fo.pack(spec, g)
    eps = 1e-6
    for i in range(theta.size):
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        lp, _ = fo.Net(spec, tp, sigma=0.7).loss_grad(f, Q, floor=0.2)
        lm, _ = fo.Net(spec, tm, sigma=0.7).loss_grad(f, Q, floor=0.2)
        gn = (lp - lm) / (2 * eps)
        assert abs(ga[i] - gn) <= 1e-6 * max(1.0, abs(gn)), (i, ga[i], gn)
    # with zero biases the kind-1 network is a quadratic form in f
    d = fo.unpack(spec, theta)
    for k in d:
        if k in ("bP", "c1", "c2") or k.startswith("b"):
            d[k][:] = 0.0
    q = fo.Net(spec, fo.pack(spec, d), sigma=0.7)
    y1, c1 = q.forward(f)
    y2, c2 = q.forward(3.0 * f)
    assert np.allclose(y1, y2)  # the input is scaled by its maximum
    assert np.allclose(q.predict(3.0 * f), 9.0 * q.predict(f))


def test_full_mode_transform_pair_is_identity():
    spec = fo.Spec(N=6, C=2, Km=6, L=1, Hd=2)
    _, n = spec.layout()
    net = fo.Net(spec, np.zeros(n))
    h = np.random.default_rng(0).normal(size=(2, 6, 6, 6, 2))
    back = net.inv_modes(net.fwd_modes(h))
    assert np.abs(back - h).max() < 1e-6  # the matrices hold float32 cos/sin


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 0.0])
    y = fo.bf16(x)
    assert y[0] == 1.0
    assert y[1] == 1.0          # tie -> even mantissa
    assert y[2] == 1.0078125    # above the tie
    assert abs(y[3] + 3.0e-3) <= 3.0e-3 * 2 ** -8
    assert y[4] == 0.0


def test_layout_matches_library_count(lib_built):
    import spectralbte_gb300 as sb
    spec = fo.Spec(N=32, C=64, Km=12, L=4, Hd=128)
    _, n = spec.layout()
    cls, ncls = spec.classes()
    # the count the library computes for the same shape (no GPU needed)
    C, Hd, L = 64, 128, 4
    want = 2 * C + L * (C * C + C + ncls * C * C) + Hd * C + 2 * Hd + 1
    assert n == want
    _, n1 = fo.Spec(N=32, C=64, Km=12, L=4, Hd=128, kind=1).layout()
    assert n1 == want - Hd // 2
    assert cls.shape == (12, 12, 12) and cls.max() == ncls - 1
    assert "spectral_fno_create" in sb.declared_symbols()


def test_gelu_erf_approximation_bound():
    """The device GELU's erf (Abramowitz and Stegun 7.1.26, fno_gemm.cuh
    erf_as), evaluated in float32 with the same constants, stays within
    1e-6 of the exact erf on [-12, 12]."""
    import re
    from scipy.special import erf
    src = open(__import__("os").path.join(__import__("os").path.dirname(__file__), "..",
                                          "spectralbte_gb300", "csrc", "fno_gemm.cuh")).read()
    body = src[src.index("float erf_as("):src.index("float gelu_f(")]
    consts = [float(c[:-1]) for c in re.findall(r"-?\d+\.\d+f", body)]
    p, a5, a4, a3, a2, a1 = consts[0], consts[2], consts[3], consts[4], consts[5], consts[6]
    f32 = np.float32
    x = np.linspace(-12, 12, 400001).astype(f32)
    ax = np.abs(x)
    t = (f32(1) / (f32(p) * ax + f32(1))).astype(f32)
    poly = ((((f32(a5) * t + f32(a4)) * t + f32(a3)) * t + f32(a2)) * t + f32(a1)) * t
    r = np.copysign((f32(1) - poly * np.exp(-(ax * ax)).astype(f32)).astype(f32), x)
    assert np.abs(r - erf(x.astype(np.float64))).max() < 1e-6


def test_gelu_forward_approximation_bound():
    """The device forward GELU (fno_gemm.cuh gelu_f / gelu2_f: the erfc form
    of the same rational approximation, max(z, 0) - |z| erfc(|z|/sqrt 2)/2,
    with halved coefficients), evaluated in float32 with the constants parsed
    from the source, against the exact z Phi(z) on [-12, 12]: within
    2.5e-7 max(1, |z|).  (The device takes the reciprocal and 2^x from the
    PTX approximations, about 1 ulp each; numpy rounds them exactly.)"""
    import os
    import re
    from scipy.special import erf
    src = open(os.path.join(os.path.dirname(__file__), "..", "spectralbte_gb300", "csrc",
                            "fno_gemm.cuh")).read()
    body = src[src.index("namespace gelu_c {"):src.index("}  // namespace gelu_c")]
    c = {k: float(v) for k, v in re.findall(r"(k\w+) = (-?[\d.]+)f", body)}
    h = [float(v) for v in re.findall(r"kH\d = 0\.5f \* (-?[\d.]+)f", body)]
    assert len(h) == 5 and {"kInvSqrt2", "kP", "kNegLog2e"} <= set(c)
    f32 = np.float32
    H = [f32(0.5) * f32(x) for x in h]
    z = np.linspace(-12, 12, 400001).astype(f32)
    a = np.abs(z)
    u = (a * f32(c["kInvSqrt2"])).astype(f32)
    t = (f32(1) / (u * f32(c["kP"]) + f32(1))).astype(f32)
    p = H[4] * t + H[3]
    for k in (2, 1, 0):
        p = (p * t + H[k]).astype(f32)
    p = (p * t).astype(f32)
    e = np.exp2((u * (u * f32(c["kNegLog2e"]))).astype(f32)).astype(f32)
    g = (np.maximum(z, f32(0)) - a * (p * e)).astype(f32)
    z64 = z.astype(np.float64)
    exact = 0.5 * z64 * (1.0 + erf(z64 / np.sqrt(2.0)))
    assert (np.abs(g - exact) / np.maximum(1.0, np.abs(z64))).max() < 2.5e-7


@pytest.mark.parametrize("power", [2.0, 3.0])
def test_power_loss_gradients_match_finite_differences(power):
    """mean_b e_b^k (k > 1 weights the worst instances up) against central
    finite differences of itself, every parameter, with the loss floor.  The
    oracle returns the gradient divided by the batch mean of the instance
    weights k e_b^(k-1), as the device does."""
    spec, theta, net = _small(seed=5)
    f, Q = _data(spec, 3, 6)
    loss, g = net.loss_grad(f, Q, floor=0.1, power=power)
    l1, _ = net.loss_grad(f, Q, floor=0.1)
    assert loss > 0 and abs(loss - l1) > 1e-6 * l1   # not the plain loss
    # the instance errors e_b and weights of the same batch
    y, c = net.forward(f)
    t = Q.reshape(3, -1) / (c["s"] ** 2 * 0.7)[:, None]
    den = (t ** 2).sum(axis=1)
    den = den + 0.1 * den.mean()
    eb = ((y.reshape(3, -1) - t) ** 2).sum(axis=1) / den
    mean_w = (power * eb ** (power - 1.0)).mean()
    ga = fo.pack(spec, g) * mean_w
    eps = 1e-6
    gn = np.empty_like(theta)
    for i in range(theta.size):
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        lp, _ = fo.Net(spec, tp, sigma=0.7).loss_grad(f, Q, floor=0.1, power=power)
        lm, _ = fo.Net(spec, tm, sigma=0.7).loss_grad(f, Q, floor=0.1, power=power)
        gn[i] = (lp - lm) / (2 * eps)
    err = np.abs(ga - gn).max() / np.abs(gn).max()
    assert err < 1e-6, err


def test_equilibrium_form_gradients_match_finite_differences():
    """The equilibrium-exact loss (network on [f; M_f], output difference)
    against central finite differences of itself, every parameter."""
    spec, theta, net = _small(seed=7)
    f, Q = _data(spec, 2, 4)
    v = np.linspace(-3.0, 3.0, spec.N)
    M = fo.maxwellian_of(f.reshape(2, -1), v).reshape(f.shape)
    loss, g = net.loss_grad(f, Q, floor=0.1, M=M)
    ga = fo.pack(spec, g)
    eps = 1e-6
    gn = np.empty_like(theta)
    for i in range(theta.size):
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        lp, _ = fo.Net(spec, tp, sigma=0.7).loss_grad(f, Q, floor=0.1, M=M)
        lm, _ = fo.Net(spec, tm, sigma=0.7).loss_grad(f, Q, floor=0.1, M=M)
        gn[i] = (lp - lm) / (2 * eps)
    assert loss > 0
    err = np.abs(ga - gn).max() / np.abs(gn).max()
    assert err < 1e-6, err


def test_equilibrium_form_vanishes_at_equilibrium():
    """Q(f) = P(f) - P(M_f) is zero for f = M_f, for any parameters."""
    spec, theta, net = _small(seed=9)
    v = np.linspace(-3.0, 3.0, spec.N)
    f = np.random.default_rng(2).uniform(0.1, 1.0, (2, spec.N ** 3))
    M = fo.maxwellian_of(f, v)
    assert np.abs(net.predict_eq(M, M)).max() == 0.0
    assert np.abs(net.predict_eq(f, M)).max() > 0.0


def test_maxwellian_of_keeps_the_moments():
    """The Maxwellian of f has f's density, bulk velocity and temperature up
    to the grid's quadrature error (a wide grid keeps it small)."""
    from spectralbte_gb300.workloads import maxwellian
    N = 24
    v = np.linspace(-8.0, 8.0, N)
    f = 0.6 * maxwellian(v, 1.0, (0.4, 0.0, -0.2), 1.3) + 0.4 * maxwellian(v, 1.0, (-0.5, 0.1, 0), 0.8)
    M = fo.maxwellian_of(f.reshape(1, -1), v).reshape(N, N, N)
    wt = np.ones(N)
    wt[0] = wt[-1] = 0.5
    dv = v[1] - v[0]
    w = wt[:, None, None] * wt[None, :, None] * wt[None, None, :] * dv ** 3
    vx = v[:, None, None]
    for g in (f, M):
        assert abs((w * g).sum() - 1.0) < 1e-6
    assert abs((w * vx * f).sum() - (w * vx * M).sum()) < 1e-6
