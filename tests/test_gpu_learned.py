"""GPU learned collision operator (fno.cu) against its FP64 oracle.

* Forward: the network output on the device equals the oracle's with the
  same BF16 rounding points within rel-L2 1e-3, or for deeper networks no
  farther than that oracle is from the pure-FP64 one (FP32 accumulation
  order flips a few BF16 roundings, and the layers amplify them), and the
  pure-FP64 oracle within rel-L2 3e-2.
* Gradients: every parameter block's gradient equals the rounding oracle's
  within rel-L2 5e-3 or twice that oracle's distance from the FP64 one
  (the lift gradient is a sum with heavy cancellation, accumulated in FP32
  atomics on the device), and the FP64 oracle's within 5e-2; the loss within
  1e-4 relative.  An indexing or formula error shows as an O(1) difference.
  Both network kinds (GELU, bilinear), both element types (BF16, FP16),
  three shapes, and batches that are not a multiple of 8 (padding).
* Training on pairs from the plain operator lowers the held-out error of the
  network well below that of the untrained network.
* The plan's SPECTRAL_LEARNED path: the output is the conservation
  projection of the network output; a spot check above the tolerance
  returns the plain FP32 operator's result bit for bit and stays on it
  until a check passes; mass, momentum and energy are conserved to 1e-12
  either way.
"""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import fno_oracle as fo

pytestmark = pytest.mark.gpu

N, WIDTH, MODES, LAYERS, HIDDEN = 8, 8, 4, 2, 16
# (N, width, modes, layers, hidden, kind, precision)
SHAPES = {"small": (8, 8, 4, 2, 16, 0, 0), "wide": (16, 16, 8, 3, 32, 0, 0),
          "odd": (12, 24, 6, 1, 48, 0, 0), "bil": (8, 8, 4, 2, 16, 1, 0),
          "wide_bil": (16, 16, 8, 3, 32, 1, 0), "small16": (8, 8, 4, 2, 16, 0, 1),
          "wide16": (16, 16, 8, 3, 32, 0, 1), "odd16": (12, 24, 6, 1, 48, 0, 1)}


def _net(gpu, seed=7, sigma=0.5, shape="small"):
    n, w, m, L, hd, kind, prec = SHAPES[shape]
    net = gpu.FourierOperator(n, w, m, L, hd, seed=seed, kind=kind, precision=prec)
    net.output_scale = sigma
    spec = fo.Spec(N=n, C=w, Km=m, L=L, Hd=hd, kind=kind)
    return net, spec, prec


def _data(B, seed, n=N):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.05, 1.0, (B, n ** 3)).astype(np.float32)
    Q = rng.normal(size=(B, n ** 3)).astype(np.float32)
    return f, Q


@pytest.mark.parametrize("B,shape", [(3, "small"), (8, "small"), (13, "small"), (5, "wide"),
                                     (9, "odd"), (6, "bil"), (4, "wide_bil"), (5, "small16"),
                                     (4, "wide16"), (9, "odd16")])
def test_forward_matches_oracle(gpu, B, shape):
    import torch
    net, spec, prec = _net(gpu, shape=shape)
    theta = net.get_params().astype(np.float64)
    f, _ = _data(B, B, spec.N)
    fd = torch.from_numpy(f.astype(np.float64)).cuda()
    Qd = torch.zeros_like(fd)
    net.predict(fd, Qd, B)
    got = Qd.cpu().numpy()
    want_r = fo.Net(spec, theta, sigma=0.5, rounding=True, precision=prec).predict(
        f.astype(np.float64))
    want = fo.Net(spec, theta, sigma=0.5).predict(f.astype(np.float64))
    gap = rel_l2(want_r, want)
    assert rel_l2(got, want_r.reshape(B, -1)) < max(1e-3, gap), gap
    assert rel_l2(got, want.reshape(B, -1)) < 3e-2


@pytest.mark.parametrize("B,shape,floor", [(5, "small", 0.0), (16, "small", 0.3),
                                           (6, "wide", 0.0), (3, "odd", 0.1),
                                           (7, "bil", 0.1), (4, "wide_bil", 0.0),
                                           (5, "small16", 0.1), (6, "wide16", 0.1),
                                           (3, "odd16", 0.1)])
def test_gradients_match_oracle(gpu, B, shape, floor):
    import torch
    net, spec, prec = _net(gpu, seed=11, shape=shape)
    net.set_loss_floor(floor)
    theta = net.get_params().astype(np.float64)
    f, Q = _data(B, 100 + B, spec.N)
    loss, g = net.loss_grad(torch.from_numpy(f).cuda(), torch.from_numpy(Q).cuda(), B)
    lr_, gr = fo.Net(spec, theta, sigma=0.5, rounding=True, precision=prec).loss_grad(
        f.astype(np.float64), Q.astype(np.float64), floor)
    l64, g64 = fo.Net(spec, theta, sigma=0.5).loss_grad(f.astype(np.float64),
                                                        Q.astype(np.float64), floor)
    assert abs(loss - lr_) <= 1e-4 * lr_
    off, _ = spec.layout()
    for k, (o, n) in off.items():
        gk = g[o:o + n].astype(np.float64)
        gap = rel_l2(gr[k].reshape(-1), g64[k].reshape(-1))
        assert rel_l2(gk, gr[k].reshape(-1)) < max(5e-3, 2 * gap), (k, gap)
        assert rel_l2(gk, g64[k].reshape(-1)) < 5e-2, k


@pytest.mark.parametrize("B,shape,power", [(5, "small", 2.0), (6, "small16", 3.0),
                                           (4, "wide16", 2.0), (7, "bil", 2.0)])
def test_power_loss_gradients_match_oracle(gpu, B, shape, power):
    """The power loss mean_b e_b^k (spectral_fno_set_loss_power): the loss
    and every parameter block's gradient against the oracle, with the loss
    scale divided by the mean instance weight on both sides."""
    import torch
    net, spec, prec = _net(gpu, seed=19, shape=shape)
    net.set_loss_floor(0.1)
    net.set_loss_power(power)
    theta = net.get_params().astype(np.float64)
    f, Q = _data(B, 200 + B, spec.N)
    loss, g = net.loss_grad(torch.from_numpy(f).cuda(), torch.from_numpy(Q).cuda(), B)
    lr_, gr = fo.Net(spec, theta, sigma=0.5, rounding=True, precision=prec).loss_grad(
        f.astype(np.float64), Q.astype(np.float64), 0.1, power=power)
    l64, g64 = fo.Net(spec, theta, sigma=0.5).loss_grad(f.astype(np.float64),
                                                        Q.astype(np.float64), 0.1, power=power)
    assert abs(loss - lr_) <= 1e-4 * lr_
    off, _ = spec.layout()
    for k, (o, n) in off.items():
        gk = g[o:o + n].astype(np.float64)
        gap = rel_l2(gr[k].reshape(-1), g64[k].reshape(-1))
        assert rel_l2(gk, gr[k].reshape(-1)) < max(5e-3, 2 * gap), (k, gap)
        assert rel_l2(gk, g64[k].reshape(-1)) < 5e-2, k
    # back to the plain loss: the result equals a fresh plain evaluation
    net.set_loss_power(1.0)
    l1, _ = net.loss_grad(torch.from_numpy(f).cuda(), torch.from_numpy(Q).cuda(), B)
    lo, _ = fo.Net(spec, theta, sigma=0.5, rounding=True, precision=prec).loss_grad(
        f.astype(np.float64), Q.astype(np.float64), 0.1)
    assert abs(l1 - lo) <= 1e-4 * lo
    with pytest.raises(gpu.SpectralError):
        net.set_loss_power(0.5)


def _plan(gpu, n=N, L_v=6.0, lam=1.0):
    v, zeta = gpu.grid_0d(n, L_v)
    plan = gpu.Plan(n, L_v, v, zeta, 256)
    plan.generate_weights_iso(lam)
    return plan


def test_training_lowers_heldout_error(gpu, shape="small"):
    import torch
    from spectralbte_gb300 import learned as lrn
    plan = _plan(gpu)
    F, Q, _ = lrn.make_dataset(plan, 768, seed=1, chunk=128)
    Fe, Qe, fam = lrn.make_dataset(plan, 96, seed=999, chunk=96, out_dtype=torch.float64)
    net, _, _ = _net(gpu, seed=3, sigma=lrn.output_scale(F, Q), shape=shape)
    net.set_loss_floor(0.1)
    e0 = lrn.evaluate(net, plan, Fe, Qe)
    log = lrn.train(net, F, Q, steps=1500, batch=16, lr=1e-2, lr_final=3e-4)
    e1 = lrn.evaluate(net, plan, Fe, Qe)
    assert log.losses[-1][1] < 0.5 * log.losses[0][1]
    assert e1.mean() < 0.5 * e0.mean(), (e0.mean().item(), e1.mean().item(),
                                         lrn.family_stats(e1, fam))


def _moments(v, Q):
    n = v.size
    wt = np.ones(n)
    wt[0] = wt[-1] = 0.5
    dv = v[1] - v[0]
    w = (wt[:, None, None] * wt[None, :, None] * wt[None, None, :] * dv ** 3).reshape(-1)
    vx, vy, vz = (a.reshape(-1) for a in np.meshgrid(v, v, v, indexing="ij"))
    e = 0.5 * (vx ** 2 + vy ** 2 + vz ** 2)
    return np.stack([Q @ w, Q @ (w * vx), Q @ (w * vy), Q @ (w * vz), Q @ (w * e)], 1)


def test_plan_learned_path_and_fallback(gpu):
    import torch
    from spectralbte_gb300 import learned as lrn
    plan = _plan(gpu)
    net, _, _ = _net(gpu, seed=5)
    B = 12
    f = lrn.sample_f(plan.v, "mixture", B, seed=4)
    scale = float(torch.linalg.vector_norm(f, dim=1).mean())
    # accepted: Q = conserve(network(f))
    plan.set_learned(net, tol=1e9, check_every=1)
    Q = torch.empty_like(f)
    plan.computeQ_device(f, Q, B, gpu.FP32 | gpu.CONSERVE | gpu.LEARNED)
    want = torch.empty_like(f)
    net.predict(f, want, B)
    plan.conserve_device(want, B)
    torch.cuda.synchronize()
    assert torch.equal(Q, want)
    st = plan.learned_stats()
    assert st["calls"] == 1 and st["checks"] == 1 and st["fallbacks"] == 0
    assert np.isfinite(st["last_err"]) and st["last_err"] > 0
    m = _moments(plan.v, Q.cpu().numpy())
    assert np.abs(m).max() < 1e-12 * max(1.0, scale)
    # rejected: the plain FP32 operator's result, bit for bit
    plan.set_learned(net, tol=1e-12, check_every=2)
    plain = torch.empty_like(f)
    plan.computeQ_device(f, plain, B, gpu.FP32 | gpu.CONSERVE)
    for call in range(3):  # checked, unchecked (stays plain), checked
        Q.zero_()
        plan.computeQ_device(f, Q, B, gpu.FP32 | gpu.CONSERVE | gpu.LEARNED)
        torch.cuda.synchronize()
        assert torch.equal(Q, plain), call
    st = plan.learned_stats()
    assert st["calls"] == 3 and st["checks"] == 2 and st["fallbacks"] == 3
    m = _moments(plan.v, Q.cpu().numpy())
    assert np.abs(m).max() < 1e-12 * max(1.0, scale)
    plan.set_learned(None)
    with pytest.raises(gpu.SpectralError):
        plan.computeQ_device(f, Q, B, gpu.FP32 | gpu.LEARNED)


def test_1d_steps_with_learned_operator(gpu, oracle):
    """The 1D-3V step with SPECTRAL_LEARNED: with every check failing it is
    the plain FP32 step bit for bit; a graph-captured step (no checks)
    replays the uncaptured one; capture with checks is refused."""
    import torch
    nX = 16
    r = oracle.Run1D(N, 6.0, nX, 2, 3, 2e-3, 0.5)
    plan = gpu.Plan(N, 6.0, r.g.v, r.g.zeta, nX)
    plan.generate_weights_iso(1.0)
    plan.setup_1d(nX, 2, 3, 2e-3, 0.5, r.x, r.dx)
    f0 = r.init()
    net, _, _ = _net(gpu, seed=5)
    a = torch.from_numpy(f0.copy()).cuda()
    b = torch.from_numpy(f0.copy()).cuda()
    plan.set_learned(net, tol=1e-12, check_every=1)
    for _ in range(3):
        plan.step_1d(a, gpu.FP32)
        plan.step_1d(b, gpu.FP32 | gpu.LEARNED)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    st = plan.learned_stats()
    assert st["calls"] == 6 and st["fallbacks"] == 6
    plan.set_learned(net, tol=1.0, check_every=0)
    c = torch.from_numpy(f0.copy()).cuda()
    d = torch.from_numpy(f0.copy()).cuda()
    for _ in range(3):
        plan.step_1d(c, gpu.FP32 | gpu.LEARNED)
    plan.capture(1, d, flags=gpu.FP32 | gpu.LEARNED)
    for _ in range(3):
        plan.launch()
    torch.cuda.synchronize()
    assert torch.equal(c, d)
    assert not torch.equal(c, a)  # the network, not the plain operator, ran
    plan.set_learned(net, tol=1.0, check_every=1)
    with pytest.raises(gpu.SpectralError):
        plan.capture(1, d, flags=gpu.FP32 | gpu.LEARNED)


def test_channel_mix_profiling_counts_launches(gpu):
    """spectral_fno_set_profiling: one event pair per channel-mix launch (one
    per layer and forward pass); the timed output equals the untimed one."""
    import torch
    net, spec, _ = _net(gpu, shape="wide")
    B = 6
    f, _ = _data(B, 21, spec.N)
    fd = torch.from_numpy(f.astype(np.float64)).cuda()
    Q0, Q1 = torch.zeros_like(fd), torch.zeros_like(fd)
    net.predict(fd, Q0, B)
    net.set_profiling(True)
    for _ in range(3):
        net.predict(fd, Q1, B)
    ms, n = net.kernel_time()
    net.set_profiling(False)
    assert n == 3 * spec.L
    assert ms > 0.0
    assert torch.equal(Q0, Q1)
    net.set_profiling(True)   # switching on again starts a new count
    assert net.kernel_time() == (0.0, 0)
    net.set_profiling(False)


def _eq_data(B, seed, n, L_v=4.0):
    """f from the mixture family on an n-point grid, its Maxwellian (oracle),
    and random targets; f rounded to FP32 as the training path stores it."""
    import math
    rng = np.random.default_rng(seed)
    v = np.linspace(-L_v, L_v, n)
    vx, vy, vz = v[:, None, None], v[None, :, None], v[None, None, :]
    f = np.zeros((B, n, n, n))
    for b in range(B):
        for _ in range(2):
            u = rng.uniform(-0.8, 0.8, 3)
            T = rng.uniform(0.6, 1.6)
            f[b] += rng.uniform(0.3, 1.0) * (2 * math.pi * T) ** -1.5 * np.exp(
                -((vx - u[0]) ** 2 + (vy - u[1]) ** 2 + (vz - u[2]) ** 2) / (2 * T))
    f = f.reshape(B, -1).astype(np.float32).astype(np.float64)
    M = fo.maxwellian_of(f, v)
    Q = rng.normal(size=(B, n ** 3)).astype(np.float32)
    return v, f, M, Q


@pytest.mark.parametrize("B,shape", [(3, "small16"), (5, "wide16"), (4, "small")])
def test_equilibrium_form_forward_matches_oracle(gpu, B, shape):
    """P(f) - P(M_f) on the device (one batch [f; M_f], the Maxwellian built
    by the device) against the oracle with the same rounding points."""
    import torch
    net, spec, prec = _net(gpu, seed=13, shape=shape)
    v, f, M, _ = _eq_data(B, 40 + B, spec.N)
    net.set_equilibrium(True, v)
    assert net.equilibrium
    theta = net.get_params().astype(np.float64)
    fd = torch.from_numpy(f).cuda()
    Qd = torch.zeros_like(fd)
    net.predict(fd, Qd, B)
    got = Qd.cpu().numpy()
    o_r = fo.Net(spec, theta, sigma=0.5, rounding=True, precision=prec)
    o64 = fo.Net(spec, theta, sigma=0.5)
    want_r = o_r.predict_eq(f, M).reshape(B, -1)
    want = o64.predict_eq(f, M).reshape(B, -1)
    # the difference of two outputs: the scale of the rounding gap is that of
    # either output, not of their difference
    ref = np.linalg.norm(o64.predict(f))
    gap = np.linalg.norm(want_r - want) / ref
    assert np.linalg.norm(got - want_r) / ref < max(1e-3, 2 * gap), gap
    assert np.linalg.norm(got - want) / ref < 3e-2
    # switching the form off restores the plain network output
    net.set_equilibrium(False)
    P = torch.zeros_like(fd)
    net.predict(fd, P, B)
    assert rel_l2(P.cpu().numpy(), o_r.predict(f).reshape(B, -1)) < max(1e-3, 2 * gap)


@pytest.mark.parametrize("B,shape,floor", [(4, "small16", 0.1), (3, "wide16", 0.1),
                                           (5, "small", 0.0)])
def test_equilibrium_form_gradients_match_oracle(gpu, B, shape, floor):
    import torch
    net, spec, prec = _net(gpu, seed=17, shape=shape)
    v, f, M, Q = _eq_data(B, 60 + B, spec.N)
    net.set_equilibrium(True, v)
    net.set_loss_floor(floor)
    theta = net.get_params().astype(np.float64)
    loss, g = net.loss_grad(torch.from_numpy(f.astype(np.float32)).cuda(),
                            torch.from_numpy(Q).cuda(), B)
    lr_, gr = fo.Net(spec, theta, sigma=0.5, rounding=True, precision=prec).loss_grad(
        f, Q.astype(np.float64), floor, M=M)
    l64, g64 = fo.Net(spec, theta, sigma=0.5).loss_grad(f, Q.astype(np.float64), floor, M=M)
    assert abs(loss - lr_) <= 1e-4 * lr_
    off, _ = spec.layout()
    # The halves f and M_f push the gradients of the lift (P, bP) in nearly
    # opposite directions, so those blocks are small sums with heavy
    # cancellation: 16-bit rounding alone moves them by several percent (the
    # rounding oracle's distance from FP64, gap).  Every block is held to the
    # rounding oracle within max(5e-3, 3 gap) and to FP64 within
    # max(5e-2, 4 gap) (the two distances add); an indexing or formula error
    # is O(1).
    for k, (o, n) in off.items():
        gk = g[o:o + n].astype(np.float64)
        ref_r, ref_64 = gr[k].reshape(-1), g64[k].reshape(-1)
        gap = rel_l2(ref_r, ref_64)
        assert rel_l2(gk, ref_r) < max(5e-3, 3 * gap), (k, gap, rel_l2(gk, ref_r))
        assert rel_l2(gk, ref_64) < max(5e-2, 4 * gap), (k, gap, rel_l2(gk, ref_64))


def test_equilibrium_form_is_small_at_equilibrium(gpu):
    """On a Maxwellian the equilibrium form returns (nearly) zero for any
    parameters: M_f differs from f = M only by the grid's moment quadrature,
    and the network output of the difference scales with it.  The plain form
    of the same untrained network returns an O(1) output there."""
    import torch
    from spectralbte_gb300.workloads import maxwellian
    n = 16
    net = gpu.FourierOperator(n, 16, 8, 3, 32, seed=21, precision=1)
    net.output_scale = 0.5
    v = np.linspace(-7.0, 7.0, n)
    f = np.stack([maxwellian(v, 1.0, (0.3, -0.1, 0.0), 1.1).reshape(-1),
                  maxwellian(v, 0.7, (0.0, 0.2, 0.4), 0.9).reshape(-1)])
    fd = torch.from_numpy(f).cuda()
    P = torch.zeros_like(fd)
    net.predict(fd, P, 2)
    net.set_equilibrium(True, v)
    D = torch.zeros_like(fd)
    net.predict(fd, D, 2)
    torch.cuda.synchronize()
    ratio = (torch.linalg.vector_norm(D, dim=1) / torch.linalg.vector_norm(P, dim=1)).max()
    assert ratio < 1e-2, float(ratio)


def test_floored_spot_check(gpu):
    """With a floor eps the check divides by sqrt(|Q|^2 + eps mean |Q_net|^2):
    the recorded distance equals that formula for the checked instance, and is
    below the unfloored one."""
    import torch
    from spectralbte_gb300 import learned as lrn
    plan = _plan(gpu)
    net, _, _ = _net(gpu, seed=5)
    B = 6
    f = lrn.sample_f(plan.v, "mixture", B, seed=8)
    Qn = torch.empty_like(f)
    net.predict(f, Qn, B)
    plan.conserve_device(Qn, B)
    Qp = torch.empty_like(f)
    plan.computeQ_device(f, Qp, B, gpu.FP32 | gpu.CONSERVE)
    torch.cuda.synchronize()
    d = torch.linalg.vector_norm(Qn[0] - Qp[0]).item()
    q2 = torch.linalg.vector_norm(Qp[0]).item() ** 2
    msq = (Qn.pow(2).sum() / B).item()
    Q = torch.empty_like(f)
    for eps, want in ((0.0, d / np.sqrt(q2)), (0.5, d / np.sqrt(q2 + 0.5 * msq))):
        plan.set_learned(net, tol=1e9, check_every=1)
        plan.set_learned_floor(eps)
        plan.computeQ_device(f, Q, B, gpu.FP32 | gpu.CONSERVE | gpu.LEARNED)
        torch.cuda.synchronize()
        got = plan.learned_stats()["last_err"]
        assert abs(got - want) <= 1e-9 * want, (eps, got, want)
    plan.set_learned(None)


@pytest.mark.parametrize("B,prec", [(64, 1), (128, 0), (40, 1)])
def test_tma_channel_mix_matches_gemm(gpu, B, prec):
    """The inference channel mix through the TMA warp-specialised kernel
    (width 64, instances padded to a multiple of 64) equals the general
    tensor-core GEMM: same products in the same order, same epilogue.  At
    B = 40 (padded to 40) the general GEMM runs either way."""
    import torch
    net = gpu.FourierOperator(16, 64, 8, 3, 32, seed=4, precision=prec)
    net.output_scale = 0.5
    rng = np.random.default_rng(B)
    f = torch.from_numpy(rng.uniform(0.05, 1.0, (B, 16 ** 3))).cuda()
    out = {}
    for mode in range(7):   # 0: the general GEMM; 1-6: shapes of the TMA kernel
        net.set_channel_mix_kernel(mode)
        Q = torch.empty_like(f)
        net.predict(f, Q, B)
        torch.cuda.synchronize()
        out[mode] = Q.cpu().numpy()
    assert net.status() == 0
    for mode in range(1, 7):
        assert np.abs(out[mode] - out[0]).max() <= 1e-6 * np.abs(out[0]).max(), mode


@pytest.mark.parametrize("B,prec", [(64, 1), (128, 0)])
def test_tma_readout_matches_gemm(gpu, B, prec):
    """The inference readout through the TMA warp-specialised kernel (width
    64, hidden 128, instances padded to a multiple of 64) against the general
    GEMM: the hidden rows are summed in another order (two partial sums of 64
    rows each, added atomically), so the outputs agree to FP32 rounding of the
    readout, far below the 16-bit resolution of the activations."""
    import torch
    net = gpu.FourierOperator(16, 64, 8, 2, 128, seed=6, precision=prec)
    net.output_scale = 0.5
    rng = np.random.default_rng(B + 1)
    f = torch.from_numpy(rng.uniform(0.05, 1.0, (B, 16 ** 3))).cuda()
    out = {}
    for tma in (True, False):
        net.set_readout_kernel(tma)
        Q = torch.empty_like(f)
        net.predict(f, Q, B)
        torch.cuda.synchronize()
        out[tma] = Q.cpu().numpy()
    assert net.status() == 0
    assert np.abs(out[True] - out[False]).max() <= 1e-5 * np.abs(out[False]).max()
    # deterministic: a second call gives the same bits
    net.set_readout_kernel(True)
    Q2 = torch.empty_like(f)
    net.predict(f, Q2, B)
    torch.cuda.synchronize()
    assert np.array_equal(Q2.cpu().numpy(), out[True])


@pytest.mark.parametrize("B,modes,prec", [(8, 12, 1), (24, 8, 0)])
def test_tma_axis_k_matches_gemm(gpu, B, modes, prec):
    """The first forward and the last inverse axis pass of every layer through
    the TMA warp-specialised kernel (N = 32) against the general GEMM: the same
    products in the same K blocks, so the network output is the same."""
    import torch
    net = gpu.FourierOperator(32, 16, modes, 2, 32, seed=8, precision=prec)
    net.output_scale = 0.5
    rng = np.random.default_rng(B + 3)
    f = torch.from_numpy(rng.uniform(0.05, 1.0, (B, 32 ** 3))).cuda()
    out = {}
    for tma in (True, False):
        net.set_axis_kernel(tma)
        Q = torch.empty_like(f)
        net.predict(f, Q, B)
        torch.cuda.synchronize()
        out[tma] = Q.cpu().numpy()
    assert net.status() == 0
    assert np.abs(out[True] - out[False]).max() <= 1e-6 * np.abs(out[False]).max()


def test_learned_path_gain_over_plain_fp32(gpu):
    """What the trained network gains over the method without it, at N = 32
    on 256 fresh two-Maxwellian instances (config 2's family; a seed no
    training or selection used): Q evals/s of the plain FP32 operator against
    the network + FP64 projection, unchecked and with a spot check of one
    instance per call (plain FP32 fallback).  Asserted: the checked learned
    path is at least 1.5x the plain one, its batch rel-L2 against the plain
    operator is within 1e-3, its floored per-instance median within 1e-3, and
    the projection conserves the moments.  (Every instance within 1e-3 is
    what the benchmark requires before it reports the learned path as its
    headline; the committed network misses that on a few of 1024.)"""
    import os
    import torch
    from spectralbte_gb300.workloads import moment_residual, two_maxwellian_batch
    sb = gpu
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "spectralbte_gb300", "models", "fno_n32.npz")
    net = sb.FourierOperator.load(path)
    N, L_v, B = 32, 6.0, 256
    v, zeta = sb.grid_0d(N, L_v)
    plan = sb.Plan(N, L_v, v, zeta, B)
    plan.generate_weights_closed(1.0, fp64_table=False)
    f = torch.from_numpy(two_maxwellian_batch(v, B, 61001)).cuda()
    flags = sb.FP32 | sb.CONSERVE

    def rate(fl, reps=3):
        Q = torch.empty_like(f)
        plan.computeQ_device(f, Q, B, fl)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            plan.computeQ_device(f, Q, B, fl)
        e1.record()
        torch.cuda.synchronize()
        return B * reps / (e0.elapsed_time(e1) / 1e3), Q

    r_plain, Qp = rate(flags)
    plan.set_learned(net, tol=1e-3, check_every=0)
    r_net, Ql = rate(flags | sb.LEARNED)
    plan.set_learned(net, tol=1e-3, check_every=1)
    plan.set_learned_floor(0.1)
    r_checked, _ = rate(flags | sb.LEARNED)
    st = plan.learned_stats()
    num = (Ql - Qp).pow(2).sum(dim=1)
    q2 = Qp.pow(2).sum(dim=1)
    batch_rel = float((num.sum() / q2.sum()).sqrt())
    floored = (num / (q2 + 0.1 * q2.mean())).sqrt()
    res = moment_residual(v, Ql)
    print(f"plain {r_plain:.0f} Q/s, network {r_net:.0f}, checked {r_checked:.0f} "
          f"({st['fallbacks']} fallbacks in {st['calls']}); batch rel-L2 {batch_rel:.2e}, "
          f"floored median {float(floored.median()):.2e} max {float(floored.max()):.2e}")
    assert st["fallbacks"] == 0
    assert r_checked >= 1.5 * r_plain, (r_plain, r_checked)
    assert batch_rel <= 1e-3
    assert float(floored.median()) <= 1e-3
    assert max(res.values()) <= 1e-12
    plan.set_learned(None)
    plan.close()


def test_committed_network_accuracy_by_family(gpu):
    """The committed N = 32 network against the plain FP32 operator on 1,024
    fresh instances of each training family (a seed no training or selection
    used), floored distance with eps = 0.1 over each family's batch.  The
    thresholds record what the network does, with margin: the two-Maxwellian
    family (the benchmark's) at a mean of about 4e-4 with its worst instance
    near 1e-3; shock blends and Maxwellian mixtures well above 1e-3, which is
    why the spot check returns those calls to the plain operator."""
    import os
    import torch
    from spectralbte_gb300.learned import evaluate, make_dataset
    sb = gpu
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "spectralbte_gb300", "models", "fno_n32.npz")
    net = sb.FourierOperator.load(path)
    N, L_v = 32, 6.0
    v, zeta = sb.grid_0d(N, L_v)
    plan = sb.Plan(N, L_v, v, zeta, 512)
    plan.generate_weights_closed(1.0, fp64_table=False)
    bounds = {"two_maxwellian": (6e-4, 1.5e-3), "shock": (2e-2, 1e-1), "mixture": (6e-3, 5e-2)}
    got = {}
    for fam, (mean_max, worst_max) in bounds.items():
        F, Q, _ = make_dataset(plan, 1024, seed=130001, families=(fam,), out_dtype=torch.float64)
        e = evaluate(net, plan, F, Q, floor=0.1).cpu().numpy()
        got[fam] = (float(e.mean()), float(e.max()))
        assert e.mean() <= mean_max and e.max() <= worst_max, (fam, got[fam])
    print(got)
    assert got["two_maxwellian"][0] < 1e-3 < got["shock"][0]
    plan.close()
