"""GPU learned collision operator (fno.cu) against its FP64 oracle.

* Forward: the network output on the device equals the oracle's with the
  same BF16 rounding points within rel-L2 1e-3, and the pure-FP64 oracle
  within rel-L2 3e-2 (the BF16 operands).
* Gradients: every parameter block's gradient equals the rounding oracle's
  within rel-L2 5e-3 and the FP64 oracle's within 5e-2; the loss within
  1e-4 relative.  Batches that are not a multiple of 8 exercise the padding.
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


def _net(gpu, seed=7, sigma=0.5):
    net = gpu.FourierOperator(N, WIDTH, MODES, LAYERS, HIDDEN, seed=seed)
    net.output_scale = sigma
    spec = fo.Spec(N=N, C=WIDTH, Km=MODES, L=LAYERS, Hd=HIDDEN)
    return net, spec


def _data(B, seed):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.05, 1.0, (B, N ** 3)).astype(np.float32)
    Q = rng.normal(size=(B, N ** 3)).astype(np.float32)
    return f, Q


@pytest.mark.parametrize("B", [3, 8, 13])
def test_forward_matches_oracle(gpu, B):
    import torch
    net, spec = _net(gpu)
    theta = net.get_params().astype(np.float64)
    f, _ = _data(B, B)
    fd = torch.from_numpy(f.astype(np.float64)).cuda()
    Qd = torch.zeros_like(fd)
    net.predict(fd, Qd, B)
    got = Qd.cpu().numpy()
    want_r = fo.Net(spec, theta, sigma=0.5, rounding=True).predict(f.astype(np.float64))
    want = fo.Net(spec, theta, sigma=0.5).predict(f.astype(np.float64))
    assert rel_l2(got, want_r.reshape(B, -1)) < 1e-3
    assert rel_l2(got, want.reshape(B, -1)) < 3e-2


@pytest.mark.parametrize("B", [5, 16])
def test_gradients_match_oracle(gpu, B):
    import torch
    net, spec = _net(gpu, seed=11)
    theta = net.get_params().astype(np.float64)
    f, Q = _data(B, 100 + B)
    loss, g = net.loss_grad(torch.from_numpy(f).cuda(), torch.from_numpy(Q).cuda(), B)
    lr_, gr = fo.Net(spec, theta, sigma=0.5, rounding=True).loss_grad(
        f.astype(np.float64), Q.astype(np.float64))
    l64, g64 = fo.Net(spec, theta, sigma=0.5).loss_grad(f.astype(np.float64),
                                                        Q.astype(np.float64))
    assert abs(loss - lr_) <= 1e-4 * lr_
    off, _ = spec.layout()
    for k, (o, n) in off.items():
        gk = g[o:o + n].astype(np.float64)
        assert rel_l2(gk, gr[k].reshape(-1)) < 5e-3, k
        assert rel_l2(gk, g64[k].reshape(-1)) < 5e-2, k


def _plan(gpu, n=N, L_v=6.0, lam=1.0):
    v, zeta = gpu.grid_0d(n, L_v)
    plan = gpu.Plan(n, L_v, v, zeta, 256)
    plan.generate_weights_iso(lam)
    return plan


def test_training_lowers_heldout_error(gpu):
    import torch
    from spectralbte_gb300 import learned as lrn
    plan = _plan(gpu)
    F, Q = lrn.make_dataset(plan, 768, seed=1, chunk=128)
    Fe, Qe = lrn.make_dataset(plan, 96, seed=999, chunk=96, out_dtype=torch.float64)
    net, _ = _net(gpu, seed=3, sigma=lrn.output_scale(F, Q))
    e0 = lrn.evaluate(net, plan, Fe, Qe).mean().item()
    log = lrn.train(net, F, Q, steps=400, batch=16, lr=3e-3, lr_final=1e-4)
    e1 = lrn.evaluate(net, plan, Fe, Qe).mean().item()
    assert log.losses[-1][1] < log.losses[0][1]
    assert e1 < 0.5 * e0, (e0, e1)


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
    net, _ = _net(gpu, seed=5)
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
