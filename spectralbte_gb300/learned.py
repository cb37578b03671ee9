"""Training and evaluation of the learned collision operator.

The network (``FourierOperator``, fno.cu) is trained on (f, Q(f)) pairs
whose Q comes from the plain operator of this library: the FP32 batched
convolution plus the FP64 conservation projection.  The initial data f are
drawn on the device from five seeded families of velocity distributions:

* ``two_maxwellian``: discontinuous in v_x, density 1 and temperature 1 for
  v_x < 0, density 1, temperature 2 and drift 0.5 for v_x >= 0, each
  parameter jittered by +-5%;
* ``shock``: states inside a Mach-1.2 normal shock, a blend
  a M_up + (1 - a) M_down of the upstream Maxwellian (density 1, velocity
  1.2 sqrt(5/3), temperature 1) and its Rankine-Hugoniot downstream state,
  a ~ U(0, 1), with +-5% jitter;
* ``mixture``: 2-3 Maxwellians with density U(0.2, 1), drift components
  U(-1, 1) and temperature U(0.5, 2), normalised to unit mass;
* ``half_space``: the states next to a diffuse wall, one Maxwellian for
  v_x < 0 and another for v_x >= 0, densities U(0.5, 1.5), temperatures
  U(0.8, 2.2), x-drifts U(-0.3, 0.3) (the walls of the heat-transfer run sit
  at temperatures 1 and 2);
* ``near_eq``: states close to equilibrium, (1 - e) M1 + e M2 with
  e = 10^U(-3, -0.5), M1 a Maxwellian (density U(0.5, 1.5), drift
  U(-0.5, 0.5)^3, temperature U(0.7, 2)) and M2 a full or half-space
  Maxwellian drifted by U(-1, 1)^3 from it with temperature U(0.5, 2).

Everything here is host orchestration in PyTorch (device memory, random
parameters); the network's forward, backward and optimiser step are the
library's CUDA kernels.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import CONSERVE, FP32, LEARNED, FourierOperator, Plan  # noqa: F401

FAMILIES = ("two_maxwellian", "shock", "mixture", "half_space", "near_eq")
# the families of the earlier networks (before half_space and near_eq)
BASE_FAMILIES = FAMILIES[:3]


def rankine_hugoniot(mach: float, gamma: float = 5.0 / 3.0, rho1=1.0, T1=1.0):
    """Downstream (rho, u, T) of a normal shock with upstream (rho1, M sqrt(gamma T1), T1)."""
    u1 = mach * math.sqrt(gamma * T1)
    r = (gamma + 1) * mach ** 2 / ((gamma - 1) * mach ** 2 + 2)
    pr = 1 + 2 * gamma / (gamma + 1) * (mach ** 2 - 1)
    return (rho1, u1, T1), (rho1 * r, u1 / r, T1 * pr / r)


def _components(family: str, B: int, rng: np.random.Generator):
    """Per instance up to 3 Maxwellian components: (rho, ux, uy, uz, T, half)
    with half = 0 (everywhere), -1 (v_x < 0) or +1 (v_x >= 0)."""
    comp = np.zeros((B, 3, 6))
    comp[:, :, 4] = 1.0
    if family == "two_maxwellian":
        j = 1.0 + rng.uniform(-0.05, 0.05, (B, 5))
        comp[:, 0] = np.stack([j[:, 0], 0 * j[:, 0], 0 * j[:, 0], 0 * j[:, 0], j[:, 1],
                               -np.ones(B)], 1)
        comp[:, 1] = np.stack([j[:, 2], 0.5 * j[:, 4], 0 * j[:, 0], 0 * j[:, 0], 2.0 * j[:, 3],
                               np.ones(B)], 1)
    elif family == "shock":
        (r1, u1, t1), (r2, u2, t2) = rankine_hugoniot(1.2)
        a = rng.uniform(0, 1, B)
        j = 1.0 + rng.uniform(-0.05, 0.05, (B, 6))
        comp[:, 0, 0], comp[:, 0, 1], comp[:, 0, 4] = a * r1 * j[:, 0], u1 * j[:, 1], t1 * j[:, 2]
        comp[:, 1, 0], comp[:, 1, 1], comp[:, 1, 4] = (1 - a) * r2 * j[:, 3], u2 * j[:, 4], \
            t2 * j[:, 5]
    elif family == "mixture":
        k = rng.integers(2, 4, B)
        for c in range(3):
            on = (c < k).astype(float)
            comp[:, c, 0] = on * rng.uniform(0.2, 1.0, B)
            comp[:, c, 1:4] = rng.uniform(-1, 1, (B, 3))
            comp[:, c, 4] = rng.uniform(0.5, 2.0, B)
    elif family == "half_space":
        comp[:, 0, 0], comp[:, 1, 0] = rng.uniform(0.5, 1.5, B), rng.uniform(0.5, 1.5, B)
        comp[:, 0, 1], comp[:, 1, 1] = rng.uniform(-0.3, 0.3, B), rng.uniform(-0.3, 0.3, B)
        comp[:, 0, 4], comp[:, 1, 4] = rng.uniform(0.8, 2.2, B), rng.uniform(0.8, 2.2, B)
        comp[:, 0, 5], comp[:, 1, 5] = -1.0, 1.0
    elif family == "near_eq":
        e = 10.0 ** rng.uniform(-3.0, -0.5, B)
        rho = rng.uniform(0.5, 1.5, B)
        u = rng.uniform(-0.5, 0.5, (B, 3))
        comp[:, 0, 0], comp[:, 0, 1:4], comp[:, 0, 4] = (1 - e) * rho, u, rng.uniform(0.7, 2.0, B)
        comp[:, 1, 0] = e * rho
        comp[:, 1, 1:4] = u + rng.uniform(-1, 1, (B, 3))
        comp[:, 1, 4] = rng.uniform(0.5, 2.0, B)
        comp[:, 1, 5] = rng.integers(-1, 2, B)
    else:
        raise ValueError(family)
    return comp


def sample_f(v: np.ndarray, family: str, B: int, seed: int, device="cuda"):
    """B distributions of one family on the grid v, FP64 [B][N^3] on the device."""
    import torch
    rng = np.random.default_rng(seed)
    comp = torch.from_numpy(_components(family, B, rng)).to(device)
    vt = torch.from_numpy(np.asarray(v, dtype=np.float64)).to(device)
    N = vt.numel()
    vx, vy, vz = vt.view(1, N, 1, 1), vt.view(1, 1, N, 1), vt.view(1, 1, 1, N)
    f = torch.zeros(B, N, N, N, dtype=torch.float64, device=device)
    for c in range(3):
        rho, ux, uy, uz, T, half = (comp[:, c, i].view(B, 1, 1, 1) for i in range(6))
        m = rho * (2 * math.pi * T) ** -1.5 * torch.exp(
            -((vx - ux) ** 2 + (vy - uy) ** 2 + (vz - uz) ** 2) / (2 * T))
        mask = torch.where(half < 0, (vx < 0).double(),
                           torch.where(half > 0, (vx >= 0).double(), torch.ones_like(vx)))
        f += m * mask
    if family == "mixture":
        dv = float(v[1] - v[0])
        wt = torch.ones(N, dtype=torch.float64, device=device)
        wt[0] = wt[-1] = 0.5
        w3 = wt.view(N, 1, 1) * wt.view(1, N, 1) * wt.view(1, 1, N) * dv ** 3
        f /= (f * w3).sum(dim=(1, 2, 3)).view(B, 1, 1, 1)
    return f.reshape(B, -1).contiguous()


def make_dataset(plan: Plan, n: int, seed: int, chunk: int = 512,
                 families=FAMILIES, out_dtype=None):
    """n pairs (f, Q) with Q = conserve(plain FP32 Q(f)), stored as float32 on
    the device (out_dtype float64 keeps FP64), and the family index of each
    pair.  Instance i belongs to family i mod len(families)."""
    import torch
    out_dtype = out_dtype or torch.float32
    F = torch.empty(n, plan.n3, dtype=out_dtype, device="cuda")
    Q = torch.empty_like(F)
    Qc = torch.empty(chunk, plan.n3, dtype=torch.float64, device="cuda")
    nf = len(families)
    fam = torch.arange(n, device="cuda") % nf
    i, k = 0, 0
    while i < n:
        b = min(chunk, n - i)
        f = torch.empty(b, plan.n3, dtype=torch.float64, device="cuda")
        for j, name in enumerate(families):
            idx = [r for r in range(b) if (i + r) % nf == j]
            if idx:
                f[idx] = sample_f(plan.v, name, len(idx), seed + 7919 * k + 104729 * j)
        plan.computeQ_device(f, Qc, b, FP32 | CONSERVE)
        F[i:i + b] = f.to(out_dtype)
        Q[i:i + b] = Qc[:b].to(out_dtype)
        i += b
        k += 1
    torch.cuda.synchronize()
    return F, Q, fam


def output_scale(F, Q) -> float:
    """RMS of Q / s^2 (s = max f per instance): the scale that makes the
    network's targets O(1)."""
    s = F.double().amax(dim=1).clamp_min(1e-300)
    t = Q.double() / (s * s).unsqueeze(1)
    return float(t.pow(2).mean().sqrt())


@dataclass
class TrainLog:
    steps: int = 0
    seconds: float = 0.0
    samples: int = 0
    losses: list = field(default_factory=list)


def train(net: FourierOperator, F, Q, steps: int, batch: int = 32, lr: float = 2e-3,
          lr_final: float = 1e-5, seed: int = 0, log_every: int = 50,
          time_limit: float | None = None) -> TrainLog:
    """Adam with cosine decay from lr to lr_final over the run (the larger of
    the step fraction and, with a time limit, the time fraction); random
    mini-batches drawn from (F, Q) on the device."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    n = F.shape[0]
    log = TrainLog()
    fb = torch.empty(batch, F.shape[1], dtype=torch.float32, device="cuda")
    qb = torch.empty_like(fb)
    t0 = time.time()
    for s in range(steps):
        idx = torch.randint(0, n, (batch,), device="cuda", generator=g)
        torch.index_select(F, 0, idx, out=fb)
        torch.index_select(Q, 0, idx, out=qb)
        prog = s / max(1, steps)
        if time_limit:
            prog = max(prog, (time.time() - t0) / time_limit)
        a = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * min(1.0, prog)))
        want = (s % log_every == 0) or s == steps - 1
        loss = net.train_step(fb, qb, batch, a, want_loss=want)
        if want:
            log.losses.append((s, loss))
        log.steps = s + 1
        if time_limit is not None and time.time() - t0 > time_limit:
            break
    torch.cuda.synchronize()
    log.seconds = time.time() - t0
    log.samples = log.steps * batch
    return log


def family_stats(err, fam, families=FAMILIES) -> dict:
    """Mean, median and max of per-instance errors by family."""
    out = {}
    for j, name in enumerate(families):
        e = err[fam == j]
        if e.numel():
            out[name] = {"mean": e.mean().item(), "median": e.median().item(),
                         "max": e.max().item()}
    return out


def rel_l2_per_instance(A, R):
    import torch
    d = (A.double() - R.double()).pow(2).sum(dim=1)
    return torch.sqrt(d / R.double().pow(2).sum(dim=1).clamp_min(1e-300))


def evaluate(net: FourierOperator, plan: Plan, F, Q, chunk: int = 256, floor: float = 0.0,
             fam=None):
    """rel-L2 of conserve(network(f)) against Q for every instance.  With a
    floor eps > 0 the distance of instance b is |Q_net - Q| / sqrt(|Q|^2 +
    eps * mean |Q_b'|^2), the mean over the instances of b's family (fam
    given) or over all of them: the normalisation of the training loss and of
    the plan's floored spot check."""
    import torch
    n = F.shape[0]
    num = torch.empty(n, dtype=torch.float64, device="cuda")
    den = torch.empty(n, dtype=torch.float64, device="cuda")
    Qp = torch.empty(chunk, plan.n3, dtype=torch.float64, device="cuda")
    for i in range(0, n, chunk):
        b = min(chunk, n - i)
        f = F[i:i + b].double().contiguous()
        net.predict(f, Qp, b)
        plan.conserve_device(Qp, b)
        num[i:i + b] = (Qp[:b] - Q[i:i + b].double()).pow(2).sum(dim=1)
        den[i:i + b] = Q[i:i + b].double().pow(2).sum(dim=1)
    if floor > 0.0:
        if fam is None:
            den = den + floor * den.mean()
        else:
            add = torch.zeros_like(den)
            for j in torch.unique(fam):
                sel = fam == j
                add[sel] = floor * den[sel].mean()
            den = den + add
    return torch.sqrt(num / den.clamp_min(1e-300))


def main(argv=None):
    """Train a network on pairs from the plain operator and save it:
    python -m spectralbte_gb300.learned --n 32 --pairs 200000 --minutes 10 --out net.npz"""
    import argparse
    import json

    import torch

    from . import grid_0d
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--lv", type=float, default=6.0)
    ap.add_argument("--lam", type=float, default=1.0)
    ap.add_argument("--width", type=int, default=64)
    ap.add_argument("--modes", type=int, default=12)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--hidden", type=int, default=128)
    ap.add_argument("--kind", type=int, default=0, help="0: GELU network, 1: bilinear")
    ap.add_argument("--floor", type=float, default=0.1)
    ap.add_argument("--loss-power", type=float, default=1.0,
                    help="train on mean_b e_b^k (k > 1 weights the worst instances up; "
                         "plain form only)")
    ap.add_argument("--precision", type=int, default=1, help="0: BF16, 1: FP16 elements")
    ap.add_argument("--pairs", type=int, default=200000)
    ap.add_argument("--heldout", type=int, default=512)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--minutes", type=float, default=10.0)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--init", default=None, help="start from this saved network")
    ap.add_argument("--equilibrium", type=int, default=1,
                    help="1: train the equilibrium-exact form P(f) - P(M_f) (the default for "
                         "new networks); 0: the plain form")
    ap.add_argument("--families", default=",".join(FAMILIES),
                    help="comma-separated subset of " + ",".join(FAMILIES))
    ap.add_argument("--check-batch", type=int, default=0,
                    help="also score the network on this many instances of the 0D "
                         "two-Maxwellian workload (workloads.two_maxwellian_batch)")
    # distinct from the benchmark's default seed, so that the workload the
    # benchmark accepts the network on is never the one it was scored on here
    ap.add_argument("--check-seed", type=int, default=97)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    fams = tuple(x for x in a.families.split(",") if x)
    if not fams or any(x not in FAMILIES for x in fams):
        ap.error(f"--families: choose from {','.join(FAMILIES)}")
    torch.cuda.set_device(0)
    v, zeta = grid_0d(a.n, a.lv)
    plan = Plan(a.n, a.lv, v, zeta, 512)
    plan.generate_weights_iso(a.lam)
    plan.autotune(512, FP32)
    t0 = time.time()
    F, Q, _ = make_dataset(plan, a.pairs, seed=a.seed, families=fams)
    # held out: every family, whichever ones the network trains on
    Fe, Qe, fam = make_dataset(plan, a.heldout, seed=a.seed + 10 ** 6, out_dtype=torch.float64)
    Fc = Qc = None
    if a.check_batch > 0:
        from .workloads import two_maxwellian_batch
        Fc = torch.from_numpy(two_maxwellian_batch(v, a.check_batch, a.check_seed)).cuda()
        Qc = torch.empty_like(Fc)
        for i in range(0, a.check_batch, 512):
            b = min(512, a.check_batch - i)
            plan.computeQ_device(Fc[i:i + b], Qc[i:i + b], b, FP32 | CONSERVE)
    t_data = time.time() - t0
    if a.init:
        net = FourierOperator.load(a.init)
    else:
        net = FourierOperator(a.n, a.width, a.modes, a.layers, a.hidden, seed=a.seed,
                              kind=a.kind, precision=a.precision)
        net.output_scale = output_scale(F, Q)
    if a.equilibrium and not net.equilibrium:
        net.set_equilibrium(True, v)
    net.set_loss_floor(a.floor)
    if a.loss_power != 1.0:
        if net.equilibrium:
            ap.error("--loss-power needs --equilibrium 0")
        net.set_loss_power(a.loss_power)
    e0 = evaluate(net, plan, Fe, Qe)
    c0 = evaluate(net, plan, Fc, Qc) if Fc is not None else None
    log = train(net, F, Q, a.steps, batch=a.batch, lr=a.lr, seed=a.seed,
                time_limit=60.0 * a.minutes)
    e1 = evaluate(net, plan, Fe, Qe)
    e1f = evaluate(net, plan, Fe, Qe, floor=a.floor, fam=fam)
    c1 = evaluate(net, plan, Fc, Qc) if Fc is not None else None
    net.save(a.out)

    def stats(e):
        return None if e is None else {"mean": e.mean().item(), "median": e.median().item(),
                                       "max": e.max().item()}
    print(json.dumps({
        "families": list(fams),
        "heldout_by_family_untrained": family_stats(e0, fam),
        "workload_check_untrained": stats(c0),
        "workload_check_trained": stats(c1),
        "pairs": a.pairs, "data_seconds": round(t_data, 1), "steps": log.steps,
        "train_seconds": round(log.seconds, 1), "samples_per_s": log.samples / log.seconds,
        "loss_first_last": [log.losses[0], log.losses[-1]],
        "heldout_rel_l2_untrained": {"mean": e0.mean().item(), "max": e0.max().item()},
        "heldout_rel_l2_trained": {"mean": e1.mean().item(), "median": e1.median().item(),
                                   "max": e1.max().item()},
        "heldout_by_family": family_stats(e1, fam),
        "heldout_by_family_floored": family_stats(e1f, fam),
        "floor": a.floor, "loss_power": a.loss_power, "equilibrium_form": net.equilibrium,
        "out": a.out}))


if __name__ == "__main__":
    main()
