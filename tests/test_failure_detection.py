"""Failure detection without a GPU fault.

Where the reference calls exit() -- a short weight file (weights.c:83-86), a
missing anisotropic weight file (weights.c:95-97), a singular CC^T
(conserve.c:130-135) -- the library records a status and returns, and the
process survives.  NaN or infinity in f or Q sets the non-finite bit of the
device status word (and the legacy conserveAllMoments reports it).  A bounded
device wait that runs out sets the timeout bit and the kernel returns; the
test makes one run out through the stall test hook: the convolution's first
CTA waits on a barrier that nothing completes, with a short clock limit.

The first three cases fail before any device call, so they run on the CPU.
"""
import ctypes as C
import os

import numpy as np
import pytest

ERR_WEIGHTS, ERR_SINGULAR, ERR_NONFINITE = 4, 5, 8
STATUS_TIMEOUT, STATUS_NONFINITE = 1, 2


def _grid(sb, N=4, L_v=5.0):
    return sb.grid_0d(N, L_v)


def test_short_weight_file_returns_an_error(lib_built, tmp_path, monkeypatch):
    sb = lib_built
    N, L_v, lam = 4, 5.0, 0.0
    v, zeta = _grid(sb, N, L_v)
    monkeypatch.chdir(tmp_path)
    os.makedirs("Weights")
    name = f"Weights/N{N}_isotropic_L_v{L_v:g}_lambda{lam:g}.wts"
    # one row and a half of the N^3 x N^3 table: a truncated cache file
    np.zeros(N ** 3 + N ** 3 // 2).tofile(name)
    ref = sb.ReferenceAPI()
    (table,) = ref.alloc_weights(N)
    ref.initialize_weights(N, zeta, L_v, lam, 0, 0, table)
    L = sb.lib()
    assert L.spectral_last_error() == ERR_WEIGHTS
    assert b"short read" in L.spectral_last_error_message()


def test_missing_anisotropic_weights_return_an_error(lib_built, tmp_path, monkeypatch):
    sb = lib_built
    N, L_v = 4, 5.0
    v, zeta = _grid(sb, N, L_v)
    monkeypatch.chdir(tmp_path)
    os.makedirs("Weights")
    ref = sb.ReferenceAPI()
    (table,) = ref.alloc_weights(N)
    ref.initialize_weights(N, zeta, L_v, 0.0, 0, 1, table)   # isoFlag = 1, no file
    L = sb.lib()
    assert L.spectral_last_error() == ERR_WEIGHTS
    assert b"not found" in L.spectral_last_error_message()


def test_singular_conservation_matrix_returns_an_error(lib_built):
    """A species of mass 0 zeroes every row of C, so CC^T = 0.  The reference's
    pivot test sees 0/0 there; the library reports the matrix as singular."""
    sb = lib_built
    N, L_v = 4, 5.0
    v, _ = _grid(sb, N, L_v)
    ref = sb.ReferenceAPI()
    ref.initialize_conservation(N, v[1] - v[0], v, masses=(0.0,))
    L = sb.lib()
    assert L.spectral_last_error() == ERR_SINGULAR
    assert b"singular" in L.spectral_last_error_message()


# ----------------------------------------------------------------- GPU ---
def _bkw_batch(v, B, seed):
    from spectralbte_gb300 import workloads as wl
    rng = np.random.default_rng(seed)
    f = wl.bkw(v, 0.65)
    return np.stack([f * (1 + 0.05 * rng.uniform(-1, 1, f.size)) for _ in range(B)])


@pytest.mark.gpu
def test_plan_conservation_with_mass_zero_is_singular(gpu):
    sb = gpu
    N, L_v = 8, 5.0
    v, zeta = _grid(sb, N, L_v)
    plan = sb.Plan(N, L_v, v, zeta, 2)
    rc = plan.L.spectral_plan_set_conservation(plan.h, C.c_double(0.0))
    assert rc == ERR_SINGULAR
    assert rc == plan.L.spectral_plan_set_conservation(plan.h, C.c_double(0.0))
    assert plan.L.spectral_plan_set_conservation(plan.h, C.c_double(1.0)) == 0
    plan.close()


@pytest.mark.gpu
def test_nan_in_f_sets_the_nonfinite_status(gpu):
    import torch
    sb = gpu
    N, L_v, B = 8, 5.0, 3
    v, zeta = _grid(sb, N, L_v)
    plan = sb.Plan(N, L_v, v, zeta, B)
    plan.generate_weights_iso(0.0)
    f = _bkw_batch(v, B, 5)
    fd = torch.from_numpy(f).cuda()
    Qd = torch.empty_like(fd)
    for flags in (sb.FP64 | sb.CONSERVE, sb.FP32 | sb.CONSERVE,
                  sb.FP32 | sb.MAXPRESERVE | sb.CONSERVE):
        assert plan.status() == 0
        bad = fd.clone()
        bad[1, 17] = float("nan")
        plan.computeQ_device(bad, Qd, B, flags)
        torch.cuda.synchronize()
        assert plan.status() & STATUS_NONFINITE, flags
        assert plan.status() == 0          # the read clears it
        plan.computeQ_device(fd, Qd, B, flags)   # the plan stays usable
        torch.cuda.synchronize()
        assert torch.isfinite(Qd).all()
        assert plan.status() == 0
    # the output moments of an infinite f
    bad = fd.clone()
    bad[0, 3] = float("inf")
    mom = torch.empty((B, 8), dtype=torch.float64, device="cuda")
    plan.moments_device(bad, B, mom)
    torch.cuda.synchronize()
    assert plan.status() & STATUS_NONFINITE
    plan.close()


@pytest.mark.gpu
def test_nan_in_a_weight_file_is_reported_by_conserveAllMoments(gpu, tmp_path, monkeypatch):
    """A weight cache of the right size whose values are corrupt (one NaN):
    the legacy path loads it, ComputeQ carries the NaN into Q, and
    conserveAllMoments reports non-finite moments instead of conserving NaN."""
    sb = gpu
    N, L_v, lam = 8, 5.0, 0.0
    v, zeta = _grid(sb, N, L_v)
    monkeypatch.chdir(tmp_path)
    os.makedirs("Weights")
    from oracle import pyoracle as po
    g = po.Grid(N, L_v, "0d")
    W = po.weights_iso(g, lam)
    W[5, 9] = np.nan
    W.tofile(f"Weights/N{N}_isotropic_L_v{L_v:g}_lambda{lam:g}.wts")
    ref = sb.ReferenceAPI()
    ref.initialize_coll(N, L_v, v, zeta)
    ref.initialize_conservation(N, v[1] - v[0], v)
    (table,) = ref.alloc_weights(N)
    ref.initialize_weights(N, zeta, L_v, lam, 0, 0, table)
    f = _bkw_batch(v, 1, 9)[0]
    Q = ref.ComputeQ(f, None, table)
    assert not np.isfinite(Q).all()
    ref.conserveAllMoments([Q])
    L = sb.lib()
    assert L.spectral_last_error() == ERR_NONFINITE
    assert b"non-finite" in L.spectral_last_error_message()
    # a finite Q conserves as before
    W2 = po.weights_iso(g, lam)
    Q2 = po.computeQ(g, W2, f)
    (Qc,) = ref.conserveAllMoments([Q2])
    assert np.isfinite(Qc).all()
    ref.dealloc_weights(N, table)


@pytest.mark.gpu
@pytest.mark.parametrize("slot", [0, 5])
def test_bounded_wait_times_out_and_the_plan_stays_usable(gpu, slot):
    """The stall hook makes the first CTA of the next FP32 convolution skip
    one pipeline slot's copies; that CTA's waits give up after 1e5 clocks
    (about 50 us), set the timeout bit and return.  The call completes, and
    the next call without the hook equals an earlier clean call bit for bit."""
    import torch
    sb = gpu
    N, L_v, B = 16, 5.0, 40
    v, zeta = _grid(sb, N, L_v)
    plan = sb.Plan(N, L_v, v, zeta, B)
    plan.generate_weights_iso(1.0)
    plan.set_tuning(32, 3, 16, variant=3, zs=8)
    fd = torch.from_numpy(_bkw_batch(v, B, 11)).cuda()
    Q0 = torch.empty_like(fd)
    Q1 = torch.empty_like(fd)
    plan.computeQ_device(fd, Q0, B, sb.FP32 | sb.CONSERVE)
    torch.cuda.synchronize()
    assert plan.status() == 0
    plan.inject_stall(slot, 100_000)
    plan.computeQ_device(fd, Q1, B, sb.FP32 | sb.CONSERVE)
    torch.cuda.synchronize()
    st = plan.status()
    assert st & STATUS_TIMEOUT, st
    plan.computeQ_device(fd, Q1, B, sb.FP32 | sb.CONSERVE)
    torch.cuda.synchronize()
    assert plan.status() == 0
    assert torch.equal(Q0, Q1)
    plan.close()


@pytest.mark.gpu
def test_stall_hook_rejects_bad_limits(gpu):
    sb = gpu
    N, L_v = 8, 5.0
    v, zeta = _grid(sb, N, L_v)
    plan = sb.Plan(N, L_v, v, zeta, 1)
    for slot, limit in ((0, 10), (-1, 100_000), (0, 1 << 40)):
        with pytest.raises(sb.SpectralError):
            plan.inject_stall(slot, limit)
    plan.close()
