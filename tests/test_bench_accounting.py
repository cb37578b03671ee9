"""CPU checks of the work accounting behind bench.py's roofline figures.

* learned_work: the learned operator's algorithmic bytes per evaluation,
  against an explicit list of every pass of the kernel sequence (what each
  kernel reads and writes once), and the ncu-measured layer-0 traffic.
* The row-pair convolution: its term count against a brute-force count of the
  slots every zeta-row runs, and the scaling of its measured traffic.
* Both arms of the bench describe the same workload.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _passes(N, C, Km, L):
    """(name, bytes) of every tensor read or written once by one evaluation."""
    P = N ** 3
    act = 2 * P * C                       # 16-bit activations [P][C]
    t1 = 2 * N * N * (2 * Km) * C         # after the forward k pass (2 Km real rows)
    t2 = 2 * N * (2 * Km) * Km * C        # after the forward j pass
    xm = 2 * (2 * Km) * Km * Km * C       # the mode block
    out = [("inst_max reads f", 8 * P), ("to_pb reads f", 8 * P), ("to_pb writes x", 4 * P),
           ("lift reads x", 4 * P), ("lift writes H0", act)]
    for layer in range(L):
        out += [(f"{layer}: fwd k reads H", act), (f"{layer}: fwd k writes T1", t1),
                (f"{layer}: fwd j reads T1", t1), (f"{layer}: fwd j writes T2", t2),
                (f"{layer}: fwd i reads T2", t2), (f"{layer}: fwd i writes X", xm),
                (f"{layer}: mix reads X", xm), (f"{layer}: mix writes Y", xm),
                (f"{layer}: inv i reads Y", xm), (f"{layer}: inv i writes U1", t2),
                (f"{layer}: inv j reads U1", t2), (f"{layer}: inv j writes U2", t1),
                (f"{layer}: inv k reads U2", t1), (f"{layer}: inv k writes S", act),
                (f"{layer}: channel mix reads H", act), (f"{layer}: channel mix reads S", act),
                (f"{layer}: channel mix writes H'", act)]
    out += [("readout reads H_L", act), ("readout writes y", 4 * P),
            ("scaling reads y", 4 * P), ("scaling writes Q", 8 * P),
            ("conservation moments read Q", 8 * P), ("projection reads Q", 8 * P),
            ("projection writes Q", 8 * P)]
    return out


@pytest.mark.parametrize("N,C,Km,L,Hd", [(32, 64, 12, 4, 128), (16, 16, 8, 3, 32)])
def test_learned_bytes_match_the_pass_list(N, C, Km, L, Hd):
    w = bench.learned_work(N, C, Km, L, Hd)
    assert w["bytes"] == sum(b for _, b in _passes(N, C, Km, L))
    assert w["channel_mix_bytes"] == 3 * 2 * N ** 3 * C


def test_learned_layer_bytes_match_ncu():
    """ncu, layer 0 at 256 instances:
    9.93 GB over the eight GEMMs of the layer."""
    layer = sum(b for name, b in _passes(32, 64, 12, 4) if name.startswith("0:"))
    measured = 9.93e9 / 256
    assert abs(layer - measured) / measured < 0.05
    # and the channel mix alone, captured at LEARNED_CM_TRAFFIC["B"] instances:
    # the reads equal the algorithmic reads, and part of the 16-bit output is
    # still in L2 when the kernel ends, so DRAM traffic sits a few percent
    # below the algorithmic bytes
    cm = bench.learned_work(32, 64, 12, 4, 128)["channel_mix_bytes"]
    cap = bench.LEARNED_CM_TRAFFIC
    assert 0.9 < cap["bytes"] / (cm * cap["B"]) <= 1.0


@pytest.mark.parametrize("N", [8, 16, 24, 32])
def test_row_pair_term_count(N):
    """5 (N^6 + N^4) flop per instance = 10 flop x the terms the slots run."""
    h = N // 2
    slots = 0
    for zx in range(N):
        for zy in range(N):
            for r in range(N * N):
                sx, sy = (zx + h - r // N) % N, (zy + h - r % N) % N
                slots += (sx * N + sy) >= r
    terms = slots * N * N            # each slot: N zeta_z x N xi_z
    assert 10 * terms == 5 * (N ** 6 + N ** 4)


def test_row_pair_traffic_scaling():
    """The capture at N=24, B=128 scales with the table size N^2 (N^4 + N^2)/2
    and the number of instance groups."""
    t24, cap = bench.scaled_traffic(3, 24, 128, 32, sym=True)
    assert t24 == pytest.approx(cap["bytes"])
    t32, _ = bench.scaled_traffic(3, 32, 1024, 64, sym=True)
    table = lambda n: n ** 2 * (n ** 4 + n ** 2) / 2  # noqa: E731
    assert t32 == pytest.approx(cap["bytes"] / 4 * 16 * table(32) / table(24))
    # every-row capture scales with N^6
    t_all, cap_all = bench.scaled_traffic(3, 32, 1024, 64)
    assert t_all == pytest.approx(cap_all["bytes"] / 4 * 16 * (32 / 24) ** 6)


def test_variant5_traffic_capture():
    """The register-capped variant has its own capture at the headline N
    (N=32, 128 instances in groups of 64): DRAM bytes per launch scale with the
    number of instance groups, and one group reads the 2.15 GB row-pair table
    once, plus the transforms."""
    t128, cap = bench.scaled_traffic(5, 32, 128, 64, sym=True)
    assert cap["N"] == 32 and t128 == pytest.approx(cap["bytes"])
    t1024, _ = bench.scaled_traffic(5, 32, 1024, 64, sym=True)
    assert t1024 == pytest.approx(8 * cap["bytes"])
    table = 32 ** 2 * (32 ** 4 + 32 ** 2) / 2 * 4
    assert 1.0 < cap["bytes"] / (2 * table) < 1.2


def test_both_arms_describe_one_workload():
    c = bench.headline_config(32, 6.0, 1.0, 1024, 1)
    assert c["N"] == 32 and c["batch_per_gpu"] == 1024
    assert "1024 instances per GPU" in c["workload"]
