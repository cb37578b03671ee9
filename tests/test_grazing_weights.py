"""Grazing-collision weights: gHat3 of the reference's stand-alone generator
(exec/MPIcollisionRoutines.c:33-205, driven by exec/MPIWeightGenerator.c).

The reference integrates with GSL QAG (r, phi) and CQUAD (theta) to a
tolerance of 1e-6, and no GSL exists here, so parity with the reference's
numbers is not pinned.  The oracle (oracle/spectral_oracle.c) restates the
integrals with composite Gauss-Legendre rules; these CPU tests show that its
rules are converged (doubling every panel count changes a weight by
< 1e-11 relative) and that grouping the table by (|zeta|^2, zeta.xi, |xi|^2)
only merges entries with equal arguments.  The GPU tests compare the
library's kernel with the oracle: every entry within 1e-10 relative at
N = 4, 6, and at N = 8 on a sample of the distinct entries; and the
generator entry point writes the reference's file name, which
initialize_weights_AnIso then loads.
"""
import ctypes as C
import os

import numpy as np
import pytest

TOL = 1e-10


def generator_grid(N, L_v):
    """eta of MPIWeightGenerator.c:63-74."""
    h_v = 2.0 * L_v / (N - 1)
    h_eta = (2.0 * np.pi / N) / h_v
    return -0.5 * N * h_eta + h_eta * np.arange(N)


def test_oracle_rules_are_converged(oracle):
    L = oracle.lib()
    N, L_v = 8, 5.0
    eta = generator_grid(N, L_v)
    npan = L.oracle_graze_panels(float(np.abs(eta).max()), L_v)
    rng = np.random.default_rng(3)
    for glance, lam in ((0.1, 0.0), (0.01, 1.0)):
        for _ in range(3):
            z = eta[rng.integers(0, N, 3)]
            x = eta[rng.integers(0, N, 3)]
            a = L.oracle_ghat3_graze(*z, *x, L_v, lam, glance, npan)
            b = L.oracle_ghat3_graze(*z, *x, L_v, lam, glance, 2 * npan)
            assert abs(a - b) <= 1e-11 * abs(b), (glance, lam, a, b)


def test_grouping_merges_only_equal_arguments(oracle):
    N, L_v = 6, 4.0
    eta = generator_grid(N, L_v)
    pairs, inverse = oracle.graze_unique(N, eta)
    n3 = N ** 3
    idx = np.stack(np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij"),
                   -1).reshape(-1, 3)
    Z = eta[idx]
    zz = (Z * Z).sum(1)
    zx = Z @ Z.T
    key = np.stack([np.broadcast_to(zz[:, None], (n3, n3)), zx,
                    np.broadcast_to(zz[None, :], (n3, n3))], -1).reshape(-1, 3)
    rz, rx = pairs[:, :3], pairs[:, 3:]
    rep = np.stack([(rz * rz).sum(1), (rz * rx).sum(1), (rx * rx).sum(1)], -1)
    assert len(pairs) < n3 * n3 / 10
    assert np.abs(key - rep[inverse]).max() <= 1e-12 * np.abs(key).max()


@pytest.mark.gpu
@pytest.mark.parametrize("N,L_v,lam,glance", [(4, 4.0, 0.0, 0.1), (6, 5.0, 1.0, 0.05)])
def test_gpu_grazing_weights_match_oracle(gpu, oracle, N, L_v, lam, glance):
    sb = gpu
    eta = generator_grid(N, L_v)
    v = np.linspace(-L_v, L_v, N)
    plan = sb.Plan(N, L_v, v, eta, 1)
    plan.generate_weights_grazing(lam, glance)
    W = plan.get_weights()
    want = oracle.weights_graze(N, eta, L_v, lam, glance)
    plan.close()
    assert np.isfinite(W).all()
    assert np.abs(W - want).max() <= TOL * np.abs(want).max()
    assert np.linalg.norm(W - want) <= TOL * np.linalg.norm(want)


@pytest.mark.gpu
def test_gpu_grazing_weights_n8_sample(gpu, oracle):
    sb = gpu
    N, L_v, lam, glance = 8, 5.0, 1.0, 0.01
    eta = generator_grid(N, L_v)
    v = np.linspace(-L_v, L_v, N)
    plan = sb.Plan(N, L_v, v, eta, 1)
    plan.generate_weights_grazing(lam, glance)
    W = plan.get_weights().reshape(-1)
    plan.close()
    pairs, inverse = oracle.graze_unique(N, eta)
    npan = oracle.lib().oracle_graze_panels(float(np.abs(eta).max()), L_v)
    rng = np.random.default_rng(8)
    pick = rng.choice(len(pairs), 400, replace=False)
    want = oracle.weights_graze(N, eta, L_v, lam, glance, (pairs[pick], npan))
    # the table entries of each picked distinct pair all hold its value
    first = np.array([np.flatnonzero(inverse == u)[0] for u in pick])
    got = W[first]
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= TOL * scale
    for u, w in zip(pick[:20], want[:20]):
        assert np.abs(W[inverse == u] - w).max() <= TOL * scale


@pytest.mark.gpu
def test_generator_writes_the_file_initialize_weights_aniso_loads(gpu, oracle, tmp_path,
                                                                   monkeypatch):
    """spectral_weights_generator(N, glance, beta, lambda, L_v) writes
    Weights/N%d_AnIso_L_v%g_lambda%g_glance%g.wts (MPIWeightGenerator.c:79-83)
    with the grazing weights; initialize_weights_AnIso with that glance loads
    them (not the Landau weights it would generate without the file); a
    second generator call leaves the file as it is."""
    sb = gpu
    N, L_v, lam, glance = 4, 4.0, 0.0, 0.1
    monkeypatch.chdir(tmp_path)
    os.makedirs("Weights")
    L = sb.lib()
    assert L.spectral_weights_generator(N, glance, 1.0, lam, L_v) == 0
    name = f"Weights/N{N}_AnIso_L_v{L_v:g}_lambda{lam:g}_glance{glance:g}.wts"
    assert os.path.exists(name)
    eta = generator_grid(N, L_v)
    Wf = np.fromfile(name).reshape(N ** 3, N ** 3)
    want = oracle.weights_graze(N, eta, L_v, lam, glance)
    assert np.abs(Wf - want).max() <= TOL * np.abs(want).max()
    mtime = os.path.getmtime(name)
    assert L.spectral_weights_generator(N, glance, 1.0, lam, L_v) == 0
    assert os.path.getmtime(name) == mtime
    ref = sb.ReferenceAPI()
    (table,) = ref.alloc_weights(N)
    ref.initialize_weights_AnIso(N, eta, L_v, lam, 0, table, glance)
    Wl = ref.table_to_numpy(table, N)
    assert np.array_equal(Wl, Wf)
    landau = oracle.weights_landau(N, eta, L_v, lam)
    assert np.linalg.norm(Wl - landau) > 1e-3 * np.linalg.norm(landau)
    ref.dealloc_weights(N, table)
    # glance = 0: the Landau weights under the Landau file name
    assert L.spectral_weights_generator(N, 0.0, 1.0, lam, L_v) == 0
    Wlan = np.fromfile(f"Weights/N{N}_Aniso_L_v{L_v:g}_lambda{lam:g}_Landau.wts")
    assert np.abs(Wlan.reshape(landau.shape) - landau).max() <= 1e-12 * np.abs(landau).max()


@pytest.mark.gpu
def test_grazing_rejects_bad_arguments(gpu):
    sb = gpu
    N, L_v = 4, 4.0
    eta = generator_grid(N, L_v)
    plan = sb.Plan(N, L_v, np.linspace(-L_v, L_v, N), eta, 1)
    for glance in (0.0, -0.1, 3.0):
        with pytest.raises(sb.SpectralError):
            plan.generate_weights_grazing(0.0, glance)
    plan.close()
