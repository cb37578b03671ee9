"""Pin the CPU oracle to the reference's own golden data (CPU only).

* The two shipped .wts fixtures (tests/BKW8/target, tests/heat_transport/
  target of the reference), stored subsampled with full-array checksums in
  golden_w_n8.npz.  The reference produced them with GSL's adaptive
  quadrature and diffs them byte for byte (run_test.sh:41-53).  A
  reimplementation can match only to round-off, so the bar here is
  rel-L2 <= 1e-13.
* Outputs of the reference's own collisions.c / conserve.c, compiled here
  with stand-in FFT/GSL/MPI, in golden_q.npz (make_golden.py).  The oracle
  must match these bit for bit, within 1e-14 for safety.
* The reference's BKW8 golden moment table (moments_BKW8.test.in), to
  every printed digit.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_case, rel_l2

CASES = ["bkw8", "heat8", "n6", "n7", "n16"]


def _weights(po, G, name):
    N, L_v, kind, lam = golden_case(G, name)
    g = po.Grid(N, L_v, kind)
    return g, po.weights_iso(g, lam)


@pytest.mark.parametrize("tag,L_v,kind,lam", [("bkw8", 5.0, "0d", 0.0),
                                              ("heat", 9.0, "1d", 1.0)])
def test_weights_match_reference_fixture(oracle, golden_w, tag, L_v, kind, lam):
    g = oracle.Grid(8, L_v, kind)
    W = oracle.weights_iso(g, lam)
    rows = golden_w[f"{tag}_row_index"]
    assert rel_l2(W[rows], golden_w[f"{tag}_rows"]) < 1e-13
    # full-array checksums of the fixture
    assert abs(W.sum() - golden_w[f"{tag}_sum"]) <= 1e-12 * golden_w[f"{tag}_abssum"]
    assert abs((W * W).sum() / golden_w[f"{tag}_sumsq"] - 1) < 1e-13


@pytest.mark.parametrize("name", CASES)
def test_fft_matches_reference(oracle, golden_q, name):
    N, L_v, kind, _ = golden_case(golden_q, name)
    g = oracle.Grid(N, L_v, kind)
    f = golden_q[name + "_f"]
    fh = oracle.fft3d(g, f, 0)
    assert rel_l2(fh, golden_q[name + "_fhat"]) < 1e-14
    assert rel_l2(oracle.fft3d(g, fh, 1), golden_q[name + "_finv"]) < 1e-14


@pytest.mark.parametrize("name", CASES)
def test_computeQ_matches_reference(oracle, golden_q, name):
    g, W = _weights(oracle, golden_q, name)
    f = golden_q[name + "_f"]
    Q = oracle.computeQ(g, W, f)
    assert rel_l2(Q, golden_q[name + "_Q"]) < 1e-13
    Qmp = oracle.computeQ_maxPreserve(g, W, f)
    assert rel_l2(Qmp, golden_q[name + "_Qmp"]) < 1e-13
    cons = oracle.Conservation(g)
    assert rel_l2(cons(Q), golden_q[name + "_Qc"]) < 1e-13
    assert rel_l2(cons(Qmp), golden_q[name + "_Qmpc"]) < 1e-13


def _moments5(g, Q, absolute=False):
    """The five conserved moments of Q (conserve.c:217-239); with
    absolute=True the sums of absolute terms (their natural scale)."""
    v = g.v
    dv = v[1] - v[0]
    wt = np.ones(g.N)
    wt[0] = wt[-1] = 0.5
    w3 = (wt[:, None, None] * wt[None, :, None] * wt[None, None, :]) * dv ** 3
    vx = v[:, None, None]
    vy = v[None, :, None]
    vz = v[None, None, :]
    q = Q.reshape(g.N, g.N, g.N)
    if absolute:
        q = np.abs(q)
        vx, vy, vz = np.abs(vx), np.abs(vy), np.abs(vz)
    return np.array([(w3 * q).sum(), (w3 * vx * q).sum(), (w3 * vy * q).sum(),
                     (w3 * vz * q).sum(),
                     (w3 * 0.5 * (vx ** 2 + vy ** 2 + vz ** 2) * q).sum()])


@pytest.mark.parametrize("name", CASES)
def test_conservation_known_answer(oracle, golden_q, name):
    """After conserveAllMoments the five moments of Q vanish to round-off."""
    N, L_v, kind, _ = golden_case(golden_q, name)
    g = oracle.Grid(N, L_v, kind)
    Qc = oracle.Conservation(g)(golden_q[name + "_Q"])
    scale = _moments5(g, golden_q[name + "_Q"], absolute=True)
    assert np.all(np.abs(_moments5(g, Qc)) <= 1e-13 * scale)


def test_bkw8_golden_moments(oracle):
    """The BKW8 regression of the reference (0D, maxPreserve, RK2,
    dt = 0.01, 100 steps) to every printed digit (%le)."""
    g = oracle.Grid(8, 5.0, "0d")
    W = oracle.weights_iso(g, 0.0)
    rows = oracle.run_0d(8, 5.0, W, oracle.init_bkw(g), 0.01, 1.0, 100, 2, True)
    want = np.loadtxt(os.path.join(GOLDEN, "moments_BKW8.txt"))
    printed = np.array([[float("%e" % x) for x in r] for r in rows])
    cols = [c for c in range(want.shape[1]) if c != 2]  # u_x is round-off noise
    assert np.array_equal(printed[:, cols], want[:, cols])
    assert np.abs(rows[:, 2]).max() < 1e-15


def test_gauss_legendre(oracle):
    x, w = oracle.gauss_legendre(16)
    assert abs(w.sum() - 2) < 1e-14
    # exact for x^30
    assert abs((w * x ** 30).sum() - 2 / 31) < 1e-14


def test_heat_transport_golden_moments(oracle):
    """The heat_transport regression of the reference (1D, 250 cells, N=8,
    L_v=9, lambda=1, Kn=3.2, first-order upwind between diffuse walls at
    T=1 and T=2, dt=1e-4, 10 steps).  x, density, temperature and pressure
    match to every printed digit.  u_x is round-off noise (~1e-15) in the
    interior, where it depends on the last bits of W; the wall cells carry
    a real velocity, which matches to the printed precision."""
    r = oracle.Run1D(8, 9.0, 250, 1, 3, 1e-4, 3.2)
    W = oracle.weights_iso(r.g, 1.0)
    rows = r.run(W, r.init(), 10)
    want = np.loadtxt(os.path.join(GOLDEN, "moments_heat_transport.txt")).reshape(11, 250, 6)
    printed = np.vectorize(lambda x: float("%e" % x))(rows)
    for c in (0, 1, 2, 4, 5):
        assert np.array_equal(printed[..., c], want[..., c]), c
    ux, wux = rows[..., 3], want[..., 3]
    real = np.abs(wux) > 1e-10
    assert real.sum() > 10
    assert np.all(np.abs(ux[real] - wux[real]) <= 1e-6 * np.abs(wux[real]))
    assert np.all(np.abs(ux[~real] - wux[~real]) < 1e-13)


def test_landau_weights_match_reference(oracle):
    """The oracle's gHat3L restatement against the reference's own
    initialize_weights_AnIso (aniso_weights.c, Landau kernel), N = 4 and 5."""
    import os
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "golden_landau.npz"))
    for name in ("n4", "n5", "g4"):
        N, L_v, lam, _glance = d[f"{name}_meta"]
        W = oracle.weights_landau(int(N), d[f"{name}_zeta"], L_v, lam)
        ref = d[f"{name}_W"]
        assert np.abs(W - ref).max() <= 1e-13 * np.abs(ref).max(), name


def test_landau_weights_ignore_glance_in_reference():
    """The reference's generator branches on a file-scope glance that its
    parameter shadows (aniso_weights.c:31,37,417), so glance = 0.3 gives the
    Landau weights under the *_glance0.3.wts name (:68)."""
    import os
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "golden_landau.npz"))
    assert d["g4_meta"][3] == 0.3
    assert np.array_equal(d["g4_W"], d["n4_W"])
    assert str(d["g4_file"]) == "Weights/N4_AnIso_L_v4_lambda0_glance0.3.wts"
    assert str(d["n4_file"]) == "Weights/N4_Aniso_L_v4_lambda0_Landau.wts"


@pytest.mark.parametrize("tag,L_v,kind,lam", [("bkw8", 5.0, "0d", 0.0),
                                              ("heat", 9.0, "1d", 1.0)])
def test_closed_form_weights_match_reference_fixture(oracle, golden_w, tag, L_v, kind, lam):
    """The radial integral of ghat (weights.c:156-160) in closed form for
    lambda = 0 and 1 against the reference's own .wts fixtures (the same
    bounds as the quadrature) and against the quadrature itself."""
    g = oracle.Grid(8, L_v, kind)
    W = oracle.weights_iso(g, lam, closed=True)
    rows = golden_w[f"{tag}_row_index"]
    assert rel_l2(W[rows], golden_w[f"{tag}_rows"]) < 1e-13
    assert abs(W.sum() - golden_w[f"{tag}_sum"]) <= 1e-12 * golden_w[f"{tag}_abssum"]
    assert abs((W * W).sum() / golden_w[f"{tag}_sumsq"] - 1) < 1e-13
    assert rel_l2(W, oracle.weights_iso(g, lam)) < 1e-14


@pytest.mark.parametrize("N,L_v,lam", [(16, 5.0, 0.0), (24, 6.0, 1.0), (32, 6.0, 1.0)])
def test_closed_form_weights_match_quadrature_rows(oracle, N, L_v, lam):
    """Sampled rows at the bench grids: closed form against the converged
    composite Gauss-Legendre quadrature."""
    g = oracle.Grid(N, L_v, "0d")
    n3 = N ** 3
    for r0 in (0, n3 // 2 + N // 3, n3 - 2):
        a = oracle.weights_iso(g, lam, rows=(r0, r0 + 2), closed=True)
        b = oracle.weights_iso(g, lam, rows=(r0, r0 + 2))
        assert rel_l2(a, b) < 1e-13, r0


def test_closed_form_limits():
    """Exact zero arguments, the small-argument loss series, and a lambda
    without a closed form (quadrature) against the quadrature."""
    from oracle import pyoracle as po
    L = po.lib()
    cases = [(0.0, 0.0, 0.0), (0.0, 0.4, 0.9), (0.8, 0.0, 0.6), (0.4, 1.3, 0.0),
             (0.55, 0.01, 0.55), (0.3, 0.7, 1.1), (2.0, 3.0, 1.7), (0.02, 0.3, 0.5)]
    for lam in (0.0, 1.0, 0.5):
        for a0, a1, a2 in cases:
            q = L.oracle_ghat_integral(a0, a1, a2, lam, 6.0)
            c = L.oracle_ghat_closed(a0, a1, a2, lam, 6.0)
            assert abs(c - q) <= 1e-13 * max(abs(q), 1.0), (lam, a0, a1, a2, q, c)
