"""Host-side checks of the symmetric (row-pair) form of the FP32 convolution.

The weighted sum of compute_Qhat (collisions.c:141-163),
    qhat[zeta] = sum_xi W[zeta][xi] ghat[xi] fhat[s(zeta, xi)],
    s_a = (zeta_a + N/2 - xi_a) mod N per axis,
is run on the GPU over xi-row pairs (r, s(r)) with pre-summed weight tiles
when g = f.  These tests restate the kernel's slot enumeration and the
builder of the summed tiles in numpy and check, on the CPU:
  * the closed-form slot count the kernel runs against a brute-force count;
  * that the row-pair sum equals the plain sum for Q(f,f) and for the
    maxPreserve form sum W [ghat fhat[s] + Mhat ghat[s]] with fhat = Mhat +
    ghat, in FP64, at N = 8 and 6.
"""
import numpy as np
import pytest


def sym_slots(N, zx, zy):
    """Slots per zeta-row, as the kernels' sym_slots computes them."""
    h = N // 2
    return (N * N) // 2 + (2 if ((zx + h) % 2 == 0 and (zy + h) % 2 == 0) else 0)


def partner(N, zx, zy, r):
    h = N // 2
    return ((zx + h - r // N) % N) * N + (zy + h - r % N) % N


def run_rows(N, zx, zy):
    """Rows a zeta-row runs, in the producer's order."""
    return [r for r in range(N * N) if partner(N, zx, zy, r) >= r]


@pytest.mark.parametrize("N", [6, 8, 16, 24, 32])
def test_slot_count_matches_enumeration(N):
    for zx in range(N):
        for zy in range(N):
            rows = run_rows(N, zx, zy)
            assert len(rows) == sym_slots(N, zx, zy)
            # every row is run itself or through its partner, exactly once
            seen = set(rows) | {partner(N, zx, zy, r) for r in rows}
            assert seen == set(range(N * N))


def plain_sum(W, P, R, N):
    """qhat[zeta] = sum_xi W[zeta][xi] P[xi] R[s(zeta, xi)] (collisions.c:141-163)."""
    n3 = N ** 3
    h = N // 2
    idx = np.arange(n3)
    x, y, z = idx // (N * N), (idx // N) % N, idx % N
    out = np.zeros(n3, complex)
    for zeta in range(n3):
        zi, zj, zk = zeta // (N * N), (zeta // N) % N, zeta % N
        s = ((zi + h - x) % N) * N * N + ((zj + h - y) % N) * N + (zk + h - z) % N
        out[zeta] = np.sum(W[zeta] * P * R[s])
    return out


def sym_tables(W, N):
    """Wsym[zrow][slot][zz][xz] of the builder (weights_to_sym_f32), FP64."""
    n3, nn, h = N ** 3, N * N, N // 2
    ms = nn // 2 + 2
    T = np.zeros((nn, ms, N, N))
    for zrow in range(nn):
        zx, zy = zrow // N, zrow % N
        for slot, r in enumerate(run_rows(N, zx, zy)):
            sr = partner(N, zx, zy, r)
            for zz in range(N):
                zeta = zrow * N + zz
                for xz in range(N):
                    w = W[zeta, r * N + xz]
                    if sr != r:
                        w += W[zeta, sr * N + (zz + h - xz) % N]
                    T[zrow, slot, zz, xz] = w
    return T


def sym_sum(T, P, R, N, S=None, Tw=None):
    """The kernel's loop: per zeta-row, per run slot, the row r of P (and S)
    against the window of its partner row of R (and Tw)."""
    nn, h = N * N, N // 2
    out = np.zeros(N ** 3, complex)
    for zrow in range(nn):
        zx, zy = zrow // N, zrow % N
        for slot, r in enumerate(run_rows(N, zx, zy)):
            sr = partner(N, zx, zy, r)
            for zz in range(N):
                xz = np.arange(N)
                win = sr * N + (zz + h - xz) % N
                prod = P[r * N + xz] * R[win]
                if S is not None:
                    prod = prod + S[r * N + xz] * Tw[win]
                out[zrow * N + zz] += np.sum(T[zrow, slot, zz] * prod)
    return out


def _random(N, seed):
    rng = np.random.default_rng(seed)
    n3 = N ** 3
    W = rng.standard_normal((n3, n3))
    cplx = lambda: rng.standard_normal(n3) + 1j * rng.standard_normal(n3)  # noqa: E731
    return W, cplx(), cplx()


@pytest.mark.parametrize("N", [6, 8])
def test_row_pair_sum_equals_plain_sum(N):
    W, fhat, Mhat = _random(N, 3 + N)
    T = sym_tables(W, N)
    ref = plain_sum(W, fhat, fhat, N)
    got = sym_sum(T, fhat, fhat, N)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    # maxPreserve form: P = ghat, R = fhat = Mhat + ghat, S = Mhat, T = ghat
    ghat = fhat
    fsum = Mhat + ghat
    ref2 = plain_sum(W, ghat, fsum, N) + plain_sum(W, Mhat, ghat, N)
    got2 = sym_sum(T, ghat, fsum, N, S=Mhat, Tw=ghat)
    assert np.abs(got2 - ref2).max() <= 1e-12 * np.abs(ref2).max()


def test_row_pair_sum_needs_g_equal_f():
    """With g != f the pair products differ, and the row-pair form is wrong:
    the library uses it only for its g = f calls."""
    N = 6
    W, fhat, ghat = _random(N, 11)
    T = sym_tables(W, N)
    ref = plain_sum(W, ghat, fhat, N)
    got = sym_sum(T, ghat, fhat, N)
    assert np.abs(got - ref).max() > 1e-3 * np.abs(ref).max()
