"""GPU tests of the bidiagonal SVD route of split (svd method 4) against the oracle's LAPACK dgesvd
split at the size of the benchmark's centre bond.

The two-site tensor has the U(1) block structure of the centre bond of the L=100 XXZ chain at chi=2048
(45 centre charges, sector matrices up to ~460 x 460, 1.3 M entries) and a prescribed spectrum: each
centre sector is U diag(s) V^T with random orthogonal U, V and s log-uniform in [1e-16, 1], so the
global top-chi cut falls among densely spaced values near 1e-9, where a Gram-matrix route cannot
resolve them.  The
split must keep the oracle's block structure exactly (chi, sectors, kept count per sector), every
kept value to 1e-13 (absolute, values <= 1), the truncated weight, and orthonormal U and V^T whose
columns / rows agree with the oracle's up to the sensitivity eps / gap of each singular vector.
"""
import numpy as np
import pytest

from mpstools_gb300 import api, lib, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _theta(N, chi, seed, lo=-16.0, c=None, chi_right=None):
    """Blocks (a, b, s1, s2) of a two-site tensor on sites (c, c+1) of an N-site spin-1/2 chain (Sz = 0,
    bond dimension chi, chi_right on the right bond; default the centre) with a log-uniform spectrum in
    every centre-charge sector."""
    c = N // 2 - 1 if c is None else c
    left = M.bond_sectors(N, N // 2, chi)[c]
    right = M.bond_sectors(N, N // 2, chi_right or chi)[c + 2]
    rng = np.random.default_rng(seed)
    th = {}
    for q in sorted(set(a + s for a in left for s in (0, 1))):
        rows = [(q - s1, s1) for s1 in (0, 1) if (q - s1) in left]
        cols = [(q + s2, s2) for s2 in (0, 1) if (q + s2) in right]
        if not rows or not cols:
            continue
        m = sum(left[a] for a, _ in rows)
        n = sum(right[b] for b, _ in cols)
        k = min(m, n)
        U = np.linalg.qr(rng.standard_normal((m, k)))[0]
        V = np.linalg.qr(rng.standard_normal((n, k)))[0]
        s = np.sort(10.0 ** rng.uniform(lo, 0.0, k))[::-1]
        Mq = (U * s) @ V.T
        r0 = 0
        for a, s1 in rows:
            c0 = 0
            for b, s2 in cols:
                th[(a, b, s1, s2)] = Mq[r0:r0 + left[a], c0:c0 + right[b]].copy()
                c0 += right[b]
            r0 += left[a]
    return th


def _rows_by_centre(V):
    g = {}
    for (qc, b, s), v in sorted(V.items()):
        g.setdefault(qc, []).append(v)
    return {q: np.hstack(x) for q, x in g.items()}


def _cols_by_centre(U):
    g = {}
    for (a, qc, s), u in sorted(U.items(), key=lambda t: (t[0][1], t[0][2])):
        g.setdefault(qc, []).append(u)
    return {q: np.vstack(x) for q, x in g.items()}


@pytest.mark.parametrize("N,chi,chimax,site,chi_right",
                         [(100, 2048, 2048, None, None), (40, 512, 400, None, None), (100, 2048, 2048, 11, 1024)])
def test_bidiag_split_matches_dgesvd_at_the_centre_bond(ctx, N, chi, chimax, site, chi_right):
    """Sites (11, 12) with bond dimensions 2048 | 1024: tall sector matrices up to 924 x 460 (as in a
    converged chi = 2048 sweep near the chain ends), too large for the shared-memory bidiagonalisation
    of a 16-CTA cluster; they run on its global-memory variant."""
    th = _theta(N, chi, seed=11, c=site, chi_right=chi_right)
    ik = M.u1_itokeys(N)[0]
    U0, V0, l0, tw0, chi0 = O.split(th, ik, ik, chimax, nthreads=8)
    ctx.set_svd_method("bidiag")
    f0 = ctx.L.mpsg_split_fallbacks()
    try:
        U1, V1, l1, tw1, chi1 = api.split(th, (ik, ik), chimax, ctx=ctx)
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)
    assert ctx.L.mpsg_split_fallbacks() == f0
    assert chi1 == chi0
    assert chi0 == chimax or site is not None  # the tall case has fewer than chimax values above 1e-15
    assert set(l1) == set(l0)
    assert {q: len(v) for q, v in l1.items()} == {q: len(v) for q, v in l0.items()}
    assert set(U1) == set(U0) and set(V1) == set(V0)
    err = max(np.abs(np.asarray(l1[q]) - np.asarray(l0[q])).max() for q in l0 if len(l0[q]))
    assert err <= 1e-13, err
    assert abs(tw1 - tw0) <= 1e-13 * max(1.0, abs(tw0))  # tw = 1 - sum of kept s^2 (unnormalised here)
    # orthonormality and agreement of the singular vectors (FixPhase fixes the signs)
    Ug, Uo = _cols_by_centre(U1), _cols_by_centre(U0)
    Vg, Vo = _rows_by_centre(V1), _rows_by_centre(V0)
    worst = 0.0
    for q in l0:
        lam = np.asarray(l0[q])
        if not len(lam):
            continue
        assert np.abs(Ug[q].T @ Ug[q] - np.eye(len(lam))).max() < 1e-12
        assert np.abs(Vg[q] @ Vg[q].T - np.eye(len(lam))).max() < 1e-12
        # sensitivity of singular vector j: eps * s_max / (gap to its neighbours), s_max <= 1
        gaps = np.full(len(lam), np.inf)
        d = np.abs(np.diff(lam))
        gaps[:-1] = np.minimum(gaps[:-1], d)
        gaps[1:] = np.minimum(gaps[1:], d)
        tol = 1e-9 + 64 * np.finfo(float).eps / np.maximum(gaps, 1e-300)
        du = np.abs(Ug[q] - Uo[q]).max(axis=0)
        dv = np.abs(Vg[q] - Vo[q]).max(axis=1)
        worst = max(worst, float(np.max(np.maximum(du, dv) / tol)))
    assert worst <= 1.0, worst


def test_bidiag_split_weight_truncation_and_tiny_sectors(ctx):
    """doTrunc with a truncated-weight bound, sectors of one row or one column, a zero sector."""
    rng = np.random.default_rng(3)
    th = {(0, 0, 0, 0): rng.standard_normal((1, 7)), (1, 1, 0, 0): rng.standard_normal((9, 1)),
          (2, 2, 0, 0): 1e-3 * rng.standard_normal((30, 25)), (3, 3, 0, 0): np.zeros((4, 5)),
          (4, 4, 0, 0): rng.standard_normal((60, 61))}
    ik = [0, 0]
    U0, V0, l0, tw0, chi0 = O.split(th, ik, ik, 1000, doTrunc=True, tr_weight=1e-4)
    ctx.set_svd_method("bidiag")
    try:
        U1, V1, l1, tw1, chi1 = api.split(th, (ik, ik), 1000, doTrunc=True, tr_weight=1e-4, ctx=ctx)
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)
    assert chi1 == chi0
    assert {q: len(v) for q, v in l1.items()} == {q: len(v) for q, v in l0.items()}
    for q in l0:
        assert np.abs(np.asarray(l1[q]) - np.asarray(l0[q])).max(initial=0.0) <= 1e-13
    assert abs(tw1 - tw0) <= 1e-13


@pytest.mark.parametrize("chimax,tr_weight", [(60, 1e-2), (90, 1e-2), (70, 3e-2)])
def test_bidiag_split_weight_truncation_against_the_norm_of_all_values(ctx, chimax, tr_weight):
    """truncate(tr_weight, chimax) (src/BlockTensor.hpp:84-136) measures the discarded weight against
    the norm of all singular values, those below a top-chimax cut included: slowly decaying spectra
    in four sectors (98 values), chimax binding (60) or the weight bound first (90, 70): kept count,
    values and returned weight as the oracle's dgesvd split.  A norm of only the values above the
    top-chimax cut keeps 56 instead of 60 values in the first case and returns another weight in all."""
    rng = np.random.default_rng(5)
    th = {}
    for q, (m, n) in enumerate([(40, 36), (30, 34), (24, 20), (12, 16)]):
        k = min(m, n)
        U = np.linalg.qr(rng.standard_normal((m, k)))[0]
        V = np.linalg.qr(rng.standard_normal((n, k)))[0]
        th[(q, q, 0, 0)] = (U * np.exp(-np.arange(k) * 0.12 - 0.3 * q)) @ V.T
    nrm = np.sqrt(sum(float((v * v).sum()) for v in th.values()))
    th = {k: v / nrm for k, v in th.items()}
    ik = [0, 0]
    U0, V0, l0, tw0, chi0 = O.split(th, ik, ik, chimax, doTrunc=True, tr_weight=tr_weight)
    ctx.set_svd_method("bidiag")
    try:
        U1, V1, l1, tw1, chi1 = api.split(th, (ik, ik), chimax, doTrunc=True, tr_weight=tr_weight, ctx=ctx)
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)
    assert chi1 == chi0
    assert {q: len(v) for q, v in l1.items() if len(v)} == {q: len(v) for q, v in l0.items() if len(v)}
    for q in l0:
        if len(l0[q]):
            assert np.abs(np.asarray(l1[q]) - np.asarray(l0[q])).max() <= 1e-13
    assert abs(tw1 - tw0) <= 1e-12


def test_bidiag_split_sector_with_more_than_512_kept_vectors(ctx):
    """One 1016 x 792 sector (as converged chi = 2048 sweeps produce) whose 792 values are all kept:
    beyond the shared-memory Cholesky of a 16-CTA cluster, the CholeskyQR runs on its global-memory
    variant (no fallback to the Jacobi route)."""
    rng = np.random.default_rng(8)
    m, n = 1016, 792
    U = np.linalg.qr(rng.standard_normal((m, n)))[0]
    V = np.linalg.qr(rng.standard_normal((n, n)))[0]
    s = np.sort(10.0 ** rng.uniform(-10.0, 0.0, n))[::-1]
    th = {(0, 0, 0, 0): (U * s) @ V.T}
    ik = [0, 0]
    U0, V0, l0, tw0, chi0 = O.split(th, ik, ik, 1000, normalize=False)
    ctx.set_svd_method("bidiag")
    f0 = ctx.L.mpsg_split_fallbacks()
    try:
        U1, V1, l1, tw1, chi1 = api.split(th, (ik, ik), 1000, normalize=False, ctx=ctx)
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)
    assert ctx.L.mpsg_split_fallbacks() == f0
    assert chi1 == chi0 == n
    assert np.abs(np.asarray(l1[0]) - np.asarray(l0[0])).max() <= 1e-13
    Ug = U1[(0, 0, 0)]
    Vg = V1[(0, 0, 0)]
    assert np.abs(Ug.T @ Ug - np.eye(n)).max() < 1e-12
    assert np.abs(Vg @ Vg.T - np.eye(n)).max() < 1e-12
    assert np.abs((Ug * np.asarray(l1[0])) @ Vg - th[(0, 0, 0, 0)]).max() < 1e-12
