"""GPU tests of the SVD routes of split / canonicalisation against the oracle.

method 4: the library's own bidiagonal SVD (default), exact;
method 0: one-sided Jacobi SVD (cuSOLVER gesvdj), exact;
method 1: density matrix (FP64 Gram + batched eigensolver per size class);
method 2: density matrix (FP64 Gram + concurrent per-sector eigensolvers);
method 3: density matrix (FP64 Gram + the library's own batched eigensolver).
Checks: singular values, orthonormality of the kept left / right vectors and right-canonical form
after orthonormalize("rl").  The exact routes (bidiagonal, Jacobi) keep the oracle's block structure
(the same chi, the same sectors with the same kept counts) and every kept value to 1e-10.  The density routes square
the condition number: eigenvalues of M^T M below 32 n eps lambda_max are dropped (fewer kept values
than the oracle at most), a kept singular value s agrees with the oracle to 1e-10 + 64 n eps s_max^2 / s
(the Gram matrix's resolution), and both U and V are orthonormal to 1e-10 (CholeskyQR2 on U).
"""
import numpy as np
import pytest

from mpstools_gb300 import api, lib, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _case(N=12, chi=16, seed=7, site=4):
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, seed), W, ik, maxthreads=4)
    g.prepare()
    for s in range(site):
        g.do_step(s, 1, chi)
    return g, W, ik


def _left_ortho_err(U):
    groups = {}
    for (a, qc, s), u in U.items():
        groups.setdefault(qc, []).append(u)
    return max(np.abs(np.vstack(g).T @ np.vstack(g) - np.eye(g[0].shape[1])).max() for g in groups.values())


def _by_centre(U):
    groups = {}
    for (a, qc, s), u in U.items():
        groups.setdefault(qc, []).append(u)
    return groups


def _right_ortho_err(V):
    groups = {}
    for (qc, b, s), v in V.items():
        groups.setdefault(qc, []).append(v)
    return max(np.abs(np.hstack(g) @ np.hstack(g).T - np.eye(g[0].shape[0])).max() for g in groups.values())


EXACT = ("bidiag", "jacobi")


@pytest.mark.parametrize("method", ["bidiag", "jacobi", "density", "density_mt", "density_eig"])
@pytest.mark.parametrize("chimax,N,chi,site", [(10, 12, 16, 4), (200, 12, 16, 4), (100, 14, 128, 6), (1000, 14, 128, 6)])
def test_split_methods(ctx, method, chimax, N, chi, site):
    """Sector widths up to 16 (one eigensolver size class) and up to 70 (classes 32, 64, 128)."""
    g, W, ik = _case(N=N, chi=chi, site=site)
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    _, _, psi = O.lanczos(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
    U0, V0, l0, tw0, chi0 = O.split(psi, ik[site], ik[site + 1], chimax)
    ctx.set_svd_method(method)
    try:
        U1, V1, l1, tw1, chi1 = api.split(psi, (ik[site], ik[site + 1]), chimax, ctx=ctx)
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)
    eu, ev = _left_ortho_err(U1), _right_ortho_err(V1)
    nmax = max(np.vstack(g).shape[0] for g in _by_centre(U1).values())
    smax = max(v.max() for v in l0.values() if len(v))
    tol = 1e-10 if method in EXACT else None
    ratio = 0.0
    if method in EXACT:  # the reference's block structure: same sectors, same kept count in each
        assert set(l1) == set(l0)
        assert {q: len(v) for q, v in l1.items()} == {q: len(v) for q, v in l0.items()}
        assert set(U1) == set(U0) and set(V1) == set(V0)
    for q in l1:
        if q not in l0:
            continue
        m = min(len(l1[q]), len(l0[q]))
        ref = np.asarray(l0[q][:m])
        bound = 1e-10 + (0.0 if tol else 64 * nmax * np.finfo(float).eps * smax**2 / ref)
        ratio = max(ratio, (np.abs(np.asarray(l1[q][:m]) - ref) / bound).max(initial=0.0))
    print(f"{method} chimax={chimax}: chi {chi1}/{chi0} tw {tw1:.3e}/{tw0:.3e} lambda err/bound {ratio:.2e} "
          f"U ortho {eu:.2e} V ortho {ev:.2e}")
    assert eu < 1e-10 and ev < 1e-10
    assert ratio <= 1.0
    if method in EXACT:
        assert chi1 == chi0
        assert abs(tw1 - tw0) <= 1e-12
    else:
        assert chi1 <= chi0


@pytest.mark.parametrize("method", ["bidiag", "jacobi", "density", "density_mt", "density_eig"])
def test_orthonormalize_methods(ctx, method):
    """orthonormalize("rl") of a random MPS: every site right-canonical."""
    N = 10
    W = M.heisenberg_mpo(np.ones(N - 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    sites = M.random_u1_mps(N, N // 2, 16, 3)
    ctx.set_svd_method(method)
    try:
        e = api.DMRGengine(sites, W, ik, ctx=ctx)
        e.prepare()
        errs = [_right_ortho_err(e.site(s)) for s in range(1, N)]
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)
    print(f"{method}: max right-canonical error {max(errs):.2e}")
    assert max(errs) < 1e-10


@pytest.mark.parametrize("log2_scale", [140, 300, -40])
def test_density_eig_badly_scaled_sectors(ctx, log2_scale):
    """Sectors far from unit norm (an unnormalised state being orthonormalised reaches norms of 2^200
    and more): the own eigensolver scales each Gram matrix by a power of two, so its singular values
    match the exact route relative to the largest one, with no sector falling back to the Jacobi route."""
    rng = np.random.default_rng(5)
    scale = 2.0 ** log2_scale
    th = {(0, 0, 0, 0): scale * rng.standard_normal((15, 56)), (1, 1, 0, 0): scale * rng.standard_normal((40, 33)),
          (2, 2, 0, 0): scale * rng.standard_normal((7, 9))}
    ik = [0, 0]
    out = {}
    L = ctx.L
    for method in ("jacobi", "density_eig", "bidiag"):
        ctx.set_svd_method(method)
        f0 = L.mpsg_split_fallbacks()
        U, Vt, lam, tw, chi = api.split(th, (ik, ik), 1000, doTrunc=False, normalize=False, ctx=ctx)
        out[method] = (lam, L.mpsg_split_fallbacks() - f0)
    ctx.set_svd_method(lib.DEFAULT_SVD)
    assert out["density_eig"][1] == 0 and out["bidiag"][1] == 0
    lj = out["jacobi"][0]
    for other in ("density_eig", "bidiag"):
        ld = out[other][0]
        assert set(lj) == set(ld)
        for q in lj:
            a, b = np.sort(np.asarray(lj[q]))[::-1], np.sort(np.asarray(ld[q]))[::-1]
            assert len(a) == len(b)
            assert np.abs(a - b).max() <= 1e-10 * a[0], (other, q, np.abs(a - b).max() / a[0])
