"""GPU tests of the three SVD routes of split / canonicalisation against the oracle.

method 0: one-sided Jacobi SVD (cuSOLVER gesvdj), exact;
method 1: density matrix (FP64 Gram + batched eigensolver per size class);
method 2: density matrix (FP64 Gram + concurrent per-sector eigensolvers).
Checks: singular values (kept ones, 1e-10 absolute for the density routes), orthonormality of the
kept left / right vectors (1e-10), reconstruction of the truncated state, and right-canonical form
after orthonormalize("rl").
"""
import numpy as np
import pytest

from mpstools_gb300 import api, models as M
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


def _right_ortho_err(V):
    groups = {}
    for (qc, b, s), v in V.items():
        groups.setdefault(qc, []).append(v)
    return max(np.abs(np.hstack(g) @ np.hstack(g).T - np.eye(g[0].shape[0])).max() for g in groups.values())


@pytest.mark.parametrize("method", ["jacobi", "density", "density_mt"])
@pytest.mark.parametrize("chimax", [10, 200])
def test_split_methods(ctx, method, chimax):
    g, W, ik = _case()
    site = 4
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    _, _, psi = O.lanczos(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
    U0, V0, l0, tw0, chi0 = O.split(psi, ik[site], ik[site + 1], chimax)
    ctx.set_svd_method(method)
    try:
        U1, V1, l1, tw1, chi1 = api.split(psi, (ik[site], ik[site + 1]), chimax, ctx=ctx)
    finally:
        ctx.set_svd_method("jacobi")
    eu, ev = _left_ortho_err(U1), _right_ortho_err(V1)
    lam_err = max(np.abs(l1[q][:min(len(l1[q]), len(l0.get(q, [])))] - l0[q][:min(len(l1[q]), len(l0.get(q, [])))]).max()
                  for q in l1 if q in l0 and len(l1[q]) and len(l0[q]))
    print(f"{method} chimax={chimax}: chi {chi1}/{chi0} tw {tw1:.3e}/{tw0:.3e} lam err {lam_err:.2e} "
          f"U ortho {eu:.2e} V ortho {ev:.2e}")
    assert eu < 1e-10 and ev < 1e-10
    assert lam_err < 1e-10
    if method == "jacobi":
        assert chi1 == chi0


@pytest.mark.parametrize("method", ["jacobi", "density", "density_mt"])
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
        ctx.set_svd_method("jacobi")
    print(f"{method}: max right-canonical error {max(errs):.2e}")
    assert max(errs) < 1e-10
