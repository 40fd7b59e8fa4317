"""GPU parity of TEBD (complex FP64 on the device) against the oracle's restatement of
getNNGate / applyGate / doTimeSlice / second-order TEBDengine: local observables and the Schmidt
spectra after the evolution (Gamma tensors are compared only through those: inside degenerate
Schmidt subspaces the singular vectors are not unique).  Truncation by weight (doTrunc = true, the
TEBD setting of the benchmarked configuration), with and without a binding chi cap.  With
doTrunc = false the reference keeps every singular value above 1e-15, where values at the noise
level of the SVD fall on either side depending on the SVD algorithm (LAPACK in the oracle, Jacobi on
the GPU), and Gamma = U / lambda then amplifies that noise; that setting is not a parity case."""
import numpy as np
import pytest

from mpstools_gb300 import api, lib, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
SZ = [-0.5, 0.5]


def test_nn_gate_matches_oracle(ctx):
    N = 6
    W = M.heisenberg_mpo(M.xxz_couplings(N, 4, 0.8, 1.2), np.ones(N - 1), 0.3 * np.arange(N))
    for s in range(N - 1):
        for dt in (0.05, 0.05 - 0.01j):
            got = api.getNNGate(W[s], W[s + 1], s, N, dt)
            ref = O.nn_gate(W[s], W[s + 1], s, N, dt)
            assert np.abs(got - ref).max() < 1e-14


def _spectra(lam):
    return np.sort(np.concatenate([np.asarray(v) for v in lam.values()]))[::-1]


@pytest.mark.parametrize("N,steps,chimax,doTrunc", [(10, 12, 64, True), (14, 20, 12, True), (14, 20, 64, True)])
def test_tebd_matches_oracle(ctx, N, steps, chimax, doTrunc):
    dt = 0.05
    W = M.heisenberg_mpo(M.xxz_couplings(N, 4, 0.8, 1.2), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    local = M.neel_state(N)
    ref = O.TEBD(local, W, ik)
    ref.second_order(steps, dt, chimax, doTrunc=doTrunc, tr_weight=1e-10)
    f0 = ctx.L.mpsg_split_fallbacks()
    got = api.TEBDengine(local, W, ik, ctx=ctx)
    got.second_order(steps, dt, chimax, doTrunc=doTrunc, tr_weight=1e-10)
    assert ctx.L.mpsg_split_fallbacks() == f0  # every split on the complex bidiagonal route
    err_sz = max(abs(got.measure_diag(s, SZ) - ref.measure_diag(s, SZ)) for s in range(N))
    err_lam = 0.0
    for b in range(N - 1):
        lg, lo = got.lam(b), ref.lam(b)
        assert set(lg) == set(lo), b
        for q in lo:
            assert len(lg[q]) == len(lo[q]), (b, q)
        err_lam = max(err_lam, np.abs(_spectra(lg) - _spectra(lo)).max())
    print(f"N={N} chimax={chimax} trunc={doTrunc}: <Sz> err {err_sz:.2e}, lambda err {err_lam:.2e}, "
          f"stats {got.stats()}")
    assert err_sz < 1e-10 and err_lam < 1e-10
    assert abs(got.measure_diag(N // 2, SZ)) < 0.5 - 1e-3  # the state evolved
    got.close()


@pytest.mark.parametrize("N,steps,chimax", [(10, 12, 64), (14, 20, 12), (14, 20, 64)])
def test_tebd_density_split_matches_oracle(ctx, N, steps, chimax):
    """The density-matrix split (complex Gram matrix, batched Hermitian eigensolver, U = M V / s):
    a singular value s carries an absolute error ~ eps s_max^2 / s, so the comparison is at 1e-8."""
    dt = 0.05
    W = M.heisenberg_mpo(M.xxz_couplings(N, 4, 0.8, 1.2), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    local = M.neel_state(N)
    ref = O.TEBD(local, W, ik)
    ref.second_order(steps, dt, chimax, doTrunc=True, tr_weight=1e-10)
    ctx.set_svd_method("density")
    try:
        got = api.TEBDengine(local, W, ik, ctx=ctx)
        got.second_order(steps, dt, chimax, doTrunc=True, tr_weight=1e-10)
        err_sz = max(abs(got.measure_diag(s, SZ) - ref.measure_diag(s, SZ)) for s in range(N))
        err_lam = 0.0
        for b in range(N - 1):
            lg, lo = got.lam(b), ref.lam(b)
            common = set(lg) & set(lo)
            for q in common:
                a, c = np.sort(np.asarray(lg[q]))[::-1], np.sort(np.asarray(lo[q]))[::-1]
                k = min(len(a), len(c))
                err_lam = max(err_lam, np.abs(a[:k] - c[:k]).max())
        print(f"density split N={N} chimax={chimax}: <Sz> err {err_sz:.2e}, lambda err {err_lam:.2e}, {got.stats()}")
        assert err_sz < 1e-8 and err_lam < 1e-8
        got.close()
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)


@pytest.mark.parametrize("svd", ["jacobi", "density"])
def test_tebd_layer_batching_matches_bond_by_bond(ctx, svd):
    """A time slice updated as one direct sum of its bonds gives the bond-by-bond results."""
    N, steps, dt, chimax = 14, 20, 0.05, 24
    W = M.heisenberg_mpo(M.xxz_couplings(N, 4, 0.8, 1.2), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    ctx.set_svd_method(svd)
    try:
        out = []
        for batched in (False, True):
            e = api.TEBDengine(M.neel_state(N), W, ik, ctx=ctx)
            e.set_batch_layers(batched)
            e.second_order(steps, dt, chimax, doTrunc=True, tr_weight=1e-10)
            out.append(([e.measure_diag(s, SZ) for s in range(N)], [e.lam(b) for b in range(N - 1)], e.stats()))
            e.close()
        (sz0, l0, st0), (sz1, l1, st1) = out
        print(f"{svd}: bond by bond {st0['seconds']:.3f} s, batched slices {st1['seconds']:.3f} s")
        assert max(abs(a - b) for a, b in zip(sz0, sz1)) < 1e-12
        for a, b in zip(l0, l1):
            assert set(a) == set(b)
            for q in a:
                assert len(a[q]) == len(b[q])
                assert np.abs(np.sort(a[q]) - np.sort(b[q])).max() < 1e-12
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)


def test_tebd_bidiagonal_split_matches_jacobi_split(ctx):
    """The complex bidiagonal route (default) and cuSOLVER's zgesvdj give the same lambdas, block
    structure and local magnetisation after 20 second-order steps at a binding chi."""
    N, steps, dt, chimax = 14, 20, 0.05, 24
    W = M.heisenberg_mpo(M.xxz_couplings(N, 4, 0.8, 1.2), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    local = M.neel_state(N)
    res = {}
    for svd in ("bidiag", "jacobi"):
        ctx.set_svd_method(svd)
        try:
            f0 = ctx.L.mpsg_split_fallbacks()
            e = api.TEBDengine(local, W, ik, ctx=ctx)
            e.second_order(steps, dt, chimax, doTrunc=True, tr_weight=1e-10)
            res[svd] = ([e.lam(b) for b in range(N - 1)], [e.measure_diag(s, SZ) for s in range(N)],
                        e.stats()["split_seconds"], ctx.L.mpsg_split_fallbacks() - f0)
            e.close()
        finally:
            ctx.set_svd_method(lib.DEFAULT_SVD)
    (lb, szb, tb, fb), (lj, szj, tj, _) = res["bidiag"], res["jacobi"]
    assert fb == 0
    for b in range(N - 1):
        assert {q: len(v) for q, v in lb[b].items()} == {q: len(v) for q, v in lj[b].items()}, b
        assert np.abs(_spectra(lb[b]) - _spectra(lj[b])).max() < 1e-12, b
    assert max(abs(a - c) for a, c in zip(szb, szj)) < 1e-11
    print(f"split seconds: bidiagonal {tb:.3f}, zgesvdj {tj:.3f}")
