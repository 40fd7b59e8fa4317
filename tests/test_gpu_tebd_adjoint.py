"""GPU TEBD adjoint: the gradient of <Sz_c(T)> after the second-order evolution with respect to the
per-bond XXZ anisotropies Delta_b, against central finite differences (h = 1e-5) of the oracle's
TEBD (the reference's forward map restated on the CPU; the differences are pinned against dense
state vectors in test_tebd_adjoint_host.py), against the dense adjoint formula, across checkpoint
intervals, and on a chi-capped evolution where the truncation is not differentiated."""
import numpy as np
import pytest

import ed
from mpstools_gb300 import api, models as M
from test_tebd_adjoint_host import _dense_gates, _xxz, oracle_fd_gradient

pytestmark = pytest.mark.gpu
SZ = [-0.5, 0.5]


def _gpu_adjoint(ctx, N, theta, steps, dt, obs, chimax, doTrunc=True, tr_weight=1e-15, every=0):
    ik = M.u1_itokeys(N)
    dh = api.couplingDerivatives(lambda t: _xxz(N, t), theta, ik)
    eng = api.TEBDengine(M.neel_state(N), _xxz(N, theta), ik, ctx=ctx)
    v, g = eng.adjoint_second_order(steps, dt, chimax, obs, SZ, dh, doTrunc=doTrunc, tr_weight=tr_weight,
                                    checkpoint_every=every)
    after = eng.measure_diag(obs, SZ)
    secs = eng.adjoint_seconds()
    eng.close()
    return v, g, after, secs


@pytest.mark.parametrize("obs", [0, 3, 7])
def test_adjoint_matches_oracle_differences(ctx, obs):
    N, steps, dt = 8, 10, 0.05
    theta = M.xxz_couplings(N, 5, 0.8, 1.2)
    v, g, after, _ = _gpu_adjoint(ctx, N, theta, steps, dt, obs, chimax=64)
    fd = oracle_fd_gradient(N, theta, steps, dt, obs, chimax=64, doTrunc=False)
    print(f"obs={obs}: value {v:.12f}, max |grad| {np.abs(g).max():.3e}, max |grad - fd| {np.abs(g - fd).max():.2e}")
    assert abs(v - after) < 1e-15
    assert np.abs(fd).max() > 1e-5
    assert np.abs(g - fd).max() < 1e-8


def test_adjoint_matches_dense_formula(ctx):
    N, steps, dt, obs = 10, 8, 0.05, 5
    theta = M.xxz_couplings(N, 6, 0.8, 1.2)
    W = _xxz(N, theta)
    dh = api.couplingDerivatives(lambda t: _xxz(N, t), theta, M.u1_itokeys(N))
    tf = [api.gateTangent(W[s], W[s + 1], s, N, dt, dh[s]) for s in range(N - 1)]
    th = [api.gateTangent(W[s], W[s + 1], s, N, dt / 2, dh[s]) for s in range(N - 1)]
    vd, gd = ed.dense_tebd_adjoint(M.neel_state(N), _dense_gates(N, theta, dt), _dense_gates(N, theta, dt / 2), tf,
                                   th, steps, obs)
    v, g, _, _ = _gpu_adjoint(ctx, N, theta, steps, dt, obs, chimax=64)
    print(f"dense: |value diff| {abs(v - vd):.2e}, max |grad diff| {np.abs(g - gd).max():.2e}")
    # the GPU run truncates by weight 1e-15 (the dense evolution keeps everything): ~1e-11 in <Sz>
    assert abs(v - vd) < 1e-10
    assert np.abs(g - gd).max() < 1e-10


def test_adjoint_checkpoint_intervals_agree(ctx):
    N, steps, dt, obs = 10, 6, 0.05, 4
    theta = M.xxz_couplings(N, 7, 0.8, 1.2)
    ref = None
    for every in (1, 0, 3, 1000):
        v, g, _, _ = _gpu_adjoint(ctx, N, theta, steps, dt, obs, chimax=64, every=every)
        if ref is None:
            ref = (v, g)
        assert abs(v - ref[0]) < 1e-14
        assert np.abs(g - ref[1]).max() < 1e-13, every


def test_adjoint_with_binding_chi_cap(ctx):
    # chi capped at 12 with truncation by weight: the adjoint treats the truncation as exact, so it
    # agrees with the differences of the truncated evolution only up to the truncation's own effect
    N, steps, dt, obs, chimax = 14, 20, 0.05, 7, 12
    theta = M.xxz_couplings(N, 8, 0.8, 1.2)
    v, g, _, secs = _gpu_adjoint(ctx, N, theta, steps, dt, obs, chimax=chimax, tr_weight=1e-10)
    fd = oracle_fd_gradient(N, theta, steps, dt, obs, chimax=chimax, doTrunc=True, tr_weight=1e-10)
    fd_exact = oracle_fd_gradient(N, theta, steps, dt, obs, chimax=256, doTrunc=False)
    err, err_exact = np.abs(g - fd).max(), np.abs(g - fd_exact).max()
    print(f"chi cap {chimax}: max |grad| {np.abs(g).max():.3e}, vs truncated differences {err:.2e}, "
          f"vs untruncated differences {err_exact:.2e}, adjoint {secs:.2f} s")
    assert np.abs(g).max() > 1e-3
    assert err < 1e-3 * np.abs(g).max()
