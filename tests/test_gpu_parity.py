"""GPU parity tests: libmpsg (through the C ABI) against the CPU oracle on the same inputs.

Tolerances (FP64 path): block structure identical; values within 1e-11 relative to the block
norm; energies within 1e-10 relative.
"""
import os

import numpy as np
import pytest

from mpstools_gb300 import api, lib, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
RTOL = 1e-11


def _close_bm(a, b, rtol=RTOL, keys_equal=True):
    if keys_equal:
        assert set(a) == set(b), (sorted(set(a) ^ set(b)))[:5]
    scale = max([np.abs(v).max() for v in b.values()] + [1e-300])
    for k in b:
        if k not in a:
            assert np.abs(b[k]).max() <= rtol * scale
            continue
        assert a[k].shape == b[k].shape, k
        assert np.abs(a[k] - b[k]).max() <= rtol * scale, (k, np.abs(a[k] - b[k]).max(), scale)


def _case(model="xxz", N=12, chi=12, seed=7, site=4):
    if model == "xxz":
        W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    else:
        W = M.spinless_fermions_mpo(2.0 * M.uniform01(2, N - 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, seed), W, ik, maxthreads=4)
    g.prepare()
    for s in range(site):
        g.do_step(s, 1, chi)
    return g, W, ik


@pytest.mark.parametrize("model", ["xxz", "tv"])
def test_matvec_matches_oracle(ctx, model):
    g, W, ik = _case(model)
    site = 4
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    rng = np.random.default_rng(1)
    th = {k: rng.standard_normal(v.shape) for k, v in th.items()}
    ref = O.contract_twosite(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
    got = api.contractTwosite(L, R, th, W[site], W[site + 1], (ik[site], ik[site + 1]), ctx=ctx)
    _close_bm(got, ref)


def test_matvec_golden_fixture(ctx):
    from golden_io import load_case
    c = load_case(np.load(os.path.join(GOLDEN, "matvec_small.npz")))
    got = api.contractTwosite(c["L"], c["R"], c["theta"], c["W1"], c["W2"], (c["ik0"], c["ik1"]), ctx=ctx)
    _close_bm(got, c["out"])


@pytest.mark.parametrize("direction", [1, -1])
def test_env_update_matches_oracle(ctx, direction):
    g, W, ik = _case(chi=16, site=5)
    if direction > 0:
        site, env, A = 5, g.env("L", 4), g.site(5)
    else:
        site, env, A = 7, g.env("R", 8), g.site(7)
    ref = O.add_contraction_layer(env, A, W[site], ik[site], direction)
    got = api.addContractionLayer(env, A, W[site], ik[site], direction, ctx=ctx)
    _close_bm(got, ref)


def test_theta_matches_oracle(ctx):
    g, W, ik = _case()
    ref = O.theta(g.site(4), g.site(5))
    got = api.theta(g.site(4), g.site(5), ctx=ctx)
    _close_bm(got, ref)


def _recompose(U, lam, Vt):
    out = {}
    for (a, qc, s1), u in U.items():
        for (qc2, b, s2), v in Vt.items():
            if qc2 != qc:
                continue
            out[(a, b, s1, s2)] = (u * lam[qc][None, :]) @ v
    return out


@pytest.mark.parametrize("chimax", [6, 10, 200])
def test_split_matches_oracle(ctx, chimax):
    g, W, ik = _case(chi=12)
    site = 4
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    _, _, psi = O.lanczos(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
    U0, V0, l0, tw0, chi0 = O.split(psi, ik[site], ik[site + 1], chimax)
    U1, V1, l1, tw1, chi1 = api.split(psi, (ik[site], ik[site + 1]), chimax, ctx=ctx)
    assert chi1 == chi0
    assert abs(tw1 - tw0) < 1e-12
    assert set(l1) == set(l0) and all(len(l1[q]) == len(l0[q]) for q in l0)
    for q in l0:
        assert np.abs(l1[q] - l0[q]).max() < 1e-12
    assert set(U1) == set(U0) and set(V1) == set(V0)
    _close_bm(_recompose(U1, l1, V1), _recompose(U0, l0, V0), rtol=1e-10)


def test_lanczos_matches_oracle(ctx):
    g, W, ik = _case(chi=12)
    site = 4
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    E0, it0, psi0 = O.lanczos(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
    lan = api.TSLanzcosEngine(L, R, g.site(site), g.site(site + 1), W[site], W[site + 1], ik[site], ik[site + 1],
                              ctx=ctx)
    lan.simulate(500, 1e-12, True)
    assert abs(lan.E(0) - E0) <= 1e-10 * abs(E0)
    psi1 = lan.getState(0)
    keys = set(psi0) | set(psi1)
    ov = sum(float(np.vdot(psi0.get(k, 0 * psi1.get(k, 0)), psi1.get(k, 0 * psi0.get(k, 0)))) for k in keys)
    n0 = np.sqrt(sum(np.vdot(v, v) for v in psi0.values()))
    n1 = np.sqrt(sum(np.vdot(v, v) for v in psi1.values()))
    assert abs(abs(ov) / (n0 * n1) - 1.0) < 1e-9


def _bond_structure(lams):
    return {b: {q: len(v) for q, v in l.items()} for b, l in lams.items()}


def _run_both(W, sites, ik, chi, sweeps, ctx):
    N = len(sites)
    go = O.DMRG(sites, W, ik, maxthreads=8)
    Eo = go.simulate(maxsteps=sweeps, EnConv=1e-300, chimax=chi, delta=1e-12)
    gg = api.DMRGengine(sites, W, ik, ctx=ctx)
    Eg = gg.simulate(maxsteps=sweeps, EnConv=1e-300, chimax=chi, delta=1e-12)
    return go, Eo, gg, Eg


def test_dmrg_small_xxz_matches_oracle(ctx):
    N = 16
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    sites = M.random_u1_mps(N, N // 2, 24, 12345)
    go, Eo, gg, Eg = _run_both(W, sites, ik, 24, 3, ctx)
    assert abs(Eg - Eo) <= 1e-10 * abs(Eo)
    assert abs(gg.measure_energy() - go.measure()) <= 1e-10 * abs(Eo)
    so, sg = go.steps(), gg.steps()
    assert len(so) == len(sg)


def test_dmrg_heisenberg_L32_chi64(ctx):
    """Heisenberg J=1, L=32, Sz=0, chi=64, 6 sweeps from a random N(0,1) MPS (seed 12345): the
    reference's CPU-sized DMRG run."""
    N = 32
    W = M.heisenberg_mpo(np.ones(N - 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    sites = M.random_u1_mps(N, N // 2, 64, 12345)
    go, Eo, gg, Eg = _run_both(W, sites, ik, 64, 6, ctx)
    assert abs(Eg - Eo) <= 1e-10 * abs(Eo)
    Em = gg.measure_energy()
    assert abs(Em - go.measure()) <= 1e-10 * abs(Eo)


def test_dmrg_tv_product_state_matches_oracle(ctx):
    N = 14
    W = M.spinless_fermions_mpo(2.0 * M.uniform01(2, N - 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    sites = M.product_state(M.filling_state(N, N // 2), ik)
    go, Eo, gg, Eg = _run_both(W, sites, ik, 32, 3, ctx)
    assert abs(Eg - Eo) <= 1e-10 * abs(Eo)


def test_split_density_method_matches_oracle(ctx):
    """Density-matrix SVD (Gram + syevd): same kept structure and lambdas within 1e-10 (chi cut)."""
    g, W, ik = _case(chi=12)
    site = 4
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    _, _, psi = O.lanczos(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
    U0, V0, l0, tw0, chi0 = O.split(psi, ik[site], ik[site + 1], 8)
    ctx.set_svd_method("density")
    try:
        U1, V1, l1, tw1, chi1 = api.split(psi, (ik[site], ik[site + 1]), 8, ctx=ctx)
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)
    assert chi1 == chi0 and abs(tw1 - tw0) < 1e-10
    assert set(l1) == set(l0)
    for q in l0:
        assert np.abs(l1[q] - l0[q]).max() < 1e-10
    _close_bm(_recompose(U1, l1, V1), _recompose(U0, l0, V0), rtol=1e-8)


def test_dmrg_heisenberg_L32_chi64_density_svd(ctx):
    """The Heisenberg L=32, chi=64 run with the density-matrix SVD: energy within 1e-10 relative of
    the oracle."""
    N = 32
    W = M.heisenberg_mpo(np.ones(N - 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    sites = M.random_u1_mps(N, N // 2, 64, 12345)
    go = O.DMRG(sites, W, ik, maxthreads=8)
    Eo = go.simulate(maxsteps=6, EnConv=1e-300, chimax=64, delta=1e-12)
    ctx.set_svd_method("density")
    try:
        gg = api.DMRGengine(sites, W, ik, ctx=ctx)
        Eg = gg.simulate(maxsteps=6, EnConv=1e-300, chimax=64, delta=1e-12)
        Em = gg.measure_energy()
    finally:
        ctx.set_svd_method(lib.DEFAULT_SVD)
    print(f"density svd: E {Eg:.15f} measured {Em:.15f} oracle {Eo:.15f}")
    assert abs(Eg - Eo) <= 1e-10 * abs(Eo)
    assert abs(Em - go.measure()) <= 1e-10 * abs(Eo)
