"""GPU tests of the tensor-core (tcgen05) matvec and the mixed-precision Lanczos / DMRG paths.

Tolerances: max |mixed - FP64| relative to the largest |FP64| entry of the output:
TF32X3 2e-5, BF16X3 3e-4, TF32 5e-3, BF16 4e-2 (FP32 accumulation over K <= a few hundred;
hi/lo splits carry ~22 / ~16 significant bits, single TF32 / BF16 operands 11 / 8 bits).
Energies of the AUTO path (TF32X3 Lanczos finished in FP64) and of the MIXED path (TF32X3 Lanczos,
energy = FP64 Rayleigh quotient of its ground state) agree with the FP64 oracle to 1e-10.
The tensor-core environment update (addContractionLayer in each precision) meets the same
tolerances against the oracle's FP64 layer.
"""
import numpy as np
import pytest

from mpstools_gb300 import api, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

TOL = {"tf32x3": 2e-5, "bf16x3": 3e-4, "tf32": 5e-3, "bf16": 4e-2}


def _case(N=16, chi=48, seed=7, site=6, model="xxz"):
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


def _max_rel(a, b):
    scale = max(np.abs(v).max() for v in b.values())
    return max(np.abs(a[k] - b[k]).max() for k in b) / scale


@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3", "tf32", "bf16"])
@pytest.mark.parametrize("model", ["xxz", "tv"])
def test_tc_matvec_matches_fp64(ctx, prec, model):
    g, W, ik = _case(model=model)
    site = 6
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    rng = np.random.default_rng(3)
    th = {k: rng.standard_normal(v.shape) for k, v in th.items()}
    ref = api.contractTwosite(L, R, th, W[site], W[site + 1], (ik[site], ik[site + 1]), prec="fp64", ctx=ctx)
    got = api.contractTwosite(L, R, th, W[site], W[site + 1], (ik[site], ik[site + 1]), prec=prec, ctx=ctx)
    assert set(got) == set(ref)
    err = _max_rel(got, ref)
    print(f"{model} {prec}: max rel err {err:.2e}")
    assert err < TOL[prec], err


def test_tc_matvec_large_blocks(ctx):
    """Blocks larger than one 128x128 tile and K spanning several chunks (N = 22, chi = 1000)."""
    g, W, ik = _case(N=22, chi=1000, site=10)
    site = 10
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    rng = np.random.default_rng(4)
    th = {k: rng.standard_normal(v.shape) for k, v in th.items()}
    ref = api.contractTwosite(L, R, th, W[site], W[site + 1], (ik[site], ik[site + 1]), prec="fp64", ctx=ctx)
    assert max(max(v.shape) for v in th.values()) > 128
    for prec in ("tf32x3", "bf16x3"):
        got = api.contractTwosite(L, R, th, W[site], W[site + 1], (ik[site], ik[site + 1]), prec=prec, ctx=ctx)
        err = _max_rel(got, ref)
        print(f"large {prec}: {err:.2e}")
        assert err < TOL[prec], (prec, err)


def test_mixed_lanczos_energy_is_the_fp64_rayleigh_quotient(ctx):
    g, W, ik = _case()
    site = 6
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    A1, A2 = g.site(site), g.site(site + 1)
    res = {}
    for prec in ("fp64", "tf32x3", "mixed"):
        lz = api.TSLanzcosEngine(L, R, A1, A2, W[site], W[site + 1], ik[site], ik[site + 1], prec=prec, ctx=ctx)
        n = lz.simulate(500, 1e-12, True)
        res[prec] = (lz.E(0), lz.getState(0), n)
    E64 = res["fp64"][0]
    Em, psi, n = res["mixed"]
    H = api.contractTwosite(L, R, psi, W[site], W[site + 1], (ik[site], ik[site + 1]), prec="fp64", ctx=ctx)
    rq = sum(float(np.vdot(psi[k], H[k])) for k in psi) / sum(float(np.vdot(v, v)) for v in psi.values())
    print(f"fp64 {E64!r} ({res['fp64'][2]} matvecs), tf32x3 Ritz value {res['tf32x3'][0]!r}, "
          f"mixed {Em!r} ({n} TF32X3 iterations + one FP64 matvec), host Rayleigh quotient {rq!r}")
    assert n == res["tf32x3"][2]  # the same TF32X3 Lanczos
    assert abs(Em - rq) <= 1e-13 * abs(rq)
    assert abs(Em - E64) <= 1e-10 * abs(E64)


@pytest.mark.parametrize("prec", ["auto", "tf32x3", "mixed"])
def test_mixed_dmrg_energy(ctx, prec):
    N = 20
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    sites = M.random_u1_mps(N, N // 2, 32, 12345)
    go = O.DMRG(sites, W, ik, maxthreads=8)
    Eo = go.simulate(maxsteps=4, EnConv=1e-300, chimax=32, delta=1e-12)
    gg = api.DMRGengine(sites, W, ik, prec=prec, ctx=ctx)
    Eg = gg.simulate(maxsteps=4, EnConv=1e-300, chimax=32, delta=1e-12)
    Em = gg.measure_energy()
    rel = abs(Em - go.measure()) / abs(Eo)
    print(f"{prec}: E_lanczos {Eg:.15f} E_measured {Em:.15f} oracle {Eo:.15f} rel {rel:.2e}")
    if prec in ("auto", "mixed"):
        assert abs(Eg - Eo) <= 1e-10 * abs(Eo)
        assert rel <= 1e-10
    else:
        assert rel <= 1e-7


@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3", "tf32", "bf16"])
@pytest.mark.parametrize("direction", [1, -1])
def test_tc_env_update_matches_fp64_oracle(ctx, prec, direction):
    g, W, ik = _case()
    if direction > 0:
        site, env, A = 6, g.env("L", 5), g.site(6)
    else:
        site, env, A = 8, g.env("R", 9), g.site(8)
    ref = O.add_contraction_layer(env, A, W[site], ik[site], direction)
    got = api.addContractionLayer(env, A, W[site], ik[site], direction, prec=prec, ctx=ctx)
    assert set(got) == set(ref)
    err = _max_rel(got, ref)
    print(f"env {direction:+d} {prec}: max rel err {err:.2e}")
    assert err < TOL[prec], err


def test_tc_env_update_large_blocks_and_two_tensor(ctx):
    """Blocks beyond one 128-row tile (N = 22, chi = 1000) and the two-tensor form (A lower, Ap upper)."""
    g, W, ik = _case(N=22, chi=1000, site=10)
    site = 10
    env, A = g.env("L", site - 1), g.site(site)
    ref = O.add_contraction_layer(env, A, W[site], ik[site], 1)
    got = api.addContractionLayer(env, A, W[site], ik[site], 1, prec="tf32x3", ctx=ctx)
    err = _max_rel(got, ref)
    assert err < TOL["tf32x3"], err
    rng = np.random.default_rng(5)
    Ap = {k: v + 1e-3 * rng.standard_normal(v.shape) for k, v in A.items()}
    ref2 = O.add_contraction_layer2(env, A, Ap, W[site], ik[site], 1)
    got2 = api.addContractionLayer2(env, A, W[site], Ap, ik[site], 1, prec="tf32x3", ctx=ctx)
    assert set(got2) == set(ref2)
    err2 = _max_rel(got2, ref2)
    assert err2 < TOL["tf32x3"], err2


def test_dmrg_with_tensor_core_environments(ctx):
    """doStep's environment updates on the tensor cores (TF32X3) with the MIXED Lanczos: the energy
    carries the environments' ~1e-7 relative error (it is not a 1e-10 mode), then FP64 environments
    for the last sweep bring it back within the MIXED tolerance of the oracle."""
    N = 20
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    sites = M.random_u1_mps(N, N // 2, 32, 12345)
    go = O.DMRG(sites, W, ik, maxthreads=8)
    Eo = go.simulate(maxsteps=4, EnConv=1e-300, chimax=32, delta=1e-12)
    gg = api.DMRGengine(sites, W, ik, prec="mixed", ctx=ctx)
    gg.set_env_prec("tf32x3")
    Et = gg.simulate(maxsteps=3, EnConv=1e-300, chimax=32, delta=1e-12)
    rel_t = abs(Et - Eo) / abs(Eo)
    assert rel_t <= 1e-5, rel_t
    gg.set_env_prec("fp64")
    Ef = gg.simulate(maxsteps=1, EnConv=1e-300, chimax=32, delta=1e-12)
    rel_f = abs(gg.measure_energy() - Eo) / abs(Eo)
    print(f"tensor-core environments: {rel_t:.2e}; after an FP64 sweep {rel_f:.2e} (E {Ef!r}, oracle {Eo!r})")
    assert rel_f <= 1e-9, rel_f
