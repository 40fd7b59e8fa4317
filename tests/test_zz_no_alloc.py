"""GPU test of mpsg_matvec2_plan_execute_noalloc, the matvec entry point that allocates nothing.

It serves callers that may not allocate device memory when they need a matvec (hosts whose
allocator owns the whole memory budget, latency-bound loops): the stage-A intermediate sits in a fixed 8 MiB array inside the library.
Two consecutive calls through the C ABI must agree with mpsg_matvec2_plan_execute on the same plan
within the parity tolerance of the FP64 tests (1e-11 relative to the largest output entry).
The file name sorts last so that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from mpstools_gb300 import lib, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _closure(ctx, L, R, T0, w1, w2, k0, k1):
    h = C.c_void_p()
    lib.check(ctx.L.mpsg_theta_closure(ctx.h, L.h, R.h, T0.h, w1.ref(), w2.ref(), k0.ref(), k1.ref(), C.byref(h)))
    return lib.Tensor(ctx, h)


def test_noalloc_matvec_matches_allocating_entry_point(ctx):
    N, chi, site = 12, 16, 4
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, 7), W, ik, maxthreads=2)
    g.prepare()
    for s in range(site):
        g.do_step(s, 1, chi)
    L = lib.Tensor.from_dict(ctx, g.env("L", site - 1), 1)
    R = lib.Tensor.from_dict(ctx, g.env("R", site + 2), 1)
    th = O.theta(g.site(site), g.site(site + 1))
    rng = np.random.default_rng(5)
    T0 = lib.Tensor.from_dict(ctx, {k: rng.standard_normal(v.shape) for k, v in th.items()}, 2)
    w1, w2 = lib.MPOArg(W[site]), lib.MPOArg(W[site + 1])
    k0, k1 = lib.ItoKeyArg(ik[site]), lib.ItoKeyArg(ik[site + 1])
    tin = _closure(ctx, L, R, T0, w1, w2, k0, k1)
    outs = [_closure(ctx, L, R, T0, w1, w2, k0, k1) for _ in range(3)]
    plan = lib.MatvecPlan(ctx, L, R, tin, W[site], W[site + 1], ik[site], ik[site + 1], lib.PREC["fp64"])
    din, _ = tin.device_view()
    dref, _ = outs[0].device_view()
    plan.execute(din, dref)
    for t in outs[1:]:  # two calls in a row through the C ABI
        dout, _ = t.device_view()
        lib.check(ctx.L.mpsg_matvec2_plan_execute_noalloc(plan.h, C.c_void_p(din), C.c_void_p(dout)))
    ctx.sync()
    ref = outs[0].to_dict()
    scale = max(np.abs(v).max() for v in ref.values())
    assert scale > 0
    # the oracle's contractTwosite on the same input, restricted to the blocks it produces
    ora = O.contract_twosite(g.env("L", site - 1), g.env("R", site + 2), tin.to_dict(), W[site], W[site + 1],
                             ik[site], ik[site + 1])
    for t in outs[1:]:
        got = t.to_dict()
        assert set(got) == set(ref)
        for k in ref:
            assert np.abs(got[k] - ref[k]).max() <= 1e-11 * scale
        for k, v in ora.items():
            assert np.abs(got[k] - v).max() <= 1e-11 * scale
        for k in set(got) - set(ora):  # blocks the reference never creates stay zero
            assert np.abs(got[k]).max() == 0.0


def _plan_case(ctx, N, chi, site, seed, prec="fp64"):
    """Environments and theta of a seeded random U(1) MPS, built on the GPU (the plan only needs
    their block structure and values, not a canonical form)."""
    from mpstools_gb300 import api
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    eng = api.DMRGengine(M.random_u1_mps(N, N // 2, chi, seed), W, ik, ctx=ctx)
    eng.build_environments(site)
    L, R = eng.env_tensor("L", site - 1), eng.env_tensor("R", site + 2)
    A1, A2 = eng.site_tensor(site), eng.site_tensor(site + 1)  # handles alive across the call
    T0 = C.c_void_p()
    lib.check(ctx.L.mpsg_theta(ctx.h, A1.h, A2.h, C.byref(T0)))
    T0 = lib.Tensor(ctx, T0)
    w1, w2 = lib.MPOArg(W[site]), lib.MPOArg(W[site + 1])
    k0, k1 = lib.ItoKeyArg(ik[site]), lib.ItoKeyArg(ik[site + 1])
    tin = _closure(ctx, L, R, T0, w1, w2, k0, k1)
    tout = _closure(ctx, L, R, T0, w1, w2, k0, k1)
    plan = lib.MatvecPlan(ctx, L, R, tin, W[site], W[site + 1], ik[site], ik[site + 1], lib.PREC[prec])
    eng.close()
    return plan, tin, tout, (L, R, T0)


def test_noalloc_rejects_large_and_mixed_plans_and_shares_the_array(ctx):
    # an intermediate above the 1 Mi-element limit is refused with MPSG_ERR_ARG and a message
    big, bin_, bout, keep = _plan_case(ctx, 24, 1024, 11, 3)
    din, _ = bin_.device_view()
    dout, _ = bout.device_view()
    rc = ctx.L.mpsg_matvec2_plan_execute_noalloc(big.h, C.c_void_p(din), C.c_void_p(dout))
    assert rc == 1
    assert b"limit" in ctx.L.mpsg_last_error()
    # a tensor-core plan is refused
    tc, tin, tout, keep2 = _plan_case(ctx, 12, 16, 4, 9, prec="tf32x3")
    din, _ = tin.device_view()
    dout, _ = tout.device_view()
    assert ctx.L.mpsg_matvec2_plan_execute_noalloc(tc.h, C.c_void_p(din), C.c_void_p(dout)) == 1
    # two different plans one after the other share the array: each result matches its own
    # allocating execute
    for N, chi, site, seed in ((12, 16, 4, 11), (14, 24, 6, 12)):
        p, a, b, keep3 = _plan_case(ctx, N, chi, site, seed)
        ref = _closure(ctx, keep3[0], keep3[1], keep3[2], *_args(N, site))
        da, _ = a.device_view()
        db, _ = b.device_view()
        dr, _ = ref.device_view()
        p.execute(da, dr)
        lib.check(ctx.L.mpsg_matvec2_plan_execute_noalloc(p.h, C.c_void_p(da), C.c_void_p(db)))
        ctx.sync()
        r, got = ref.to_dict(), b.to_dict()
        scale = max(np.abs(v).max() for v in r.values())
        for k in r:
            assert np.abs(got[k] - r[k]).max() <= 1e-11 * scale


def _args(N, site):
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    return (lib.MPOArg(W[site]), lib.MPOArg(W[site + 1]), lib.ItoKeyArg(ik[site]), lib.ItoKeyArg(ik[site + 1]))
