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
    for t in outs[1:]:
        got = t.to_dict()
        assert set(got) == set(ref)
        for k in ref:
            assert np.abs(got[k] - ref[k]).max() <= 1e-11 * scale
