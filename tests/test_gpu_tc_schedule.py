"""GPU tests of the block-schedule autotuner of the tensor-core matvec (tcgen05 grouped GEMM).

The three block schedules (round robin, snake, greedy longest-processing-time with padding tiles)
only change which persistent CTA computes which output tile; every tile is computed the same way,
so the matvec output must be bit-identical under each schedule.  Each schedule runs in its own
process (MPSG_TC_SCHEDULE fixes it there), on a case with tiles of uneven K (blocks up to ~500,
N = 22, chi = 1000), and the output is compared with the FP64 oracle as in the other tensor-core
tests.  The autotuner itself (timed choice, cache) runs in this process.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from mpstools_gb300 import api, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_CHILD = r"""
import sys, json, hashlib
sys.path.insert(0, sys.argv[1])
import numpy as np
from mpstools_gb300 import api, lib, models as M
from oracle import pyoracle as O
N, chi, site = 22, 1000, 10
W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
ik = M.u1_itokeys(N)
g = O.DMRG(M.random_u1_mps(N, N // 2, chi, 7), W, ik, maxthreads=8)
g.prepare()
for s in range(site):
    g.do_step(s, 1, chi)
L, R = g.env("L", site - 1), g.env("R", site + 2)
th = O.theta(g.site(site), g.site(site + 1))
rng = np.random.default_rng(3)
th = {k: rng.standard_normal(v.shape) for k, v in th.items()}
ctx = lib.Context(0)
got = api.contractTwosite(L, R, th, W[site], W[site + 1], (ik[site], ik[site + 1]), prec="tf32x3", ctx=ctx)
h = hashlib.sha256(b"".join(np.ascontiguousarray(got[k]).tobytes() for k in sorted(got))).hexdigest()
ref = O.contract_twosite(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
scale = max(np.abs(v).max() for v in ref.values())
err = max(np.abs(got[k] - ref[k]).max() for k in ref) / scale
print(json.dumps({"hash": h, "err": float(err), "info": list(ctx.tc_autotune_info()[:3])}))
"""


def _run(schedule):
    env = dict(os.environ)
    env["MPSG_TC_SCHEDULE"] = str(schedule)
    out = subprocess.run([sys.executable, "-c", _CHILD, ROOT], env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_block_schedules_give_identical_outputs():
    res = [_run(s) for s in (0, 1, 2)]
    for r in res:
        assert r["err"] < 2e-5, r
    assert res[0]["hash"] == res[1]["hash"] == res[2]["hash"]
    assert [r["info"][2] for r in res] == [[0, 0], [1, 1], [2, 2]]  # the forced schedule of both stages


def test_autotuner_times_once_per_signature(ctx):
    N, chi, site = 16, 48, 6
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, 7), W, ik, maxthreads=4)
    g.prepare()
    for s in range(site):
        g.do_step(s, 1, chi)
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    args = (L, R, th, W[site], W[site + 1], (ik[site], ik[site + 1]))
    a = api.contractTwosite(*args, prec="tf32x3", ctx=ctx)
    t0, h0, sched, ms = ctx.tc_autotune_info()
    b = api.contractTwosite(*args, prec="tf32x3", ctx=ctx)  # same block sizes: served from the cache
    t1, h1, sched1, _ = ctx.tc_autotune_info()
    assert t1 == t0 and h1 == h0 + 2
    assert sched1 == sched and all(0 <= x <= 2 for x in sched)
    assert all(np.array_equal(a[k], b[k]) for k in a)
