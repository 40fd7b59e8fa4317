"""The Lanczos iterations after the first energy checkpoint run as one replayed CUDA graph per batch
(iteration index on the device, matvec on fixed buffers).  The arithmetic is that of the
launch-by-launch path: the same DMRG run with the graph path switched off (MPSG_NO_LANCZOS_GRAPH)
gives bit-identical energies, kept dimensions and iteration counts, in FP64 and in MIXED; and the
graph path issues far fewer launches from the host."""
import os

import numpy as np
import pytest

from mpstools_gb300 import api, models as M

pytestmark = pytest.mark.gpu


def _run(ctx, prec, graph):
    N, chi = 16, 24
    W = M.heisenberg_mpo(M.xxz_couplings(N, 5), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    if graph:
        os.environ.pop("MPSG_NO_LANCZOS_GRAPH", None)
    else:
        os.environ["MPSG_NO_LANCZOS_GRAPH"] = "1"
    try:
        e = api.DMRGengine(M.random_u1_mps(N, N // 2, chi, 21), W, ik, prec=prec, ctx=ctx)
        E = e.simulate(maxsteps=2, EnConv=1e-300, chimax=chi, delta=1e-12)
        steps = e.steps()
        e.close()
    finally:
        os.environ.pop("MPSG_NO_LANCZOS_GRAPH", None)
    return E, steps


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_graph_replay_is_bit_identical(ctx, prec):
    E0, s0 = _run(ctx, prec, graph=False)
    E1, s1 = _run(ctx, prec, graph=True)
    assert E1 == E0
    assert [(s["iters"], s["chi"], s["E"], s["tw"]) for s in s1] == [(s["iters"], s["chi"], s["E"], s["tw"]) for s in s0]
    assert max(s["iters"] for s in s1) > 6  # batches beyond the first ran (as graphs)
