"""Single-site DMRG on the GPU (SSDMRGengine through the dummy-site matvec) against the oracle's
restatement: the same sweep sequence and the same energies step by step (1e-10 relative), the same
final energy; the AUTO matvec precision gives the FP64 final energy to 1e-10."""
import numpy as np
import pytest

from mpstools_gb300 import api, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,chi,model", [(10, 16, "xxz"), (12, 24, "tv")])
def test_ssdmrg_matches_oracle(ctx, N, chi, model):
    if model == "xxz":
        W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    else:
        W = M.spinless_fermions_mpo(2.0 * M.uniform01(2, N - 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    start = M.random_u1_mps(N, N // 2, chi, 7)
    ref = O.SSDMRG(start, W, ik)
    E_ref = ref.simulate(maxsteps=2, EnConv=1e-12, delta=1e-12)
    e = api.DMRGengine(start, W, ik, ctx=ctx)
    E = e.ss_simulate(maxsteps=2, EnConv=1e-12, delta=1e-12)
    steps = e.steps()
    assert [(s["site"], s["dir"]) for s in steps] == [(s["site"], s["dir"]) for s in ref.steps]
    worst = max(abs(a["E"] - b["E"]) / abs(b["E"]) for a, b in zip(steps, ref.steps))
    print(f"{model} N={N} chi={chi}: {len(steps)} steps, worst relative step energy difference {worst:.2e}")
    assert worst < 1e-10
    assert abs(E - E_ref) < 1e-10 * abs(E_ref)
    assert abs(e.measure_energy() - E_ref) < 1e-9 * abs(E_ref)
    e.close()


def test_ssdmrg_auto_precision(ctx):
    N, chi = 12, 24
    W = M.heisenberg_mpo(M.xxz_couplings(N, 3), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    start = M.random_u1_mps(N, N // 2, chi, 8)
    Es = {}
    for prec in ("fp64", "auto"):
        e = api.DMRGengine(start, W, ik, prec=prec, ctx=ctx)
        Es[prec] = e.ss_simulate(maxsteps=3, EnConv=1e-12, delta=1e-12)
        e.close()
    assert abs(Es["auto"] - Es["fp64"]) < 1e-10 * abs(Es["fp64"])
