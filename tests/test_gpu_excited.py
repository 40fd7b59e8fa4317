"""Excited-state DMRG on the GPU (projected Lanczos, overlap environments) against the oracle's
restatement: the same sweep, step energies to 1e-9 relative, and the first excited energy of exact
diagonalisation at full bond dimension."""
import numpy as np
import pytest

import ed
from mpstools_gb300 import api, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def test_excited_dmrg_matches_oracle(ctx):
    N, chi = 8, 16
    Jz = M.xxz_couplings(N, 1)
    W = M.heisenberg_mpo(Jz, np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    H = ed.xxz_hamiltonian(Jz, np.ones(N - 1), np.zeros(N), N // 2).toarray()
    E1 = np.linalg.eigvalsh(H)[1]
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, 3), W, ik, maxthreads=2)
    g.simulate(maxsteps=6, EnConv=1e-12, chimax=chi, delta=1e-12)
    target = [g.site(s) for s in range(N)]
    start = M.random_u1_mps(N, N // 2, chi, 4)
    ref = O.ExcitedDMRG(start, W, ik, target)
    E_ref = ref.simulate(maxsteps=4, EnConv=1e-12, chimax=chi, delta=1e-12)
    e = api.DMRGengine(start, W, ik, ctx=ctx)
    E = e.excited_simulate(target, maxsteps=4, EnConv=1e-12, chimax=chi, delta=1e-12)
    steps = e.steps()
    assert [(s["site"], s["dir"]) for s in steps] == [(s["site"], s["dir"]) for s in ref.steps]
    worst = max(abs(a["E"] - b["E"]) / abs(b["E"]) for a, b in zip(steps, ref.steps))
    print(f"excited: {len(steps)} steps, worst relative step energy difference {worst:.2e}, E {E:.12f} E1 {E1:.12f}")
    assert worst < 1e-9
    assert abs(E - E_ref) < 1e-10 * abs(E_ref)
    assert abs(E - E1) < 1e-8 * abs(E1)
    e.close()
