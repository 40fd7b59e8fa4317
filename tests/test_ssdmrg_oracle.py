"""The oracle's single-site DMRG (SSDMRGengine restated on the oracle's kernels) pinned against exact
diagonalisation: with the full bond dimension of a small chain it converges to the ground-state
energy; with a smaller one it stays variational (above it)."""
import numpy as np

import ed
from mpstools_gb300 import models as M
from oracle import pyoracle as O


def test_ssdmrg_reaches_the_exact_ground_state():
    N = 10
    Jz = M.xxz_couplings(N, 1)
    W = M.heisenberg_mpo(Jz, np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    E_ed = ed.xxz_ground_energy(Jz, np.ones(N - 1), np.zeros(N), N // 2)
    g = O.SSDMRG(M.random_u1_mps(N, N // 2, 32, 5), W, ik)
    E = g.simulate(maxsteps=6, EnConv=1e-12, delta=1e-12)
    assert abs(E - E_ed) < 1e-9 * abs(E_ed)
    g2 = O.SSDMRG(M.random_u1_mps(N, N // 2, 8, 5), W, ik)
    E2 = g2.simulate(maxsteps=4, EnConv=1e-12, delta=1e-12)
    assert E2 > E_ed - 1e-10
