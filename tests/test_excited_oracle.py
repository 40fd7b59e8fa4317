"""The oracle's excited-state DMRG (DMRGengine::simulate(mps, ...) restated on the oracle's kernels:
projected two-site Lanczos, overlap environments) pinned against exact diagonalisation: targeting
the ground state it converges to the first excited energy of the same sector."""
import numpy as np

import ed
from mpstools_gb300 import models as M
from oracle import pyoracle as O


def _xxz(N, seed):
    Jz = M.xxz_couplings(N, seed)
    return Jz, M.heisenberg_mpo(Jz, np.ones(N - 1), np.zeros(N)), M.u1_itokeys(N)


def test_excited_dmrg_reaches_the_first_excited_energy():
    N, chi = 8, 16
    Jz, W, ik = _xxz(N, 1)
    H = ed.xxz_hamiltonian(Jz, np.ones(N - 1), np.zeros(N), N // 2).toarray()
    E0, E1 = np.linalg.eigvalsh(H)[:2]
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, 3), W, ik, maxthreads=2)
    Eg = g.simulate(maxsteps=6, EnConv=1e-12, chimax=chi, delta=1e-12)
    assert abs(Eg - E0) < 1e-9 * abs(E0)
    target = [g.site(s) for s in range(N)]
    x = O.ExcitedDMRG(M.random_u1_mps(N, N // 2, chi, 4), W, ik, target)
    E = x.simulate(maxsteps=6, EnConv=1e-12, chimax=chi, delta=1e-12)
    assert abs(E - E1) < 1e-8 * abs(E1), (E, E1, E0)
