"""The oracle's applyMPO and compressTwoSite (restated on the oracle's kernels) pinned against dense
vectors: applyMPO(H, psi) is H psi; with a bond dimension large enough for H psi the two-site fit
reproduces H psi; with a small one the fit is the better approximation the more sweeps it gets."""
import numpy as np

import ed
from mpstools_gb300 import models as M
from oracle import pyoracle as O


def _case(N=8, chi=8, seed=3):
    Jz = M.xxz_couplings(N, 1)
    W = M.heisenberg_mpo(Jz, np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    H = ed.xxz_hamiltonian(Jz, np.ones(N - 1), np.zeros(N), N // 2)
    return W, ik, H, M.random_u1_mps(N, N // 2, chi, seed)


def test_apply_mpo_is_the_dense_product():
    W, ik, H, psi = _case()
    N = len(psi)
    got = ed.mps_sector_vector(O.apply_mpo(psi, W, ik), N // 2)
    ref = H @ ed.mps_sector_vector(psi, N // 2)
    assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()


def test_compress_reproduces_the_product_when_chi_suffices():
    W, ik, H, psi = _case()
    N = len(psi)
    ref = H @ ed.mps_sector_vector(psi, N // 2)
    conv, fit = O.compress_two_site(psi, W, ik, chimax=200, maxstep=2, delta=1e-14, doTrunc=True, tr_weight=1e-14)
    got = ed.mps_sector_vector(fit, N // 2)
    assert np.abs(got - ref).max() < 1e-9 * np.abs(ref).max()
    assert np.isfinite(conv)
