"""The oracle's applyMPO, compressTwoSite, compress and compressSingleSite (restated on the oracle's
kernels) pinned against dense vectors: applyMPO(H, psi) is H psi; with a bond dimension large enough
the fits reproduce H psi (psi for compress, psi / |psi| with normalize); with a small one the
compress measure is the squared relative distance and more sweeps give a closer fit."""
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


def _dense(sites, N):
    return ed.mps_sector_vector(sites, N // 2)


def test_compress_reproduces_psi_when_chi_suffices():
    W, ik, H, psi = _case()
    N = len(psi)
    ref = _dense(psi, N)
    conv, _, fit = O.compress(psi, ik, chimax=200, maxstep=2, delta=1e-14)
    assert np.abs(_dense(fit, N) - ref).max() < 1e-12 * np.abs(ref).max()
    assert abs(conv) < 1e-12


def test_compress_normalize_gives_the_normalised_state():
    W, ik, H, psi = _case()
    N = len(psi)
    ref = _dense(psi, N)
    conv, prepared, fit = O.compress(psi, ik, chimax=200, maxstep=2, delta=1e-14, normalize=True)
    # the norm goes into the boundary dummies with the sign of the boundary SVD (a choice of the SVD
    # routine, in the reference as here): the state is psi / |psi| up to a sign
    unit = ref / np.linalg.norm(ref)
    for v in (_dense(prepared, N), _dense(fit, N)):
        sign = np.sign(v @ unit)
        assert np.abs(sign * v - unit).max() < 1e-12
    assert abs(conv) < 1e-12


def test_compress_binding_chi_measure_is_the_distance_and_sweeps_help():
    W, ik, H, psi = _case(chi=16)
    N = len(psi)
    ref = _dense(psi, N)
    conv1, _, fit1 = O.compress(psi, ik, chimax=4, maxstep=1, delta=1e-14)
    conv3, _, fit3 = O.compress(psi, ik, chimax=4, maxstep=3, delta=1e-14)
    for conv, fit in ((conv1, fit1), (conv3, fit3)):
        v = _dense(fit, N)
        assert abs(conv - np.linalg.norm(v - ref) ** 2 / np.linalg.norm(ref) ** 2) < 1e-12
        assert max(max(b.shape[1] for b in s.values()) for s in fit[:-1]) <= 4
    assert 0 < conv3 <= conv1 + 1e-14


def test_compress_single_site_reproduces_the_product_when_chi_suffices():
    W, ik, H, psi = _case()
    N = len(psi)
    ref = H @ _dense(psi, N)
    conv, fit = O.compress_single_site(psi, W, ik, chimax=200, maxstep=2, delta=1e-14)
    assert np.abs(_dense(fit, N) - ref).max() < 1e-11 * np.abs(ref).max()
    assert np.isfinite(conv)


def test_compress_single_site_sweeps_approach_the_product():
    W, ik, H, psi = _case(chi=16)
    N = len(psi)
    ref = H @ _dense(psi, N)
    d = []
    for maxstep in (1, 3):
        conv, fit = O.compress_single_site(psi, W, ik, chimax=15, maxstep=maxstep, delta=1e-14)
        d.append(np.linalg.norm(_dense(fit, N) - ref) / np.linalg.norm(ref))
    assert 0 < d[1] <= d[0] + 1e-13
