"""Host-side checks of the TEBD adjoint (no GPU): the gate tangent (dG/dtheta) G^H of the library
against central differences of scipy's matrix exponential, the adjoint formula itself on dense
state vectors against central differences of the dense second-order evolution, and the oracle's
TEBD (the reference's forward map restated) differenced at h = 1e-5 against the same dense
differences, which pins the finite-difference gradient the GPU adjoint is checked against."""
import numpy as np
import pytest
import scipy.linalg as sl

import ed
from mpstools_gb300 import api, models as M
from oracle import pyoracle as O

SZ = [-0.5, 0.5]


def _xxz(N, theta):
    return M.heisenberg_mpo(theta, np.ones(N - 1), 0.2 * np.cos(np.arange(N)))


@pytest.mark.parametrize("site", [0, 3, 6])
def test_gate_tangent_matches_expm_differences(site):
    N = 8
    theta = M.xxz_couplings(N, 4, 0.8, 1.2)
    W = _xxz(N, theta)
    dh = api.couplingDerivatives(lambda t: _xxz(N, t), theta, M.u1_itokeys(N))
    sz = np.diag([-0.5, 0.5])
    assert np.abs(dh[site] - np.kron(sz, sz)).max() < 1e-15
    H = api.bondHamiltonian(W[site], W[site + 1], site, N)
    for tau in (0.05, 0.025, 0.7):
        B = api.gateTangent(W[site], W[site + 1], site, N, tau, dh[site])
        e = 1e-6
        dG = (sl.expm(-1j * tau * (H + e * dh[site])) - sl.expm(-1j * tau * (H - e * dh[site]))) / (2 * e)
        ref = dG @ sl.expm(-1j * tau * H).conj().T
        assert np.abs(B - ref).max() < 1e-9 * max(1.0, tau), (site, tau)


def _dense_gates(N, theta, tau):
    W = _xxz(N, theta)
    return [api.getNNGate(W[s], W[s + 1], s, N, tau) for s in range(N - 1)]


def _dense_value(N, theta, steps, dt, obs):
    psi = ed.dense_tebd_second_order(M.neel_state(N), _dense_gates(N, theta, dt), _dense_gates(N, theta, dt / 2),
                                     steps)
    return ed.sz_expect(psi, obs, N)


def _dense_fd(N, theta, steps, dt, obs, h=1e-5):
    g = np.zeros(N - 1)
    for b in range(N - 1):
        tp, tm = theta.copy(), theta.copy()
        tp[b] += h
        tm[b] -= h
        g[b] = (_dense_value(N, tp, steps, dt, obs) - _dense_value(N, tm, steps, dt, obs)) / (2 * h)
    return g


def test_dense_adjoint_formula_matches_differences():
    N, steps, dt, obs = 8, 10, 0.05, 4
    theta = M.xxz_couplings(N, 4, 0.8, 1.2)
    W = _xxz(N, theta)
    dh = api.couplingDerivatives(lambda t: _xxz(N, t), theta, M.u1_itokeys(N))
    tf = [api.gateTangent(W[s], W[s + 1], s, N, dt, dh[s]) for s in range(N - 1)]
    th = [api.gateTangent(W[s], W[s + 1], s, N, dt / 2, dh[s]) for s in range(N - 1)]
    v, g = ed.dense_tebd_adjoint(M.neel_state(N), _dense_gates(N, theta, dt), _dense_gates(N, theta, dt / 2), tf, th,
                                 steps, obs)
    fd = _dense_fd(N, theta, steps, dt, obs)
    assert abs(v - _dense_value(N, theta, steps, dt, obs)) < 1e-14
    assert np.abs(g).max() > 1e-3
    assert np.abs(g - fd).max() < 1e-8


def oracle_fd_gradient(N, theta, steps, dt, obs, chimax, doTrunc=True, tr_weight=1e-10, h=1e-5, bonds=None):
    """Central differences of <Sz_obs> after the oracle's second-order TEBD, one bond at a time."""
    ik = M.u1_itokeys(N)
    local = M.neel_state(N)

    def value(t):
        ref = O.TEBD(local, _xxz(N, t), ik)
        ref.second_order(steps, dt, chimax, doTrunc=doTrunc, tr_weight=tr_weight)
        return ref.measure_diag(obs, SZ)

    g = np.zeros(N - 1)
    for b in (range(N - 1) if bonds is None else bonds):
        tp, tm = theta.copy(), theta.copy()
        tp[b] += h
        tm[b] -= h
        g[b] = (value(tp) - value(tm)) / (2 * h)
    return g


def test_oracle_differences_match_dense_differences():
    # without truncation (doTrunc = false keeps every value above 1e-15): truncation by weight makes
    # <Sz> jump by ~1e-12 between neighbouring couplings, which h = 1e-5 turns into ~1e-7 noise
    N, steps, dt, obs = 8, 10, 0.05, 3
    theta = M.xxz_couplings(N, 5, 0.8, 1.2)
    g_or = oracle_fd_gradient(N, theta, steps, dt, obs, chimax=64, doTrunc=False)
    g_de = _dense_fd(N, theta, steps, dt, obs)
    assert np.abs(g_de).max() > 1e-4
    assert np.abs(g_or - g_de).max() < 1e-9


def test_nn_gate_matches_oracle_and_expm_on_the_host():
    """The library's getNNGate (host code, no GPU) against the oracle's MPO::getNNGate restatement
    and against expm of the library's own bond Hamiltonian (boundary-aware on-site weights), for
    real and complex time steps: the reference exponentiates -(imag(dt) + i real(dt)) h
    (src/MPOTypes.hpp:1190)."""
    N = 6
    W = M.heisenberg_mpo(M.xxz_couplings(N, 4, 0.8, 1.2), np.ones(N - 1), 0.3 * np.arange(N))
    for s in range(N - 1):
        H = api.bondHamiltonian(W[s], W[s + 1], s, N)
        assert np.abs(H - H.T).max() < 1e-15
        for dt in (0.05 + 0j, 0.05 - 0.01j):
            got = api.getNNGate(W[s], W[s + 1], s, N, dt)
            assert np.abs(got - O.nn_gate(W[s], W[s + 1], s, N, dt)).max() < 1e-14
            assert np.abs(got - sl.expm(-(dt.imag + 1j * dt.real) * H)).max() < 1e-13
