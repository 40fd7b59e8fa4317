"""CPU tests: the oracle's two-site Lanczos against an independent numpy restatement of the
reference's TSLanzcosEngine::simulate (src/lanzcos.hpp:165-278) and getState (:81-92), with the
effective Hamiltonian applied by dense contraction (tests/ed.py).

The restatement follows the reference: k = |A1|, stop when k < delta; A1 /= k; A2 = H A1;
e = <A2, A1>; every Ndiag = 5 iterations (it > 0) the lowest eigenvalue of the tridiagonal matrix
(dstev) is compared with the previous test's and the loop stops when they differ by less than
delta; the three-term recurrence A3 = A2 - e A1 - k A0 without reorthogonalisation; the loop also
stops after itmax iterations.  The energy is the lowest eigenvalue of the final tridiagonal matrix
and the state sum_i A_i z_i0 with z from dstev.  The oracle reports the number of Krylov vectors
(matvecs) entering the state.
"""
import numpy as np
import pytest
from scipy.linalg import eigh_tridiagonal

import ed
from mpstools_gb300 import models as M
from oracle import pyoracle as O


def _dot(x, y):
    return sum(float((x[k] * y[k]).sum()) for k in x if k in y)


def _lincomb(*terms):
    out = {}
    for c, x in terms:
        for k, v in x.items():
            out[k] = out[k] + c * v if k in out else c * v
    return out


def _lanczos_np(matvec, th, itmax, delta, ndiag=5, testenergy=True):
    A1, A0 = dict(th), None
    es, ks, As = [], [], []
    eold, it, first, tests = 1e100, 0, True, []
    while True:
        k = np.sqrt(_dot(A1, A1))
        if abs(k) < delta:
            break
        if not first:
            ks.append(k)
        A1 = {key: v / k for key, v in A1.items()}
        A2 = matvec(A1)
        As.append(A1)
        e = _dot(A2, A1)
        es.append(e)
        if it % ndiag == 0 and it != 0 and testenergy:
            e0 = eigh_tridiagonal(np.array(es), np.array(ks), eigvals_only=True, lapack_driver="stev")[0]
            tests.append(abs(e0 - eold))
            if abs(e0 - eold) < delta:
                break
            eold = e0
        elif it % ndiag == 0 and it != 0:
            # residual of the current Ritz vector, one extra matvec
            w, z = eigh_tridiagonal(np.array(es), np.array(ks), lapack_driver="stev")
            A4 = _lincomb(*[(z[i, 0], As[i]) for i in range(len(As))])
            A6 = _lincomb((1.0, matvec(A4)), (-w[0], A4))
            resi = np.sqrt(_dot(A6, A6))
            tests.append(resi)
            if resi < delta:
                break
        if not first:
            A3 = _lincomb((1.0, A2), (-e, A1), (-k, A0))
        else:
            A3 = _lincomb((1.0, A2), (-e, A1))
            first = False
        A0, A1 = A1, A3
        it += 1
        if it >= itmax:
            break
    w, z = eigh_tridiagonal(np.array(es), np.array(ks), lapack_driver="stev")
    psi = _lincomb(*[(z[i, 0], As[i]) for i in range(len(As))])
    return w[0], len(es), psi, tests


def _case(seed, N=10, chi=8, site=4, model="xxz"):
    if model == "xxz":
        W = M.heisenberg_mpo(M.xxz_couplings(N, seed), np.ones(N - 1), np.zeros(N))
    else:
        W = M.spinless_fermions_mpo(2.0 * M.uniform01(seed, N - 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, seed), W, ik, maxthreads=2)
    g.prepare()
    for s in range(site):
        g.do_step(s, 1, chi)
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    return L, R, th, W[site], W[site + 1], ik[site], ik[site + 1]


@pytest.mark.parametrize("seed,model,itmax,delta,testenergy",
                         [(1, "xxz", 500, 1e-12, True), (2, "xxz", 500, 1e-9, True), (3, "tv", 500, 1e-12, True),
                          (4, "xxz", 7, 1e-12, True), (1, "xxz", 500, 5e-9, False), (3, "tv", 500, 1e-9, False)])
def test_lanczos_matches_restatement(seed, model, itmax, delta, testenergy):
    """testenergy = False: the reference tests the residual |H A4 - E0 A4| of the current Ritz vector
    instead of the energy change (src/lanzcos.hpp:215-235)."""
    L, R, th, W1, W2, ik0, ik1 = _case(seed, model=model)
    E, n, st = O.lanczos(L, R, th, W1, W2, ik0, ik1, itmax=itmax, delta=delta, testenergy=testenergy, nthreads=2)
    keys, shapes, H, to_vec, to_blocks = ed.dense_heff_matrix(L, R, th, W1, W2, ik0, ik1)
    E_np, n_np, psi, tests = _lanczos_np(lambda x: to_blocks(H @ to_vec(x)), th, itmax, delta, testenergy=testenergy)
    # the stopping test must not sit at the threshold, or rounding could move the stop
    assert all(t < 0.1 * delta or t > 10 * delta for t in tests), tests
    assert n == n_np
    assert abs(E - E_np) < 1e-12 * abs(E_np)
    keys = set(st) | set(psi)
    zero = lambda k: np.zeros_like(st[k] if k in st else psi[k])
    diff = max(float(np.abs(st.get(k, zero(k)) - psi.get(k, zero(k))).max()) for k in keys)
    assert diff < 1e-8, diff
    if itmax == 7:
        assert n == 7  # the cap stops the loop before the second energy test


def test_lanczos_state_is_the_ground_state_of_the_dense_operator():
    """With a converged Lanczos the energy is the lowest eigenvalue of the effective Hamiltonian on
    the charge-allowed blocks and the state its eigenvector (up to sign)."""
    L, R, th, W1, W2, ik0, ik1 = _case(5)
    E, n, st = O.lanczos(L, R, th, W1, W2, ik0, ik1, itmax=500, delta=1e-13, nthreads=2)
    keys, shapes, H, to_vec, to_blocks = ed.dense_heff_matrix(L, R, th, W1, W2, ik0, ik1)
    assert set(st) <= set(keys)
    assert np.abs(H - H.T).max() < 1e-12 * np.abs(H).max()
    w, v = np.linalg.eigh(0.5 * (H + H.T))
    # the Krylov space of theta may miss a symmetry sector of H: compare with the lowest eigenvalue
    # whose eigenvector overlaps theta
    x0 = to_vec(th)
    j = next(j for j in range(len(w)) if abs(float(v[:, j] @ x0)) > 1e-8 * np.linalg.norm(x0))
    assert abs(E - w[j]) < 1e-11 * abs(w[j])
    psi = to_vec(st)
    assert abs(abs(float(psi @ v[:, j])) - 1.0) < 1e-8
