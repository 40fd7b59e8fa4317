"""CPU tests: the oracle against exact diagonalisation, dense contractions and the golden fixtures."""
import json
import os

import numpy as np
import pytest

import ed
from mpstools_gb300 import models as M
from oracle import pyoracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _dmrg(W, sites, ik, chi, sweeps, threads=4):
    g = O.DMRG(sites, W, ik, maxthreads=threads)
    E = g.simulate(maxsteps=sweeps, EnConv=1e-300, chimax=chi, delta=1e-12)
    return g, E


@pytest.mark.parametrize("N", [6, 10, 12])
def test_heisenberg_energy_matches_ed(N):
    Nup = N // 2
    Jz, Jxy, B = np.ones(N - 1), np.ones(N - 1), np.zeros(N)
    W = M.heisenberg_mpo(Jz, Jxy, B)
    ik = M.u1_itokeys(N)
    g, E = _dmrg(W, M.product_state(M.filling_state(N, Nup), ik), ik, 256, 4)
    assert abs(E - ed.xxz_ground_energy(Jz, Jxy, B, Nup)) < 1e-10
    assert abs(g.measure() - E) < 1e-10


def test_xxz_random_start_matches_ed():
    N, Nup = 12, 6
    Jz, Jxy, B = M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N)
    W = M.heisenberg_mpo(Jz, Jxy, B)
    ik = M.u1_itokeys(N)
    _, E = _dmrg(W, M.random_u1_mps(N, Nup, 16, 12345), ik, 64, 4)
    assert abs(E - ed.xxz_ground_energy(Jz, Jxy, B, Nup)) < 1e-10


def test_tv_fermions_match_ed():
    N, Nf = 10, 5
    V, t, mu = 2.0 * M.uniform01(2, N - 1), np.ones(N - 1), np.zeros(N)
    W = M.spinless_fermions_mpo(V, t, mu)
    ik = M.u1_itokeys(N)
    _, E = _dmrg(W, M.product_state(M.filling_state(N, Nf), ik), ik, 64, 4)
    assert abs(E - ed.tv_ground_energy(V, t, mu, Nf)) < 1e-10


def test_mpo_builders_agree():
    N = 7
    Jz, Jxy, B = M.xxz_couplings(N, 3), np.full(N - 1, 0.7), np.linspace(-0.3, 0.4, N)
    assert M.heisenberg_mpo(Jz, Jxy, B) == O.heisenberg_mpo(Jz, Jxy, B)
    V, t, mu = M.uniform01(4, N - 1), np.ones(N - 1), np.full(N, 0.25)
    assert M.spinless_fermions_mpo(V, t, mu) == O.spinless_fermions_mpo(V, t, mu)


def _env_case(seed=7, N=12, chi=12, site=4):
    Jz = M.xxz_couplings(N, 1)
    W = M.heisenberg_mpo(Jz, np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, seed), W, ik, maxthreads=2)
    g.prepare()
    for s in range(site):
        g.do_step(s, 1, chi)
    return g, W, ik


def test_oracle_matvec_matches_dense_contraction():
    g, W, ik = _env_case()
    site = 4
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    rng = np.random.default_rng(0)
    th = {k: rng.standard_normal(v.shape) for k, v in th.items()}
    out = O.contract_twosite(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
    ref = ed.dense_heff_apply(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
    assert set(out) <= set(ref)
    for k, v in ref.items():
        got = out.get(k, np.zeros_like(v))
        assert np.abs(got - v).max() < 1e-12 * max(1.0, np.abs(v).max())


def test_oracle_env_update_matches_dense():
    g, W, ik = _env_case()
    site = 4
    Lprev = g.env("L", site - 1)
    A = g.site(site)
    out = O.add_contraction_layer(Lprev, A, W[site], ik[site], 1)
    # dense: L'[b',b;w'] = sum W[w,w'](out,in) A(a',b';in)^T L(a',a;w) A(a,b;out)
    for (b1, b, w1), blk in out.items():
        acc = np.zeros_like(blk)
        for (wl, wr, so, si, v) in W[site][0]:
            if wr != w1:
                continue
            for (a1, a, w), Lb in Lprev.items():
                if w != wl:
                    continue
                au = A.get((a1, b1, si))
                ad = A.get((a, b, so))
                if au is None or ad is None:
                    continue
                acc += v * au.T @ Lb @ ad
        assert np.abs(acc - blk).max() < 1e-12


def test_oracle_env_update_right_matches_dense():
    """addContractionLayer with direction <= 0 (src/MPSfunctions.hpp:276-352, add_out_sub_2):
    R'[a',a;wl] = sum over W[wl,wr](out,in) of A(a',b';in) R[b',b;wr] A(a,b;out)^T."""
    g, W, ik = _env_case()
    site = 6
    Rprev = g.env("R", site + 1)
    A = g.site(site)
    out = O.add_contraction_layer(Rprev, A, W[site], ik[site], -1)
    assert out
    for (a1, a, w0), blk in out.items():
        acc = np.zeros_like(blk)
        for (wl, wr, so, si, v) in W[site][0]:
            if wl != w0:
                continue
            for (b1, b, w), Rb in Rprev.items():
                if w != wr:
                    continue
                au = A.get((a1, b1, si))
                ad = A.get((a, b, so))
                if au is None or ad is None:
                    continue
                acc += v * au @ Rb @ ad.T
        assert np.abs(acc - blk).max() < 1e-12


def test_golden_fixtures_reproduce():
    """The committed fixtures (tests/golden/make_golden.py) are reproduced by the oracle."""
    with open(os.path.join(GOLDEN, "ed_energies.json")) as f:
        cases = json.load(f)
    for c in cases:
        assert abs(c["E_oracle"] - c["E_ed"]) < 1e-10
    z = np.load(os.path.join(GOLDEN, "matvec_small.npz"), allow_pickle=False)
    from golden_io import load_case
    case = load_case(z)
    out = O.contract_twosite(case["L"], case["R"], case["theta"], case["W1"], case["W2"], case["ik0"], case["ik1"])
    assert set(out) == set(case["out"])
    for k in out:
        assert np.abs(out[k] - case["out"][k]).max() < 1e-13


def test_golden_step_fixture_reproduces():
    """tests/golden/step_small.npz (made by tests/golden/make_golden.py from the oracle): the left
    environment update, the split at a binding chimax and the Lanczos ground state of one update of
    a 12-site XXZ chain are reproduced by the oracle from the stored inputs."""
    from golden_io import unpack_bm, unpack_mpo
    z = np.load(os.path.join(GOLDEN, "step_small.npz"), allow_pickle=False)
    L, R, A1, A2 = (unpack_bm(n, z) for n in ("L", "R", "A1", "A2"))
    W1, W2 = unpack_mpo("W1", z), unpack_mpo("W2", z)
    ik0, ik1 = [int(x) for x in z["ik0"]], [int(x) for x in z["ik1"]]

    def same(a, b, tol):
        assert set(a) == set(b)
        for k in a:
            assert a[k].shape == b[k].shape and np.abs(a[k] - b[k]).max() <= tol, k

    same(O.add_contraction_layer(L, A1, W1, ik0, 1), unpack_bm("Lnext", z), 1e-13)
    chimax, tw0, chi0 = z["split_scalars"]
    U, Vt, lam, tw, chi = O.split(unpack_bm("split_theta", z), ik0, ik1, int(chimax), doTrunc=False,
                                  tr_weight=1e-12, normalize=True)
    assert chi == int(chi0) and abs(tw - tw0) < 1e-14
    kept = {q: v for q, v in lam.items() if len(v)}
    assert sorted(kept) == [int(q) for q in z["split_lam_q"]]
    np.testing.assert_allclose(np.concatenate([kept[q] for q in sorted(kept)]), z["split_lam"], rtol=1e-13)
    same(U, unpack_bm("split_U", z), 1e-11)
    same(Vt, unpack_bm("split_Vt", z), 1e-11)
    E0, n0 = z["lanczos_scalars"]
    E, n, st = O.lanczos(L, R, O.theta(A1, A2), W1, W2, ik0, ik1, itmax=500, delta=1e-12)
    assert n == int(n0) and abs(E - E0) < 1e-13 * abs(E0)
    same(st, unpack_bm("lanczos_state", z), 1e-10)


def test_oracle_overlap_and_measure_match_dense():
    """computeOverlap and MPO::measure (energy, local Sz) against dense state vectors."""
    N, Nup = 8, 4
    ik = M.u1_itokeys(N)
    a, b = M.random_u1_mps(N, Nup, 6, 1), M.random_u1_mps(N, Nup, 6, 2)
    va, vb = ed.mps_sector_vector(a, Nup), ed.mps_sector_vector(b, Nup)
    assert abs(O.overlap(a, b, ik) - va @ vb) <= 1e-12 * abs(va @ vb)
    assert abs(O.overlap(b, a, ik) - va @ vb) <= 1e-12 * abs(va @ vb)
    Jz = M.xxz_couplings(N, 1)
    W = M.heisenberg_mpo(Jz, np.ones(N - 1), np.zeros(N))
    H = ed.xxz_hamiltonian(Jz, np.ones(N - 1), np.zeros(N), Nup)
    e_dense = va @ (H @ va)
    assert abs(O.mpo_measure(a, W, ik) - e_dense) <= 1e-12 * abs(e_dense)
    states, _ = ed._basis(N, Nup)
    for site in (0, 3, N - 1):
        sz = np.array([0.5 if (s >> site) & 1 else -0.5 for s in states])
        ref = (va ** 2 * sz).sum()
        got = O.mpo_measure(a, M.local_operator_mpo(N, site, np.diag([-0.5, 0.5])), ik)
        assert abs(got - ref) <= 1e-12 * np.abs(va ** 2).sum()


def _bond_weights(s, N):
    if s == 0:
        return 1.0, 0.5
    if s + 1 == N - 1:
        return 0.5, 1.0
    return 0.5, 0.5


def test_oracle_nn_gate_matches_expm():
    """MPO::getNNGate restatement: exp(-i dt h_b) with boundary-aware halves of the field terms."""
    import scipy.linalg as sla
    N = 6
    Jz, B = M.xxz_couplings(N, 4, 0.8, 1.2), 0.3 * np.arange(1, N + 1)
    W = M.heisenberg_mpo(Jz, np.ones(N - 1), B)
    for s in range(N - 1):
        for dt in (0.05, 0.05 - 0.02j):
            g = O.nn_gate(W[s], W[s + 1], s, N, dt)
            w1, w2 = _bond_weights(s, N)
            h = ed.bond_hamiltonian(Jz[s], 1.0, B[s], B[s + 1], w1, w2)
            ref = sla.expm(-1j * complex(dt).real * h - complex(dt).imag * h)
            assert np.abs(g - ref).max() < 1e-13, (s, dt)


def test_oracle_tebd_matches_dense_trotter():
    """Second-order TEBD without truncation against the same gate sequence on the dense state."""
    N, steps, dt = 8, 10, 0.05
    Jz = M.xxz_couplings(N, 4, 0.8, 1.2)
    W = M.heisenberg_mpo(Jz, np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    local = M.neel_state(N)
    t = O.TEBD(local, W, ik)
    t.second_order(steps, dt, chimax=64)
    full = [O.nn_gate(W[s], W[s + 1], s, N, dt) for s in range(N - 1)]
    half = [O.nn_gate(W[s], W[s + 1], s, N, dt / 2) for s in range(N - 1)]
    psi = ed.dense_tebd_second_order(local, full, half, steps)
    for site in range(N):
        ref = ed.sz_expect(psi, site, N)
        got = t.measure_diag(site, [-0.5, 0.5])
        assert abs(got - ref) < 1e-12, (site, got, ref)
    assert abs(ed.sz_expect(psi, 0, N) - (-0.5)) > 1e-3  # the state did evolve


def test_oracle_truncation_ties_keep_the_later_sector():
    """DiagBlockMatrix::truncate (src/BlockTensor.hpp:234-276) walks the values of a reversed
    std::multimap: by value descending, equal values in reverse insertion order (later charge sector
    first).  Two 1x1 sectors with the same singular value and chimax = 1: the second one is kept."""
    th = {(0, 0, 0, 0): np.array([[0.6]]), (0, 1, 1, 0): np.array([[0.6]])}
    ik = [0, 1]
    U, Vt, lam, tw, chi = O.split(th, ik, ik, 1, doTrunc=False, tr_weight=1e-12, normalize=True)
    assert chi == 1
    kept = {q: v for q, v in lam.items() if len(v)}
    assert list(kept) == [1] and abs(kept[1][0] - 1.0) < 1e-15
    assert abs(tw - (1.0 - 0.36)) < 1e-15  # 1 - the kept value squared, before normalisation


def _right_orthonormal_error(site):
    acc = {}
    for (a, b, s), m in site.items():
        acc[a] = acc.get(a, 0) + m @ m.T
    return max(np.abs(x - np.eye(x.shape[0])).max() for x in acc.values())


def test_oracle_prepare_is_right_canonical_and_keeps_the_state():
    """orthonormalize(mps, "rl") (src/MPSfunctions.hpp:1756-1792, prepareSite "r" with truncation of
    values <= 1e-16): every site right-orthonormal, the state unchanged up to its norm (the norm
    goes to the left boundary and is dropped), and a bond direction that carries no weight is cut."""
    N = 10
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    sites = M.random_u1_mps(N, N // 2, 6, 5)
    v0 = ed.mps_sector_vector(sites, N // 2)

    def prepared(s):
        g = O.DMRG(s, W, ik, maxthreads=2)
        g.prepare()
        return [g.site(x) for x in range(N)]

    ps = prepared(sites)
    v1 = ed.mps_sector_vector(ps, N // 2)
    assert abs(np.linalg.norm(v1) - 1.0) < 1e-13
    assert abs(abs(float(v0 @ v1)) / np.linalg.norm(v0) - 1.0) < 1e-13
    for x in range(N):
        assert _right_orthonormal_error(ps[x]) < 1e-13, x
    # a redundant direction on bond x: a zero row in the left sector q of site x and a random
    # column in the right sector q of site x - 1 (the state does not change)
    x = N // 2
    q = sorted({k[0] for k in sites[x]} & {k[1] for k in sites[x - 1]})[1]
    rng = np.random.default_rng(0)
    aug = [dict(t) for t in sites]
    for k, m in list(aug[x].items()):
        if k[0] == q:
            aug[x][k] = np.vstack([m, np.zeros((1, m.shape[1]))])
    for k, m in list(aug[x - 1].items()):
        if k[1] == q:
            aug[x - 1][k] = np.hstack([m, rng.standard_normal((m.shape[0], 1))])
    assert np.abs(ed.mps_sector_vector(aug, N // 2) - v0).max() < 1e-12
    pa = prepared(aug)
    dims = lambda st: [sorted((k, m.shape) for k, m in t.items()) for t in st]
    assert dims(pa) == dims(ps)
    v2 = ed.mps_sector_vector(pa, N // 2)
    assert abs(abs(float(v2 @ v1)) - 1.0) < 1e-13


def _left_orthonormal_error(site):
    acc = {}
    for (a, b, s), m in site.items():
        acc[b] = acc.get(b, 0) + m.T @ m
    return max(np.abs(x - np.eye(x.shape[0])).max() for x in acc.values())


def test_oracle_do_step_absorbs_lambda_by_direction():
    """DMRGengine::doStep (src/container.hpp:292-337): split into U, lambda, V^T; lambda goes right
    (dir > 0: site keeps U, left-orthonormal; site+1 = lambda V^T) or left (dir <= 0: site = U lambda;
    site+1 keeps V^T, right-orthonormal).  Without truncation the state after the step is the
    normalised Lanczos ground state, whose energy the step returns."""
    N = 10
    W = M.heisenberg_mpo(M.xxz_couplings(N, 2), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, 32, 9), W, ik, maxthreads=2)
    g.prepare()
    for site in range(4):
        E = g.do_step(site, 1, 1000)
        assert _left_orthonormal_error(g.site(site)) < 1e-12
        lam = g.lam(site)
        nrm = sum(float(v @ v) for v in lam.values())
        assert abs(nrm - 1.0) < 1e-13
        # site+1 = lambda V^T: its rows scaled back by 1/lambda are orthonormal
        B = {k: m / lam[k[0]][:, None] for k, m in g.site(site + 1).items()}
        assert _right_orthonormal_error(B) < 1e-10
        assert abs(g.measure() - E) < 1e-11 * abs(E)
    for site in range(4, 0, -1):
        E = g.do_step(site, -1, 1000)
        assert _right_orthonormal_error(g.site(site + 1)) < 1e-12
        lam = g.lam(site)
        A = {k: m / lam[k[1]][None, :] for k, m in g.site(site).items()}
        assert _left_orthonormal_error(A) < 1e-10
        assert abs(g.measure() - E) < 1e-11 * abs(E)


def test_oracle_theta_formation():
    """BlockMatrix<2>(B1, B2) (src/BlockTensor.hpp:285-301): theta(a,b;s1,s2) = A1(a,c;s1) A2(c,b;s2)
    for every pair of blocks sharing the middle charge c (one pair per key)."""
    N = 10
    ik = M.u1_itokeys(N)
    sites = M.random_u1_mps(N, N // 2, 12, 4)
    A1, A2 = sites[4], sites[5]
    th = O.theta(A1, A2)
    want = {}
    for (a, c, s1), m1 in A1.items():
        for (c2, b, s2), m2 in A2.items():
            if c2 == c:
                assert (a, b, s1, s2) not in want
                want[(a, b, s1, s2)] = m1 @ m2
    assert set(th) == set(want)
    for k in want:
        assert np.abs(th[k] - want[k]).max() < 1e-13 * max(1.0, np.abs(want[k]).max())
