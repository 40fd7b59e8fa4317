"""Generate the golden fixtures in this directory.

ed_energies.json  exact-diagonalisation ground-state energies (scipy) of small XXZ / t-V chains
                  next to the oracle's DMRG energy for the same chain.
matvec_small.npz  one two-site matvec case (L, R, W1, W2, theta and the oracle's output) taken
                  from a DMRG run on a 12-site XXZ chain with a seeded random MPS.
step_small.npz    the other pieces of one update of the same chain, each the oracle's output on the
                  stored inputs: the left environment update of the site tensor, the split of a
                  random normalised two-site tensor at a binding chimax (U, V^T, lambda, truncated
                  weight, kept count) and the Lanczos ground state of the two-site tensor.

Run from the repository root:  python tests/golden/make_golden.py [energies] [matvec] [step]
(no argument: all three).
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import ed  # noqa: E402
from golden_io import pack_bm, pack_mpo  # noqa: E402
from mpstools_gb300 import models as M  # noqa: E402
from oracle import pyoracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def energies():
    cases = []
    for N in (8, 10, 12):
        Jz, Jxy, B = M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N)
        W = M.heisenberg_mpo(Jz, Jxy, B)
        ik = M.u1_itokeys(N)
        g = O.DMRG(M.random_u1_mps(N, N // 2, 16, 12345), W, ik, maxthreads=2)
        E = g.simulate(maxsteps=4, EnConv=1e-300, chimax=128, delta=1e-12)
        cases.append(dict(model="xxz", N=N, seed_delta=1, chi=128, E_oracle=E,
                          E_ed=ed.xxz_ground_energy(Jz, Jxy, B, N // 2)))
    for N in (8, 10):
        V, t, mu = 2.0 * M.uniform01(2, N - 1), np.ones(N - 1), np.zeros(N)
        W = M.spinless_fermions_mpo(V, t, mu)
        ik = M.u1_itokeys(N)
        g = O.DMRG(M.product_state(M.filling_state(N, N // 2), ik), W, ik, maxthreads=2)
        E = g.simulate(maxsteps=4, EnConv=1e-300, chimax=128, delta=1e-12)
        cases.append(dict(model="tv", N=N, seed_V=2, chi=128, E_oracle=E, E_ed=ed.tv_ground_energy(V, t, mu, N // 2)))
    with open(os.path.join(HERE, "ed_energies.json"), "w") as f:
        json.dump(cases, f, indent=1)
    print("wrote", len(cases), "energy cases")


def _chain12():
    N, site = 12, 4
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, 12, 7), W, ik, maxthreads=2)
    g.prepare()
    for s in range(site):
        g.do_step(s, 1, 12)
    return g, W, ik, site


def matvec():
    g, W, ik, site = _chain12()
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    th = O.theta(g.site(site), g.site(site + 1))
    rng = np.random.default_rng(0)
    th = {k: rng.standard_normal(v.shape) for k, v in th.items()}
    out = O.contract_twosite(L, R, th, W[site], W[site + 1], ik[site], ik[site + 1])
    z = {}
    pack_bm("L", L, z)
    pack_bm("R", R, z)
    pack_bm("theta", th, z)
    pack_bm("out", out, z)
    pack_mpo("W1", W[site], z)
    pack_mpo("W2", W[site + 1], z)
    z["ik0"] = np.array(ik[site], np.int64)
    z["ik1"] = np.array(ik[site + 1], np.int64)
    np.savez_compressed(os.path.join(HERE, "matvec_small.npz"), **z)
    print("wrote matvec_small.npz")


def step():
    g, W, ik, site = _chain12()
    L, R = g.env("L", site - 1), g.env("R", site + 2)
    A1, A2 = g.site(site), g.site(site + 1)
    z = {}
    pack_bm("L", L, z)
    pack_bm("R", R, z)
    pack_bm("A1", A1, z)
    pack_bm("A2", A2, z)
    pack_mpo("W1", W[site], z)
    pack_mpo("W2", W[site + 1], z)
    z["ik0"] = np.array(ik[site], np.int64)
    z["ik1"] = np.array(ik[site + 1], np.int64)
    # environment update of the site tensor (direction +1)
    pack_bm("Lnext", O.add_contraction_layer(L, A1, W[site], ik[site], 1), z)
    # split of a random normalised two-site tensor at a binding chimax
    rng = np.random.default_rng(1)
    th = {k: rng.standard_normal(v.shape) for k, v in O.theta(A1, A2).items()}
    nrm = np.sqrt(sum(float((v * v).sum()) for v in th.values()))
    th = {k: v / nrm for k, v in th.items()}
    chimax = 10
    U, Vt, lam, tw, chi = O.split(th, ik[site], ik[site + 1], chimax, doTrunc=False, tr_weight=1e-12, normalize=True)
    pack_bm("split_theta", th, z)
    pack_bm("split_U", U, z)
    pack_bm("split_Vt", Vt, z)
    lq = sorted(q for q, v in lam.items() if len(v))
    z["split_lam_q"] = np.array(lq, np.int64)
    z["split_lam_n"] = np.array([len(lam[q]) for q in lq], np.int64)
    z["split_lam"] = np.concatenate([lam[q] for q in lq])
    z["split_scalars"] = np.array([chimax, tw, chi], np.float64)
    # Lanczos ground state of the two-site tensor
    E0, n, st = O.lanczos(L, R, O.theta(A1, A2), W[site], W[site + 1], ik[site], ik[site + 1], itmax=500, delta=1e-12)
    pack_bm("lanczos_state", st, z)
    z["lanczos_scalars"] = np.array([E0, n], np.float64)
    np.savez_compressed(os.path.join(HERE, "step_small.npz"), **z)
    print("wrote step_small.npz")


if __name__ == "__main__":
    todo = sys.argv[1:] or ["energies", "matvec", "step"]
    for name in todo:
        {"energies": energies, "matvec": matvec, "step": step}[name]()
