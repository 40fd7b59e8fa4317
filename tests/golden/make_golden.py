"""Generate the golden fixtures in this directory.

ed_energies.json  exact-diagonalisation ground-state energies (scipy) of small XXZ / t-V chains
                  next to the oracle's DMRG energy for the same chain.
matvec_small.npz  one two-site matvec case (L, R, W1, W2, theta and the oracle's output) taken
                  from a DMRG run on a 12-site XXZ chain with a seeded random MPS.

Run from the repository root:  python tests/golden/make_golden.py
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


def main():
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

    N, site = 12, 4
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, 12, 7), W, ik, maxthreads=2)
    g.prepare()
    for s in range(site):
        g.do_step(s, 1, 12)
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
    print("wrote", len(cases), "energy cases and matvec_small.npz")


if __name__ == "__main__":
    main()
