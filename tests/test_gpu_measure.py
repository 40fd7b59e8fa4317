"""GPU parity of the measurement entry points against the oracle (FP64, 1e-12 relative):
computeOverlap, MPO::measure (energy and local operators), the two-tensor addContractionLayer, and
DMRGengine measurements of a converged state."""
import numpy as np
import pytest

from mpstools_gb300 import api, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _close(a, b, tol=1e-12):
    return abs(a - b) <= tol * max(abs(b), 1e-300)


def test_overlap_matches_oracle(ctx):
    N, Nup = 12, 6
    ik = M.u1_itokeys(N)
    a, b = M.random_u1_mps(N, Nup, 16, 3), M.random_u1_mps(N, Nup, 16, 4)
    for x, y in ((a, b), (b, a), (a, a)):
        ref = O.overlap(x, y, ik)
        got = api.computeOverlap(x, y, ik, ctx=ctx)
        assert _close(got, ref), (got, ref)


def test_mpo_measure_matches_oracle(ctx):
    N, Nup = 12, 6
    ik = M.u1_itokeys(N)
    a = M.random_u1_mps(N, Nup, 16, 5)
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    assert _close(api.measureMPO(a, W, ik, ctx=ctx), O.mpo_measure(a, W, ik))
    for site in (0, 5, N - 1):
        Wl = M.local_operator_mpo(N, site, np.diag([-0.5, 0.5]))
        assert _close(api.measureMPO(a, Wl, ik, ctx=ctx), O.mpo_measure(a, Wl, ik))


@pytest.mark.parametrize("direction", [1, -1])
def test_two_tensor_contraction_layer(ctx, direction):
    N, Nup, chi = 12, 6, 16
    ik = M.u1_itokeys(N)
    W = M.heisenberg_mpo(np.ones(N - 1), np.ones(N - 1), np.zeros(N))
    a, b = M.random_u1_mps(N, Nup, chi, 6), M.random_u1_mps(N, Nup, chi, 7)
    site = 5
    g = O.DMRG(a, W, ik, maxthreads=4)
    g.prepare()
    g.build_environments(site + 1)
    env = g.env("L", site - 1) if direction > 0 else g.env("R", site + 1)
    ref = O.add_contraction_layer2(env, a[site], b[site], W[site], ik[site], direction)
    got = api.addContractionLayer2(env, a[site], W[site], b[site], ik[site], direction, ctx=ctx)
    assert set(got) == set(ref)
    for k in ref:
        assert np.abs(got[k] - ref[k]).max() <= 1e-12 * max(np.abs(ref[k]).max(), 1.0)


def test_dmrg_local_measurements(ctx):
    """<Sz_i> and the energy of a converged DMRG state: engine measurement vs the oracle's MPO::measure
    on the engine's own site tensors, and the energy vs the oracle's DMRG run."""
    N = 16
    # a random longitudinal field breaks the spin-flip symmetry, so <Sz_i> is not zero
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), 0.5 * (M.uniform01(9, N) - 0.5))
    ik = M.u1_itokeys(N)
    sites = M.random_u1_mps(N, N // 2, 32, 11)
    go = O.DMRG(sites, W, ik, maxthreads=8)
    Eo = go.simulate(maxsteps=4, EnConv=1e-300, chimax=32, delta=1e-12)
    e = api.DMRGengine(sites, W, ik, ctx=ctx)
    Eg = e.simulate(maxsteps=4, EnConv=1e-300, chimax=32, delta=1e-12)
    assert abs(Eg - Eo) <= 1e-10 * abs(Eo)
    mine = [e.site(s) for s in range(N)]
    theirs = [go.site(s) for s in range(N)]
    for site in (0, 7, N - 1):
        Wl = M.local_operator_mpo(N, site, np.diag([-0.5, 0.5]))
        got = e.measure(Wl)
        assert abs(got - O.mpo_measure(mine, Wl, ik)) <= 1e-12      # same state, oracle arithmetic
        assert abs(got - O.mpo_measure(theirs, Wl, ik)) <= 1e-8     # the oracle's own DMRG state
        assert abs(got) > 1e-4
    assert _close(e.measure(W), O.mpo_measure(mine, W, ik), 1e-11)
    assert abs(e.measure(W) - Eo) <= 1e-10 * abs(Eo)
