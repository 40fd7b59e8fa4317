"""MPSGCKP1 checkpoints through the C ABI: a state written by the oracle side (numpy writer) loads
into the GPU engine with the oracle's energy; the GPU engine's own checkpoint reads back (numpy
reader) as its exported tensors; and a run that is saved, loaded and continued matches a run that
was never interrupted."""
import numpy as np
import pytest

from mpstools_gb300 import api, checkpoint, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def test_oracle_state_loads_into_the_engine(ctx, tmp_path):
    N, chi = 12, 16
    W = M.heisenberg_mpo(M.xxz_couplings(N, 2), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, 9), W, ik, maxthreads=2)
    g.simulate(maxsteps=1, EnConv=1e-300, chimax=chi, delta=1e-12)
    sites = [g.site(s) for s in range(N)]
    p = str(tmp_path / "oracle.mpsg")
    checkpoint.save(p, sites, W, ik, {b: g.lam(b) for b in range(N - 1)})
    e = api.DMRGengine.load(p, ctx=ctx)
    E = O.mpo_measure(sites, W, ik)
    assert abs(e.measure_energy() - E) <= 1e-12 * abs(E)
    e.close()


def test_engine_checkpoint_roundtrip_and_resume(ctx, tmp_path):
    N, chi = 12, 16
    W = M.heisenberg_mpo(M.xxz_couplings(N, 3), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    start = M.random_u1_mps(N, N // 2, chi, 11)
    a = api.DMRGengine(start, W, ik, ctx=ctx)
    a.simulate(maxsteps=1, EnConv=1e-300, chimax=chi, delta=1e-12)
    p = str(tmp_path / "engine.mpsg")
    a.save(p)
    sites, W2, ik2, lam = checkpoint.load(p)
    for s in range(N):
        exp = a.site(s)
        assert set(exp) == set(sites[s])
        for k in exp:
            assert np.array_equal(np.asarray(exp[k]), sites[s][k])
    assert len(lam) > 0
    b = api.DMRGengine.load(p, ctx=ctx)
    assert abs(b.measure_energy() - a.measure_energy()) <= 1e-13 * abs(a.measure_energy())
    Ea = a.simulate(maxsteps=1, EnConv=1e-300, chimax=chi, delta=1e-12)
    Eb = b.simulate(maxsteps=1, EnConv=1e-300, chimax=chi, delta=1e-12)
    assert abs(Ea - Eb) <= 1e-12 * abs(Ea)
    a.close()
    b.close()
