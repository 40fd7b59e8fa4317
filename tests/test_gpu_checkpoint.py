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


def test_options_are_restored_and_corrupt_files_are_rejected(ctx, tmp_path):
    import ctypes as C
    from mpstools_gb300 import lib
    N, chi = 10, 8
    W = M.heisenberg_mpo(M.xxz_couplings(N, 4), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    a = api.DMRGengine(M.random_u1_mps(N, N // 2, chi, 13), W, ik, prec="mixed", lanmax=321, ctx=ctx)
    a.simulate(maxsteps=1, EnConv=1e-300, chimax=chi, delta=1e-12)
    p = tmp_path / "mixed.mpsg"
    a.save(str(p))
    assert checkpoint.read_settings(str(p))["prec"] == lib.PREC["mixed"]
    b = api.DMRGengine.load(str(p), ctx=ctx)
    assert b.options() == {"prec": lib.PREC["mixed"], "reorth": 0, "lanmax": 321}
    b.close()
    a.close()
    # an MPO term whose wl index exceeds Dl, and a file cut inside the block data: MPSG_ERR_ARG
    sites, W2, ik2, lam = checkpoint.load(str(p))
    bad = list(W2)
    terms, Dl, Dr = bad[3]
    bad[3] = ([(Dl + 2,) + tuple(terms[0][1:])] + list(terms[1:]), Dl, Dr)
    checkpoint.save(str(tmp_path / "bad.mpsg"), sites, bad, ik2, lam)
    h = C.c_void_p()
    assert ctx.L.mpsg_dmrg_load(ctx.h, str(tmp_path / "bad.mpsg").encode(), C.byref(h)) == 1
    assert b"out of range" in ctx.L.mpsg_last_error()
    data = p.read_bytes()
    (tmp_path / "cut.mpsg").write_bytes(data[: len(data) * 2 // 3])
    assert ctx.L.mpsg_dmrg_load(ctx.h, str(tmp_path / "cut.mpsg").encode(), C.byref(h)) == 1
    assert b"truncated" in ctx.L.mpsg_last_error()
