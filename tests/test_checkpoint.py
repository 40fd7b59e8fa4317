"""MPSGCKP1 checkpoints on the CPU: a DMRG state made by the oracle written and read back by
mpstools_gb300.checkpoint is identical, and the oracle's energy of the re-read state equals the
original one; a truncated file is rejected."""
import numpy as np
import pytest

from mpstools_gb300 import checkpoint, models as M
from oracle import pyoracle as O


def _state(N=10, chi=12, seed=3):
    W = M.heisenberg_mpo(M.xxz_couplings(N, 1), np.ones(N - 1), np.zeros(N))
    ik = M.u1_itokeys(N)
    g = O.DMRG(M.random_u1_mps(N, N // 2, chi, seed), W, ik, maxthreads=2)
    g.simulate(maxsteps=1, EnConv=1e-300, chimax=chi, delta=1e-12)
    sites = [g.site(s) for s in range(N)]
    lam = {b: g.lam(b) for b in range(N - 1)}
    return g, sites, W, ik, lam


def test_roundtrip_of_an_oracle_state(tmp_path):
    g, sites, W, ik, lam = _state()
    p = str(tmp_path / "state.mpsg")
    checkpoint.save(p, sites, W, ik, lam)
    s2, W2, ik2, lam2 = checkpoint.load(p)
    assert checkpoint.read_header(p) == {"version": 2, "N": len(sites)}
    assert checkpoint.read_settings(p) == checkpoint.DEFAULT_SETTINGS
    assert ik2 == [list(map(int, k)) for k in ik]
    for a, b in zip(sites, s2):
        assert set(a) == set(b)
        for k in a:
            assert np.array_equal(np.asarray(a[k]), b[k])
    for (t, Dl, Dr), (t2, Dl2, Dr2) in zip(W, W2):
        assert (Dl, Dr) == (Dl2, Dr2)
        assert sorted(t, key=lambda x: (x[0], x[1], x[3], x[2])) == [tuple(x) for x in t2]
    for b in lam:
        assert set(lam[b]) == set(lam2[b])
        for q in lam[b]:
            assert np.array_equal(np.asarray(lam[b][q]), lam2[b][q])
    E = O.mpo_measure(sites, W, ik)
    assert abs(O.mpo_measure(s2, W2, ik2) - E) <= 1e-14 * abs(E)


def test_truncated_file_is_rejected(tmp_path):
    g, sites, W, ik, lam = _state(N=6, chi=4)
    p = tmp_path / "state.mpsg"
    checkpoint.save(str(p), sites, W, ik, lam)
    data = p.read_bytes()
    (tmp_path / "cut.mpsg").write_bytes(data[: len(data) // 2])
    with pytest.raises(ValueError):
        checkpoint.load(str(tmp_path / "cut.mpsg"))


def test_settings_record_and_version_1_files(tmp_path):
    g, sites, W, ik, lam = _state(N=6, chi=4)
    p = tmp_path / "state.mpsg"
    st = {"prec": 6, "reorth": 1, "lanmax": 123, "updates": 77}
    checkpoint.save(str(p), sites, W, ik, lam, settings=st)
    assert checkpoint.read_settings(str(p)) == st
    # the same file as version 1: no settings record, read with the defaults
    data = p.read_bytes()
    v1 = data[:8] + (1).to_bytes(4, "little") + data[12:16] + data[36:]
    (tmp_path / "v1.mpsg").write_bytes(v1)
    assert checkpoint.read_settings(str(tmp_path / "v1.mpsg")) == checkpoint.DEFAULT_SETTINGS
    s2, W2, ik2, lam2 = checkpoint.load(str(tmp_path / "v1.mpsg"))
    for a, b in zip(sites, s2):
        for k in a:
            assert np.array_equal(np.asarray(a[k]), b[k])
