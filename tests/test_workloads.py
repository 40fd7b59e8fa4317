"""The benchmark's synthetic inputs on the CPU: the mixed-canonical random U(1) MPS of the centre
update (left isometries left of the centre, right isometries right of it, charge conservation,
bond dimensions <= chi) and the batched-chains generator (lengths in 24..96, Delta in [0.5, 1.5),
deterministic)."""
import os
import sys

import numpy as np
import pytest

from mpstools_gb300 import models as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _orthonormal(Mx):
    r, c = Mx.shape
    G = Mx.T @ Mx if r >= c else Mx @ Mx.T
    return np.abs(G - np.eye(G.shape[0])).max()


@pytest.mark.parametrize("N,chi,center", [(14, 16, 6), (12, 8, 3)])
def test_mixed_canonical_state(N, chi, center):
    ik = M.u1_itokeys(N)
    sites = M.random_mixed_canonical_mps(N, N // 2, chi, 5, center)
    for x, blocks in enumerate(sites):
        for (a, b, s), v in blocks.items():
            assert b == a + int(ik[x][s])  # U(1) charge flows through every block
        for bond_side in (0, 1):
            dims = {}
            for k, v in blocks.items():
                dims.setdefault(k[bond_side], v.shape[bond_side])
                assert dims[k[bond_side]] == v.shape[bond_side]  # one dimension per charge and bond
            assert sum(dims.values()) <= chi
        if x < center or x > center + 1:
            left = x < center
            groups = {}
            for k in sorted(blocks):
                groups.setdefault(k[1] if left else k[0], []).append(k)
            for ks in groups.values():
                Mx = np.vstack([blocks[k] for k in ks]) if left else np.hstack([blocks[k] for k in ks])
                assert _orthonormal(Mx) < 1e-12


def test_mixed_canonical_state_bond_dimensions():
    N, chi = 16, 12
    sites = M.random_mixed_canonical_mps(N, N // 2, chi, 5, 7)
    for x in range(N - 1):
        right = {}
        for (a, b, s), v in sites[x].items():
            right.setdefault(b, v.shape[1])
        assert sum(right.values()) <= chi


def test_chains_workload_is_deterministic_and_in_range():
    l1, d1, c1 = bench.chains_workload(8, 64)  # chi >= the 49 charge sectors of a 96-site chain
    l2, d2, c2 = bench.chains_workload(8, 64)
    assert l1 == l2 and np.array_equal(d1, d2)
    assert all(24 <= n <= 96 for n in l1)
    assert np.all((d1 >= 0.5) & (d1 < 1.5))
    for (sites, W, ik), n in zip(c1, l1):
        assert len(sites) == n and len(W) == n and len(ik) == n


@pytest.mark.parametrize("model", ["xxz", "tv"])
def test_centre_workload(model):
    W, ik, sites, center = bench.workload(8, 10, model)
    assert center == 4 and len(W) == len(sites) == len(ik) == 10
    ref = (M.spinless_fermions_mpo(2.0 * M.uniform01(bench.SEED_V, 9), np.ones(9), np.zeros(10)) if model == "tv"
           else M.heisenberg_mpo(M.xxz_couplings(10, bench.SEED_DELTA), np.ones(9), np.zeros(10)))
    for a, b in zip(W, ref):
        assert a[1:] == b[1:] and sorted(a[0]) == sorted(b[0])
