"""CPU tests: the oracle's two-site split against an independent numpy restatement of the
reference's split, on random block-sparse states.

The restatement follows the reference step by step:
* split (src/MPSfunctions.hpp:1142-1278): one matrix per centre charge qc = a + q(s1), rows stacked
  by s1 ascending, columns by s2 ascending; U blocks keyed (qc - q(s1), qc; s1), V^T blocks
  (qc, qc + q(s2); s2);
* BoostSVD (blas/lapack_routines.cpp:614-634) followed by FixPhase (blas/helperfunctions.hpp:18-51):
  the first entry of largest modulus of every V^T row made positive, U's column flipped with it;
* DiagBlockMatrix::truncate(chimax) (src/BlockTensor.hpp:234-276): all values in a multimap,
  walked from the largest (equal values: the later insertion first), at most chimax kept, values
  <= 1e-15 never kept, tw = 1 - sum of the kept squares (before normalisation);
* DiagBlockMatrix::truncate(tr_weight, chimax) (src/BlockTensor.hpp:84-136): tw starts at norm()
  (which is sqrt(sum s^2)), each kept value subtracts s^2 / norm, the walk stops when
  |tw| <= norm * tr_weight or chimax values are kept; tiny negative tw clamped to 0;
* normalize() divides by sqrt(sum s^2) of the kept values; dropDangling (src/MPSfunctions.hpp:
  1444-1484) removes the blocks of sectors with no kept value and cuts U / V^T to the kept count.

numpy's SVD (gesdd) stands in for the reference's gesvd: the values agree to rounding and the
vectors, after FixPhase, to rounding over the gap; the random sectors here have no degenerate values.
"""
import numpy as np
import pytest

from oracle import pyoracle as O


def _vec_abs_max_ind(v):
    ind, val = 0, 0.0
    for i, x in enumerate(v):
        if abs(x) > val:
            ind, val = i, abs(x)
    return ind


def _split_np(th, ik0, ik1, chimax, doTrunc, tr_weight, normalize):
    secs = {}
    for key, blk in th.items():
        a, b, s1, s2 = key
        secs.setdefault(a + ik0[s1], []).append((key, blk))
    full = {}
    for qc in sorted(secs):
        rows, cols = {}, {}
        for (a, b, s1, s2), blk in secs[qc]:
            rows[s1], cols[s2] = blk.shape
        r0, c0, m, n = {}, {}, 0, 0
        for s1 in sorted(rows):
            r0[s1], m = m, m + rows[s1]
        for s2 in sorted(cols):
            c0[s2], n = n, n + cols[s2]
        M = np.zeros((m, n))
        for (a, b, s1, s2), blk in secs[qc]:
            M[r0[s1]:r0[s1] + blk.shape[0], c0[s2]:c0[s2] + blk.shape[1]] = blk
        U, S, Vt = np.linalg.svd(M, full_matrices=False)
        for i in range(len(S)):
            if not Vt[i, _vec_abs_max_ind(Vt[i])] > 0:
                Vt[i] *= -1
                U[:, i] *= -1
        full[qc] = (U, S, Vt, r0, rows, c0, cols)
    # the multimap of all values: insertion by sector ascending, values in SVD order; the walk
    # from the largest takes equal values in reverse insertion order
    ins = [(float(s), qc) for qc in sorted(full) for s in full[qc][1]]
    walk = [ins[i] for i in reversed(sorted(range(len(ins)), key=lambda i: ins[i][0]))]
    if not chimax and doTrunc:
        chimax = 100
    if not chimax and not doTrunc:
        chimax = 200
    kept = {}
    if not doTrunc:
        tw, cnt = 1.0, 0
        for s, qc in walk:
            if cnt == chimax or not abs(s) > 1e-15:
                break
            tw -= s * s
            kept.setdefault(qc, []).append(s)
            cnt += 1
    else:
        norm = np.sqrt(sum(s * s for s, _ in ins))
        tw, cnt = norm, 0
        for s, qc in walk:
            if not (abs(tw) > norm * tr_weight and cnt < chimax):
                break
            tw -= s * s / norm
            kept.setdefault(qc, []).append(s)
            cnt += 1
        if tw < 0 and abs(tw) < 1e-14:
            tw = 0.0
    lam = {qc: np.array(v) for qc, v in kept.items()}
    if normalize and lam:
        nrm = np.sqrt(sum(float(v @ v) for v in lam.values()))
        lam = {qc: v / nrm for qc, v in lam.items()}
    Ub, Vb = {}, {}
    for qc, v in lam.items():
        U, S, Vt, r0, rows, c0, cols = full[qc]
        k = len(v)
        for s1 in rows:
            Ub[(qc - ik0[s1], qc, s1)] = U[r0[s1]:r0[s1] + rows[s1], :k]
        for s2 in cols:
            Vb[(qc, qc + ik1[s2], s2)] = Vt[:k, c0[s2]:c0[s2] + cols[s2]]
    return Ub, Vb, lam, tw, cnt


def _random_theta(rng, dims, ik0, ik1, scale=1.0):
    th = {}
    for a in dims:
        for s1 in range(len(ik0)):
            for s2 in range(len(ik1)):
                b = a + ik0[s1] + ik1[s2]
                if b in dims:
                    th[(a, b, s1, s2)] = scale * rng.standard_normal((dims[a], dims[b]))
    return th


def _compare(got, want, tol_vec=1e-10):
    U, Vt, lam, tw, chi = got
    Uw, Vw, lw, tww, chiw = want
    assert chi == chiw
    assert abs(tw - tww) <= 1e-12 * max(1.0, abs(tww)), (tw, tww)
    kept = {q: v for q, v in lam.items() if len(v)}
    assert sorted(kept) == sorted(lw)
    for q in lw:
        np.testing.assert_allclose(kept[q], lw[q], rtol=1e-12, atol=1e-14)
    assert sorted(U) == sorted(Uw) and sorted(Vt) == sorted(Vw)
    for k in Uw:
        assert U[k].shape == Uw[k].shape, k
        np.testing.assert_allclose(U[k], Uw[k], atol=tol_vec)
    for k in Vw:
        assert Vt[k].shape == Vw[k].shape, k
        np.testing.assert_allclose(Vt[k], Vw[k], atol=tol_vec)


SPIN = [0, 1]  # i_to_key of a spin-1/2 site: down -> 0, up -> 1


@pytest.mark.parametrize("seed,chimax", [(0, 6), (1, 12), (2, 1000), (3, 1)])
@pytest.mark.parametrize("normalize", [True, False])
def test_split_by_chimax_matches_restatement(seed, chimax, normalize):
    rng = np.random.default_rng(seed)
    dims = {q: int(rng.integers(1, 7)) for q in range(2, 8)}
    th = _random_theta(rng, dims, SPIN, SPIN)
    got = O.split(th, SPIN, SPIN, chimax, doTrunc=False, tr_weight=1e-12, normalize=normalize, nthreads=2)
    _compare(got, _split_np(th, SPIN, SPIN, chimax, False, 1e-12, normalize))


@pytest.mark.parametrize("seed,tr_weight,chimax", [(4, 1e-2, 100), (5, 1e-1, 100), (6, 1e-12, 5), (7, 0.3, 3)])
def test_split_by_weight_matches_restatement(seed, tr_weight, chimax):
    rng = np.random.default_rng(seed)
    dims = {q: int(rng.integers(1, 6)) for q in range(0, 5)}
    th = _random_theta(rng, dims, SPIN, SPIN)
    nrm = np.sqrt(sum(float((v * v).sum()) for v in th.values()))
    th = {k: v / nrm for k, v in th.items()}  # the weight-based cut measures against the norm
    got = O.split(th, SPIN, SPIN, chimax, doTrunc=True, tr_weight=tr_weight, normalize=True, nthreads=2)
    _compare(got, _split_np(th, SPIN, SPIN, chimax, True, tr_weight, True))


def test_split_weight_variant_returns_discarded_weight_over_the_norm():
    """truncate(tr_weight, chimax) starts tw at norm() = sqrt(sum s^2) and subtracts s^2 / norm: the
    returned weight is the discarded sum of squares divided by the norm (not a relative weight)."""
    th = {(0, 0, 0, 0): np.array([[3.0]]), (0, 1, 1, 0): np.array([[4.0]])}
    U, Vt, lam, tw, chi = O.split(th, SPIN, SPIN, 1, doTrunc=True, tr_weight=1e-12, normalize=False)
    assert chi == 1
    assert abs(tw - 9.0 / 5.0) < 1e-14
    kept = {q: v for q, v in lam.items() if len(v)}
    assert list(kept) == [1] and abs(kept[1][0] - 4.0) < 1e-14


def test_split_drops_zero_sectors_and_fixes_phases():
    """A sector whose matrix is zero keeps no value (<= 1e-15) and loses its U / V^T blocks; the
    largest-modulus entry of every kept V^T row is positive."""
    rng = np.random.default_rng(11)
    dims = {2: 3, 3: 4, 4: 2, 5: 3}
    th = _random_theta(rng, dims, SPIN, SPIN)
    zero_qc = 4  # every block with a + q(s1) = 4
    for k in th:
        if k[0] + SPIN[k[2]] == zero_qc:
            th[k] = np.zeros_like(th[k])
    got = O.split(th, SPIN, SPIN, 1000, doTrunc=False, tr_weight=1e-12, normalize=True, nthreads=2)
    want = _split_np(th, SPIN, SPIN, 1000, False, 1e-12, True)
    _compare(got, want)
    U, Vt, lam, tw, chi = got
    assert not len(lam.get(zero_qc, []))
    assert all(k[1] != zero_qc for k in U) and all(k[0] != zero_qc for k in Vt)
    for qc in {k[0] for k in Vt}:
        rows = np.hstack([Vt[k] for k in sorted(Vt) if k[0] == qc])
        for r in rows:
            assert r[_vec_abs_max_ind(r)] > 0
