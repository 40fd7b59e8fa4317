"""Exact diagonalisation and dense effective-Hamiltonian helpers (numpy/scipy).

Independent pins for the oracle: they build the Hamiltonian from its physics
definition (not from the MPO code) and contract environments densely.
"""
from __future__ import annotations

import itertools

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _basis(N, Nup):
    states = []
    for occ in itertools.combinations(range(N), Nup):
        s = 0
        for i in occ:
            s |= 1 << i
        states.append(s)
    states.sort()
    return states, {s: i for i, s in enumerate(states)}


def xxz_ground_energy(Jz, Jxy, B, Nup):
    """H = sum_i Jxy_i/2 (S+S- + h.c.) + Jz_i Sz Sz - sum_i B_i Sz_i, fixed up-count Nup."""
    H = xxz_hamiltonian(Jz, Jxy, B, Nup)
    if H.shape[0] <= 64:
        return float(np.linalg.eigvalsh(H.toarray())[0])
    return float(spla.eigsh(H, k=1, which="SA", tol=1e-14)[0][0])


def mps_sector_vector(sites, Nup):
    """Amplitudes of a U(1) block MPS on the basis of _basis(N, Nup) (site i <-> bit i, index 1 = up).

    Blocks (a, b, s) are placed at offsets of their charges on each bond; psi is contracted left to
    right over all 2^N configurations (N <= 12)."""
    N = len(sites)
    lays = []
    for i in range(N + 1):
        dims = {}
        if i > 0:
            for (a, b, s), m in sites[i - 1].items():
                dims[b] = m.shape[1]
        if i < N:
            for (a, b, s), m in sites[i].items():
                dims.setdefault(a, m.shape[0])
        lays.append(_bond_layout(dims))
    psi = np.zeros((1, lays[0][1]))
    psi[0, lays[0][0][0][0]] = 1.0
    for i in range(N):
        (lay_l, _), (lay_r, Dr) = lays[i], lays[i + 1]
        new = np.zeros((psi.shape[0] * 2, Dr))
        for (a, b, s), m in sites[i].items():
            oa, da = lay_l[a]
            ob, db = lay_r[b]
            rows = np.arange(psi.shape[0]) + s * psi.shape[0]
            new[rows, ob:ob + db] += psi[:, oa:oa + da] @ m
        psi = new
    full = psi[:, lays[N][0][Nup][0]] if Nup in lays[N][0] else np.zeros(psi.shape[0])
    states, _ = _basis(N, Nup)
    return full[np.asarray(states)]


def xxz_hamiltonian(Jz, Jxy, B, Nup):
    """Sparse H on the basis of _basis(N, Nup)."""
    N = len(B)
    states, idx = _basis(N, Nup)
    rows, cols, vals = [], [], []
    for k, s in enumerate(states):
        diag = 0.0
        for i in range(N):
            szi = 0.5 if (s >> i) & 1 else -0.5
            diag -= B[i] * szi
        for i in range(N - 1):
            a, b = (s >> i) & 1, (s >> (i + 1)) & 1
            diag += Jz[i] * (0.5 if a else -0.5) * (0.5 if b else -0.5)
            if a != b:
                t = s ^ (1 << i) ^ (1 << (i + 1))
                rows.append(idx[t]); cols.append(k); vals.append(Jxy[i] / 2.0)
        rows.append(k); cols.append(k); vals.append(diag)
    return sp.csr_matrix((vals, (rows, cols)), shape=(len(states), len(states)))


def tv_ground_energy(V, t, mu, Nf):
    """Spinless fermions H = sum_i -t_i (c+_i c_i+1 + h.c.) + V_i n_i n_i+1 - mu_i n_i (open chain)."""
    N = len(mu)
    states, idx = _basis(N, Nf)
    rows, cols, vals = [], [], []
    for k, s in enumerate(states):
        diag = 0.0
        for i in range(N):
            diag -= mu[i] * ((s >> i) & 1)
        for i in range(N - 1):
            a, b = (s >> i) & 1, (s >> (i + 1)) & 1
            diag += V[i] * a * b
            if a != b:  # nearest-neighbour hop: no fermion sign for adjacent sites
                u = s ^ (1 << i) ^ (1 << (i + 1))
                rows.append(idx[u]); cols.append(k); vals.append(-t[i])
        rows.append(k); cols.append(k); vals.append(diag)
    H = sp.csr_matrix((vals, (rows, cols)), shape=(len(states), len(states)))
    if H.shape[0] <= 64:
        return float(np.linalg.eigvalsh(H.toarray())[0])
    return float(spla.eigsh(H, k=1, which="SA", tol=1e-14)[0][0])


# --------------------------------------------------------------------------- dense H_eff
def _bond_layout(charges_dims):
    """charges_dims: {q: dim} -> {q: (offset, dim)}, total."""
    off, lay = 0, {}
    for q in sorted(charges_dims):
        lay[q] = (off, charges_dims[q])
        off += charges_dims[q]
    return lay, off


def _dense_parts(Lenv, Renv, theta, W1, W2, ik0, ik1):
    """Dense L[wl][a'(global), a(global)], R[wr][b', b], W as [wl, wr, out, in], and the bond layouts."""
    lq, rq = {}, {}
    for (q0, q1, w), m in Lenv.items():
        lq.setdefault(q0, m.shape[0]); lq.setdefault(q1, m.shape[1])
    for (q0, q1, w), m in Renv.items():
        rq.setdefault(q0, m.shape[0]); rq.setdefault(q1, m.shape[1])
    for (a, b, s1, s2), m in theta.items():
        lq.setdefault(a, m.shape[0]); rq.setdefault(b, m.shape[1])
    llay, nl = _bond_layout(lq)
    rlay, nr = _bond_layout(rq)
    d0, d1 = len(ik0), len(ik1)
    DW = max(max(t[0] for t in W1[0]), max(t[1] for t in W1[0]), max(t[0] for t in W2[0]),
             max(t[1] for t in W2[0]), max(k[2] for k in Lenv), max(k[2] for k in Renv)) + 1
    Ld = np.zeros((DW, nl, nl))
    Rd = np.zeros((DW, nr, nr))
    for (q0, q1, w), m in Lenv.items():
        o0, o1 = llay[q0][0], llay[q1][0]
        Ld[w, o0:o0 + m.shape[0], o1:o1 + m.shape[1]] = m
    for (q0, q1, w), m in Renv.items():
        o0, o1 = rlay[q0][0], rlay[q1][0]
        Rd[w, o0:o0 + m.shape[0], o1:o1 + m.shape[1]] = m
    W1d = np.zeros((DW, DW, d0, d0))
    W2d = np.zeros((DW, DW, d1, d1))
    for (wl, wr, o, i, v) in W1[0]:
        W1d[wl, wr, o, i] += v
    for (wl, wr, o, i, v) in W2[0]:
        W2d[wl, wr, o, i] += v
    # the charge-allowed blocks (a, b; s1, s2), b = a + q(s1) + q(s2)
    allowed = [(a, b, s1, s2) for a in lq for b in rq for s1 in range(d0) for s2 in range(d1)
               if a + ik0[s1] + ik1[s2] == b]
    return llay, rlay, nl, nr, d0, d1, Ld, Rd, W1d, W2d, allowed


def dense_heff_apply(Lenv, Renv, theta, W1, W2, ik0, ik1):
    """Apply L.W1.W2.R to theta by dense contraction (reference operator convention).

    out(a',b';s1',s2') = sum L[a',a;wl] W1[wl,wm](out=s1,in=s1') W2[wm,wr](out=s2,in=s2')
                         theta(a,b;s1,s2) R[b',b;wr]
    Result blocks are keyed like theta and restricted to blocks with nonzero support.
    """
    llay, rlay, nl, nr, d0, d1, Ld, Rd, W1d, W2d, allowed = _dense_parts(Lenv, Renv, theta, W1, W2, ik0, ik1)
    T = np.zeros((nl, d0, d1, nr))
    for (a, b, s1, s2), m in theta.items():
        oa, ob = llay[a][0], rlay[b][0]
        T[oa:oa + m.shape[0], s1, s2, ob:ob + m.shape[1]] = m
    # out[a', s1', s2', b'] = L[wl,a',a] W1[wl,wm,s1,s1'] W2[wm,wr,s2,s2'] T[a,s1,s2,b] R[wr,b',b]
    out = np.einsum("lxa,lmpP,mrqQ,apqb,ryb->xPQy", Ld, W1d, W2d, T, Rd, optimize=True)
    res = {}
    for (a, b, s1, s2) in allowed:
        oa, na = llay[a]
        ob, nb = rlay[b]
        res[(a, b, s1, s2)] = out[oa:oa + na, s1, s2, ob:ob + nb].copy()
    return res


def dense_heff_matrix(Lenv, Renv, theta, W1, W2, ik0, ik1):
    """The operator of dense_heff_apply as a matrix on the charge-allowed blocks (the blocks
    dense_heff_apply returns, in sorted key order, each flattened row-major).

    Returns (keys, shapes, H, to_vec, to_blocks) with to_vec(blocks) -> flat vector (missing blocks
    zero) and to_blocks(vector) -> {key: block}."""
    llay, rlay, nl, nr, d0, d1, Ld, Rd, W1d, W2d, allowed = _dense_parts(Lenv, Renv, theta, W1, W2, ik0, ik1)
    # the full operator on (a, s1, s2, b) x (a', s1', s2', b'), then restricted to the allowed blocks
    full = np.einsum("lxa,lmpP,mrqQ,ryb->xPQyapqb", Ld, W1d, W2d, Rd, optimize=True)
    nfull = nl * d0 * d1 * nr
    full = full.reshape(nfull, nfull)
    keys = sorted(allowed)
    shapes = {k: (llay[k[0]][1], rlay[k[1]][1]) for k in keys}
    idx = []
    for (a, b, s1, s2) in keys:
        oa, na = llay[a]
        ob, nb = rlay[b]
        ii = np.arange(oa, oa + na)[:, None] * (d0 * d1 * nr) + (s1 * d1 + s2) * nr + np.arange(ob, ob + nb)[None, :]
        idx.append(ii.ravel())
    idx = np.concatenate(idx) if idx else np.zeros(0, int)
    sizes = [int(np.prod(shapes[k])) for k in keys]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
    H = full[np.ix_(idx, idx)]

    def to_vec(x):
        v = np.zeros(len(idx))
        for i, k in enumerate(keys):
            if k in x:
                v[off[i]:off[i + 1]] = np.asarray(x[k]).ravel()
        return v

    def to_blocks(v):
        return {k: v[off[i]:off[i + 1]].reshape(shapes[k]).copy() for i, k in enumerate(keys)}

    return keys, shapes, H, to_vec, to_blocks


# --------------------------------------------------------------------------- dense TEBD reference
def spin_ops():
    sz = np.diag([-0.5, 0.5])
    sp = np.array([[0.0, 0.0], [1.0, 0.0]])  # |up><down| with index 1 = up
    return sz, sp, sp.T


def bond_hamiltonian(Jz, Jxy, B1, B2, w1, w2):
    """h_b = Jz SzSz + Jxy/2 (S+S- + S-S+) - w1 B1 Sz (x) 1 - w2 B2 1 (x) Sz, dense index o1 + 2*o2
    (site 1 is the fast index, numpy kron(op_site2, op_site1))."""
    sz, sp, sm = spin_ops()
    one = np.eye(2)
    h = Jz * np.kron(sz, sz) + 0.5 * Jxy * (np.kron(sm, sp) + np.kron(sp, sm))
    h -= w1 * B1 * np.kron(one, sz) + w2 * B2 * np.kron(sz, one)
    return h


def apply_two_site(psi, gate, s, N):
    """psi: full 2^N vector (site i <-> bit i, 1 = up); gate on sites (s, s+1), index o1 + 2*o2."""
    t = psi.reshape((2,) * N, order="F")  # axis i = site i
    g = gate.reshape((2, 2, 2, 2), order="F")  # (o1, o2, i1, i2)
    t = np.moveaxis(t, (s, s + 1), (0, 1))
    t = np.tensordot(g, t, axes=([2, 3], [0, 1]))
    t = np.moveaxis(t, (0, 1), (s, s + 1))
    return t.reshape(-1, order="F")


def dense_tebd_second_order(local, gates_full, gates_half, steps):
    N = len(local)
    psi = np.zeros(2 ** N, complex)
    psi[sum(int(v) << i for i, v in enumerate(local))] = 1.0
    def slice_(gates, start):
        nonlocal psi
        for s in range(start, N - 1, 2):
            psi = apply_two_site(psi, gates[s], s, N)
    slice_(gates_half, 1)
    for step in range(1, steps + 1):
        slice_(gates_full, 0)
        slice_(gates_full if step < steps else gates_half, 1)
    return psi


def sz_expect(psi, site, N):
    idx = np.arange(2 ** N)
    sz = np.where((idx >> site) & 1, 0.5, -0.5)
    return float(np.real(np.vdot(psi, sz * psi)))


def tebd_schedule(steps):
    """Layers of the second-order schedule: (first bond, half step?)."""
    out = [(1, True)]
    for step in range(1, steps + 1):
        out += [(0, False), (1, step == steps)]
    return out


def dense_tebd_adjoint(local, gates_full, gates_half, tang_full, tang_half, steps, obs_site):
    """<Sz_obs_site> after the dense second-order evolution and its gradient by the adjoint formula
    d<O>/dtheta_b = sum over layers holding b of 2 Re <chi_l| B_b |psi_l>, B_b = (dG_b/dtheta) G_b^H,
    psi_l the state after layer l, chi_l = (later layers)^H O psi_T."""
    N = len(local)
    psi = np.zeros(2 ** N, complex)
    psi[sum(int(v) << i for i, v in enumerate(local))] = 1.0
    states = []
    for start, half in tebd_schedule(steps):
        gates = gates_half if half else gates_full
        for s in range(start, N - 1, 2):
            psi = apply_two_site(psi, gates[s], s, N)
        states.append(psi)
    idx = np.arange(2 ** N)
    sz = np.where((idx >> obs_site) & 1, 0.5, -0.5)
    value = float(np.real(np.vdot(psi, sz * psi)))
    chi = sz * psi
    grad = np.zeros(N - 1)
    for li in range(len(states) - 1, -1, -1):
        start, half = tebd_schedule(steps)[li]
        tang = tang_half if half else tang_full
        gates = gates_half if half else gates_full
        for s in range(start, N - 1, 2):
            grad[s] += 2.0 * np.real(np.vdot(chi, apply_two_site(states[li], tang[s], s, N)))
        for s in range(start, N - 1, 2):
            chi = apply_two_site(chi, gates[s].conj().T, s, N)
    return value, grad
