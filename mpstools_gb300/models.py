"""Model MPOs, charge maps and initial states for the DMRG path.

MPO matrices are lists of terms ``(wl, wr, out, in, value)`` plus the bond
dimensions ``(Dl, Dr)``: the entry ``W[wl, wr]`` is a sparse single-site
operator whose element ``(out, in)`` carries ``value`` (the reference's
``MPOMat<1,T>`` of ``SparseOperator<1,T>`` keyed by ``OpKeyType<1>(out, in)``,
src/MPOTypes.hpp:50-128,839-889).  Terms are listed in the reference's map order:
``(wl, wr)`` ascending, then ``(in, out)`` ascending.

Charges are packed ``AbKeyType`` words (src/keyTypes.hpp:20-124): with one
U(1) charge the word is just the particle / up-spin count.
"""
from __future__ import annotations

import numpy as np

MASK64 = (1 << 64) - 1

# --------------------------------------------------------------------------- operators
# single-site operators as {(out, in): value}
SZ = {(0, 0): -0.5, (1, 1): 0.5}
SP = {(1, 0): 1.0}
SM = {(0, 1): 1.0}
ID2 = {(0, 0): 1.0, (1, 1): 1.0}
NUM = {(0, 0): 0.0, (1, 1): 1.0}
CDAG = {(1, 0): 1.0}
CANN = {(0, 1): 1.0}
PJW = {(0, 0): 1.0, (1, 1): -1.0}


def op_scale(o, s):
    return {k: v * s for k, v in o.items()}


def op_mul(a, b):
    """Operator product (a*b)(out,in) = sum_k a(out,k) b(k,in) (src/MPOTypes.hpp:200-230)."""
    out = {}
    for (ao, ai), av in a.items():
        for (bo, bi), bv in b.items():
            if ai == bo:
                out[(ao, bi)] = out.get((ao, bi), 0.0) + av * bv
    return out


def _mpomat(entries, Dl, Dr, thresh=1e-16):
    """entries: {(wl, wr): op}; squeeze elements below thresh; reference map order."""
    terms = []
    for (wl, wr) in sorted(entries):
        o = entries[(wl, wr)]
        for (out, inn) in sorted(o, key=lambda k: (k[1], k[0])):
            v = o[(out, inn)]
            if abs(v) < thresh:
                continue
            terms.append((wl, wr, out, inn, float(v)))
    return (terms, Dl, Dr)


def heisenberg_mpo(Jz, Jxy, B):
    """XXZ / Heisenberg chain, D=5 (src/Hamiltonians.hpp:84-131).

    H = sum_i Jxy_i/2 (S+_i S-_{i+1} + h.c.) + Jz_i Sz_i Sz_{i+1} - sum_i B_i Sz_i.
    Jz, Jxy have N-1 entries (one per bond), B has N entries.
    """
    B = np.asarray(B, np.float64)
    N = len(B)
    Jz = np.r_[np.asarray(Jz, np.float64), 0.0]
    Jxy = np.r_[np.asarray(Jxy, np.float64), 0.0]
    W = []
    W.append(_mpomat({(0, 0): op_scale(SZ, -B[0]), (0, 1): op_scale(SM, Jxy[0] / 2.0),
                      (0, 2): op_scale(SP, Jxy[0] / 2.0), (0, 3): op_scale(SZ, Jz[0]), (0, 4): ID2}, 1, 5))
    for s in range(1, N - 1):
        W.append(_mpomat({(0, 0): ID2, (1, 0): SP, (2, 0): SM, (3, 0): SZ, (4, 0): op_scale(SZ, -B[s]),
                          (4, 1): op_scale(SM, Jxy[s] / 2.0), (4, 2): op_scale(SP, Jxy[s] / 2.0),
                          (4, 3): op_scale(SZ, Jz[s]), (4, 4): ID2}, 5, 5))
    W.append(_mpomat({(0, 0): ID2, (1, 0): SP, (2, 0): SM, (3, 0): SZ, (4, 0): op_scale(SZ, -B[N - 1])}, 5, 1))
    return W


def spinless_fermions_mpo(V, t, mu):
    """t-V chain with Jordan-Wigner string, D=5 (src/Hamiltonians.hpp:527-566).

    H = sum_i -t_i (c+_i c_{i+1} + h.c.) + V_i n_i n_{i+1} - sum_i mu_i n_i.
    """
    mu = np.asarray(mu, np.float64)
    N = len(mu)
    V = np.r_[np.asarray(V, np.float64), 0.0]
    t = np.r_[np.asarray(t, np.float64), 0.0]
    cp = op_mul(CANN, PJW)
    cdp = op_mul(CDAG, PJW)
    W = []
    W.append(_mpomat({(0, 0): op_scale(NUM, -mu[0]), (0, 1): op_scale(cp, t[0]), (0, 2): op_scale(cdp, -t[0]),
                      (0, 3): op_scale(NUM, V[0]), (0, 4): ID2}, 1, 5))
    for s in range(1, N - 1):
        W.append(_mpomat({(0, 0): ID2, (1, 0): CDAG, (2, 0): CANN, (3, 0): NUM, (4, 0): op_scale(NUM, -mu[s]),
                          (4, 1): op_scale(cp, t[s]), (4, 2): op_scale(cdp, -t[s]), (4, 3): op_scale(NUM, V[s]),
                          (4, 4): ID2}, 5, 5))
    W.append(_mpomat({(0, 0): ID2, (1, 0): CDAG, (2, 0): CANN, (3, 0): NUM, (4, 0): op_scale(NUM, -mu[N - 1])}, 5, 1))
    return W


def local_operator_mpo(N, site, op):
    """D = 1 MPO of the d x d operator `op` (op[out, in]) on `site`, identity elsewhere: MPO::measure
    with it gives the local expectation value <op_site> (the role of SparseLocalOperator::measure,
    src/MPOTypes.hpp:532-563, for states that are not in Vidal form)."""
    op = np.asarray(op, dtype=np.float64)
    d = op.shape[0]
    W = []
    for s in range(N):
        if s == site:
            terms = [(0, 0, o, i, float(op[o, i])) for i in range(d) for o in range(d) if op[o, i] != 0.0]
        else:
            terms = [(0, 0, i, i, 1.0) for i in range(d)]
        W.append((terms, 1, 1))
    return W


def u1_itokeys(N, d=2):
    """itokey per site: local state n -> charge n (spin-1/2: down->0, up->1; fermions: empty->0, full->1)."""
    return [[k for k in range(d)] for _ in range(N)]


# --------------------------------------------------------------------------- seeded generators
def splitmix64(seed: int, n: int) -> np.ndarray:
    """n outputs of the splitmix64 generator started at `seed` (uint64 array)."""
    with np.errstate(over="ignore"):
        g = np.uint64(0x9E3779B97F4A7C15)
        s = (np.uint64(seed & MASK64) + g * np.arange(1, n + 1, dtype=np.uint64)).astype(np.uint64)
        z = s
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int) -> np.ndarray:
    """n doubles in [0,1) from the top 53 bits of splitmix64."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def normal(seed: int, n: int) -> np.ndarray:
    """n N(0,1) doubles by Box-Muller on splitmix64 uniforms."""
    m = (n + 1) // 2
    u = uniform01(seed, 2 * m)
    u1 = 1.0 - u[0::2]  # (0,1]
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.empty(2 * m)
    z[0::2] = r * np.cos(2 * np.pi * u2)
    z[1::2] = r * np.sin(2 * np.pi * u2)
    return z[:n]


# --------------------------------------------------------------------------- MPS initial states
def product_state(local_state, itokeys):
    """Product-state MPS (src/MPSTypes.hpp:449-476): 1x1 blocks (q_l, q_l + q(s); s)."""
    sites = []
    ql = 0
    for s, ls in enumerate(local_state):
        qr = ql + itokeys[s][ls]
        sites.append({(ql, qr, int(ls)): np.ones((1, 1))})
        ql = qr
    return sites


def filling_state(N, Nup):
    """Filling of the reference drivers (main/mainHeisenberg.cpp:175-191): every (N//Nup)-th site up."""
    mod = N // Nup
    st, q = [], 0
    for s in range(N):
        if s % mod == 0 and q < Nup:
            st.append(1)
            q += 1
        else:
            st.append(0)
    if q != Nup:
        raise ValueError("could not generate filling")
    return st


def neel_state(N):
    return [s % 2 for s in range(N)]


def _comb(n, k):
    from math import comb
    return comb(n, k) if 0 <= k <= n else 0


def bond_sectors(N, Nup, chi):
    """Charge sectors and sizes on the N+1 bonds of a spin-1/2 / spinless chain with Nup particles.

    Bond b sits to the right of site b-1 (b=0: left edge, b=N: right edge).  Sector q on bond b
    has the exact Schmidt dimension min(C(b,q), C(N-b,Nup-q)); when the bond total exceeds chi
    the sizes are scaled down by that weight (largest remainders first), keeping every sector >= 1.
    """
    bonds = []
    for b in range(N + 1):
        qs = [q for q in range(max(0, Nup - (N - b)), min(b, Nup) + 1)]
        ex = {q: min(_comb(b, q), _comb(N - b, Nup - q)) for q in qs}
        tot = sum(ex.values())
        if tot <= chi:
            bonds.append(ex)
            continue
        if len(qs) > chi:
            raise ValueError("chi smaller than the number of charge sectors")
        base = {q: max(1, int(np.floor(chi * ex[q] / tot))) for q in qs}
        base = {q: min(base[q], ex[q]) for q in qs}
        rem = chi - sum(base.values())
        order = sorted(qs, key=lambda q: (-(chi * ex[q] / tot - np.floor(chi * ex[q] / tot)), q))
        while rem > 0:
            moved = False
            for q in order:
                if rem == 0:
                    break
                if base[q] < ex[q]:
                    base[q] += 1
                    rem -= 1
                    moved = True
            if not moved:
                break
        while rem < 0:
            for q in sorted(qs, key=lambda q: -base[q]):
                if rem == 0:
                    break
                if base[q] > 1:
                    base[q] -= 1
                    rem += 1
        bonds.append(base)
    return bonds


def random_u1_mps(N, Nup, chi, seed, itokeys=None):
    """Random MPS with U(1) blocks on every bond for all reachable charges (entries N(0,1)).

    Block (a, b; s) of site x exists when a is a sector of bond x, b = a + q(s) a sector of
    bond x+1.  Entries are drawn in site order, block key order, column-major.
    """
    if itokeys is None:
        itokeys = u1_itokeys(N)
    bonds = bond_sectors(N, Nup, chi)
    sizes = []
    for x in range(N):
        blocks = []
        for a in sorted(bonds[x]):
            for s in range(len(itokeys[x])):
                b = a + itokeys[x][s]
                if b in bonds[x + 1]:
                    blocks.append((a, b, s, bonds[x][a], bonds[x + 1][b]))
        blocks.sort(key=lambda t: (t[0], t[1], t[2]))
        sizes.append(blocks)
    total = sum(r * c for blk in sizes for (_, _, _, r, c) in blk)
    z = normal(seed, total)
    off = 0
    sites = []
    for blk in sizes:
        d = {}
        for (a, b, s, r, c) in blk:
            d[(a, b, s)] = z[off:off + r * c].reshape((r, c), order="F").copy()
            off += r * c
        sites.append(d)
    return sites


def random_mixed_canonical_mps(N, Nup, chi, seed, center, itokeys=None):
    """Random U(1) MPS in mixed-canonical form around bond (center, center+1).

    Sites left of `center` are left isometries (for every right charge b the stacked blocks
    [A(a,b;s)] over (a,s) have orthonormal columns), sites right of center+1 are right
    isometries (for every left charge a the blocks [B(a,b;s)] over (b,s) have orthonormal
    rows); the two centre sites keep their N(0,1) entries.  Where a charge group has fewer
    rows than columns the orthonormal side is swapped (the bond is larger than the sector's
    exact dimension).  Isometries come from the QR factorisation of the seeded N(0,1) blocks.
    """
    sites = random_u1_mps(N, Nup, chi, seed, itokeys)
    for x in list(range(center)) + list(range(center + 2, N)):
        blocks = sites[x]
        left = x < center
        groups = {}
        for k in sorted(blocks):
            groups.setdefault(k[1] if left else k[0], []).append(k)
        for _, ks in groups.items():
            if left:
                M = np.vstack([blocks[k] for k in ks])
            else:
                M = np.hstack([blocks[k] for k in ks]).T
            r, c = M.shape
            if r >= c:
                Qm, _ = np.linalg.qr(M)
            else:
                Qm, _ = np.linalg.qr(M.T)
                Qm = Qm.T
            if not left:
                Qm = Qm.T
            off = 0
            for k in ks:
                if left:
                    n = blocks[k].shape[0]
                    blocks[k] = np.ascontiguousarray(Qm[off:off + n, :])
                else:
                    n = blocks[k].shape[1]
                    blocks[k] = np.ascontiguousarray(Qm[:, off:off + n])
                off += n
    for x in (center, center + 1):
        nrm = np.sqrt(sum(float(np.vdot(v, v)) for v in sites[x].values()))
        for k in sites[x]:
            sites[x][k] = sites[x][k] / nrm
    return sites


def xxz_couplings(N, seed, lo=0.5, hi=1.5):
    """Delta_i ~ U[lo,hi] per bond (N-1 values) from splitmix64(seed)."""
    return lo + (hi - lo) * uniform01(seed, N - 1)
