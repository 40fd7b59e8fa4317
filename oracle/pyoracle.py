"""ctypes binding of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker and by bench.py for the timed CPU baseline.  The product package
(mpstools_gb300) never imports this module.

Parity unpinned: MPSTools has no tests or golden vectors and cannot be built here, so
no output of the reference itself checks the oracle; tests/ check it against exact
diagonalisation, dense contractions and numpy restatements of the reference's split,
truncation and Lanczos instead.

Block matrices cross this boundary as plain dicts:
  single-site / environment:  {(q0, q1, p0): 2-D float64 array}
  two-site theta:             {(q0, q1, p0, p1): 2-D float64 array}
  lambda:                     {q: 1-D float64 array}
MPO matrices as lists of (wl, wr, out, in, value) plus (Dl, Dr).
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def openblas_path() -> str:
    """Locate the LP64 OpenBLAS bundled with scipy (exports scipy_dgemm_ & co)."""
    import scipy

    base = os.path.dirname(os.path.dirname(scipy.__file__))
    cands = sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas-*.so")))
    cands = [c for c in cands if "openblas64" not in c]
    if not cands:
        raise RuntimeError("scipy's bundled OpenBLAS (libscipy_openblas-*.so) not found")
    return cands[0]


def build(force: bool = False) -> str:
    """Compile oracle.cpp into oracle/liboracle.so (g++, OpenMP)."""
    out = os.path.join(_HERE, "liboracle.so")
    src = os.path.join(_HERE, "oracle.cpp")
    if force or not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", out,
                               src, "-ldl"])
    return out


def lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    path = build()
    L = C.CDLL(path)
    vp, i32, f64 = C.c_void_p, C.c_int, C.c_double
    P = C.POINTER
    L.orc_init.argtypes = [C.c_char_p]
    L.orc_bm_new.restype = vp
    L.orc_bm_new.argtypes = [i32, i32, vp, vp, vp, vp, vp]
    L.orc_bm_nblocks.argtypes = [vp]
    L.orc_bm_nphys.argtypes = [vp]
    L.orc_bm_size.argtypes = [vp]
    L.orc_bm_size.restype = C.c_long
    L.orc_bm_export.argtypes = [vp, vp, vp, vp, vp, vp]
    L.orc_bm_free.argtypes = [vp]
    L.orc_mpo_new.restype = vp
    L.orc_mpo_new.argtypes = [i32, vp, vp, vp, vp, vp, i32, i32]
    L.orc_mpo_nterms.argtypes = [vp]
    L.orc_mpo_export.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.orc_mpo_free.argtypes = [vp]
    L.orc_mpo_heisenberg.argtypes = [i32, vp, vp, vp, vp]
    L.orc_mpo_spinless.argtypes = [i32, vp, vp, vp, vp]
    L.orc_theta.restype = vp
    L.orc_theta.argtypes = [vp, vp]
    L.orc_contract_twosite.restype = vp
    L.orc_contract_twosite.argtypes = [vp, vp, vp, vp, vp, vp, i32, vp, i32, i32]
    L.orc_add_contraction_layer.restype = vp
    L.orc_add_contraction_layer.argtypes = [vp, vp, vp, vp, i32, i32, i32]
    L.orc_add_contraction_layer2.restype = vp
    L.orc_add_contraction_layer2.argtypes = [vp, vp, vp, vp, vp, i32, i32, i32]
    L.orc_overlap.restype = f64
    L.orc_overlap.argtypes = [i32, vp, vp, vp, vp, i32]
    L.orc_mpo_measure.restype = f64
    L.orc_mpo_measure.argtypes = [i32, vp, vp, vp, vp, i32]
    L.orc_split.argtypes = [vp, vp, i32, vp, i32, i32, i32, f64, i32, i32, P(vp), P(vp), P(vp),
                            P(f64), P(i32)]
    L.orc_lanczos.argtypes = [vp, vp, vp, vp, vp, vp, i32, vp, i32, i32, f64, i32, i32, P(f64),
                              P(i32), P(vp)]
    L.orc_dmrg_new.restype = vp
    L.orc_dmrg_new.argtypes = [i32, vp, vp, vp, i32]
    L.orc_dmrg_set_threads.argtypes = [vp, i32, i32]
    L.orc_dmrg_simulate.restype = f64
    L.orc_dmrg_simulate.argtypes = [vp, i32, f64, i32, i32, f64, f64, i32]
    L.orc_dmrg_prepare.argtypes = [vp]
    L.orc_dmrg_build_envs.argtypes = [vp, i32]
    L.orc_dmrg_set_env.argtypes = [vp, i32, i32, vp]
    L.orc_dmrg_do_step.restype = f64
    L.orc_dmrg_do_step.argtypes = [vp, i32, i32, i32, i32, f64, f64, i32]
    L.orc_dmrg_nsteps.argtypes = [vp]
    L.orc_dmrg_steps.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.orc_dmrg_times.argtypes = [vp, vp]
    L.orc_dmrg_site.restype = vp
    L.orc_dmrg_site.argtypes = [vp, i32]
    L.orc_dmrg_lambda.restype = vp
    L.orc_dmrg_lambda.argtypes = [vp, i32]
    L.orc_dmrg_env.restype = vp
    L.orc_dmrg_env.argtypes = [vp, i32, i32]
    L.orc_dmrg_measure.restype = f64
    L.orc_dmrg_measure.argtypes = [vp, i32]
    L.orc_dmrg_free.argtypes = [vp]
    L.orc_tebd_new.restype = vp
    L.orc_tebd_new.argtypes = [i32, vp, vp, vp, vp]
    L.orc_tebd_second_order.argtypes = [vp, i32, f64, i32, i32, f64, i32]
    L.orc_tebd_measure_diag.restype = f64
    L.orc_tebd_measure_diag.argtypes = [vp, i32, vp, i32]
    L.orc_tebd_gamma_info.restype = i32
    L.orc_tebd_gamma_info.argtypes = [vp, i32, P(C.c_long)]
    L.orc_tebd_gamma_export.argtypes = [vp, i32, vp, vp, vp, vp, vp]
    L.orc_tebd_lambda.restype = vp
    L.orc_tebd_lambda.argtypes = [vp, i32]
    L.orc_nn_gate.argtypes = [vp, vp, i32, i32, f64, f64, i32, i32, vp]
    L.orc_tebd_free.argtypes = [vp]
    rc = L.orc_init(openblas_path().encode())
    if rc != 0:
        raise RuntimeError(f"oracle: orc_init failed ({rc})")
    _LIB = L
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None and a.size else None


# ------------------------------------------------------------------ conversion
def bm_to_handle(bm: dict, nphys: int):
    L = lib()
    keys = sorted(bm.keys())
    n = len(keys)
    q = np.zeros(2 * max(n, 1), np.uint64)
    p = np.zeros(max(1, nphys) * max(n, 1), np.uint32)
    rows = np.zeros(max(n, 1), np.int32)
    cols = np.zeros(max(n, 1), np.int32)
    chunks = []
    for i, k in enumerate(keys):
        a = np.asarray(bm[k], dtype=np.float64)
        if nphys == 0:
            q[2 * i] = q[2 * i + 1] = k
            a = a.reshape(-1, 1)
        else:
            q[2 * i], q[2 * i + 1] = k[0], k[1]
            for j in range(nphys):
                p[nphys * i + j] = k[2 + j]
        rows[i], cols[i] = a.shape
        chunks.append(np.asfortranarray(a).ravel(order="F"))
    data = np.concatenate(chunks) if chunks else np.zeros(1)
    return L.orc_bm_new(nphys, n, _ptr(q), _ptr(p), _ptr(rows), _ptr(cols), _ptr(data))


def handle_to_bm(h, free: bool = True) -> dict:
    L = lib()
    n = L.orc_bm_nblocks(h)
    nphys = L.orc_bm_nphys(h)
    size = L.orc_bm_size(h)
    q = np.zeros(2 * max(n, 1), np.uint64)
    p = np.zeros(max(1, nphys) * max(n, 1), np.uint32)
    rows = np.zeros(max(n, 1), np.int32)
    cols = np.zeros(max(n, 1), np.int32)
    data = np.zeros(max(size, 1))
    L.orc_bm_export(h, _ptr(q), _ptr(p), _ptr(rows), _ptr(cols), _ptr(data))
    out = {}
    off = 0
    for i in range(n):
        r, c = int(rows[i]), int(cols[i])
        a = data[off:off + r * c].reshape((r, c), order="F").copy()
        off += r * c
        if nphys == 0:
            out[int(q[2 * i])] = a[:, 0].copy()
        elif nphys == 1:
            out[(int(q[2 * i]), int(q[2 * i + 1]), int(p[i]))] = a
        else:
            out[(int(q[2 * i]), int(q[2 * i + 1]), int(p[2 * i]), int(p[2 * i + 1]))] = a
    if free:
        L.orc_bm_free(h)
    return out


def mpo_to_handle(terms, Dl, Dr):
    L = lib()
    n = len(terms)
    arr = lambda j, dt: np.array([t[j] for t in terms] or [0], dtype=dt)
    wl, wr, out, inn = (arr(j, np.uint32) for j in range(4))
    val = arr(4, np.float64)
    return L.orc_mpo_new(n, _ptr(wl), _ptr(wr), _ptr(out), _ptr(inn), _ptr(val), Dl, Dr)


def handle_to_mpo(h, free=True):
    L = lib()
    n = L.orc_mpo_nterms(h)
    wl, wr, out, inn = (np.zeros(max(n, 1), np.uint32) for _ in range(4))
    val = np.zeros(max(n, 1))
    d = np.zeros(2, np.int32)
    L.orc_mpo_export(h, _ptr(wl), _ptr(wr), _ptr(out), _ptr(inn), _ptr(val), _ptr(d))
    terms = [(int(wl[i]), int(wr[i]), int(out[i]), int(inn[i]), float(val[i])) for i in range(n)]
    if free:
        L.orc_mpo_free(h)
    return terms, int(d[0]), int(d[1])


# ------------------------------------------------------------------ API mirroring the reference
def heisenberg_mpo(Jz, Jxy, B):
    L = lib()
    N = len(B)
    Jz = np.ascontiguousarray(np.r_[Jz, 0.0], np.float64)
    Jxy = np.ascontiguousarray(np.r_[Jxy, 0.0], np.float64)
    B = np.ascontiguousarray(B, np.float64)
    hs = (C.c_void_p * N)()
    L.orc_mpo_heisenberg(N, _ptr(Jz), _ptr(Jxy), _ptr(B), hs)
    return [handle_to_mpo(hs[i]) for i in range(N)]


def spinless_fermions_mpo(V, t, mu):
    L = lib()
    N = len(mu)
    V = np.ascontiguousarray(np.r_[V, 0.0], np.float64)
    t = np.ascontiguousarray(np.r_[t, 0.0], np.float64)
    mu = np.ascontiguousarray(mu, np.float64)
    hs = (C.c_void_p * N)()
    L.orc_mpo_spinless(N, _ptr(V), _ptr(t), _ptr(mu), hs)
    return [handle_to_mpo(hs[i]) for i in range(N)]


def theta(A1, A2):
    L = lib()
    h1, h2 = bm_to_handle(A1, 1), bm_to_handle(A2, 1)
    out = handle_to_bm(L.orc_theta(h1, h2))
    L.orc_bm_free(h1)
    L.orc_bm_free(h2)
    return out


def contract_twosite(Lenv, Renv, th, W1, W2, ik0, ik1, nthreads=8):
    L = lib()
    hL, hR, hT = bm_to_handle(Lenv, 1), bm_to_handle(Renv, 1), bm_to_handle(th, 2)
    w1, w2 = mpo_to_handle(*W1), mpo_to_handle(*W2)
    a, b = np.asarray(ik0, np.uint64), np.asarray(ik1, np.uint64)
    out = handle_to_bm(L.orc_contract_twosite(hL, hR, hT, w1, w2, _ptr(a), len(a), _ptr(b), len(b), nthreads))
    for h in (hL, hR, hT):
        L.orc_bm_free(h)
    L.orc_mpo_free(w1)
    L.orc_mpo_free(w2)
    return out


def add_contraction_layer(BL, A, W, ik, direction, nthreads=8):
    L = lib()
    hB, hA = bm_to_handle(BL, 1), bm_to_handle(A, 1)
    w = mpo_to_handle(*W)
    a = np.asarray(ik, np.uint64)
    out = handle_to_bm(L.orc_add_contraction_layer(hB, hA, w, _ptr(a), len(a), int(direction), nthreads))
    L.orc_bm_free(hB)
    L.orc_bm_free(hA)
    L.orc_mpo_free(w)
    return out


def add_contraction_layer2(BL, A, Ap, W, ik, direction, nthreads=8):
    """Two-tensor addContractionLayer(BL, A, mpo, Ap, itokey, direction): A lower, Ap upper."""
    L = lib()
    hB, hA, hP = bm_to_handle(BL, 1), bm_to_handle(A, 1), bm_to_handle(Ap, 1)
    w = mpo_to_handle(*W)
    a = np.asarray(ik, np.uint64)
    out = handle_to_bm(L.orc_add_contraction_layer2(hB, hA, hP, w, _ptr(a), len(a), int(direction), nthreads))
    for h in (hB, hA, hP):
        L.orc_bm_free(h)
    L.orc_mpo_free(w)
    return out


def _site_handles(sites):
    hs = [bm_to_handle(s, 1) for s in sites]
    arr = (C.c_void_p * len(hs))(*hs)
    return hs, arr


def _ik_tables(iks):
    flat = np.ascontiguousarray(np.concatenate([np.asarray(k, np.uint64) for k in iks]), np.uint64)
    d = np.ascontiguousarray([len(k) for k in iks], np.int32)
    return flat, d


def overlap(a, b, iks, nthreads=8):
    """computeOverlap(a, b): a lower (ket), b upper (bra)."""
    L = lib()
    ha, pa = _site_handles(a)
    hb, pb = _site_handles(b)
    flat, d = _ik_tables(iks)
    try:
        return L.orc_overlap(len(a), pa, pb, _ptr(flat), _ptr(d), nthreads)
    finally:
        for h in ha + hb:
            L.orc_bm_free(h)


def mpo_measure(sites, W, iks, nthreads=8):
    """MPO::measure(mps) on the given site tensors and MPO (list of (terms, Dl, Dr))."""
    L = lib()
    hs, ps = _site_handles(sites)
    ws = [mpo_to_handle(*w) for w in W]
    pw = (C.c_void_p * len(ws))(*ws)
    flat, d = _ik_tables(iks)
    try:
        return L.orc_mpo_measure(len(sites), ps, pw, _ptr(flat), _ptr(d), nthreads)
    finally:
        for h in hs:
            L.orc_bm_free(h)
        for w in ws:
            L.orc_mpo_free(w)


def split(th, ik0, ik1, chimax, doTrunc=False, tr_weight=1e-12, normalize=True, nthreads=8):
    L = lib()
    hT = bm_to_handle(th, 2)
    a, b = np.asarray(ik0, np.uint64), np.asarray(ik1, np.uint64)
    U, V, lam = C.c_void_p(), C.c_void_p(), C.c_void_p()
    tw, chi = C.c_double(), C.c_int()
    L.orc_split(hT, _ptr(a), len(a), _ptr(b), len(b), int(chimax), int(doTrunc), float(tr_weight),
                int(normalize), nthreads, C.byref(U), C.byref(V), C.byref(lam), C.byref(tw), C.byref(chi))
    L.orc_bm_free(hT)
    return handle_to_bm(U.value), handle_to_bm(V.value), handle_to_bm(lam.value), tw.value, chi.value


def lanczos(Lenv, Renv, th, W1, W2, ik0, ik1, itmax=500, delta=1e-12, testenergy=True, nthreads=8):
    L = lib()
    hL, hR, hT = bm_to_handle(Lenv, 1), bm_to_handle(Renv, 1), bm_to_handle(th, 2)
    w1, w2 = mpo_to_handle(*W1), mpo_to_handle(*W2)
    a, b = np.asarray(ik0, np.uint64), np.asarray(ik1, np.uint64)
    E0, it, st = C.c_double(), C.c_int(), C.c_void_p()
    L.orc_lanczos(hL, hR, hT, w1, w2, _ptr(a), len(a), _ptr(b), len(b), itmax, delta, int(testenergy),
                  nthreads, C.byref(E0), C.byref(it), C.byref(st))
    for h in (hL, hR, hT):
        L.orc_bm_free(h)
    L.orc_mpo_free(w1)
    L.orc_mpo_free(w2)
    return E0.value, it.value, handle_to_bm(st.value)


class DMRG:
    """Oracle DMRGengine: sites = list of single-site dicts, mpo = list of (terms, Dl, Dr)."""

    def __init__(self, sites, mpo, itokeys, maxthreads=None, matvec_threads=8):
        L = lib()
        N = len(sites)
        self.N = N
        hs = (C.c_void_p * N)(*[bm_to_handle(s, 1) for s in sites])
        ws = (C.c_void_p * N)(*[mpo_to_handle(*w) for w in mpo])
        d = len(itokeys[0])
        ik = np.ascontiguousarray(np.asarray(itokeys, np.uint64).ravel())
        self.h = L.orc_dmrg_new(N, hs, ws, _ptr(ik), d)
        for i in range(N):
            L.orc_bm_free(hs[i])
            L.orc_mpo_free(ws[i])
        if maxthreads is None:
            maxthreads = os.cpu_count() or 1
        L.orc_dmrg_set_threads(self.h, int(maxthreads), int(matvec_threads))

    def simulate(self, maxsteps=5, EnConv=1e-10, chimax=100, doTrunc=False, tr_weight=1e-12, delta=1e-13,
                 testenergy=True):
        return lib().orc_dmrg_simulate(self.h, maxsteps, EnConv, chimax, int(doTrunc), tr_weight, delta,
                                       int(testenergy))

    def prepare(self):
        lib().orc_dmrg_prepare(self.h)

    def build_environments(self, center):
        lib().orc_dmrg_build_envs(self.h, int(center))

    def set_env(self, which, site, bm):
        h = bm_to_handle(bm, 1)
        lib().orc_dmrg_set_env(self.h, 1 if which == "R" else 0, int(site), h)
        lib().orc_bm_free(h)

    def do_step(self, site, direction, chimax, doTrunc=False, tr_weight=1e-12, delta=1e-12, testenergy=True):
        return lib().orc_dmrg_do_step(self.h, site, direction, chimax, int(doTrunc), tr_weight, delta,
                                      int(testenergy))

    def steps(self):
        L = lib()
        n = L.orc_dmrg_nsteps(self.h)
        a = [np.zeros(max(n, 1), np.int32) for _ in range(4)]
        E, tw = np.zeros(max(n, 1)), np.zeros(max(n, 1))
        L.orc_dmrg_steps(self.h, *[_ptr(x) for x in a], _ptr(E), _ptr(tw))
        return [dict(site=int(a[0][i]), dir=int(a[1][i]), iters=int(a[2][i]), chi=int(a[3][i]),
                     E=float(E[i]), tw=float(tw[i])) for i in range(n)]

    def times(self):
        t = np.zeros(4)
        lib().orc_dmrg_times(self.h, _ptr(t))
        return dict(total=t[0], matvec=t[1], env=t[2], split=t[3])

    def site(self, s):
        return handle_to_bm(lib().orc_dmrg_site(self.h, s))

    def lam(self, bond):
        return handle_to_bm(lib().orc_dmrg_lambda(self.h, bond))

    def env(self, which, s):
        return handle_to_bm(lib().orc_dmrg_env(self.h, 1 if which == "R" else 0, s))

    def measure(self, nthreads=1):
        return lib().orc_dmrg_measure(self.h, nthreads)

    def __del__(self):
        try:
            lib().orc_dmrg_free(self.h)
        except Exception:
            pass


# ------------------------------------------------------------------ single-site DMRG (CPU restatement)
def _svd_groups(mats):
    """Economy SVD (LAPACK through numpy) of each group matrix, no truncation (prepareBlock with
    truncate=false, src/MPSfunctions.hpp:21-142)."""
    return {q: np.linalg.svd(m, full_matrices=False) for q, m in mats.items()}


def prepare_left(A, B=None):
    """prepareMatrix(A, lambda, B, "l", multiply=true): per right charge the blocks of A stacked by rows
    = U D Vd; A <- U, lambda = D, B <- D Vd B for B's blocks with that left charge."""
    groups = {}
    for k in sorted(A):
        groups.setdefault(k[1], []).append(k)
    mats = {q: np.vstack([A[k] for k in ks]) for q, ks in groups.items()}
    out, lam, dv = {}, {}, {}
    for q, (U, D, Vd) in _svd_groups(mats).items():
        r0 = 0
        for k in groups[q]:
            out[k] = U[r0:r0 + A[k].shape[0], :].copy()
            r0 += A[k].shape[0]
        lam[q] = D.copy()
        dv[q] = D[:, None] * Vd
    if B is not None:
        B = {k: (dv[k[0]] @ v if k[0] in dv else v) for k, v in B.items()}
    return out, B, lam


def prepare_right(A, B):
    """prepareMatrix(A, lambda, B, "r", multiply=true): per left charge the blocks of B side by side =
    U D Vd; B <- Vd, lambda = D, A <- A U D for A's blocks with that right charge (A may be None)."""
    groups = {}
    for k in sorted(B):
        groups.setdefault(k[0], []).append(k)
    mats = {q: np.hstack([B[k] for k in ks]) for q, ks in groups.items()}
    out, lam, ud = {}, {}, {}
    for q, (U, D, Vd) in _svd_groups(mats).items():
        c0 = 0
        for k in groups[q]:
            out[k] = Vd[:, c0:c0 + B[k].shape[1]].copy()
            c0 += B[k].shape[1]
        lam[q] = D.copy()
        ud[q] = U * D[None, :]
    if A is not None:
        A = {k: (v @ ud[k[1]] if k[1] in ud else v) for k, v in A.items()}
    return A, out, lam


class SSDMRG:
    """SSDMRGengine (src/container.hpp:827-925) restated on the oracle's kernels: the single-site
    Lanczos (SSLanzcosEngine, src/lanzcos.hpp:503-600) is the oracle's Lanczos on contractSingle,
    written as the two-site contraction with a dummy second site (identity MPO tensor on the right
    channels, one local state of charge 0); prepareSite without truncation; addContractionLayer for
    the environments."""

    def __init__(self, sites, mpo, itokeys):
        self.N = len(sites)
        self.W, self.ik = mpo, itokeys
        g = DMRG(sites, mpo, itokeys, maxthreads=2)
        g.prepare()  # orthonormalize("rl")
        self.sites = [g.site(s) for s in range(self.N)]
        last = self.sites[-1]
        dims = {}
        for (q0, q1, p), v in last.items():
            dims.setdefault(q1, v.shape[1])
        self.R = {self.N: {(q, q, 0): np.eye(n) for q, n in dims.items()}}  # getRMax
        for s in range(self.N - 1, 0, -1):  # computeR(mps, mpo, 1)
            self.R[s] = add_contraction_layer(self.R[s + 1], self.sites[s], mpo[s], itokeys[s], 0)
        self.L = {-1: {(0, 0, 0): np.ones((1, 1))}}  # getLMin
        self.steps = []

    def do_step(self, site, direction, delta=1e-12, testenergy=True, itmax=500):
        W1 = self.W[site]
        D = W1[2]
        W2 = ([(w, w, 0, 0, 1.0) for w in range(D)], D, D)
        th = {(a, b, p, 0): v for (a, b, p), v in self.sites[site].items()}
        E, it, psi = lanczos(self.L[site - 1], self.R[site + 1], th, W1, W2, self.ik[site], [0], itmax, delta,
                             testenergy)
        A = {(a, b, p): v for (a, b, p, _), v in psi.items()}
        if direction > 0:
            nxt = self.sites[site + 1] if site + 1 < self.N else None
            A, nxt, lam = prepare_left(A, nxt)
            if nxt is not None:
                self.sites[site + 1] = nxt
            self.sites[site] = A
            self.L[site] = add_contraction_layer(self.L[site - 1], A, W1, self.ik[site], 1)
        else:
            prv = self.sites[site - 1] if site > 0 else None
            prv, A, lam = prepare_right(prv, A)
            if prv is not None:
                self.sites[site - 1] = prv
            self.sites[site] = A
            self.R[site] = add_contraction_layer(self.R[site + 1], A, W1, self.ik[site], -1)
        self.steps.append(dict(site=site, dir=direction, iters=it, E=E))
        return E

    def simulate(self, maxsteps=5, EnConv=1e-10, delta=1e-12, testenergy=True):
        globalE, step = 1e100, 0
        while True:
            for site in range(self.N - 1):
                out = self.do_step(site, 1, delta, testenergy)
            for site in range(self.N - 1, 0, -1):
                out = self.do_step(site, -1, delta, testenergy)
            step += 1
            conv = abs(globalE - out) < EnConv or step > maxsteps
            globalE = out
            if conv:
                break
        return self.do_step(0, -1, delta, testenergy)


# ------------------------------------------------------------------ excited states (CPU restatement)
def _dot(a, b):
    return float(sum(np.vdot(a[k], b[k]) for k in a.keys() & b.keys()))


def _axpy(y, a, x):
    """y + a x over the union of the blocks (BlockMatrix arithmetic)."""
    out = {k: v.copy() for k, v in y.items()}
    for k, v in x.items():
        out[k] = out[k] + a * v if k in out else a * v
    return out


def identity_mpo(d):
    return ([(0, 0, i, i, 1.0) for i in range(d)], 1, 1)


def lanczos_projected(Lenv, Renv, th, W1, W2, ik0, ik1, state, itmax=500, delta=1e-12, testenergy=True):
    """TSLanzcosEngine::simulate(itmax, delta, testenergy, state, delta_ortho) (src/lanzcos.hpp:282-400):
    the Lanczos of the oracle with the start vector and every new Krylov vector projected orthogonal
    to `state` (squeezed at 1e-15).  Returns (E0, iterations, lowest Ritz vector)."""
    from scipy.linalg import eigh_tridiagonal
    state = {k: v for k, v in state.items() if np.abs(v).max() > 1e-15}
    sn = _dot(state, state)
    A1 = _axpy(th, -_dot(state, th) / sn, state) if sn > 0 else dict(th)
    As, es, ks = [], [], []
    eold, it, first, A0 = 1e100, 0, True, None
    while True:
        k = np.sqrt(_dot(A1, A1))
        if abs(k) < delta:
            break
        if not first:
            ks.append(k)
        A1 = {key: v / k for key, v in A1.items()}
        A2 = contract_twosite(Lenv, Renv, A1, W1, W2, ik0, ik1)
        As.append(A1)
        e = _dot(A2, A1)
        es.append(e)
        if it % 5 == 0 and it != 0 and testenergy:
            E0 = eigh_tridiagonal(np.array(es), np.array(ks), eigvals_only=True)[0]
            if abs(E0 - eold) < delta:
                break
            eold = E0
        A3 = _axpy(A2, -e, A1)
        if not first:
            A3 = _axpy(A3, -k, A0)
        if sn > 0:
            A3 = _axpy(A3, -_dot(state, A3) / sn, state)
        A0, A1, first = A1, A3, False
        it += 1
        if it >= itmax:
            break
    w, z = eigh_tridiagonal(np.array(es), np.array(ks))
    psi = {}
    for zi, Ai in zip(z[:, 0], As):
        psi = _axpy(psi, zi, Ai)
    return float(w[0]), len(es), psi


class ExcitedDMRG:
    """DMRGengine::simulate(mps, delta_ortho, ...) (src/container.hpp:441-570) restated on the oracle's
    kernels: two-site sweeps with the projected Lanczos; the target state enters each update through
    the overlap environments <target|state> and contractTwosite with identity MPOs.  The last update
    uses the target's sites 0 and 1 (the reference pairs site 0 with itself there)."""

    def __init__(self, sites, mpo, itokeys, target):
        self.N = len(sites)
        self.W, self.ik, self.tgt = mpo, itokeys, target
        g = DMRG(sites, mpo, itokeys, maxthreads=2)
        g.prepare()
        self.sites = [g.site(s) for s in range(self.N)]
        self.R = {s: g.env("R", s) for s in range(2, self.N + 1)}
        self.L = {-1: {(0, 0, 0): np.ones((1, 1))}}
        ids = [identity_mpo(len(k)) for k in itokeys]
        self.ids = ids
        last = target[-1]
        dims = {}
        for (q0, q1, p), v in last.items():
            dims.setdefault(q1, v.shape[1])
        self.oR = {self.N: {(q, q, 0): np.eye(n) for q, n in dims.items()}}
        for s in range(self.N - 1, -1, -1):
            self.oR[s] = add_contraction_layer2(self.oR[s + 1], target[s], self.sites[s], ids[s], itokeys[s], 0)
        self.oL = {-1: {(0, 0, 0): np.ones((1, 1))}}
        self.steps = []

    def do_step(self, site, direction, chimax, doTrunc=False, tr_weight=1e-12, delta=1e-12, testenergy=True):
        ik0, ik1 = self.ik[site], self.ik[site + 1]
        old = theta(self.tgt[site], self.tgt[site + 1])
        state = contract_twosite(self.oL[site - 1], self.oR[site + 2], old, self.ids[site], self.ids[site + 1], ik0,
                                 ik1)
        th = theta(self.sites[site], self.sites[site + 1])
        E, it, psi = lanczos_projected(self.L[site - 1], self.R[site + 2], th, self.W[site], self.W[site + 1], ik0,
                                       ik1, state, 500, delta, testenergy)
        U, Vt, lam, tw, chi = split(psi, ik0, ik1, chimax, doTrunc, tr_weight)
        if direction > 0:
            self.sites[site] = U
            self.sites[site + 1] = {k: lam[k[0]][:, None] * v for k, v in Vt.items()}
            self.L[site] = add_contraction_layer(self.L[site - 1], self.sites[site], self.W[site], ik0, 1)
        else:
            self.sites[site] = {k: v * lam[k[1]][None, :] for k, v in U.items()}
            self.sites[site + 1] = Vt
            self.R[site + 1] = add_contraction_layer(self.R[site + 2], Vt, self.W[site + 1], ik1, -1)
        self.steps.append(dict(site=site, dir=direction, iters=it, chi=chi, E=E))
        return E

    def simulate(self, maxsteps=5, EnConv=1e-10, chimax=100, doTrunc=False, tr_weight=1e-12, delta=1e-12,
                 testenergy=True, leaveoutlast=False):
        N = self.N
        globalE, step = 1e100, 0
        while True:
            for site in range(N - 2):
                out = self.do_step(site, 1, chimax, doTrunc, tr_weight, delta, testenergy)
                self.oL[site] = add_contraction_layer2(self.oL[site - 1], self.tgt[site], self.sites[site],
                                                       self.ids[site], self.ik[site], 1)
            for site in range(N - 2, 0, -1):
                if leaveoutlast and site == N - 2:
                    continue
                out = self.do_step(site, -1, chimax, doTrunc, tr_weight, delta, testenergy)
                self.oR[site + 1] = add_contraction_layer2(self.oR[site + 2], self.tgt[site + 1], self.sites[site + 1],
                                                           self.ids[site + 1], self.ik[site + 1], -1)
            step += 1
            conv = abs(globalE - out) < EnConv or step >= maxsteps
            globalE = out
            if conv:
                break
        return self.do_step(0, -1, chimax, doTrunc, tr_weight, delta, testenergy)


# ------------------------------------------------------------------ applyMPO / compressTwoSite (CPU)
def apply_mpo(sites, W, itokeys):
    """applyMPO (src/MPSfunctions.hpp:2088-2346) restated: five-leg pieces v*A((a, wl), (b, wr); s_out)
    for every MPS block and MPO element; new charges propagated from the left ((b, wr) takes
    charge(a, wl) + q(s_out) when first seen, in key order); per new charge a coarse grid over the MPO
    channels with the largest piece size per channel (zero padding)."""
    N = len(sites)
    q0 = min(k[0] for k in sites[0])
    qleft = {(q0, w): q0 for w in range(W[0][1])}
    size_left = {q0: [1] * W[0][1]}
    out = []
    for s in range(N):
        terms, Dl, Dr = W[s]
        five = {}
        for (wl, wr, o, i, v) in terms:
            for (a, b, p), blk in sites[s].items():
                if p != i:
                    continue
                key = ((a, wl), (b, wr), o)
                five[key] = five[key] + v * blk if key in five else v * blk
        qright, size_right, kept = {}, {}, []
        for key in sorted(five):
            if key[0] not in qleft:
                continue
            qr = qleft[key[0]] + int(itokeys[s][key[2]])
            qright.setdefault(key[1], qr)
            kept.append(key)
        for key in kept:
            qr = qright[key[1]]
            v = size_right.setdefault(qr, [0] * Dr)
            v[key[1][1]] = max(v[key[1][1]], five[key].shape[1])
        site = {}
        for key in kept:
            ql, qr = qleft[key[0]], qright[key[1]]
            sl, sr = size_left[ql], size_right[qr]
            nk = (ql, qr, key[2])
            if nk not in site:
                site[nk] = np.zeros((sum(sl), sum(sr)))
            r0, c0 = sum(sl[:key[0][1]]), sum(sr[:key[1][1]])
            m = five[key]
            site[nk][r0:r0 + m.shape[0], c0:c0 + m.shape[1]] = m
        out.append(site)
        qleft, size_left = qright, size_right
    return out


def truncate_lambda(lam, chimax, tr_weight):
    """DiagBlockMatrix::truncate(tr_weight, chimax, false) (src/BlockTensor.hpp:26-136): values in the
    order (value descending, later insertion first), kept while the truncated weight exceeds
    norm * tr_weight and fewer than chimax are kept; returns the kept count per charge."""
    qs = sorted(lam)
    vals = [(float(v), q) for q in qs for v in lam[q]]
    order = sorted(range(len(vals)), key=lambda i: (-vals[i][0], -i))
    norm = np.sqrt(sum(v * v for v, _ in vals))
    tw, cnt, keep = norm, 0, {q: 0 for q in qs}
    for i in order:
        if not (abs(tw) > norm * tr_weight and cnt < chimax):
            break
        tw -= vals[i][0] ** 2 / norm
        keep[vals[i][1]] += 1
        cnt += 1
    return keep


def compress_two_site(sites, W, itokeys, chimax=100, maxstep=5, delta=1e-10, doTrunc=True, tr_weight=1e-10):
    """compressTwoSite (src/MPSfunctions.hpp:2797-2940) restated on the oracle's kernels; returns
    (conv, fitted sites).  conv = (n1^2 + n2^2 - 2 |<fit|psi>|) / n1^2 as the reference computes it."""
    N = len(sites)
    full = apply_mpo(sites, W, itokeys)
    n1 = np.sqrt(overlap(full, full, itokeys))
    t = [dict(x) for x in sites]
    lam = {}
    for s in range(N - 1):
        t[s], t[s + 1], lam[s] = prepare_left(t[s], t[s + 1])
    for s in range(N - 1, 0, -1):
        t[s - 1], t[s], lam[s - 1] = prepare_right(t[s - 1], t[s])
    _truncate_sites(t, lam, int(np.floor(chimax / W[1][2])), delta)
    comp = apply_mpo(t, W, itokeys)
    for s in range(N - 1):
        comp[s], comp[s + 1], _ = prepare_left(comp[s], comp[s + 1])
    for s in range(N - 1, 0, -1):
        comp[s - 1], comp[s], _ = prepare_right(comp[s - 1], comp[s])
    last = sites[-1]
    dims = {}
    for (a, b, p), v in last.items():
        dims.setdefault(b, v.shape[1])
    BL = {-1: {(0, 0, 0): np.ones((1, 1))}}
    BR = {N: {(q, q, 0): np.eye(n) for q, n in dims.items()}}
    for s in range(N - 1, 1, -1):
        BR[s] = add_contraction_layer2(BR[s + 1], sites[s], comp[s], W[s], itokeys[s], -1)

    def fit(s):
        return contract_twosite(BL[s - 1], BR[s + 2], theta(sites[s], sites[s + 1]), W[s], W[s + 1], itokeys[s],
                                itokeys[s + 1])

    conv, conv_old, step, converged = 0.0, 1.0, 1, maxstep == 0
    while not converged:
        for s in range(N - 2):
            U, Vt, lm, tw, ch = split(fit(s), itokeys[s], itokeys[s + 1], chimax, doTrunc, tr_weight, False)
            comp[s] = U
            comp[s + 1] = {k: lm[k[0]][:, None] * v for k, v in Vt.items()}
            BL[s] = add_contraction_layer2(BL[s - 1], sites[s], comp[s], W[s], itokeys[s], 1)
        for s in range(N - 2, 0, -1):
            U, Vt, lm, tw, ch = split(fit(s), itokeys[s], itokeys[s + 1], chimax, doTrunc, tr_weight, False)
            comp[s] = {k: v * lm[k[1]][None, :] for k, v in U.items()}
            comp[s + 1] = Vt
            BR[s + 1] = add_contraction_layer2(BR[s + 2], sites[s + 1], comp[s + 1], W[s + 1], itokeys[s + 1], -1)
        n2 = np.sqrt(overlap(comp, comp, itokeys))
        conv = (n1 * n1 + n2 * n2 - 2 * abs(overlap(comp, sites, itokeys))) / (n1 * n1)
        if conv_old < conv:
            break
        conv_old = conv
        if step >= maxstep or abs(conv) < delta:
            converged = True
        step += 1
    n2 = np.sqrt(overlap(comp, comp, itokeys))
    conv = (n1 * n1 + n2 * n2 - 2 * abs(overlap(comp, sites, itokeys))) / (n1 * n1)
    return conv, comp



def contract_single(BL, BR, A, W, ik):
    """contractSingle(out, BL, A, W, BR, itokey) (src/MPSfunctions.hpp:857-885) as the two-site
    contraction with a dummy second site (identity MPO tensor on W's right channels, one local state of
    charge 0)."""
    D = W[2]
    W2 = ([(w, w, 0, 0, 1.0) for w in range(D)], D, D)
    th = {(a, b, p, 0): v for (a, b, p), v in A.items()}
    out = contract_twosite(BL, BR, th, W, W2, ik, [0])
    return {(a, b, p): v for (a, b, p, _), v in out.items()}


def _prep_l(m, s):
    """prepareSite(mps, s, "l", true) in place (the last site multiplies into the right dummy)."""
    nxt = m[s + 1] if s + 1 < len(m) else None
    m[s], nxt, lam = prepare_left(m[s], nxt)
    if nxt is not None:
        m[s + 1] = nxt
    return lam


def _prep_r(m, s):
    """prepareSite(mps, s, "r", true) in place (site 0 multiplies into the left dummy)."""
    prv = m[s - 1] if s > 0 else None
    prv, m[s], lam = prepare_right(prv, m[s])
    if prv is not None:
        m[s - 1] = prv
    return lam


def _truncate_sites(t, lam, chimax, delta):
    """truncate(mps, chimax, delta) (src/MPSfunctions.hpp:1705-1728): per bond the kept count of
    DiagBlockMatrix::truncate, then dropDangling; chimax = 0 returns without truncating."""
    if chimax == 0:
        return
    for s in range(len(t) - 1):
        keep = truncate_lambda(lam[s], chimax, delta)
        t[s] = {k: v[:, :keep.get(k[1], 0)] for k, v in t[s].items() if keep.get(k[1], 0) > 0}
        t[s + 1] = {k: v[:keep.get(k[0], 0), :] for k, v in t[s + 1].items() if keep.get(k[0], 0) > 0}


def _rmax(sites):
    dims = {}
    for (a, b, p), v in sites[-1].items():
        dims.setdefault(b, v.shape[1])
    return {(q, q, 0): np.eye(n) for q, n in dims.items()}


def _single_site_fit(mps, comp, W, itokeys, n1, maxstep, delta):
    """The sweeps shared by compress and compressSingleSite: environments <mps| W |comp> (mps lower,
    the fit upper), sites 0 .. N-2 right (contractSingle, prepareSite "l") and N-1 .. 1 left
    (contractSingle, prepareSite "r"); after each sweep conv = (n1^2 + n2^2 - 2 |<comp|mps>|) / n1^2; stop
    when conv grows, after maxstep sweeps or when |conv| < delta.  Returns the left environments."""
    N = len(mps)
    BL = {-1: {(0, 0, 0): np.ones((1, 1))}}
    BR = {N: _rmax(mps)}
    converged = maxstep == 0
    if not converged:
        for s in range(N - 1, 0, -1):
            BR[s] = add_contraction_layer2(BR[s + 1], mps[s], comp[s], W[s], itokeys[s], -1)
    conv_old, step = 1.0, 1
    while not converged:
        for s in range(N - 1):
            comp[s] = contract_single(BL[s - 1], BR[s + 1], mps[s], W[s], itokeys[s])
            _prep_l(comp, s)
            BL[s] = add_contraction_layer2(BL[s - 1], mps[s], comp[s], W[s], itokeys[s], 1)
        for s in range(N - 1, 0, -1):
            comp[s] = contract_single(BL[s - 1], BR[s + 1], mps[s], W[s], itokeys[s])
            _prep_r(comp, s)
            BR[s] = add_contraction_layer2(BR[s + 1], mps[s], comp[s], W[s], itokeys[s], -1)
        n2 = np.sqrt(overlap(comp, comp, itokeys))
        conv = (n1 * n1 + n2 * n2 - 2 * abs(overlap(comp, mps, itokeys))) / (n1 * n1)
        if conv_old < conv:
            break
        conv_old = conv
        if step >= maxstep or abs(conv) < delta:
            converged = True
        step += 1
    return BL, BR


def compress(sites, itokeys, chimax=100, maxstep=5, delta=1e-10, normalize=False):
    """compress (src/MPSfunctions.hpp:2349-2510) restated: variational single-site compression of psi to
    bond dimension <= chimax; returns (conv, the prepared psi, the fitted sites).  psi is first swept
    with prepareSite "l" over 0 .. Nmax-1 and "r" over Nmax-1 .. Nmin (Nmax = N-1, Nmin = 1, or N and 0
    with normalize, which drops the norm into the dummies); the initial guess is psi truncated to chimax
    with those lambdas, then swept l and r; after the sweeps site 0 is fitted once more and the fit is
    swept l and r again.  conv = |fit - psi|^2 / |psi|^2."""
    N = len(sites)
    m = [dict(x) for x in sites]
    lam = {}
    nmin, nmax = (0, N) if normalize else (1, N - 1)
    for s in range(nmax):
        lam[s] = _prep_l(m, s)
    for s in range(nmax - 1, nmin - 1, -1):
        lam[s - 1] = _prep_r(m, s)
    comp = [dict(x) for x in m]
    _truncate_sites(comp, lam, chimax, delta)
    for s in range(N - 1):
        _prep_l(comp, s)
    for s in range(N - 1, 0, -1):
        _prep_r(comp, s)
    n1 = np.sqrt(overlap(m, m, itokeys))
    idW = [identity_mpo(len(k)) for k in itokeys]
    BL, BR = _single_site_fit(m, comp, idW, itokeys, n1, maxstep, delta)
    comp[0] = contract_single(BL[-1], BR[1], m[0], idW[0], itokeys[0])
    for s in range(N - 1):
        _prep_l(comp, s)
    for s in range(N - 1, 0, -1):
        _prep_r(comp, s)
    n2 = np.sqrt(overlap(comp, comp, itokeys))
    conv = (n1 * n1 + n2 * n2 - 2 * abs(overlap(comp, m, itokeys))) / (n1 * n1)
    return conv, m, comp


def compress_single_site(sites, W, itokeys, chimax=100, maxstep=5, delta=1e-10):
    """compressSingleSite (src/MPSfunctions.hpp:2667-2792) restated: variational single-site fit of
    W|psi>; n1 = |W psi| from the exact product; initial guess W applied to psi truncated to chimax / D
    (D = W's right bond dimension at site 1) after an l and an r sweep, itself swept l and r.  conv as
    in compressTwoSite (the overlap term with psi).  Returns (conv, fitted sites)."""
    N = len(sites)
    full = apply_mpo(sites, W, itokeys)
    n1 = np.sqrt(overlap(full, full, itokeys))
    t = [dict(x) for x in sites]
    lam = {}
    for s in range(N - 1):
        _prep_l(t, s)
    for s in range(N - 1, 0, -1):
        lam[s - 1] = _prep_r(t, s)
    _truncate_sites(t, lam, int(np.floor(chimax / W[1][2])), delta)
    comp = apply_mpo(t, W, itokeys)
    for s in range(N - 1):
        _prep_l(comp, s)
    for s in range(N - 1, 0, -1):
        _prep_r(comp, s)
    _single_site_fit(sites, comp, W, itokeys, n1, maxstep, delta)
    n2 = np.sqrt(overlap(comp, comp, itokeys))
    conv = (n1 * n1 + n2 * n2 - 2 * abs(overlap(comp, sites, itokeys))) / (n1 * n1)
    return conv, comp

# ------------------------------------------------------------------ TEBD (complex FP64)
def nn_gate(W1, W2, site1, N, dt, d1=2, d2=2):
    """MPO::getNNGate: dense (d1 d2 x d1 d2) complex gate exp(-i dt h_b), index o1 + d1*o2."""
    L = lib()
    w1, w2 = mpo_to_handle(*W1), mpo_to_handle(*W2)
    out = np.zeros(2 * (d1 * d2) ** 2)
    dt_c = complex(dt)
    L.orc_nn_gate(w1, w2, int(site1), int(N), dt_c.real, dt_c.imag, d1, d2, _ptr(out))
    L.orc_mpo_free(w1)
    L.orc_mpo_free(w2)
    g = out[0::2] + 1j * out[1::2]
    return g.reshape((d1 * d2, d1 * d2), order="F")


class TEBD:
    """TEBDengine from a product state (Vidal form), second-order Trotter evolution."""

    def __init__(self, local_state, W, itokeys):
        L = lib()
        self.N = len(local_state)
        loc = np.ascontiguousarray(local_state, np.int32)
        ws = [mpo_to_handle(*w) for w in W]
        pw = (C.c_void_p * len(ws))(*ws)
        flat, d = _ik_tables(itokeys)
        self.h = L.orc_tebd_new(self.N, _ptr(loc), pw, _ptr(flat), _ptr(d))
        for w in ws:
            L.orc_mpo_free(w)

    def second_order(self, steps, dt, chimax, doTrunc=False, tr_weight=1e-10, normalize=True):
        lib().orc_tebd_second_order(self.h, int(steps), float(dt), int(chimax), int(doTrunc), float(tr_weight),
                                    int(normalize))

    def measure_diag(self, site, op_diag):
        op = np.ascontiguousarray(op_diag, np.float64)
        return lib().orc_tebd_measure_diag(self.h, int(site), _ptr(op), len(op))

    def gamma(self, site):
        L = lib()
        ne = C.c_long()
        n = L.orc_tebd_gamma_info(self.h, int(site), C.byref(ne))
        q = np.zeros(2 * max(n, 1), np.uint64)
        p = np.zeros(max(n, 1), np.uint32)
        r = np.zeros(max(n, 1), np.int32)
        c = np.zeros(max(n, 1), np.int32)
        data = np.zeros(2 * max(ne.value, 1))
        L.orc_tebd_gamma_export(self.h, int(site), _ptr(q), _ptr(p), _ptr(r), _ptr(c), _ptr(data))
        z = data[0::2] + 1j * data[1::2]
        out, off = {}, 0
        for i in range(n):
            rr, cc = int(r[i]), int(c[i])
            out[(int(q[2 * i]), int(q[2 * i + 1]), int(p[i]))] = z[off:off + rr * cc].reshape((rr, cc), order="F")
            off += rr * cc
        return out

    def lam(self, bond):
        return handle_to_bm(lib().orc_tebd_lambda(self.h, int(bond)))

    def __del__(self):
        try:
            lib().orc_tebd_free(self.h)
        except Exception:
            pass
