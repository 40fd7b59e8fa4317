"""Reference-shaped Python API over libmpsg.

Names and argument meaning follow MPSTools:
  contractTwosite      src/MPSfunctions.hpp:949-981
  addContractionLayer  src/MPSfunctions.hpp:442-493
  split                src/MPSfunctions.hpp:1142-1278
  TSLanzcosEngine      src/lanzcos.hpp:96-278
  DMRGengine           src/container.hpp:236-438
  computeOverlap       src/MPSfunctions.hpp:2066-2085
  TEBDengine           src/container.hpp:1195-1406 (applyGate src/MPSfunctions.hpp:1492-1548)
  MPO::measure         src/MPOTypes.hpp:990-1020
Block matrices are dicts keyed like TensorKeyType ((q0, q1, p0) or (q0, q1, p0, p1));
lambdas are dicts {q: 1-D array}; MPO matrices are (terms, Dl, Dr) with
terms (wl, wr, out, in, value).  All arithmetic runs on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import lib
from .lib import Context, ItoKeyArg, ItoKeyArray, MPOArg, MPOArray, Tensor, check, handle_array

_CTX = None


def default_context() -> Context:
    global _CTX
    if _CTX is None:
        _CTX = Context(0)
    return _CTX


def _prec(p):
    return lib.PREC[p] if isinstance(p, str) else int(p)


def contractTwosite(BL, BR, A, mpol, mpor, itokey, prec="fp64", ctx=None):
    ctx = ctx or default_context()
    tL, tR, tA = Tensor.from_dict(ctx, BL, 1), Tensor.from_dict(ctx, BR, 1), Tensor.from_dict(ctx, A, 2)
    w1, w2 = MPOArg(mpol), MPOArg(mpor)
    k0, k1 = ItoKeyArg(itokey[0]), ItoKeyArg(itokey[1])
    h = C.c_void_p()
    check(ctx.L.mpsg_contract_twosite(ctx.h, tL.h, tR.h, tA.h, w1.ref(), w2.ref(), k0.ref(), k1.ref(),
                                      _prec(prec), C.byref(h)))
    return Tensor(ctx, h).to_dict()


def addContractionLayer(BL, A, mpo, itokey, direction, prec="fp64", ctx=None):
    ctx = ctx or default_context()
    tB, tA = Tensor.from_dict(ctx, BL, 1), Tensor.from_dict(ctx, A, 1)
    w = MPOArg(mpo)
    k = ItoKeyArg(itokey)
    h = C.c_void_p()
    check(ctx.L.mpsg_add_contraction_layer(ctx.h, tB.h, tA.h, w.ref(), k.ref(), int(direction), _prec(prec),
                                           C.byref(h)))
    return Tensor(ctx, h).to_dict()


def theta(A1, A2, ctx=None):
    ctx = ctx or default_context()
    t1, t2 = Tensor.from_dict(ctx, A1, 1), Tensor.from_dict(ctx, A2, 1)
    h = C.c_void_p()
    check(ctx.L.mpsg_theta(ctx.h, t1.h, t2.h, C.byref(h)))
    return Tensor(ctx, h).to_dict()


def addContractionLayer2(BL, A, mpo, Ap, itokey, direction, prec="fp64", ctx=None):
    """Two-tensor addContractionLayer(BL, A, mpo, Ap, itokey, direction): A lower, Ap upper."""
    ctx = ctx or default_context()
    tB, tA, tP = Tensor.from_dict(ctx, BL, 1), Tensor.from_dict(ctx, A, 1), Tensor.from_dict(ctx, Ap, 1)
    w = MPOArg(mpo)
    k = ItoKeyArg(itokey)
    h = C.c_void_p()
    check(ctx.L.mpsg_add_contraction_layer2(ctx.h, tB.h, tA.h, tP.h, w.ref(), k.ref(), int(direction),
                                            _prec(prec), C.byref(h)))
    return Tensor(ctx, h).to_dict()


def computeOverlap(a, b, itokeys, ctx=None):
    """computeOverlap(a, b) for two MPS given as lists of site dicts (a lower, b upper)."""
    ctx = ctx or default_context()
    ta = [Tensor.from_dict(ctx, x, 1) for x in a]
    tb = [Tensor.from_dict(ctx, x, 1) for x in b]
    ks = ItoKeyArray(itokeys)
    out = C.c_double()
    check(ctx.L.mpsg_overlap(ctx.h, len(ta), handle_array(ta), handle_array(tb), ks.ptr(), C.byref(out)))
    return out.value


def measureMPO(sites, mpo, itokeys, ctx=None):
    """MPO::measure(mps): <psi|W|psi> for site dicts and one MPO tensor per site."""
    ctx = ctx or default_context()
    ts = [Tensor.from_dict(ctx, x, 1) for x in sites]
    ws, ks = MPOArray(mpo), ItoKeyArray(itokeys)
    out = C.c_double()
    check(ctx.L.mpsg_mpo_measure(ctx.h, len(ts), handle_array(ts), ws.ptr(), ks.ptr(), C.byref(out)))
    return out.value


def applyMPO(mpo, sites, itokeys, ctx=None):
    """applyMPO(mpo, mps): the exact MPS of W|psi> (site dicts)."""
    ctx = ctx or default_context()
    ts = [Tensor.from_dict(ctx, x, 1) for x in sites]
    ws, ks = MPOArray(mpo), ItoKeyArray(itokeys)
    out = (C.c_void_p * len(ts))()
    check(ctx.L.mpsg_apply_mpo(ctx.h, len(ts), handle_array(ts), ws.ptr(), ks.ptr(), out))
    return [Tensor(ctx, C.c_void_p(h)).to_dict() for h in out]


def compressTwoSite(sites, mpo, itokeys, chimax=100, maxstep=5, delta=1e-10, doTrunc=True, tr_weight=1e-10,
                    ctx=None):
    """compressTwoSite(mps, mpo, ...): returns (conv, fitted site dicts)."""
    ctx = ctx or default_context()
    ts = [Tensor.from_dict(ctx, x, 1) for x in sites]
    ws, ks = MPOArray(mpo), ItoKeyArray(itokeys)
    out = (C.c_void_p * len(ts))()
    conv = C.c_double()
    check(ctx.L.mpsg_compress_two_site(ctx.h, len(ts), handle_array(ts), ws.ptr(), ks.ptr(), int(chimax), int(maxstep),
                                       float(delta), int(doTrunc), float(tr_weight), out, C.byref(conv)))
    return conv.value, [Tensor(ctx, C.c_void_p(h)).to_dict() for h in out]


def compress(sites, itokeys, chimax=100, maxstep=5, delta=1e-10, normalize=False, ctx=None):
    """compress(mps, chimax, maxstep, delta, verbose, normalize): variational single-site compression;
    returns (conv, fitted site dicts)."""
    ctx = ctx or default_context()
    ts = [Tensor.from_dict(ctx, x, 1) for x in sites]
    ks = ItoKeyArray(itokeys)
    out = (C.c_void_p * len(ts))()
    conv = C.c_double()
    check(ctx.L.mpsg_compress(ctx.h, len(ts), handle_array(ts), ks.ptr(), int(chimax), int(maxstep), float(delta),
                              int(normalize), out, C.byref(conv)))
    return conv.value, [Tensor(ctx, C.c_void_p(h)).to_dict() for h in out]


def compressSingleSite(sites, mpo, itokeys, chimax=100, maxstep=5, delta=1e-10, ctx=None):
    """compressSingleSite(mps, mpo, chimax, maxstep, delta): returns (conv, fitted site dicts)."""
    ctx = ctx or default_context()
    ts = [Tensor.from_dict(ctx, x, 1) for x in sites]
    ws, ks = MPOArray(mpo), ItoKeyArray(itokeys)
    out = (C.c_void_p * len(ts))()
    conv = C.c_double()
    check(ctx.L.mpsg_compress_single_site(ctx.h, len(ts), handle_array(ts), ws.ptr(), ks.ptr(), int(chimax),
                                          int(maxstep), float(delta), out, C.byref(conv)))
    return conv.value, [Tensor(ctx, C.c_void_p(h)).to_dict() for h in out]


def split(A, itokey, chimax, doTrunc=False, tr_weight=1e-12, normalize=True, ctx=None):
    """Returns (U, Vt, lambda, truncated_weight, chi) -- direction 0 of the reference."""
    ctx = ctx or default_context()
    tA = Tensor.from_dict(ctx, A, 2)
    k0, k1 = ItoKeyArg(itokey[0]), ItoKeyArg(itokey[1])
    U, V, lam = C.c_void_p(), C.c_void_p(), C.c_void_p()
    tw, chi = C.c_double(), C.c_uint32()
    check(ctx.L.mpsg_split2(ctx.h, tA.h, k0.ref(), k1.ref(), int(chimax), int(doTrunc), float(tr_weight),
                            int(normalize), C.byref(U), C.byref(V), C.byref(lam), C.byref(tw), C.byref(chi)))
    return (Tensor(ctx, U).to_dict(), Tensor(ctx, V).to_dict(), Tensor(ctx, lam).to_dict(), tw.value, chi.value)


class TSLanzcosEngine:
    """Two-site Lanczos: simulate(itmax, delta, testenergy) then getState(0)."""

    def __init__(self, L, R, mpsl, mpsr, mpol, mpor, itokeyl, itokeyr, prec="fp64", reorth=False, ctx=None):
        self.ctx = ctx or default_context()
        self.args = (L, R, mpsl, mpsr, mpol, mpor, itokeyl, itokeyr)
        self.prec, self.reorth = prec, reorth
        self._E0 = None
        self._state = None
        self.iterations = 0

    def simulate(self, itmax=500, delta=1e-12, testenergy=True):
        L, R, mpsl, mpsr, mpol, mpor, ikl, ikr = self.args
        ctx = self.ctx
        tL, tR = Tensor.from_dict(ctx, L, 1), Tensor.from_dict(ctx, R, 1)
        tl, tr = Tensor.from_dict(ctx, mpsl, 1), Tensor.from_dict(ctx, mpsr, 1)
        w1, w2 = MPOArg(mpol), MPOArg(mpor)
        k0, k1 = ItoKeyArg(ikl), ItoKeyArg(ikr)
        st, E0, it = C.c_void_p(), C.c_double(), C.c_int32()
        check(ctx.L.mpsg_lanczos2(ctx.h, tL.h, tR.h, tl.h, tr.h, w1.ref(), w2.ref(), k0.ref(), k1.ref(), int(itmax),
                                  float(delta), int(testenergy), _prec(self.prec), int(self.reorth), C.byref(st),
                                  C.byref(E0), C.byref(it)))
        self._state = Tensor(ctx, st)
        self._E0 = E0.value
        self.iterations = it.value
        return it.value

    def E(self, i=0):
        assert i == 0, "only the ground state is kept"
        return self._E0

    def getState(self, j=0):
        assert j == 0, "only the ground state is kept"
        return self._state.to_dict()


class DMRGengine:
    """DMRGengine<AbKeyType,Real>(mps, mpo): site tensors and MPO stay on the GPU."""

    def __init__(self, sites, mpo, itokeys, prec="fp64", reorth=False, lanmax=500, ctx=None):
        self.ctx = ctx or default_context()
        ctx = self.ctx
        self.N = len(sites)
        self._tensors = [Tensor.from_dict(ctx, s, 1) for s in sites]
        self._mpos = [MPOArg(w) for w in mpo]
        self._iks = [ItoKeyArg(k) for k in itokeys]
        harr = (C.c_void_p * self.N)(*[t.h.value for t in self._tensors])
        marr = (lib._MPOStruct * self.N)(*[m.s for m in self._mpos])
        karr = (lib._ItoKeyStruct * self.N)(*[k.s for k in self._iks])
        h = C.c_void_p()
        check(ctx.L.mpsg_dmrg_create(ctx.h, self.N, harr, marr, karr, C.byref(h)))
        self.h = h
        check(ctx.L.mpsg_dmrg_set_options(self.h, _prec(prec), int(reorth), int(lanmax)))

    def excited_simulate(self, target_sites, maxsteps=5, EnConv=1e-10, chimax=100, doTrunc=False, tr_weight=1e-12,
                         delta=1e-12, testenergy=True, leaveoutlast=False, delta_ortho=1e-10):
        """DMRGengine::simulate(mps, ...): two-site DMRG orthogonal to the target MPS (site dicts)."""
        ts = [Tensor.from_dict(self.ctx, x, 1) for x in target_sites]
        E = C.c_double()
        check(self.ctx.L.mpsg_dmrg_excited_simulate(self.h, handle_array(ts), float(delta_ortho), int(maxsteps),
                                                     float(EnConv), int(chimax), int(doTrunc), float(tr_weight),
                                                     float(delta), int(testenergy), int(leaveoutlast), C.byref(E)))
        return E.value

    def ss_simulate(self, maxsteps=5, EnConv=1e-10, delta=1e-12, testenergy=True):
        """SSDMRGengine::simulate: single-site sweeps (no bond growth) from the engine's state."""
        E = C.c_double()
        check(self.ctx.L.mpsg_dmrg_ss_simulate(self.h, int(maxsteps), float(EnConv), float(delta), int(testenergy),
                                                C.byref(E)))
        return E.value

    def save(self, path):
        """Write the state (site tensors, lambdas, charge maps, MPO) as an MPSGCKP1 checkpoint."""
        check(self.ctx.L.mpsg_dmrg_save(self.h, os.fsencode(path)))

    @classmethod
    def load(cls, path, prec=None, reorth=None, lanmax=None, ctx=None):
        """An engine holding the state of an MPSGCKP1 checkpoint (written by save() or by
        mpstools_gb300.checkpoint.save).  The run settings stored in the file (matvec precision,
        reorthogonalisation, Lanczos iteration limit) are restored; arguments that are not None
        override them."""
        self = cls.__new__(cls)
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        check(self.ctx.L.mpsg_dmrg_load(self.ctx.h, os.fsencode(path), C.byref(h)))
        self.h = h
        from . import checkpoint
        hdr = checkpoint.read_header(path)
        self.N = hdr["N"]
        self._tensors, self._mpos, self._iks = [], [], []
        st = checkpoint.read_settings(path)
        check(self.ctx.L.mpsg_dmrg_set_options(self.h, st["prec"] if prec is None else _prec(prec),
                                               st["reorth"] if reorth is None else int(reorth),
                                               st["lanmax"] if lanmax is None else int(lanmax)))
        return self

    def options(self):
        """{"prec", "reorth", "lanmax"} in effect (mpsg_dmrg_get_options)."""
        p, r, m = C.c_int32(), C.c_int32(), C.c_int32()
        check(self.ctx.L.mpsg_dmrg_get_options(self.h, C.byref(p), C.byref(r), C.byref(m)))
        return {"prec": p.value, "reorth": r.value, "lanmax": m.value}

    def simulate(self, maxsteps=5, EnConv=1e-10, chimax=100, doTrunc=False, tr_weight=1e-12, delta=1e-13,
                 testenergy=True):
        E = C.c_double()
        check(self.ctx.L.mpsg_dmrg_simulate(self.h, int(maxsteps), float(EnConv), int(chimax), int(doTrunc),
                                            float(tr_weight), float(delta), int(testenergy), C.byref(E)))
        return E.value

    def prepare(self):
        check(self.ctx.L.mpsg_dmrg_prepare(self.h))

    def do_step(self, site, direction, chimax, doTrunc=False, tr_weight=1e-12, delta=1e-12, testenergy=True):
        E = C.c_double()
        check(self.ctx.L.mpsg_dmrg_do_step(self.h, int(site), int(direction), int(chimax), int(doTrunc),
                                           float(tr_weight), float(delta), int(testenergy), C.byref(E)))
        return E.value

    def steps(self):
        n = self.ctx.L.mpsg_dmrg_nsteps(self.h)
        a = [np.zeros(max(n, 1), np.int32) for _ in range(4)]
        E, tw = np.zeros(max(n, 1)), np.zeros(max(n, 1))
        check(self.ctx.L.mpsg_dmrg_steps(self.h, *[lib.ptr(x) for x in a], lib.ptr(E), lib.ptr(tw)))
        return [dict(site=int(a[0][i]), dir=int(a[1][i]), iters=int(a[2][i]), chi=int(a[3][i]), E=float(E[i]),
                     tw=float(tw[i])) for i in range(n)]

    def set_env_prec(self, prec):
        """Arithmetic of doStep's environment updates: "fp64" (default) or a tensor-core precision."""
        check(self.ctx.L.mpsg_dmrg_set_env_prec(self.h, lib.PREC[prec]))

    def stats(self):
        s = np.zeros(12)
        check(self.ctx.L.mpsg_dmrg_stats_ext(self.h, lib.ptr(s), 12))
        keys = ["matvecs", "matvec_flops", "lanczos_iter_seconds", "env_seconds", "split_seconds",
                "lanczos_seconds", "env_flops", "wall_seconds", "step_device_seconds", "step_calls",
                "prep_seconds", "lanczos_call_seconds"]
        return dict(zip(keys, s.tolist()))

    def build_environments(self, center):
        check(self.ctx.L.mpsg_dmrg_build_environments(self.h, int(center)))

    def env_tensor(self, which, site):
        h = C.c_void_p()
        check(self.ctx.L.mpsg_dmrg_env(self.h, 1 if which == "R" else 0, int(site), C.byref(h)))
        return Tensor(self.ctx, h)

    def site_tensor(self, s):
        h = C.c_void_p()
        check(self.ctx.L.mpsg_dmrg_site(self.h, int(s), C.byref(h)))
        return Tensor(self.ctx, h)

    def site(self, s):
        h = C.c_void_p()
        check(self.ctx.L.mpsg_dmrg_site(self.h, int(s), C.byref(h)))
        return Tensor(self.ctx, h).to_dict()

    def lam(self, bond):
        h = C.c_void_p()
        check(self.ctx.L.mpsg_dmrg_lambda(self.h, int(bond), C.byref(h)))
        return Tensor(self.ctx, h).to_dict()

    def measure_energy(self):
        E = C.c_double()
        check(self.ctx.L.mpsg_dmrg_measure_energy(self.h, C.byref(E)))
        return E.value

    def measure(self, mpo):
        """MPO::measure of the current state with another MPO (one tensor per site)."""
        ws = MPOArray(mpo)
        out = C.c_double()
        check(self.ctx.L.mpsg_dmrg_measure_mpo(self.h, ws.ptr(), C.byref(out)))
        return out.value

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.mpsg_dmrg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DMRGbatch:
    """Independent DMRGengine chains swept in lockstep, every step's work batched over the chains
    (one launch per matvec stage for all chains).  The engines are updated in place."""

    def __init__(self, engines, prec="fp64", lanmax=500, ctx=None):
        self.ctx = ctx or engines[0].ctx
        self.engines = list(engines)
        arr = (C.c_void_p * len(self.engines))(*[e.h.value for e in self.engines])
        h = C.c_void_p()
        check(self.ctx.L.mpsg_batch_create(self.ctx.h, len(self.engines), arr, C.byref(h)))
        self.h = h
        check(self.ctx.L.mpsg_batch_set_options(self.h, _prec(prec), int(lanmax)))

    def simulate(self, sweeps, chimax, doTrunc=False, tr_weight=1e-12, delta=1e-12, testenergy=True):
        out = np.zeros(len(self.engines))
        check(self.ctx.L.mpsg_batch_simulate(self.h, int(sweeps), int(chimax), int(doTrunc), float(tr_weight),
                                              float(delta), int(testenergy), out.ctypes.data_as(C.c_void_p)))
        return out

    def stats(self):
        st = np.zeros(11)
        check(self.ctx.L.mpsg_batch_stats(self.h, st.ctypes.data_as(C.c_void_p)))
        keys = ["global_steps", "chain_steps", "matvecs", "matvec_flops", "matvec_launches", "lanczos_seconds",
                "split_seconds", "env_seconds", "wall_seconds", "device_seconds", "prepare_seconds"]
        return dict(zip(keys, st.tolist()))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.mpsg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def getNNGate(W1, W2, site1, N, dt, d1=2, d2=2):
    """MPO::getNNGate: dense (d1 d2 x d1 d2) complex gate exp(-i dt h_b), index o1 + d1*o2."""
    L = lib.load()
    w1, w2 = MPOArg(W1), MPOArg(W2)
    out = np.zeros(2 * (d1 * d2) ** 2)
    dt = complex(dt)
    check(L.mpsg_nn_gate(w1.ref(), w2.ref(), int(site1), int(N), dt.real, dt.imag, d1, d2,
                         out.ctypes.data_as(C.c_void_p)))
    return (out[0::2] + 1j * out[1::2]).reshape((d1 * d2, d1 * d2), order="F")


def bondHamiltonian(W1, W2, site1, N, d1=2, d2=2):
    """The bond Hamiltonian h_b that MPO::getNNGate exponentiates: real (d1 d2 x d1 d2), index o1 + d1*o2."""
    L = lib.load()
    w1, w2 = MPOArg(W1), MPOArg(W2)
    out = np.zeros((d1 * d2) ** 2)
    check(L.mpsg_bond_hamiltonian(w1.ref(), w2.ref(), int(site1), int(N), d1, d2, out.ctypes.data_as(C.c_void_p)))
    return out.reshape((d1 * d2, d1 * d2), order="F")


def gateTangent(W1, W2, site1, N, dt, dh, d1=2, d2=2):
    """(dG/dtheta) G^H for the gate G = exp(-i dt h_b) of getNNGate when dh_b/dtheta = dh (real symmetric)."""
    L = lib.load()
    w1, w2 = MPOArg(W1), MPOArg(W2)
    dhf = np.asfortranarray(dh, np.float64)
    out = np.zeros(2 * (d1 * d2) ** 2)
    check(L.mpsg_nn_gate_tangent(w1.ref(), w2.ref(), int(site1), int(N), float(dt), dhf.ctypes.data_as(C.c_void_p),
                                 d1, d2, out.ctypes.data_as(C.c_void_p)))
    return (out[0::2] + 1j * out[1::2]).reshape((d1 * d2, d1 * d2), order="F")


def couplingDerivatives(make_mpo, theta, itokeys):
    """dh_b / dtheta_b for every bond from an MPO builder that is affine in its per-bond parameters:
    make_mpo(theta) -> list of MPO tensors; the bond Hamiltonians are differenced at theta + e_b and
    theta (exact for affine dependence up to rounding)."""
    theta = np.asarray(theta, np.float64)
    N = len(itokeys)
    W0 = make_mpo(theta)
    out = []
    for b in range(N - 1):
        d1, d2 = len(itokeys[b]), len(itokeys[b + 1])
        tp = theta.copy()
        tp[b] += 1.0
        W1 = make_mpo(tp)
        out.append(bondHamiltonian(W1[b], W1[b + 1], b, N, d1, d2) - bondHamiltonian(W0[b], W0[b + 1], b, N, d1, d2))
    return out


class TEBDengine:
    """TEBDengine from a product state on the GPU: complex Gamma tensors, real lambdas."""

    def __init__(self, local_state, mpo, itokeys, ctx=None):
        self.ctx = ctx or default_context()
        self.N = len(local_state)
        loc = np.ascontiguousarray(local_state, np.int32)
        self._w, self._k = MPOArray(mpo), ItoKeyArray(itokeys)
        h = C.c_void_p()
        check(self.ctx.L.mpsg_tebd_create(self.ctx.h, self.N, loc.ctypes.data_as(C.c_void_p), self._w.ptr(),
                                           self._k.ptr(), C.byref(h)))
        self.h = h

    def second_order(self, steps, dt, chimax, doTrunc=False, tr_weight=1e-10, normalize=True):
        check(self.ctx.L.mpsg_tebd_second_order(self.h, int(steps), float(dt), int(chimax), int(doTrunc),
                                                 float(tr_weight), int(normalize)))

    def adjoint_second_order(self, steps, dt, chimax, obs_site, obs_diag, dh, doTrunc=True, tr_weight=1e-10,
                             checkpoint_every=0):
        """Second-order evolution (as second_order, normalised) and the gradient of <O_obs_site> at the end
        with respect to one parameter per bond (dh[b] = d h_b / d theta_b).  Returns (value, grad)."""
        op = np.ascontiguousarray(obs_diag, np.float64)
        flat = np.concatenate([np.asarray(m, np.float64).reshape(-1, order="F") for m in dh])
        grad = np.zeros(self.N - 1)
        val = C.c_double()
        check(self.ctx.L.mpsg_tebd_adjoint_second_order(
            self.h, int(steps), float(dt), int(chimax), int(doTrunc), float(tr_weight), int(obs_site),
            op.ctypes.data_as(C.c_void_p), len(op), flat.ctypes.data_as(C.c_void_p), int(checkpoint_every),
            C.byref(val), grad.ctypes.data_as(C.c_void_p)))
        return val.value, grad

    def set_batch_layers(self, on=True):
        check(self.ctx.L.mpsg_tebd_set_batch_layers(self.h, int(bool(on))))

    def adjoint_seconds(self):
        s = C.c_double()
        check(self.ctx.L.mpsg_tebd_adjoint_seconds(self.h, C.byref(s)))
        return s.value

    def measure_diag(self, site, op_diag):
        op = np.ascontiguousarray(op_diag, np.float64)
        out = C.c_double()
        check(self.ctx.L.mpsg_tebd_measure_diag(self.h, int(site), op.ctypes.data_as(C.c_void_p), len(op),
                                                 C.byref(out)))
        return out.value

    def lam(self, bond):
        h = C.c_void_p()
        check(self.ctx.L.mpsg_tebd_lambda(self.h, int(bond), C.byref(h)))
        return Tensor(self.ctx, h).to_dict()

    def gamma(self, site):
        n, ne = C.c_int32(), C.c_int64()
        check(self.ctx.L.mpsg_tebd_gamma_shape(self.h, int(site), C.byref(n), C.byref(ne)))
        nb = max(n.value, 1)
        q = np.zeros(2 * nb, np.uint64)
        p = np.zeros(nb, np.uint32)
        r = np.zeros(nb, np.int32)
        c = np.zeros(nb, np.int32)
        data = np.zeros(2 * max(ne.value, 1))
        ptr = lambda a: a.ctypes.data_as(C.c_void_p)
        check(self.ctx.L.mpsg_tebd_gamma_export(self.h, int(site), ptr(q), ptr(p), ptr(r), ptr(c), ptr(data)))
        z = data[0::2] + 1j * data[1::2]
        out, off = {}, 0
        for i in range(n.value):
            rr, cc = int(r[i]), int(c[i])
            out[(int(q[2 * i]), int(q[2 * i + 1]), int(p[i]))] = z[off:off + rr * cc].reshape((rr, cc), order="F")
            off += rr * cc
        return out

    def stats(self):
        s, sp, g = C.c_double(), C.c_double(), C.c_int64()
        check(self.ctx.L.mpsg_tebd_stats(self.h, C.byref(s), C.byref(sp), C.byref(g)))
        return {"seconds": s.value, "split_seconds": sp.value, "gates": g.value}

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.mpsg_tebd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
