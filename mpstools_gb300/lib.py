"""ctypes binding of libmpsg.so (include/mpsg.h).

There is no fallback: if the in-tree library is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libmpsg.so")

PREC = {"fp64": 0, "tf32": 1, "tf32x3": 2, "bf16": 3, "bf16x3": 4, "auto": 5, "mixed": 6}

_L = None


class MPSGError(RuntimeError):
    pass


def load(build_if_missing: bool = False):
    global _L
    if _L is not None:
        return _L
    if not os.path.exists(LIBPATH):
        if not build_if_missing:
            raise MPSGError(f"libmpsg.so not built ({LIBPATH}); run __graft_entry__.build()")
        from .build import build
        build()
    L = C.CDLL(LIBPATH)
    vp, i32, i64, f64, u32 = C.c_void_p, C.c_int32, C.c_int64, C.c_double, C.c_uint32
    P = C.POINTER
    L.mpsg_last_error.restype = C.c_char_p
    L.mpsg_ctx_create.argtypes = [i32, P(vp)]
    L.mpsg_ctx_destroy.argtypes = [vp]
    L.mpsg_ctx_destroy.restype = None
    L.mpsg_ctx_set_stream.argtypes = [vp, vp]
    L.mpsg_ctx_sync.argtypes = [vp]
    L.mpsg_ctx_trim.argtypes = [vp]
    L.mpsg_tc_autotune_info.argtypes = [vp, vp, vp, vp]
    L.mpsg_tc_autotune_info.restype = None
    L.mpsg_ctx_kernel_launches.argtypes = [vp]
    L.mpsg_ctx_kernel_launches.restype = i64
    L.mpsg_ctx_set_svd_method.argtypes = [vp, i32]
    L.mpsg_tensor_create.argtypes = [vp, i32, i32, vp, vp, vp, vp, vp, P(vp)]
    L.mpsg_tensor_shape.argtypes = [vp, P(i32), P(i32), P(i64)]
    L.mpsg_tensor_export.argtypes = [vp, vp, vp, vp, vp, vp]
    L.mpsg_tensor_device_view.argtypes = [vp, P(vp), vp]
    L.mpsg_tensor_destroy.argtypes = [vp]
    L.mpsg_tensor_destroy.restype = None
    L.mpsg_contract_twosite.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, i32, P(vp)]
    L.mpsg_add_contraction_layer.argtypes = [vp, vp, vp, vp, vp, i32, i32, P(vp)]
    L.mpsg_add_contraction_layer2.argtypes = [vp, vp, vp, vp, vp, vp, i32, i32, P(vp)]
    L.mpsg_overlap.argtypes = [vp, i32, vp, vp, vp, P(f64)]
    L.mpsg_mpo_measure.argtypes = [vp, i32, vp, vp, vp, P(f64)]
    L.mpsg_theta.argtypes = [vp, vp, vp, P(vp)]
    L.mpsg_split2.argtypes = [vp, vp, vp, vp, u32, i32, f64, i32, P(vp), P(vp), P(vp), P(f64), P(u32)]
    L.mpsg_lanczos2.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, i32, f64, i32, i32, i32, P(vp), P(f64), P(i32)]
    L.mpsg_dmrg_create.argtypes = [vp, i32, vp, vp, vp, P(vp)]
    L.mpsg_dmrg_set_options.argtypes = [vp, i32, i32, i32]
    L.mpsg_dmrg_get_options.argtypes = [vp, P(i32), P(i32), P(i32)]
    L.mpsg_dmrg_simulate.argtypes = [vp, u32, f64, u32, i32, f64, f64, i32, P(f64)]
    L.mpsg_dmrg_prepare.argtypes = [vp]
    L.mpsg_dmrg_do_step.argtypes = [vp, i32, i32, u32, i32, f64, f64, i32, P(f64)]
    L.mpsg_dmrg_nsteps.argtypes = [vp]
    L.mpsg_dmrg_steps.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.mpsg_dmrg_set_env_prec.argtypes = [vp, C.c_int32]
    L.mpsg_dmrg_stats.argtypes = [vp, vp]
    L.mpsg_dmrg_stats_ext.argtypes = [vp, vp, C.c_int32]
    L.mpsg_dmrg_site.argtypes = [vp, i32, P(vp)]
    L.mpsg_dmrg_lambda.argtypes = [vp, i32, P(vp)]
    L.mpsg_dmrg_measure_energy.argtypes = [vp, P(f64)]
    L.mpsg_dmrg_measure_mpo.argtypes = [vp, vp, P(f64)]
    L.mpsg_tebd_create.argtypes = [vp, i32, vp, vp, vp, P(vp)]
    L.mpsg_tebd_second_order.argtypes = [vp, i32, f64, u32, i32, f64, i32]
    L.mpsg_tebd_measure_diag.argtypes = [vp, i32, vp, i32, P(f64)]
    L.mpsg_tebd_lambda.argtypes = [vp, i32, P(vp)]
    L.mpsg_tebd_gamma_shape.argtypes = [vp, i32, P(i32), P(C.c_int64)]
    L.mpsg_tebd_gamma_export.argtypes = [vp, i32, vp, vp, vp, vp, vp]
    L.mpsg_tebd_stats.argtypes = [vp, P(f64), P(f64), P(C.c_int64)]
    L.mpsg_tebd_destroy.argtypes = [vp]
    L.mpsg_tebd_destroy.restype = None
    L.mpsg_nn_gate.argtypes = [vp, vp, i32, i32, f64, f64, i32, i32, vp]
    L.mpsg_bond_hamiltonian.argtypes = [vp, vp, i32, i32, i32, i32, vp]
    L.mpsg_nn_gate_tangent.argtypes = [vp, vp, i32, i32, f64, vp, i32, i32, vp]
    L.mpsg_tebd_adjoint_second_order.argtypes = [vp, i32, f64, u32, i32, f64, i32, vp, i32, vp, i32, P(f64), vp]
    L.mpsg_tebd_adjoint_seconds.argtypes = [vp, P(f64)]
    L.mpsg_tebd_set_batch_layers.argtypes = [vp, i32]
    L.mpsg_dmrg_ss_simulate.argtypes = [vp, u32, f64, f64, i32, P(f64)]
    L.mpsg_dmrg_excited_simulate.argtypes = [vp, vp, f64, u32, f64, u32, i32, f64, f64, i32, i32, P(f64)]
    L.mpsg_apply_mpo.argtypes = [vp, i32, vp, vp, vp, vp]
    L.mpsg_compress_two_site.argtypes = [vp, i32, vp, vp, vp, u32, u32, f64, i32, f64, vp, P(f64)]
    L.mpsg_compress.argtypes = [vp, i32, vp, vp, u32, u32, f64, i32, vp, P(f64)]
    L.mpsg_compress_single_site.argtypes = [vp, i32, vp, vp, vp, u32, u32, f64, vp, P(f64)]
    L.mpsg_dmrg_save.argtypes = [vp, C.c_char_p]
    L.mpsg_dmrg_load.argtypes = [vp, C.c_char_p, P(vp)]
    L.mpsg_split_fallbacks.argtypes = []
    L.mpsg_split_fallbacks.restype = C.c_int64
    L.mpsg_batch_create.argtypes = [vp, i32, vp, P(vp)]
    L.mpsg_batch_set_options.argtypes = [vp, i32, i32]
    L.mpsg_batch_simulate.argtypes = [vp, u32, u32, i32, f64, f64, i32, vp]
    L.mpsg_batch_stats.argtypes = [vp, vp]
    L.mpsg_batch_destroy.argtypes = [vp]
    L.mpsg_batch_destroy.restype = None
    L.mpsg_dmrg_destroy.argtypes = [vp]
    L.mpsg_dmrg_destroy.restype = None
    L.mpsg_dmrg_build_environments.argtypes = [vp, i32]
    L.mpsg_dmrg_env.argtypes = [vp, i32, i32, P(vp)]
    L.mpsg_matvec2_plan_create.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, i32, P(vp)]
    L.mpsg_matvec2_plan_execute.argtypes = [vp, vp, vp]
    L.mpsg_matvec2_plan_execute_noalloc.argtypes = [vp, vp, vp]
    L.mpsg_matvec2_plan_info.argtypes = [vp, vp]
    L.mpsg_matvec2_plan_destroy.argtypes = [vp]
    L.mpsg_matvec2_plan_destroy.restype = None
    L.mpsg_theta_closure.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, P(vp)]
    _L = L
    return L


def check(rc):
    if rc != 0:
        msg = load().mpsg_last_error().decode(errors="replace")
        raise MPSGError(f"libmpsg error {rc}: {msg}")


def ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None and a.size else None


# the SVD route a new context starts with (mpsg_ctx_set_svd_method)
DEFAULT_SVD = "bidiag"


class Context:
    """mpsg_ctx: one GPU, one stream, the device memory pool and the solver handles."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = C.c_void_p()
        check(self.L.mpsg_ctx_create(device, C.byref(h)))
        self.h = h

    def sync(self):
        check(self.L.mpsg_ctx_sync(self.h))

    def trim(self):
        check(self.L.mpsg_ctx_trim(self.h))

    def tc_autotune_info(self):
        """(signatures timed, plans served from the cache, [stage-A, stage-C] schedule of the last
        tensor-core plan: 0 round robin, 1 snake, 2 greedy longest-processing-time, best ms of each
        schedule in the last timing: stage A x3 then stage C x3, -1 where not timed)"""
        t, h, sch, ms = C.c_int64(), C.c_int64(), (C.c_int32 * 2)(), (C.c_float * 6)()
        self.L.mpsg_tc_autotune_info(C.byref(t), C.byref(h), sch, ms)
        return t.value, h.value, [sch[0], sch[1]], [float(x) for x in ms]

    def kernel_launches(self) -> int:
        return int(self.L.mpsg_ctx_kernel_launches(self.h))

    def set_svd_method(self, method):
        """'bidiag' (4, default), 'jacobi' (0), 'density' (1), 'density_mt' (2), 'density_eig' (3): see
        mpsg_ctx_set_svd_method."""
        m = {"jacobi": 0, "density": 1, "density_mt": 2, "density_eig": 3, "bidiag": 4}.get(method, method)
        check(self.L.mpsg_ctx_set_svd_method(self.h, int(m)))

    def set_stream(self, stream_ptr: int | None):
        check(self.L.mpsg_ctx_set_stream(self.h, C.c_void_p(stream_ptr) if stream_ptr else None))

    def close(self):
        if self.h:
            self.L.mpsg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tensor:
    """mpsg_tensor handle (device-resident block-sparse tensor)."""

    def __init__(self, ctx: Context, h):
        self.ctx = ctx
        self.h = h

    @staticmethod
    def from_dict(ctx: Context, bm: dict, nphys: int) -> "Tensor":
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
            chunks.append(a.ravel(order="F"))
        data = np.ascontiguousarray(np.concatenate(chunks)) if chunks else np.zeros(1)
        h = C.c_void_p()
        check(ctx.L.mpsg_tensor_create(ctx.h, nphys, n, ptr(q), ptr(p), ptr(rows), ptr(cols), ptr(data),
                                       C.byref(h)))
        return Tensor(ctx, h)

    @staticmethod
    def from_flat(ctx: Context, flat) -> "Tensor":
        """flat = (nphys, q, p, rows, cols, data) as produced by pack_flat (no Python loops)."""
        nphys, q, p, rows, cols, data = flat
        h = C.c_void_p()
        check(ctx.L.mpsg_tensor_create(ctx.h, nphys, len(rows), ptr(q), ptr(p), ptr(rows), ptr(cols), ptr(data),
                                       C.byref(h)))
        return Tensor(ctx, h)

    def device_view(self):
        """(device base pointer, element offsets of the blocks in key order)."""
        _, nb, _ = self.shape()
        d = C.c_void_p()
        offs = np.zeros(max(nb, 1), np.int64)
        check(self.ctx.L.mpsg_tensor_device_view(self.h, C.byref(d), ptr(offs)))
        return d.value, offs[:nb]

    def export_flat(self, alloc=None):
        """(nphys, q, p, rows, cols, data); alloc(n) may supply the data buffer (e.g. pinned memory)."""
        nphys, n, ne = self.shape()
        q = np.zeros(2 * max(n, 1), np.uint64)
        p = np.zeros(max(1, nphys) * max(n, 1), np.uint32)
        rows = np.zeros(max(n, 1), np.int32)
        cols = np.zeros(max(n, 1), np.int32)
        data = alloc(max(ne, 1)) if alloc else np.zeros(max(ne, 1))
        check(self.ctx.L.mpsg_tensor_export(self.h, ptr(q), ptr(p), ptr(rows), ptr(cols), ptr(data)))
        return (nphys, q, p, rows[:n], cols[:n], data)

    def shape(self):
        nphys, nb, ne = C.c_int32(), C.c_int32(), C.c_int64()
        check(self.ctx.L.mpsg_tensor_shape(self.h, C.byref(nphys), C.byref(nb), C.byref(ne)))
        return nphys.value, nb.value, ne.value

    def to_dict(self) -> dict:
        nphys, n, ne = self.shape()
        q = np.zeros(2 * max(n, 1), np.uint64)
        p = np.zeros(max(1, nphys) * max(n, 1), np.uint32)
        rows = np.zeros(max(n, 1), np.int32)
        cols = np.zeros(max(n, 1), np.int32)
        data = np.zeros(max(ne, 1))
        check(self.ctx.L.mpsg_tensor_export(self.h, ptr(q), ptr(p), ptr(rows), ptr(cols), ptr(data)))
        out, off = {}, 0
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
        return out

    def close(self):
        if self.h:
            self.ctx.L.mpsg_tensor_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pack_flat(bm: dict, nphys: int):
    """dict block matrix -> (nphys, q, p, rows, cols, data) in key order."""
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
        chunks.append(a.ravel(order="F"))
    data = np.ascontiguousarray(np.concatenate(chunks)) if chunks else np.zeros(1)
    return (nphys, q, p, rows[:n], cols[:n], data)


class MatvecPlan:
    """mpsg_matvec_plan: persistent two-site matvec on device arenas laid out like `layout`."""

    def __init__(self, ctx, L, R, layout, W1, W2, ik0, ik1, prec=0):
        self.ctx = ctx
        self._keep = (MPOArg(W1), MPOArg(W2), ItoKeyArg(ik0), ItoKeyArg(ik1))
        w1, w2, k0, k1 = self._keep
        h = C.c_void_p()
        check(ctx.L.mpsg_matvec2_plan_create(ctx.h, L.h, R.h, layout.h, w1.ref(), w2.ref(), k0.ref(), k1.ref(),
                                             int(prec), C.byref(h)))
        self.h = h

    def execute(self, din: int, dout: int):
        check(self.ctx.L.mpsg_matvec2_plan_execute(self.h, C.c_void_p(din), C.c_void_p(dout)))

    def info(self):
        a = np.zeros(4)
        check(self.ctx.L.mpsg_matvec2_plan_info(self.h, ptr(a)))
        return dict(flops=a[0], flops_ref=a[1], bytes=a[2], launches=int(a[3]))

    def close(self):
        if self.h:
            self.ctx.L.mpsg_matvec2_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _MPOStruct(C.Structure):
    _fields_ = [("nterms", C.c_int32), ("wl", C.c_void_p), ("wr", C.c_void_p), ("out", C.c_void_p),
                ("in_", C.c_void_p), ("value", C.c_void_p), ("Dl", C.c_int32), ("Dr", C.c_int32)]


class _ItoKeyStruct(C.Structure):
    _fields_ = [("d", C.c_int32), ("charge", C.c_void_p)]


class MPOArg:
    """Keeps the numpy arrays behind an mpsg_mpo alive."""

    def __init__(self, mpo):
        terms, Dl, Dr = mpo
        self.arrs = [np.ascontiguousarray([t[j] for t in terms] or [0], dtype=np.uint32) for j in range(4)]
        self.val = np.ascontiguousarray([t[4] for t in terms] or [0.0], dtype=np.float64)
        self.s = _MPOStruct(len(terms), *[ptr(a) for a in self.arrs], ptr(self.val), Dl, Dr)

    def ref(self):
        return C.byref(self.s)


class ItoKeyArg:
    def __init__(self, ik):
        self.a = np.ascontiguousarray(ik, dtype=np.uint64)
        self.s = _ItoKeyStruct(len(self.a), ptr(self.a))

    def ref(self):
        return C.byref(self.s)


class MPOArray:
    """Contiguous mpsg_mpo[N] for entry points that take one MPO tensor per site."""

    def __init__(self, mpos):
        self.items = [MPOArg(w) for w in mpos]
        self.arr = (_MPOStruct * len(self.items))(*[m.s for m in self.items])

    def ptr(self):
        return C.cast(self.arr, C.c_void_p)


class ItoKeyArray:
    """Contiguous mpsg_itokey[N]."""

    def __init__(self, iks):
        self.items = [ItoKeyArg(k) for k in iks]
        self.arr = (_ItoKeyStruct * len(self.items))(*[k.s for k in self.items])

    def ptr(self):
        return C.cast(self.arr, C.c_void_p)


def handle_array(tensors):
    return (C.c_void_p * len(tensors))(*[t.h for t in tensors])
