"""Benchmark of the DMRG hot path on GB300 (one JSON line on stdout).

Workload (config: XXZ chain L=100, Jxy=1, Delta_i ~ U[0.5,1.5] from seed 1, U(1) Sz_total=0,
MPO bond dimension 5, at the chi=2048 end of the chi ramp): a seeded random U(1) MPS with
chi=2048 on every bond, left-isometric left of the centre bond and right-isometric right of it.
One step = one two-site DMRG update at the centre bond (DMRGengine::doStep: theta formation,
Lanczos, SVD split with truncation to chi, environment update), alternating direction so
consecutive steps stay on the same bond.  Default precision MIXED (TF32X3 tensor-core Lanczos,
energy = FP64 Rayleigh quotient); the AUTO and plain FP64 paths are timed on the same updates.
--model tv: the t-V chain instead (L=128, t=1, V_i ~ U[0,2] from seed 2, mu=0, half filling).

value   = algorithmic FLOPs of the Lanczos matvecs executed inside the timed steps / total device time
          of the steps (TFLOP/s; MIXED's extra FP64 Rayleigh-quotient matvec is not counted as work);
          ms_per_step is the device time of one update.
e2e     = the same metric through the C ABI with host buffers: per step the environments and the
          two site tensors are uploaded (mpsg_tensor_create), the update runs through
          mpsg_lanczos2 + mpsg_split2 + mpsg_add_contraction_layer and the results are
          downloaded (mpsg_tensor_export); the host buffers are pinned.
roofline: the grouped matvec GEMM timed alone with CUDA events, L2 flushed before each launch.
--impl reference: the CPU oracle (restatement of the reference's C++/BLAS path) on the same
          workload, one two-site update per step, all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DMRG sweep time + matvec TFLOP/s, mixed/batched vs FP64 GPU, dE/E<1e-10"
L_SITES, NUP, CHI, SEED_MPS, SEED_DELTA = 100, 50, 2048, 12345, 1
# arithmetic of each Lanczos mode: tensor-core matvec with FP64 recurrence / energies, or plain FP64
DTYPE = {"fp64": "f64", "auto": "tf32x3+f64", "mixed": "tf32x3+f64"}
CENTER = L_SITES // 2 - 1


SEED_V = 2  # t-V chain: V_i ~ U[0,2] from this seed
MODEL_L = {"xxz": L_SITES, "tv": 128}
MODEL_TEXT = {"xxz": "XXZ (Heisenberg MPO D=5), Jxy=1, Delta~U[0.5,1.5] seed 1",
              "tv": "spinless fermions t-V (Jordan-Wigner MPO D=5), t=1, V~U[0,2] seed 2, mu=0"}


def workload(chi=CHI, L=L_SITES, model="xxz"):
    """XXZ chain (Sz_total = 0) or t-V chain at half filling, and a seeded random U(1) MPS of bond
    dimension chi in mixed-canonical form around the centre bond."""
    from mpstools_gb300 import models as M
    Nup = L // 2
    center = L // 2 - 1
    if model == "tv":
        W = M.spinless_fermions_mpo(2.0 * M.uniform01(SEED_V, L - 1), np.ones(L - 1), np.zeros(L))
    else:
        W = M.heisenberg_mpo(M.xxz_couplings(L, SEED_DELTA), np.ones(L - 1), np.zeros(L))
    ik = M.u1_itokeys(L)
    sites = M.random_mixed_canonical_mps(L, Nup, chi, SEED_MPS, center)
    return W, ik, sites, center


def config_dict(chi, L, prec, svd="density", model="xxz"):
    return {"workload": f"{model}_L{L}_chi{chi}_centre_bond_two_site_update",
            "model": MODEL_TEXT[model],
            "L": L, **({"N_particles": L // 2} if model == "tv" else {"Sz_total": 0}), "chi": chi, "mpo_bond_dim": 5,
            "state": "seeded random U(1) MPS, mixed canonical",
            "lanczos": "delta=1e-12, energy test every 5 iterations, itmax 500", "matvec_precision": prec,
            "svd": svd, "l2": "flushed (512 MiB write) before every timed step and every roofline launch"}


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def fp64_peak_tflops(torch):
    """cuBLAS DGEMM 8192^3 (best of 5) -- the FP64 denominator of the roofline."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


# ----------------------------------------------------------------------------- CPU oracle leg
def reference_arm(args):
    """--impl reference: the CPU oracle on the same workload, all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    W, ik, sites, center = workload(args.chi, args.L, args.model)
    from oracle import pyoracle as O
    g = O.DMRG(sites, W, ik, maxthreads=threads, matvec_threads=threads)
    g.build_environments(center)
    for i in range(args.warmup):
        g.do_step(center, 1 if i % 2 == 0 else -1, args.chi)
    n0 = len(g.steps())
    t0 = time.perf_counter()
    for i in range(args.steps):
        g.do_step(center, 1 if (args.warmup + i) % 2 == 0 else -1, args.chi)
    dt = time.perf_counter() - t0
    st = g.steps()[n0:]
    flops_per_mv = matvec_flops_host(g, W, ik, center)
    mv = sum(s["iters"] for s in st)
    value = flops_per_mv * mv / dt / 1e12
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": config_dict(args.chi, args.L, "fp64 (CPU oracle, OpenBLAS dgemm)", "dgesvd (CPU oracle)",
                                  args.model),
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} two-site updates at the centre bond (chi={args.chi})"},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "lanczos_iterations_per_step": mv / max(args.steps, 1)}
    print(json.dumps(line), flush=True)


def matvec_flops_host(g, W, ik, center):
    """Algorithmic FLOPs of one centre-bond matvec, counted from the block tables like the GPU plan."""
    from oracle import pyoracle as O  # noqa: F401
    L = g.env("L", center - 1)
    R = g.env("R", center + 2)
    th = {}
    A1, A2 = g.site(center), g.site(center + 1)
    for (a, c, s1), x in A1.items():
        for (c2, b, s2), y in A2.items():
            if c2 == c:
                th[(a, b, s1, s2)] = (x.shape[0], y.shape[1])
    return count_matvec_flops(L, R, th, W[center], W[center + 1], ik[center], ik[center + 1])


def count_matvec_flops(L, R, thdims, W1, W2, ik0, ik1):
    """FLOPs of the factored schedule (stage A: X = sum L~ theta; stage C: out = sum X R~^T)."""
    lt, xt, ot = {}, {}, {}
    Rk = {k: v.shape for k, v in R.items()}
    w2 = {}
    for t in W2[0]:
        w2.setdefault(t[0], []).append(t)
    for (a1, a, wl), Lb in L.items():
        for (wl_, wm, s1, s1p, v1) in W1[0]:
            if wl_ != wl:
                continue
            for (wm_, wr, s2, s2p, v2) in w2.get(wm, []):
                b = a + ik0[s1] + ik1[s2]
                if (a, b, s1, s2) not in thdims:
                    continue
                b1 = a1 + ik0[s1p] + ik1[s2p]
                if (b1, b, wr) not in Rk:
                    continue
                xk = (a1, b, wm, s1p, s2)
                xt.setdefault(xk, {})[s1] = (Lb.shape[0], Lb.shape[1], thdims[(a, b, s1, s2)][1])
                ot.setdefault((a1, b1, s1p, s2p), set()).add((xk, (b1, b, wm, s2p, s2), Rk[(b1, b, wr)][0]))
    f = 0.0
    for xk, segs in xt.items():
        for (m, k, n) in segs.values():
            f += 2.0 * m * n * k
    for ok, prs in ot.items():
        for (xk, rk, rb1) in prs:
            m = next(iter(xt[xk].values()))[0]
            kk = next(iter(xt[xk].values()))[2]
            f += 2.0 * m * rb1 * kk
    return f


# ----------------------------------------------------------------------------- GPU arm
def max_over_ranks(x, dist, device):
    """The largest x over the ranks (a job's time is its slowest rank's); x itself on one process."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gpu_arm(args):
    import torch
    from mpstools_gb300 import api, lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    prec = args.prec
    W, ik, sites, center = workload(args.chi, args.L, args.model)
    ctx = lib.Context(local)
    # one explicit stream shared by the library, the L2 flush and the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_svd_method(args.svd)
    eng = api.DMRGengine(sites, W, ik, prec=prec, ctx=ctx)
    eng.build_environments(center)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def one(i):
        eng.do_step(center, 1 if i % 2 == 0 else -1, args.chi)

    for i in range(args.warmup):
        one(i)
    st0 = eng.stats()
    n_steps0 = len(eng.steps())
    launches0 = ctx.kernel_launches()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler()
    clk.start()
    times = []
    for i in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        one(args.warmup + i)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    torch.cuda.synchronize()
    clocks = clk.stop()
    total = float(np.sum(times))
    total = max_over_ranks(total, dist, "cuda")
    st1 = eng.stats()
    launches = ctx.kernel_launches() - launches0
    mv_flops = st1["matvec_flops"] - st0["matvec_flops"]
    matvecs = st1["matvecs"] - st0["matvecs"]
    # throughput counts the Lanczos matvecs only (the reference's work); MIXED's one FP64
    # Rayleigh-quotient matvec per update is time spent, not throughput
    lanczos_mv = matvecs - (args.steps if prec == "mixed" else 0)
    value = mv_flops * (lanczos_mv / max(matvecs, 1)) * world / total / 1e12
    steps_rec = eng.steps()[n_steps0:]

    # ------------------------------------------- other precisions (plain FP64 GPU path, AUTO) on the same updates
    def other_leg(p):
        e2 = api.DMRGengine(sites, W, ik, prec=p, ctx=ctx)
        e2.build_environments(center)
        for i in range(args.warmup):
            e2.do_step(center, 1 if i % 2 == 0 else -1, args.chi)
        n2 = len(e2.steps())
        t2 = []
        for i in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            e2.do_step(center, 1 if (args.warmup + i) % 2 == 0 else -1, args.chi)
            e1.record(stream)
            e1.synchronize()
            t2.append(e0.elapsed_time(e1) * 1e-3)
        energies = [r["E"] for r in e2.steps()[n2:]]
        e2.close()
        return float(np.sum(t2)), energies

    emix = [r["E"] for r in steps_rec]
    fp64_leg, auto_leg = None, None
    if prec != "fp64" and not args.no_fp64_leg:
        t64, e64 = other_leg("fp64")
        fp64_leg = {"ms_per_step": t64 / args.steps * 1e3, "energies": e64,
                    "speedup_of_this_line": t64 / (total / world),
                    "max_rel_energy_diff": max(abs(a - b) / abs(b) for a, b in zip(emix, e64))}
        if prec == "mixed":
            ta, ea = other_leg("auto")
            auto_leg = {"ms_per_step": ta / args.steps * 1e3, "energies": ea,
                        "speedup_over_fp64": t64 / ta,
                        "max_rel_energy_diff_vs_fp64": max(abs(a - b) / abs(b) for a, b in zip(ea, e64))}
    lam_c = eng.lam(center)
    lam_all = np.sort(np.concatenate([np.asarray(v) for v in lam_c.values() if len(v)]))[::-1]
    spectrum = {"chi": int(lam_all.size), "s_max": float(lam_all[0]), "s_min_kept": float(lam_all[-1]),
                "sectors": {int(q): len(v) for q, v in lam_c.items()}}

    if args.steps_only:  # profiling runs: only warm-up + timed steps (few launches under a profiler)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "steps_only": True, "ms_per_step": total / args.steps * 1e3,
                              "gpu_launches": int(launches), "config": config_dict(args.chi, args.L, prec, args.svd, args.model),
                              "split_seconds_per_step": (st1["split_seconds"] - st0["split_seconds"]) / args.steps,
                              "energies": [s["E"] for s in steps_rec]}), flush=True)
        return

    # --------------------------------------------------------------- roofline: matvec kernel alone
    L = eng.env_tensor("L", center - 1)
    R = eng.env_tensor("R", center + 2)
    A1, A2 = eng.site_tensor(center), eng.site_tensor(center + 1)
    import ctypes as C
    th0 = C.c_void_p()
    lib.check(ctx.L.mpsg_theta(ctx.h, A1.h, A2.h, C.byref(th0)))
    th0 = lib.Tensor(ctx, th0)
    k0, k1 = lib.ItoKeyArg(ik[center]), lib.ItoKeyArg(ik[center + 1])
    w1, w2 = lib.MPOArg(W[center]), lib.MPOArg(W[center + 1])
    thc = C.c_void_p()
    lib.check(ctx.L.mpsg_theta_closure(ctx.h, L.h, R.h, th0.h, w1.ref(), w2.ref(), k0.ref(), k1.ref(), C.byref(thc)))
    thc = lib.Tensor(ctx, thc)
    thout = C.c_void_p()
    lib.check(ctx.L.mpsg_theta_closure(ctx.h, L.h, R.h, th0.h, w1.ref(), w2.ref(), k0.ref(), k1.ref(), C.byref(thout)))
    thout = lib.Tensor(ctx, thout)
    def time_matvec(p):
        plan = lib.MatvecPlan(ctx, L, R, thc, W[center], W[center + 1], ik[center], ik[center + 1], lib.PREC[p])
        din, _ = thc.device_view()
        dout, _ = thout.device_view()
        for _ in range(3):
            plan.execute(din, dout)
        mvt = []
        for _ in range(max(10, args.steps)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.execute(din, dout)
            e1.record(stream)
            e1.synchronize()
            mvt.append(e0.elapsed_time(e1) * 1e-3)
        return plan.info(), float(np.mean(mvt))

    pk, pk_kind = peaks()
    # the FP64 grouped GEMM (FP64 matvecs, environment update, the split's Gram and CholeskyQR products)
    # is the dominant kernel of an update in every mode; its roofline is the measured DGEMM peak
    info, mv64 = time_matvec("fp64")
    peak64 = fp64_peak_tflops(torch)
    roof = {"bound": "fp64", "achieved": info["flops"] / mv64 / 1e12, "peak": peak64, "unit": "TFLOP/s",
            "frac": info["flops"] / mv64 / 1e12 / peak64, "traffic": args.traffic_bytes,
            "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (MEASURED_PEAKS.json has no FP64 entry)",
            "kernel": "k_gemm_f64 (stage A + stage C of one FP64 matvec)", "flops_per_matvec": info["flops"],
            "matvec_seconds": mv64}
    roof_tc = None
    if prec != "fp64":
        mv_prec = "tf32x3" if prec in ("auto", "mixed") else prec  # the tensor-core matvec of the Lanczos
        info_tc, mv_tc = time_matvec(mv_prec)
        # hardware MMA work per algorithmic FLOP: 3 for hi/lo splits, x2 for TF32 (half the BF16 rate)
        mma_per_flop = (3 if mv_prec.endswith("x3") else 1) * (2 if mv_prec.startswith("tf32") else 1)
        ach = info_tc["flops"] / mv_tc / 1e12
        roof_tc = {"bound": "tensor", "achieved": ach, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                   "frac": ach / pk["bf16_tflops"], "peak_source": f"bf16_tflops ({pk_kind} dense BF16 cuBLAS)",
                   "kernel": f"k_tc_gemm<{mv_prec}> (conversion + stage A + stage C of one matvec)",
                   "matvec_seconds": mv_tc, "bf16_equivalent_mma_per_algorithmic_flop": mma_per_flop,
                   "tensor_issue_frac": ach * mma_per_flop / pk["bf16_tflops"]}
        tuned, hits, sched, ms6 = ctx.tc_autotune_info()
        names = ["round_robin", "snake", "lpt"]
        roof_tc["block_schedule_autotuner"] = {
            "signatures_timed": tuned, "plans_from_cache": hits,
            "stage_a": names[sched[0]] if sched[0] >= 0 else None,
            "stage_c": names[sched[1]] if sched[1] >= 0 else None,
            "last_timing_ms": {"stage_a": dict(zip(names, ms6[:3])), "stage_c": dict(zip(names, ms6[3:]))}}

    # --------------------------------------------------------------- e2e through the C ABI, host buffers
    env_leg = env_update_leg(ctx, eng, W, ik, center, torch, flush) if not args.steps_only else None
    e2e_raw = e2e_leg(ctx, eng, W, ik, center, args, stream, torch, flush, prec)
    e2e = {"value": info["flops"] * e2e_raw["matvecs"] * world / e2e_raw["seconds"] / 1e12, "unit": "TFLOP/s",
           "h2d_bytes_per_step": e2e_raw["h2d_bytes_per_step"], "d2h_bytes_per_step": e2e_raw["d2h_bytes_per_step"],
           "ms_per_step": e2e_raw["seconds"] / e2e_raw["steps"] * 1e3, "steps": e2e_raw["steps"],
           "path": "mpsg_tensor_create x4 -> mpsg_lanczos2 -> mpsg_split2 -> mpsg_add_contraction_layer -> "
                   "mpsg_tensor_export x4 (host buffers, wall clock with device sync)"}

    # --------------------------------------------------------------- CPU baseline (bounded sample)
    cpu, oracle_check = None, None
    if rank == 0 and not args.no_cpu:
        envs = (L.to_dict(), R.to_dict())
        sites_c = {center: A1.to_dict(), center + 1: A2.to_dict()}
        threads = os.cpu_count() or 1
        ts, st, g_or = cpu_update_seconds_window(W, ik, sites_c, center, args.chi, 1, threads, envs, args.L,
                                                 keep=True)
        cpu_mv = sum(s["iters"] for s in st)
        cpu_value = info["flops"] * cpu_mv / sum(ts) / 1e12
        cpu = {"value": cpu_value, "unit": "TFLOP/s", "cores": threads, "kind": "port",
               "sample": f"1 two-site update at the centre bond (chi={args.chi}), {cpu_mv} Lanczos matvecs, "
                         f"{sum(ts):.2f} s"}
        # the same update (same L, R, site tensors, direction) on the GPU, against the oracle's
        eng.do_step(center, 1, args.chi)
        g_rec, o_rec = eng.steps()[-1], st[-1]
        lg, lo = eng.lam(center), g_or.lam(center)
        common = set(lg) & set(lo)
        oracle_check = {"E_gpu": g_rec["E"], "E_oracle": o_rec["E"],
                        "rel_energy_diff": abs(g_rec["E"] - o_rec["E"]) / abs(o_rec["E"]),
                        "chi_gpu": g_rec["chi"], "chi_oracle": o_rec["chi"], "tw_gpu": g_rec["tw"],
                        "tw_oracle": o_rec["tw"],
                        "kept_per_sector_equal": {q: len(v) for q, v in lg.items()} ==
                                                 {q: len(v) for q, v in lo.items()},
                        "lambda_max_abs_diff": max((float(np.abs(np.asarray(lg[q])[:m] - np.asarray(lo[q])[:m]).max())
                                                    for q in common for m in [min(len(lg[q]), len(lo[q]))] if m),
                                                   default=0.0),
                        "what": "one two-site update at the centre bond from the same state (GPU in this "
                                "line's precision, oracle FP64 with LAPACK dgesvd)"}
        # the plain FP64 GPU path (mpsg_lanczos2 + mpsg_split2) on the same state against the same oracle
        # update: block structure, kept counts and singular values of the exact split
        w1c, w2c = lib.MPOArg(W[center]), lib.MPOArg(W[center + 1])
        k0c, k1c = lib.ItoKeyArg(ik[center]), lib.ItoKeyArg(ik[center + 1])
        st64, E64, it64 = C.c_void_p(), C.c_double(), C.c_int32()
        lib.check(ctx.L.mpsg_lanczos2(ctx.h, L.h, R.h, A1.h, A2.h, w1c.ref(), w2c.ref(), k0c.ref(), k1c.ref(), 500,
                                      1e-12, 1, lib.PREC["fp64"], 0, C.byref(st64), C.byref(E64), C.byref(it64)))
        psi64 = lib.Tensor(ctx, st64)
        U64, V64, lam64 = C.c_void_p(), C.c_void_p(), C.c_void_p()
        tw64, chi64 = C.c_double(), C.c_uint32()
        lib.check(ctx.L.mpsg_split2(ctx.h, psi64.h, k0c.ref(), k1c.ref(), args.chi, 0, 1e-12, 1, C.byref(U64),
                                    C.byref(V64), C.byref(lam64), C.byref(tw64), C.byref(chi64)))
        U64, V64 = lib.Tensor(ctx, U64), lib.Tensor(ctx, V64)
        l64 = lib.Tensor(ctx, lam64).to_dict()
        common64 = set(l64) & set(lo)
        oracle_check["fp64_gpu_path"] = {
            "E_gpu": E64.value, "rel_energy_diff": abs(E64.value - o_rec["E"]) / abs(o_rec["E"]),
            "chi_gpu": int(chi64.value), "tw_gpu": tw64.value,
            "kept_per_sector_equal": {q: len(v) for q, v in l64.items() if len(v)} ==
                                     {q: len(v) for q, v in lo.items() if len(v)},
            "lambda_max_abs_diff": max((float(np.abs(np.asarray(l64[q]) - np.asarray(lo[q])).max())
                                        for q in common64 if len(l64[q]) == len(lo[q]) and len(lo[q])), default=0.0)}
        del U64, V64, psi64

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": DTYPE.get(prec, prec),
                "data": "synthetic", "config": config_dict(args.chi, args.L, prec, args.svd, args.model), "clocks": clocks,
                "e2e": e2e, "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu,
                "lanczos_matvecs_per_step": matvecs / args.steps,
                "split_seconds_per_step": (st1["split_seconds"] - st0["split_seconds"]) / args.steps,
                "env_seconds_per_step": (st1["env_seconds"] - st0["env_seconds"]) / args.steps,
                "lanczos_seconds_per_step": (st1["lanczos_seconds"] - st0["lanczos_seconds"]) / args.steps,
                "energies": [s["E"] for s in steps_rec], "truncated_weight": [s["tw"] for s in steps_rec],
                "centre_bond_spectrum": spectrum, "fp64_gpu_path": fp64_leg, "auto_path": auto_leg,
                "roofline_tensor_matvec": roof_tc, "env_update_by_precision": env_leg,
                "matvec_flops_reference_schedule": info["flops_ref"], "oracle_check": oracle_check}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def cpu_update_seconds_window(W, ik, sites_c, center, chi, nsteps, threads, envs, N, keep=False):
    from oracle import pyoracle as O
    window = [sites_c.get(i, {}) for i in range(N)]
    g = O.DMRG(window, W, ik, maxthreads=threads, matvec_threads=threads)
    g.set_env("L", center - 1, envs[0])
    g.set_env("R", center + 2, envs[1])
    ts = []
    for i in range(nsteps):
        t0 = time.perf_counter()
        g.do_step(center, 1 if i % 2 == 0 else -1, chi)
        ts.append(time.perf_counter() - t0)
    return (ts, g.steps(), g) if keep else (ts, g.steps())


def env_update_leg(ctx, eng, W, ik, center, torch, flush, reps=5):
    """addContractionLayer at the centre bond (left environment through the centre site tensor) in
    FP64 and in each tensor-core precision, through the C ABI on device tensors: median ms (L2
    flushed before each call) and the largest deviation from the FP64 result relative to its largest
    entry."""
    import ctypes as C
    from mpstools_gb300 import lib
    Lt, A = eng.env_tensor("L", center - 1), eng.site_tensor(center)
    w, k = lib.MPOArg(W[center]), lib.ItoKeyArg(ik[center])
    out = {}
    ref = None
    for prec in ("fp64", "tf32x3", "bf16x3", "tf32", "bf16"):
        ts = []
        for rep in range(reps + 1):
            flush.zero_()
            torch.cuda.synchronize()
            a = time.perf_counter()
            h = C.c_void_p()
            lib.check(ctx.L.mpsg_add_contraction_layer(ctx.h, Lt.h, A.h, w.ref(), k.ref(), 1, lib.PREC[prec],
                                                       C.byref(h)))
            ctx.sync()
            if rep:
                ts.append(time.perf_counter() - a)
            t = lib.Tensor(ctx, h)
            if rep == reps:
                d = t.to_dict()
                if prec == "fp64":
                    ref = d
                    out[prec] = {"ms": float(np.median(ts)) * 1e3}
                else:
                    scale = max(np.abs(v).max() for v in ref.values())
                    err = max(float(np.abs(d[q] - ref[q]).max()) for q in ref) / scale
                    out[prec] = {"ms": float(np.median(ts)) * 1e3, "max_rel_diff_vs_fp64": err}
            del t
    return out


def e2e_leg(ctx, eng, W, ik, center, args, stream, torch, flush, prec):
    """Two-site update through the reference-facing C ABI from host buffers."""
    import ctypes as C
    from mpstools_gb300 import lib
    # host buffers of the inputs and results are pinned (page-locked), as an integration that streams
    # tensors through the library would allocate them
    pool = {}

    def pinned(n, tag):
        key = (tag, n)
        if key not in pool:
            pool[key] = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        return pool[key]

    def pin_flat(flat, tag):
        buf = pinned(flat[5].size, tag)
        buf[:] = flat[5]
        return flat[:5] + (buf,)

    Lh = pin_flat(eng.env_tensor("L", center - 1).export_flat(), "L")
    Rh = pin_flat(eng.env_tensor("R", center + 2).export_flat(), "R")
    A1h = pin_flat(eng.site_tensor(center).export_flat(), "A1")
    A2h = pin_flat(eng.site_tensor(center + 1).export_flat(), "A2")
    w1, w2 = lib.MPOArg(W[center]), lib.MPOArg(W[center + 1])
    k0, k1 = lib.ItoKeyArg(ik[center]), lib.ItoKeyArg(ik[center + 1])
    h2d = sum(x[5].nbytes + x[1].nbytes + x[2].nbytes + x[3].nbytes * 2 for x in (Lh, Rh, A1h, A2h))
    d2h = [0]
    flops = [0.0]

    def step(i):
        tL, tR = lib.Tensor.from_flat(ctx, Lh), lib.Tensor.from_flat(ctx, Rh)
        t1, t2 = lib.Tensor.from_flat(ctx, A1h), lib.Tensor.from_flat(ctx, A2h)
        st, E0, it = C.c_void_p(), C.c_double(), C.c_int32()
        lib.check(ctx.L.mpsg_lanczos2(ctx.h, tL.h, tR.h, t1.h, t2.h, w1.ref(), w2.ref(), k0.ref(), k1.ref(), 500,
                                      1e-12, 1, lib.PREC[prec], 0, C.byref(st), C.byref(E0), C.byref(it)))
        psi = lib.Tensor(ctx, st)
        U, V, lam = C.c_void_p(), C.c_void_p(), C.c_void_p()
        tw, chi = C.c_double(), C.c_uint32()
        lib.check(ctx.L.mpsg_split2(ctx.h, psi.h, k0.ref(), k1.ref(), args.chi, 0, 1e-12, 1, C.byref(U), C.byref(V),
                                    C.byref(lam), C.byref(tw), C.byref(chi)))
        U, V, lam = lib.Tensor(ctx, U), lib.Tensor(ctx, V), lib.Tensor(ctx, lam)
        Lo = C.c_void_p()
        lib.check(ctx.L.mpsg_add_contraction_layer(ctx.h, tL.h, U.h, w1.ref(), k0.ref(), 1, lib.PREC["fp64"],
                                                   C.byref(Lo)))
        Lo = lib.Tensor(ctx, Lo)
        outs = [t.export_flat(lambda n, tag=tag: pinned(n, tag))
                for t, tag in ((U, "U"), (V, "V"), (lam, "lam"), (Lo, "Lo"))]
        d2h[0] = sum(o[5].nbytes for o in outs)
        return it.value  # Lanczos matvecs (MIXED's FP64 Rayleigh-quotient matvec is not counted)

    for i in range(2):
        step(i)
    torch.cuda.synchronize()
    n = max(2, min(args.steps, 5))
    mvs, secs = 0, 0.0
    for i in range(n):
        flush.zero_()
        torch.cuda.synchronize()
        a = time.perf_counter()
        mvs += step(i)
        torch.cuda.synchronize()
        secs += time.perf_counter() - a
    return {"matvecs": mvs, "seconds": secs, "steps": n, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h[0])}


SWEEP_RAMP = (256, 256, 1024, 1024, 1024, 2048, 2048, 2048)


def sweep_workload(L=L_SITES, model="xxz"):
    """Config of the sweep measurement: the XXZ chain (L=100, Jxy=1, Delta_i ~ U[0.5,1.5] from seed 1,
    Sz_total=0) or the t-V chain at half filling, from the product state of the reference drivers
    (every (L/N)-th site occupied, main/mainHeisenberg.cpp:175-191)."""
    from mpstools_gb300 import models as M
    if model == "tv":
        W = M.spinless_fermions_mpo(2.0 * M.uniform01(SEED_V, L - 1), np.ones(L - 1), np.zeros(L))
    else:
        W = M.heisenberg_mpo(M.xxz_couplings(L, SEED_DELTA), np.ones(L - 1), np.zeros(L))
    ik = M.u1_itokeys(L)
    sites = M.product_state(M.filling_state(L, L // 2), ik)
    return W, ik, sites


def run_sweeps(eng, N, ramp, sync=None, on_sweep=None):
    """DMRGengine::simulate's sweep loop (src/container.hpp:381-438) with one chimax per sweep:
    orthonormalize("rl") and the right environments once, then per sweep doStep(site, +1) for
    site = 0..N-3 and doStep(site, -1) for site = N-2..1; after the last sweep doStep(0, -1).
    Returns one record per sweep (wall seconds, chi, energy of the sweep's last update)."""
    recs = []
    t0 = time.perf_counter()
    eng.prepare()
    if sync:
        sync()
    t_prep = time.perf_counter() - t0
    for k, chi in enumerate(ramp):
        n0 = len(eng.steps())
        t0 = time.perf_counter()
        for site in range(N - 2):
            eng.do_step(site, 1, chi)
        for site in range(N - 2, 0, -1):
            eng.do_step(site, -1, chi)
        if sync:
            sync()
        dt = time.perf_counter() - t0
        st = eng.steps()[n0:]
        recs.append({"sweep": k + 1, "chi": chi, "seconds": dt, "E": st[-1]["E"], "updates": len(st),
                     "lanczos_iterations": int(sum(s["iters"] for s in st)),
                     "max_chi_kept": int(max(s["chi"] for s in st)),
                     "chi_kept": [int(s["chi"]) for s in st]})
        if on_sweep:
            on_sweep(recs[-1])
    last = eng.do_step(0, -1, ramp[-1])
    return recs, t_prep, last


def sweep_leg(ctx, prec, W, ik, sites, ramp, torch):
    from mpstools_gb300 import api
    eng = api.DMRGengine(sites, W, ik, prec=prec, ctx=ctx)
    s0 = eng.stats()
    f0 = int(ctx.L.mpsg_split_fallbacks())

    def progress(r):  # one line per sweep on stderr, so that a run cut short still leaves its record
        st = eng.stats()
        print(json.dumps({"prec": prec, "sweep": r["sweep"], "chi": r["chi"], "seconds": r["seconds"], "E": r["E"],
                          "max_chi_kept": r["max_chi_kept"], "lanczos_iterations": r["lanczos_iterations"],
                          "split_seconds_total": st["split_seconds"] - s0["split_seconds"],
                          "lanczos_seconds_total": st["lanczos_seconds"] - s0["lanczos_seconds"],
                          "matvec_seconds_total": st["lanczos_iter_seconds"] - s0["lanczos_iter_seconds"],
                          "env_seconds_total": st["env_seconds"] - s0["env_seconds"],
                          "prep_seconds_total": st["prep_seconds"] - s0["prep_seconds"],
                          "lanczos_call_seconds_total": st["lanczos_call_seconds"] - s0["lanczos_call_seconds"],
                          "split_fallbacks_to_jacobi": int(ctx.L.mpsg_split_fallbacks()) - f0}),
              file=sys.stderr, flush=True)

    recs, t_prep, E = run_sweeps(eng, len(sites), ramp, sync=torch.cuda.synchronize, on_sweep=progress)
    s1 = eng.stats()
    lam_c = eng.lam(len(sites) // 2 - 1)
    vals = np.sort(np.concatenate([np.asarray(v) for v in lam_c.values() if len(v)]))[::-1]
    eng.close()
    return {"prec": prec, "sweeps": recs, "prepare_seconds": t_prep, "E_final": E,
            "split_seconds": s1["split_seconds"] - s0["split_seconds"],
            "env_seconds": s1["env_seconds"] - s0["env_seconds"],
            "lanczos_seconds": s1["lanczos_seconds"] - s0["lanczos_seconds"],
            "matvecs": s1["matvecs"] - s0["matvecs"], "matvec_flops": s1["matvec_flops"] - s0["matvec_flops"],
            "centre_bond": {"chi": int(vals.size), "s_min_kept": float(vals[-1]),
                            "sectors": {int(q): len(v) for q, v in lam_c.items()}}}


SPLIT_RAMP = (256, 256, 1024, 1024, 1024, 2048)


def split_arm(args):
    """--workload split: the split alone (mpsg_split2 with --svd) of the two-site ground state at the
    centre bond of the XXZ chain (L=100, Jxy=1, Delta_i ~ U[0.5,1.5] seed 1) after a chi ramp
    (--ramp, default 256, 256, 1024, 1024, 1024, 2048: chi grows about fourfold per sweep from the
    product state; MIXED): the sector structure of a converged
    chi=2048 state (sector matrices up to ~1000 x 1000).  The FP64 Lanczos ground state at the centre
    bond is formed once; --warmup + --steps splits of it follow, the timed ones inside the NVTX range
    "split" (profiler launch lists: ncu --nvtx --nvtx-include split/).  The oracle's split (LAPACK
    dgesvd) of the same state checks the singular values and the kept count of every sector."""
    import ctypes as C
    import torch
    from mpstools_gb300 import lib, api
    ramp = tuple(args.ramp) if args.ramp else SPLIT_RAMP
    chimax = ramp[-1]
    W, ik, sites = sweep_workload(args.L, args.model)
    ctx = lib.Context(0)
    ctx.set_svd_method(args.svd)
    eng = api.DMRGengine(sites, W, ik, prec="mixed", ctx=ctx)
    t0 = time.perf_counter()
    run_sweeps(eng, args.L, ramp, sync=torch.cuda.synchronize)
    c = args.L // 2 - 1
    for site in range(c):
        eng.do_step(site, 1, chimax)
    t_ramp = time.perf_counter() - t0
    Lt, Rt = eng.env_tensor("L", c - 1), eng.env_tensor("R", c + 2)
    A1, A2 = eng.site_tensor(c), eng.site_tensor(c + 1)
    w1, w2 = lib.MPOArg(W[c]), lib.MPOArg(W[c + 1])
    k0, k1 = lib.ItoKeyArg(ik[c]), lib.ItoKeyArg(ik[c + 1])
    st, E0, it = C.c_void_p(), C.c_double(), C.c_int32()
    lib.check(ctx.L.mpsg_lanczos2(ctx.h, Lt.h, Rt.h, A1.h, A2.h, w1.ref(), w2.ref(), k0.ref(), k1.ref(), 500, 1e-12, 1,
                                  lib.PREC["fp64"], 0, C.byref(st), C.byref(E0), C.byref(it)))
    psi = lib.Tensor(ctx, st)
    # only the state stays on the device (the engine, its environments and site tensors are released)
    del Lt, Rt, A1, A2
    eng.close()
    ctx.trim()

    def split_once():
        U, V, lam = C.c_void_p(), C.c_void_p(), C.c_void_p()
        tw, chi = C.c_double(), C.c_uint32()
        lib.check(ctx.L.mpsg_split2(ctx.h, psi.h, k0.ref(), k1.ref(), chimax, 0, 1e-12, 1, C.byref(U), C.byref(V),
                                    C.byref(lam), C.byref(tw), C.byref(chi)))
        return lib.Tensor(ctx, U), lib.Tensor(ctx, V), lib.Tensor(ctx, lam), tw.value, chi.value

    f0 = int(ctx.L.mpsg_split_fallbacks())
    for _ in range(max(args.warmup, 1)):
        out = split_once()
    clk = ClockSampler()
    clk.start()
    times = []
    torch.cuda.nvtx.range_push("split")
    for _ in range(args.steps):
        del out
        ctx.sync()
        a = time.perf_counter()
        out = split_once()
        ctx.sync()
        times.append(time.perf_counter() - a)
    torch.cuda.nvtx.range_pop()
    clocks = clk.stop()
    U, V, lam, tw, chi = out
    lam_d, u_d, v_d = lam.to_dict(), U.to_dict(), V.to_dict()
    rows, cols = {}, {}
    for (a, qc, s1), blk in u_d.items():
        rows[qc] = rows.get(qc, 0) + blk.shape[0]
    for (qc, b, s2), blk in v_d.items():
        cols[qc] = cols.get(qc, 0) + blk.shape[1]
    sectors = sorted(([int(rows[q]), int(cols[q]), len(lam_d[q])] for q in lam_d if q in rows and q in cols),
                     key=lambda x: -x[0] * x[1])
    line = {"metric": "split time of a converged chi=2048 two-site state", "value": float(np.median(times)) * 1e3,
            "unit": "ms", "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{args.model}_L{args.L}_centre_bond_split_after_ramp", "ramp": list(ramp),
                       "svd": args.svd, "state": "FP64 Lanczos ground state at the centre bond after the ramp",
                       "ramp_seconds": t_ramp},
            "ms_each": [t * 1e3 for t in times], "chi": int(chi), "truncated_weight": tw,
            "sectors_m_n_kept": sectors, "split_fallbacks_to_jacobi": int(ctx.L.mpsg_split_fallbacks()) - f0,
            "clocks": clocks}
    if not args.no_cpu:
        from oracle import pyoracle as O
        th = psi.to_dict()
        a = time.perf_counter()
        U0, V0, l0, tw0, chi0 = O.split(th, ik[c], ik[c + 1], chimax, nthreads=os.cpu_count() or 1)
        t_or = time.perf_counter() - a
        kept_eq = {q: len(v) for q, v in l0.items() if len(v)} == {q: len(v) for q, v in lam_d.items() if len(v)}
        dl = max((float(np.abs(np.asarray(lam_d[q]) - np.asarray(l0[q])).max())
                  for q in l0 if len(l0[q]) and q in lam_d and len(lam_d[q]) == len(l0[q])), default=0.0)
        line["oracle_check"] = {"chi_oracle": int(chi0), "kept_per_sector_equal": bool(kept_eq),
                                "lambda_max_abs_diff": dl, "tw_oracle": tw0, "oracle_seconds": t_or}
        line["cpu_baseline"] = {"value": t_or * 1e3, "unit": "ms", "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": "the same split in the oracle (LAPACK dgesvd per sector, all threads)"}
    print(json.dumps(line), flush=True)


def oracle_sweeps(W, ik, sites, ramp, threads):
    from oracle import pyoracle as O
    g = O.DMRG(sites, W, ik, maxthreads=threads, matvec_threads=threads)
    recs = []
    t0 = time.perf_counter()
    g.prepare()
    N = len(sites)
    for k, chi in enumerate(ramp):
        n0 = len(g.steps())
        a = time.perf_counter()
        for site in range(N - 2):
            g.do_step(site, 1, chi)
        for site in range(N - 2, 0, -1):
            g.do_step(site, -1, chi)
        st = g.steps()[n0:]
        recs.append({"sweep": k + 1, "chi": chi, "seconds": time.perf_counter() - a, "E": st[-1]["E"],
                     "chi_kept": [int(s["chi"]) for s in st]})
    return recs


def sweep_arm(args):
    """XXZ L=100 from the product state, chi ramp 256 (2 sweeps) -> 1024 (3) -> 2048 (3), in
    MIXED (tensor-core Lanczos) and in plain FP64 on the same GPU; the CPU oracle runs the first
    --oracle-sweeps sweeps of the same schedule for the energy check."""
    import torch
    from mpstools_gb300 import lib
    ramp = tuple(args.ramp) if args.ramp else SWEEP_RAMP
    W, ik, sites = sweep_workload(args.L, args.model)
    ctx = lib.Context(0)
    ctx.set_svd_method(args.svd)
    legs = {}
    clk = ClockSampler()
    clk.start()
    for p in ([args.prec] + ([] if args.prec == "fp64" or args.no_fp64_leg else ["fp64"])):
        legs[p] = sweep_leg(ctx, p, W, ik, sites, ramp, torch)
    clocks = clk.stop()
    ora = None
    if args.oracle_sweeps > 0:
        ora = oracle_sweeps(W, ik, sites, ramp[:args.oracle_sweeps], os.cpu_count() or 1)
    main = legs[args.prec]
    top = max(ramp)
    t_top = [r["seconds"] for r in main["sweeps"] if r["chi"] == top]
    out = {"metric": "DMRG sweep time (XXZ L=100, chi ramp 256 -> 1024 -> 2048)", "impl": "ours", "value": float(np.mean(t_top)),
           "unit": f"s per sweep at chi={top}", "higher_is_better": False, "n_gpus": 1,
           "dtype": DTYPE.get(args.prec, args.prec), "data": "synthetic",
           "config": {"workload": f"{args.model}_L{args.L}_product_state_chi_ramp", "ramp": list(ramp),
                      "model": MODEL_TEXT[args.model], "lanczos": "delta=1e-12, energy test every 5 iterations",
                      "svd": args.svd}, "clocks": clocks, "legs": legs}
    if "fp64" in legs and args.prec != "fp64":
        f = legs["fp64"]
        t64 = [r["seconds"] for r in f["sweeps"] if r["chi"] == top]
        out["fp64_speedup_at_top_chi"] = float(np.sum(t64) / np.sum(t_top))
        out["rel_energy_diff_per_sweep_vs_fp64"] = [abs(a["E"] - b["E"]) / abs(b["E"])
                                                     for a, b in zip(main["sweeps"], f["sweeps"])]
        out["rel_energy_diff_final_vs_fp64"] = abs(main["E_final"] - f["E_final"]) / abs(f["E_final"])
    if ora:
        out["oracle"] = {"sweeps": ora, "cores": os.cpu_count() or 1}
        for p, leg in legs.items():
            out[f"rel_energy_diff_vs_oracle_{p}"] = [abs(a["E"] - b["E"]) / abs(b["E"])
                                                     for a, b in zip(leg["sweeps"], ora)]
            out[f"chi_kept_equal_oracle_{p}"] = [a["chi_kept"] == b["chi_kept"] for a, b in zip(leg["sweeps"], ora)]
    print(json.dumps(out), flush=True)


def chains_workload(nchains, chi, seed=3):
    """Batched ground states: nchains XXZ chains, L ~ U{24..96}, one Delta ~ U[0.5,1.5] per chain
    (seeded), Jxy = 1, Sz_total = 0, each from a seeded random U(1) MPS with bond dimension chi."""
    from mpstools_gb300 import models as M
    u = M.uniform01(seed, 2 * nchains)
    lengths = [24 + min(72, int(np.floor(x * 73))) for x in u[:nchains]]
    deltas = 0.5 + u[nchains:]
    chains = []
    for c, (N, d) in enumerate(zip(lengths, deltas)):
        W = M.heisenberg_mpo(np.full(N - 1, d), np.ones(N - 1), np.zeros(N))
        chains.append((M.random_u1_mps(N, N // 2, chi, 3000 + c), W, M.u1_itokeys(N)))
    return lengths, deltas, chains


def chains_arm(args):
    """Batched chains against the same chains run one at a time on the same GPU."""
    from mpstools_gb300 import api, lib
    ctx = lib.Context(0)
    ctx.set_svd_method(args.svd)
    lengths, deltas, chains = chains_workload(args.nchains, args.chi)
    engines = [api.DMRGengine(s, W, ik, ctx=ctx) for s, W, ik in chains]
    batch = api.DMRGbatch(engines, prec=args.prec)
    t0 = time.perf_counter()
    E = batch.simulate(args.sweeps, args.chi, delta=1e-12)
    t_batch = time.perf_counter() - t0
    st = batch.stats()
    batch.close()
    for e in engines:
        e.close()
    K = max(0, min(args.seq_chains, args.nchains))
    t_seq, E_seq = 0.0, []
    for s, W, ik in chains[:K]:
        e = api.DMRGengine(s, W, ik, prec=args.prec, ctx=ctx)
        t0 = time.perf_counter()
        E_seq.append(e.simulate(maxsteps=args.sweeps, EnConv=1e-300, chimax=args.chi, delta=1e-12))
        t_seq += time.perf_counter() - t0
        e.close()
    E_k, t_batch_k, st_k = [], 0.0, {"matvec_launches": 0, "matvecs": 0}
    if K > 0:
        engines_k = [api.DMRGengine(s, W, ik, ctx=ctx) for s, W, ik in chains[:K]]
        bk = api.DMRGbatch(engines_k, prec=args.prec)
        t0 = time.perf_counter()
        E_k = bk.simulate(args.sweeps, args.chi, delta=1e-12)
        t_batch_k = time.perf_counter() - t0
        st_k = bk.stats()
        bk.close()
    rel = (float(np.max(np.abs(np.asarray(E_k) - np.asarray(E_seq)) / np.abs(np.asarray(E_seq))))
           if K > 0 else None)
    out = {"metric": "chain-sweeps per second, batched independent DMRG chains", "impl": "ours",
           "value": args.nchains * args.sweeps / t_batch, "unit": "chain-sweeps/s", "higher_is_better": True,
           "n_gpus": 1, "dtype": args.prec, "data": "synthetic",
           "config": {"workload": f"{args.nchains}_xxz_chains_L24-96_chi{args.chi}", "chains": args.nchains,
                      "chi": args.chi, "sweeps": args.sweeps, "lengths": lengths, "svd": args.svd,
                      "model": "XXZ, Jxy=1, one Delta~U[0.5,1.5] per chain (seed 3), Sz_total=0",
                      "state": "seeded random U(1) MPS per chain"},
           "seconds": t_batch, "device_seconds": st["device_seconds"], "batch_stats": st,
           "split_fallbacks_to_jacobi": int(ctx.L.mpsg_split_fallbacks()),
           "energies_first": [float(x) for x in E[:4]],
           "sequential_same_gpu": {"chains": K, "seconds": t_seq, "batched_seconds": t_batch_k,
                                   "speedup_of_batching": t_seq / t_batch_k if K > 0 else None,
                                   "max_rel_energy_diff": rel,
                                   "batched_matvec_launches": st_k["matvec_launches"],
                                   "batched_matvecs": st_k["matvecs"]}}
    print(json.dumps(out))


def tebd_arm(args):
    """TEBD of the XXZ chain L=64 from the Neel state, second order, dt=0.05, chi <= 512, truncation
    1e-10 (split by --svd: default the library's complex bidiagonal SVD; slices batched): forward
    time, the gradient of <Sz_32(T)> w.r.t. the 63 per-bond anisotropies (Delta_i ~ U[0.8,1.2],
    seed 4) by the adjoint, and central differences (h = 1e-5) of the same evolution on `--fd-bonds`
    bonds."""
    from mpstools_gb300 import api, lib, models as M
    N, dt, chimax, trw, obs = 64, 0.05, 512, 1e-10, 32
    steps = args.tebd_steps
    sz = [-0.5, 0.5]
    ctx = lib.Context(0)
    ctx.set_svd_method(args.svd)
    theta = 0.8 + 0.4 * M.uniform01(4, N - 1)
    ik = M.u1_itokeys(N)
    mk = lambda t: M.heisenberg_mpo(t, np.ones(N - 1), np.zeros(N))

    def forward(t):
        e = api.TEBDengine(M.neel_state(N), mk(t), ik, ctx=ctx)
        t0 = time.perf_counter()
        e.second_order(steps, dt, chimax, doTrunc=True, tr_weight=trw)
        sec = time.perf_counter() - t0
        v = e.measure_diag(obs, sz)
        chis = [sum(len(x) for x in e.lam(b).values()) for b in range(N - 1)]
        st = e.stats()
        e.close()
        return v, sec, max(chis), st

    v0, t_fwd, chi_max, st = forward(theta)
    dh = api.couplingDerivatives(mk, theta, ik)
    e = api.TEBDengine(M.neel_state(N), mk(theta), ik, ctx=ctx)
    t0 = time.perf_counter()
    v_adj, grad = e.adjoint_second_order(steps, dt, chimax, obs, sz, dh, doTrunc=True, tr_weight=trw)
    t_adj = time.perf_counter() - t0
    e.close()
    h, fd = 1e-5, {}
    for b in args.fd_bonds:
        tp, tm = theta.copy(), theta.copy()
        tp[b] += h
        tm[b] -= h
        fd[b] = (forward(tp)[0] - forward(tm)[0]) / (2 * h)
    out = {"metric": "TEBD second-order steps per second (XXZ L=64, chi<=512)", "impl": "ours",
           "value": steps / t_fwd, "unit": "steps/s", "higher_is_better": True, "n_gpus": 1, "dtype": "c128",
           "data": "synthetic",
           "config": {"workload": "tebd_xxz_L64_neel_dt0.05_chi512", "steps": steps, "dt": dt, "chimax": chimax,
                      "tr_weight": trw, "observable": "Sz_32", "couplings": "Delta_i ~ U[0.8,1.2] seed 4",
                      "svd": {"bidiag": "complex bidiagonal SVD (own kernels)", "jacobi": "cuSOLVER zgesvdj"}.get(
                          args.svd, "density (complex Gram, batched Hermitian eigensolver)") + ", slices batched",
                      "split_fallbacks": int(ctx.L.mpsg_split_fallbacks())},
           "forward_seconds": t_fwd, "max_chi": chi_max, "value_Sz32": v0, "gates": st["gates"],
           "split_seconds": st["split_seconds"],
           "adjoint": {"seconds_forward_plus_gradient": t_adj, "value": v_adj, "grad_max_abs": float(np.abs(grad).max()),
                       "grad_bonds_fd": {str(b): {"adjoint": float(grad[b]), "central_difference": float(fd[b])}
                                         for b in fd}}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--chi", type=int, default=CHI)
    ap.add_argument("--L", type=int, default=None, help="chain length (default: 100 for xxz, 128 for tv)")
    ap.add_argument("--model", default="xxz", choices=["xxz", "tv"],
                    help="centre-update workload: XXZ chain or t-V chain at half filling")
    ap.add_argument("--prec", default=None,
                    help="fp64 | tf32 | tf32x3 | bf16 | bf16x3 | auto | mixed (default: mixed; chains: auto)")
    ap.add_argument("--svd", default="bidiag", choices=["bidiag", "density", "density_mt", "density_eig", "jacobi"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--traffic-bytes", type=float, default=None)
    ap.add_argument("--no-fp64-leg", action="store_true",
                    help="skip the plain FP64 GPU path timed on the same updates (mixed precisions only)")
    ap.add_argument("--steps-only", action="store_true",
                    help="time the DMRG steps only (no roofline / e2e / CPU legs); for profiler launch lists")
    ap.add_argument("--workload", default="centre_update",
                    choices=["centre_update", "sweep", "split", "chains", "tebd"],
                    help="chains: batched independent chains (--nchains, --sweeps, --seq-chains; --chi 256); "
                         "tebd: L=64 TEBD forward + adjoint gradient (--tebd-steps, --fd-bonds); "
                         "split: the split of a converged chi=2048 centre-bond state (--ramp)")
    ap.add_argument("--ramp", type=int, nargs="*", default=None, help="sweep: chimax per sweep")
    ap.add_argument("--oracle-sweeps", type=int, default=2, help="sweep: sweeps the CPU oracle runs")
    ap.add_argument("--tebd-steps", type=int, default=200)
    ap.add_argument("--fd-bonds", type=int, nargs="*", default=[31])
    ap.add_argument("--nchains", type=int, default=64)
    ap.add_argument("--sweeps", type=int, default=2)
    ap.add_argument("--seq-chains", type=int, default=8)
    args = ap.parse_args()
    if args.L is None:
        args.L = MODEL_L[args.model]
    if args.prec is None:
        args.prec = "auto" if args.workload == "chains" else "mixed"
    if args.workload == "chains":
        chains_arm(args)
    elif args.workload == "tebd":
        tebd_arm(args)
    elif args.workload == "sweep":
        sweep_arm(args)
    elif args.workload == "split":
        split_arm(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
