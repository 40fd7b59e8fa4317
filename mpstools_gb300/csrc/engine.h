// DMRG engine (DMRGengine::simulate / doStep) with all tensors resident on the device: shared by the
// C ABI (capi.cpp) and the batched-chain engine (batch.cpp).
#pragma once
#include <chrono>
#include <cmath>
#include <cstring>

#include "capi_types.h"

namespace mpsg {

struct StepRec {
  int site, dir, iters, chi;
  double E, tw;
};

// DMRGengine (src/container.hpp:236-438) with all tensors resident on the device.
struct Engine {
  Ctx* ctx;
  std::shared_ptr<Ctx> keep;
  int N;
  std::vector<TensorP> mps;
  std::vector<MPO> mpo;
  std::vector<ItoKey> ik;
  std::map<int, TensorP> L, R, lam;
  mpsg_prec prec = MPSG_PREC_FP64;
  bool reorth = false;
  int lanmax = 500;
  // arithmetic of the environment updates of doStep (FP64 by default: a tensor-core environment
  // perturbs H itself, by ~1e-7 relative for TF32X3, which the FP64 energy then carries)
  mpsg_prec env_prec = MPSG_PREC_FP64;
  std::vector<StepRec> steps;
  int64_t updates_base = 0;  // doStep calls made before this engine was loaded from a checkpoint
  int64_t updates_done() const { return updates_base + (int64_t)steps.size(); }
  LanczosStats lst;
  double env_seconds = 0, split_seconds = 0, env_flops = 0, wall = 0;
  // wall seconds of doStep before the eigensolver (theta layout, closure and formation) and of the
  // eigensolver call as a whole (matvec plan, Lanczos, the FP64 energy of MIXED, AUTO's finish)
  double prep_seconds = 0, lanczos_call_seconds = 0;

  static TensorP lmin(Ctx* ctx) {  // getLMin: (0,0;0) = [[1]]
    uint64_t q[2] = {0, 0};
    uint32_t p[1] = {0};
    int32_t r[1] = {1}, c[1] = {1};
    double d[1] = {1.0};
    return tensor_from_host(ctx, 1, 1, q, p, r, c, d);
  }
  static TensorP rmax(Ctx* ctx, const Tensor& last) {  // getRMax: identity per right charge
    std::map<Q, int> dims;
    for (auto& b : last.b)
      if (!dims.count(b.k.q1)) dims[b.k.q1] = b.c;
    std::vector<uint64_t> q;
    std::vector<uint32_t> p;
    std::vector<int32_t> r, c;
    std::vector<double> d;
    for (auto& x : dims) {
      q.push_back(x.first);
      q.push_back(x.first);
      p.push_back(0);
      r.push_back(x.second);
      c.push_back(x.second);
      for (int j = 0; j < x.second; ++j)
        for (int i = 0; i < x.second; ++i) d.push_back(i == j ? 1.0 : 0.0);
    }
    return tensor_from_host(ctx, 1, (int)dims.size(), q.data(), p.data(), r.data(), c.data(), d.data());
  }

  void prepare() {
    // orthonormalize(mps, "rl") (src/MPSfunctions.hpp:1776-1784) with truncation of values <= 1e-16
    for (int site = N - 1; site >= 0; --site) {
      TensorP lamt;
      if (site > 0) prepare_matrix_r(ctx, &mps[site - 1], mps[site], &lamt, 1e-16);
      else prepare_matrix_r(ctx, nullptr, mps[0], &lamt, 1e-16);
      lam[site - 1] = lamt;
    }
    auto t0 = std::chrono::steady_clock::now();
    R.clear();
    R[N] = rmax(ctx, *mps[N - 1]);
    for (int s = N - 1; s >= 2; --s) R[s] = env_update(ctx, *R[s + 1], *mps[s], mpo[s], ik[s], 0, &env_flops);
    ctx->sync();
    env_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    L.clear();
    L[-1] = lmin(ctx);
  }

  void build_environments(int c) {
    MPSG_CHECK(c >= 0 && c + 1 < N, "center out of range");
    auto t0 = std::chrono::steady_clock::now();
    L.clear();
    L[-1] = lmin(ctx);
    for (int s = 0; s < c; ++s) L[s] = env_update(ctx, *L[s - 1], *mps[s], mpo[s], ik[s], 1, &env_flops);
    R.clear();
    R[N] = rmax(ctx, *mps[N - 1]);
    for (int s = N - 1; s >= c + 2; --s) R[s] = env_update(ctx, *R[s + 1], *mps[s], mpo[s], ik[s], 0, &env_flops);
    ctx->sync();
    env_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double step_device_seconds = 0;
  int64_t nstep_calls = 0;

  StepRec do_step(int site, int dir, int chimax, bool doTrunc, double tr_weight, double delta, bool testenergy) {
    if (!ev0) {
      MPSG_CUDA(cudaEventCreate(&ev0));
      MPSG_CUDA(cudaEventCreate(&ev1));
    }
    MPSG_CUDA(cudaEventRecord(ev0, ctx->stream));
    StepRec r = do_step_impl(site, dir, chimax, doTrunc, tr_weight, delta, testenergy);
    MPSG_CUDA(cudaEventRecord(ev1, ctx->stream));
    MPSG_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    step_device_seconds += ms * 1e-3;
    ++nstep_calls;
    return r;
  }
  ~Engine() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }

  // Identity MPO tensor of a site (IdentityMPO, Dl = Dr = 1): overlap environments and basis changes.
  static MPO identity_mpo(int d) {
    MPO m;
    m.Dl = m.Dr = 1;
    MPOEntry en;
    en.wl = en.wr = 0;
    for (uint32_t i = 0; i < (uint32_t)d; ++i) en.ops.push_back(OpEl{i, i, 1.0});
    m.e.push_back(en);
    return m;
  }

  // The dummy second site of a single-site contraction: identity on D MPO channels, one local state
  // (of charge 0, ItoKey(1, 0)).
  static MPO dummy_site_mpo(int D) {
    MPO m;
    m.Dl = m.Dr = D;
    for (int w = 0; w < D; ++w) {
      MPOEntry en;
      en.wl = en.wr = (uint32_t)w;
      en.ops.push_back(OpEl{0, 0, 1.0});
      m.e.push_back(en);
    }
    return m;
  }

  // excited-state targeting: the target MPS and its overlap environments with the engine's state
  const std::vector<TensorP>* target = nullptr;
  std::map<int, TensorP> ovL, ovR;

  StepRec do_step_impl(int site, int dir, int chimax, bool doTrunc, double tr_weight, double delta,
                       bool testenergy) {
    MPSG_CHECK(site >= 0 && site + 1 < N, "site out of range");
    MPSG_CHECK(L.count(site - 1) && R.count(site + 2), "environments missing (call prepare first)");
    const auto tp0 = std::chrono::steady_clock::now();
    const Tensor& Le = *L[site - 1];
    const Tensor& Re = *R[site + 2];
    // theta structure: blocks of BlockMatrix<2>(mps[site], mps[site+1]) and everything the matvec reaches
    Layout s0;
    {
      std::map<Q, std::vector<int>> by_left;
      for (int j = 0; j < (int)mps[site + 1]->b.size(); ++j) by_left[mps[site + 1]->b[j].k.q0].push_back(j);
      for (auto& a : mps[site]->b) {
        auto it = by_left.find(a.k.q1);
        if (it == by_left.end()) continue;
        for (int j : it->second) {
          const Block& b = mps[site + 1]->b[j];
          s0.add(K2(a.k.q0, b.k.q1, a.k.p0, b.k.p0), a.r, b.c);
        }
      }
      s0.finalize();
    }
    // doStepExcited: the target's two-site state in the current basis (contractTwosite with the
    // overlap environments and identity MPOs, src/container.hpp:488-498), projected out of the Lanczos
    TensorP tstate;
    const MPO id0 = identity_mpo((int)ik[site].size()), id1 = identity_mpo((int)ik[site + 1].size());
    if (target) {
      TensorP told = theta_form(ctx, *(*target)[site], *(*target)[site + 1], nullptr);
      auto nat = build_matvec(ctx, *ovL.at(site - 1), *ovR.at(site + 2), layout_of(*told), id0, id1, ik[site],
                              ik[site + 1], nullptr, MPSG_PREC_FP64);
      for (auto& b : nat->out.b)
        if (!s0.idx.count(b.k)) s0.add(b.k, b.r, b.c);
      s0.finalize();
      told.reset();
    }
    Layout sx = theta_closure(Le, Re, s0, mpo[site], mpo[site + 1], ik[site], ik[site + 1]);
    if (target) {
      TensorP told = theta_form(ctx, *(*target)[site], *(*target)[site + 1], nullptr);
      auto mvs = build_matvec(ctx, *ovL.at(site - 1), *ovR.at(site + 2), layout_of(*told), id0, id1, ik[site],
                              ik[site + 1], &sx, MPSG_PREC_FP64);
      tstate = make_tensor(ctx, 2, sx, true);
      mvs->run(told->d, tstate->d);
    }
    TensorP th = theta_form(ctx, *mps[site], *mps[site + 1], &sx);
    TensorP psi = make_tensor(ctx, 2, sx, true);
    const auto tp1 = std::chrono::steady_clock::now();
    prep_seconds += std::chrono::duration<double>(tp1 - tp0).count();
    // MIXED: the FP64 energy of psi runs on the side stream beside the split (both only read psi)
    EnergyJob energy;
    LanczosResult lr = lanczos_prec(ctx, Le, Re, sx, mpo[site], mpo[site + 1], ik[site], ik[site + 1], *th, *psi,
                                    lanmax, delta, testenergy, reorth, (int)prec, &lst, tstate ? tstate->d : nullptr,
                                    &energy);
    tstate.reset();
    th.reset();
    auto t0 = std::chrono::steady_clock::now();
    lanczos_call_seconds += std::chrono::duration<double>(t0 - tp1).count();
    // the energy matvec is queued once the bidiagonalisation launches are (their clusters are placed
    // first), or after the split when it takes another route
    std::function<void(cudaEvent_t)> hook;
    if (energy.pending())
      hook = [&energy](cudaEvent_t after) {
        if (!energy.launched) energy.launch(after);
      };
    SplitResult sp = split2(ctx, *psi, ik[site], ik[site + 1], chimax, doTrunc, tr_weight, true, dir > 0 ? 1 : -1,
                            nullptr, nullptr, hook);
    ctx->sync();
    auto t1 = std::chrono::steady_clock::now();
    split_seconds += std::chrono::duration<double>(t1 - t0).count();
    if (energy.pending()) {
      lr.E0 = energy.finish();
      const auto t2 = std::chrono::steady_clock::now();
      lanczos_call_seconds += std::chrono::duration<double>(t2 - t1).count();
      t1 = t2;
    }
    psi.reset();
    mps[site] = sp.U;
    mps[site + 1] = sp.Vt;
    lam[site] = sp.lam;
    if (dir > 0) L[site] = env_update(ctx, *L[site - 1], *mps[site], mpo[site], ik[site], 1, &env_flops, nullptr, env_prec);
    else
      R[site + 1] = env_update(ctx, *R[site + 2], *mps[site + 1], mpo[site + 1], ik[site + 1], -1, &env_flops, nullptr,
                               env_prec);
    ctx->sync();
    env_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    StepRec r{site, dir, lr.iterations, sp.chi, lr.E0, sp.tw};
    steps.push_back(r);
    return r;
  }

  double simulate(int maxsteps, double EnConv, int chimax, bool doTrunc, double tr_weight, double delta,
                  bool testenergy) {
    auto t0 = std::chrono::steady_clock::now();
    prepare();
    double globalE = 1e100;
    StepRec out{};
    int step = 0;
    while (true) {
      for (int site = 0; site < N - 2; ++site) out = do_step(site, 1, chimax, doTrunc, tr_weight, delta, testenergy);
      for (int site = N - 2; site > 0; --site) out = do_step(site, -1, chimax, doTrunc, tr_weight, delta, testenergy);
      ++step;
      bool conv = std::fabs(globalE - out.E) < EnConv;
      if (step >= maxsteps) conv = true;
      globalE = out.E;
      if (conv) break;
    }
    out = do_step(0, -1, chimax, doTrunc, tr_weight, delta, testenergy);
    wall += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return out.E;
  }

  // ---------------------------------------------------------------- single-site DMRG
  // SSDMRGengine::doStep (src/container.hpp:865-883): SSLanzcosEngine on site with L[site-1] and
  // R[site+1] (contractSingle, src/MPSfunctions.hpp:857-885), prepareSite "l" (dir > 0, D Vd into the
  // right neighbour) or "r" (dir <= 0, U D into the left neighbour) without truncation, then the
  // environment update.  contractSingle is the two-site matvec with a dummy second site: an identity
  // MPO tensor carrying the right MPO channel and a one-state local space of charge 0, so the
  // grouped matvec, its closure and every Lanczos precision serve the single-site update unchanged.
  StepRec ss_do_step(int site, int dir, double delta, bool testenergy) {
    MPSG_CHECK(site >= 0 && site < N, "site out of range");
    MPSG_CHECK(L.count(site - 1) && R.count(site + 1), "environments missing (single-site)");
    const Tensor& Le = *L[site - 1];
    const Tensor& Re = *R[site + 1];
    const MPO& W1 = mpo[site];
    const MPO W2 = dummy_site_mpo(W1.Dr);
    const ItoKey ikd(1, (Q)0);
    const Tensor& A = *mps[site];
    Layout s0;
    for (auto& b : A.b) s0.add(K2(b.k.q0, b.k.q1, b.k.p0, 0), b.r, b.c);
    s0.finalize();
    Layout sx = theta_closure(Le, Re, s0, W1, W2, ik[site], ikd);
    TensorP th = make_tensor(ctx, 2, sx, true);
    {
      std::vector<CopyOp> ops;
      for (auto& b : A.b) {
        const int j = th->find(K2(b.k.q0, b.k.q1, b.k.p0, 0));
        ops.push_back(CopyOp{A.d + b.off, th->d + th->b[j].off, nullptr, nullptr, b.r, b.c, b.r, b.r, 0, 1.0});
      }
      run_copyops(ctx, ops);
    }
    TensorP psi = make_tensor(ctx, 2, sx, true);
    LanczosResult lr = lanczos_prec(ctx, Le, Re, sx, W1, W2, ik[site], ikd, *th, *psi, lanmax, delta, testenergy,
                                    reorth, (int)prec, &lst);
    th.reset();
    // the ground state as a single-site tensor (every block of the closure)
    Layout l1;
    for (auto& b : psi->b) l1.add(K1(b.k.q0, b.k.q1, b.k.p0), b.r, b.c);
    l1.finalize();
    TensorP a = make_tensor(ctx, 1, l1, false);
    MPSG_CHECK(a->nelem == psi->nelem, "single-site state layout mismatch");
    MPSG_CUDA(cudaMemcpyAsync(a->d, psi->d, sizeof(double) * std::max<int64_t>(psi->nelem, 1), cudaMemcpyDeviceToDevice,
                              ctx->stream));
    psi.reset();
    auto t0 = std::chrono::steady_clock::now();
    mps[site] = a;
    TensorP lamt;
    if (dir > 0) {
      prepare_matrix_l(ctx, mps[site], site + 1 < N ? &mps[site + 1] : nullptr, &lamt, 0.0);
      lam[site] = lamt;
    } else {
      prepare_matrix_r(ctx, site > 0 ? &mps[site - 1] : nullptr, mps[site], &lamt, 0.0);
      lam[site - 1] = lamt;
    }
    ctx->sync();
    auto t1 = std::chrono::steady_clock::now();
    split_seconds += std::chrono::duration<double>(t1 - t0).count();
    if (dir > 0) L[site] = env_update(ctx, *L[site - 1], *mps[site], mpo[site], ik[site], 1, &env_flops);
    else R[site] = env_update(ctx, *R[site + 1], *mps[site], mpo[site], ik[site], -1, &env_flops);
    ctx->sync();
    env_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    int chi = 0;
    if (lamt)
      for (auto& b : lamt->b) chi += b.r;
    StepRec r{site, dir, lr.iterations, chi, lr.E0, 0.0};
    steps.push_back(r);
    return r;
  }

  // SSDMRGengine::simulate (src/container.hpp:886-925): orthonormalize("rl"), computeR(mps, mpo, 1),
  // sweeps 0 .. N-2 right and N-1 .. 1 left until the energy changes by less than EnConv or more than
  // maxsteps sweeps were made (the reference's step > maxsteps test), then doStep(0, -1).
  double ss_simulate(int maxsteps, double EnConv, double delta, bool testenergy) {
    auto t0 = std::chrono::steady_clock::now();
    prepare();
    R[1] = env_update(ctx, *R[2], *mps[1], mpo[1], ik[1], 0, &env_flops);
    double globalE = 1e100;
    StepRec out{};
    int step = 0;
    while (true) {
      for (int site = 0; site < N - 1; ++site) out = ss_do_step(site, 1, delta, testenergy);
      for (int site = N - 1; site > 0; --site) out = ss_do_step(site, -1, delta, testenergy);
      ++step;
      bool conv = std::fabs(globalE - out.E) < EnConv;
      if (step > maxsteps) conv = true;
      globalE = out.E;
      if (conv) break;
    }
    out = ss_do_step(0, -1, delta, testenergy);
    wall += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return out.E;
  }

  // DMRGengine::simulate(mps, delta_ortho, ...) (src/container.hpp:441-570): two-site sweeps whose
  // Lanczos stays orthogonal to the target state `tgt` (e.g. a ground state), giving the lowest state
  // orthogonal to it.  Overlap environments <tgt|engine> are kept left and right of the updated bond.
  // Sweeps 0 .. N-3 right and N-2 .. 1 left (skipping N-2 when leaveoutlast) until |dE| < EnConv or
  // maxsteps sweeps, then the update of bond (0, 1) leftwards.  The reference forms the target's
  // two-site state of that last update from tgt[0] twice (state_oldbasis(mps[site], mps[site])); here
  // it is tgt[0] tgt[1] as in every other update.
  double excited_simulate(const std::vector<TensorP>& tgt, int maxsteps, double EnConv, int chimax, bool doTrunc,
                          double tr_weight, double delta, bool testenergy, bool leaveoutlast) {
    MPSG_CHECK((int)tgt.size() == N, "target state has a different length");
    auto t0 = std::chrono::steady_clock::now();
    prepare();
    target = &tgt;
    ovR.clear();
    ovL.clear();
    try {
      ovR[N] = rmax(ctx, *tgt[N - 1]);
      for (int s = N - 1; s >= 0; --s)
        ovR[s] = env_update(ctx, *ovR[s + 1], *tgt[s], identity_mpo((int)ik[s].size()), ik[s], 0, nullptr,
                            mps[s].get());
      ovL[-1] = lmin(ctx);
      double globalE = 1e100;
      StepRec out{};
      int step = 0;
      while (true) {
        for (int site = 0; site < N - 2; ++site) {
          out = do_step(site, 1, chimax, doTrunc, tr_weight, delta, testenergy);
          ovL[site] = env_update(ctx, *ovL[site - 1], *tgt[site], identity_mpo((int)ik[site].size()), ik[site], 1,
                                 nullptr, mps[site].get());
        }
        for (int site = N - 2; site > 0; --site) {
          if (leaveoutlast && site == N - 2) continue;
          out = do_step(site, -1, chimax, doTrunc, tr_weight, delta, testenergy);
          ovR[site + 1] = env_update(ctx, *ovR[site + 2], *tgt[site + 1], identity_mpo((int)ik[site + 1].size()),
                                     ik[site + 1], -1, nullptr, mps[site + 1].get());
        }
        ++step;
        bool conv = std::fabs(globalE - out.E) < EnConv;
        if (step >= maxsteps) conv = true;
        globalE = out.E;
        if (conv) break;
      }
      out = do_step(0, -1, chimax, doTrunc, tr_weight, delta, testenergy);
      target = nullptr;
      wall += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      return out.E;
    } catch (...) {
      target = nullptr;
      throw;
    }
  }

  double measure_energy() { return measure(mpo); }

  // MPO::measure (src/MPOTypes.hpp:990-1020): left environments through the chain, then the sum of
  // the diagonals of the charge-diagonal blocks.
  double measure(const std::vector<MPO>& W) {
    std::vector<const Tensor*> s;
    for (auto& t : mps) s.push_back(t.get());
    return mpo_expectation(ctx, s, W, ik);
  }
  static double mpo_expectation(Ctx* ctx, const std::vector<const Tensor*>& sites, const std::vector<MPO>& W,
                                const std::vector<ItoKey>& ik) {
    TensorP l = lmin(ctx);
    for (size_t s = 0; s < sites.size(); ++s) l = env_update(ctx, *l, *sites[s], W[s], ik[s], 1, nullptr);
    std::vector<double> h;
    tensor_to_host(*l, h);
    double e = 0;
    int64_t off = 0;
    for (auto& b : l->b) {
      if (b.k.q0 == b.k.q1)
        for (int i = 0; i < std::min(b.r, b.c); ++i) e += h[off + i + (int64_t)i * b.r];
      off += (int64_t)b.r * b.c;
    }
    return e;
  }
  // computeOverlap(a, b) (src/MPSfunctions.hpp:2066-2085): identity MPO layers with a lower and b upper;
  // the value is entry (0,0) of the first block of the last environment (0 if there is none).
  static double overlap(Ctx* ctx, const std::vector<const Tensor*>& a, const std::vector<const Tensor*>& b,
                        const std::vector<ItoKey>& ik) {
    TensorP l = lmin(ctx);
    for (size_t s = 0; s < a.size(); ++s) {
      MPO id;
      id.Dl = id.Dr = 1;
      MPOEntry en;
      en.wl = en.wr = 0;
      for (uint32_t i = 0; i < (uint32_t)ik[s].size(); ++i) en.ops.push_back(OpEl{i, i, 1.0});
      id.e.push_back(en);
      l = env_update(ctx, *l, *a[s], id, ik[s], 1, nullptr, b[s]);
    }
    if (l->b.empty()) return 0.0;
    double v = 0;
    MPSG_CUDA(cudaMemcpyAsync(&v, l->d + l->b[0].off, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    return v;
  }
};

}  // namespace mpsg

struct mpsg_dmrg_s {
  mpsg::Engine* e = nullptr;
};
