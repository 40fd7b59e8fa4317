// Batched ground states of independent chains (many DMRGengine runs, src/container.hpp:292-438, in
// lockstep): at every global step each active chain performs its own next two-site update
// (doStep), and all chains' work of that step goes through the single-chain machinery once, on the
// DIRECT SUM of the chains: chain i's charges are shifted by i << 32 and its MPO channels by the
// sum of the previous chains' MPO dimensions, so the chains' theta, environments and MPO tensors
// form one block-diagonal problem.  One grouped-GEMM (or tcgen05) launch per matvec stage then
// serves every chain, the split batches every chain's charge sectors, and the environment update
// runs once per sweep direction.  What must stay per chain is per chain: the Lanczos reductions
// and scalars (segmented kernels over each chain's contiguous range of the concatenated vectors,
// one tridiagonal solve per chain), the convergence test, the truncation / normalisation of the
// split and the absorbed lambda side.
#include <algorithm>

#include "engine.h"

namespace mpsg {
namespace {

constexpr int kChainShiftBits = 32;
inline Q chain_shift(int i) { return (Q)i << kChainShiftBits; }

// Direct sum of per-chain tensors (chain i: charges + i << 32, p0 + pshift[i]).  Shifting keeps every
// chain's key order and puts chain i after chain i - 1, so the arena is the concatenation of the
// chains' arenas (one device copy per chain).
// `slot` (optional, ascending) puts part i at slot[i] instead of i.
TensorP direct_sum(Ctx* ctx, const std::vector<const Tensor*>& parts, const std::vector<uint32_t>& pshift, int nphys,
                   const std::vector<int>* slot = nullptr) {
  Layout lay;
  for (size_t i = 0; i < parts.size(); ++i)
    for (const Block& b : parts[i]->b) {
      MPSG_CHECK(b.k.q0 < chain_shift(1) && b.k.q1 < chain_shift(1), "charge too large for the chain direct sum");
      const int si = slot ? (*slot)[i] : (int)i;
      MPSG_CHECK(i == 0 || !slot || (*slot)[i] > (*slot)[i - 1], "direct-sum slots must ascend");
      BKey k = b.k;
      k.q0 += chain_shift(si);
      k.q1 += chain_shift(si);
      k.p0 += pshift.empty() ? 0u : pshift[i];
      lay.add(k, b.r, b.c);
    }
  lay.finalize();
  TensorP t = make_tensor(ctx, nphys, lay, false);
  int64_t pre = 0;
  size_t j = 0;
  for (size_t i = 0; i < parts.size(); ++i) {
    const Tensor& p = *parts[i];
    for (const Block& b : p.b) {
      MPSG_CHECK(t->b[j].off == pre + b.off, "direct-sum layout is not the concatenation of the parts");
      ++j;
    }
    MPSG_CHECK(pre + p.nelem <= t->nelem, "direct-sum arena smaller than its parts");
    if (p.nelem > 0)
      MPSG_CUDA(cudaMemcpyAsync(t->d + pre, p.d, sizeof(double) * p.nelem, cudaMemcpyDeviceToDevice, ctx->stream));
    pre += p.nelem;
  }
  return t;
}

// Part i of a direct sum (charges in [i << 32, (i + 1) << 32)), keys shifted back.
TensorP unsum(Ctx* ctx, const Tensor& t, int i, uint32_t pshift) {
  Layout lay;
  int j0 = -1, j1 = -1;
  for (int j = 0; j < (int)t.b.size(); ++j) {
    const Block& b = t.b[j];
    if (b.k.q0 < chain_shift(i) || b.k.q0 >= chain_shift(i + 1)) continue;
    if (j0 < 0) j0 = j;
    j1 = j + 1;
    BKey k = b.k;
    k.q0 -= chain_shift(i);
    k.q1 -= chain_shift(i);
    MPSG_CHECK(k.p0 >= pshift, "direct-sum index below the chain's shift");
    k.p0 -= pshift;
    lay.add(k, b.r, b.c);
  }
  lay.finalize();
  TensorP o = make_tensor(ctx, t.nphys, lay, false);
  if (j0 >= 0) {
    const int64_t off0 = t.b[j0].off;
    for (int j = j0; j < j1; ++j) MPSG_CHECK(o->b[j - j0].off == t.b[j].off - off0, "direct-sum part is not contiguous");
    MPSG_CHECK(off0 + o->nelem <= t.nelem, "direct-sum part outside the arena");
    if (o->nelem > 0)
      MPSG_CUDA(cudaMemcpyAsync(o->d, t.d + off0, sizeof(double) * o->nelem, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return o;
}

// Block-diagonal MPO tensor of the chains' tensors (left channels shifted by offl, right by offr).
MPO mpo_direct_sum(const std::vector<const MPO*>& W, const std::vector<uint32_t>& offl,
                   const std::vector<uint32_t>& offr) {
  MPO m;
  for (size_t i = 0; i < W.size(); ++i) {
    for (const MPOEntry& e : W[i]->e) {
      MPOEntry x = e;
      x.wl += offl[i];
      x.wr += offr[i];
      m.e.push_back(x);
    }
    m.Dl += W[i]->Dl;
    m.Dr += W[i]->Dr;
  }
  return m;
}

struct SegLanczos {
  std::vector<double> E0;
  std::vector<int> iters;
};

// <psi_c|H|psi_c> / <psi_c|psi_c> of every chain c of a direct sum (segments [segoff[c], segoff[c+1])
// of the block-diagonal problem): one matvec, two segmented dot products.
std::vector<double> rayleigh_quotient_seg(Ctx* ctx, MatvecPlan& mv, const Tensor& psi,
                                          const std::vector<int64_t>& segoff, LanczosStats* st) {
  const int C = (int)segoff.size() - 1;
  const int64_t n = psi.nelem;
  cudaStream_t s = ctx->stream;
  auto t0 = std::chrono::steady_clock::now();
  double* w = (double*)ctx->dmalloc(sizeof(double) * (std::max<int64_t>(n, 2) + 2 * (size_t)C));
  double* q = w + std::max<int64_t>(n, 2);
  double* part = (double*)ctx->dmalloc(sizeof(double) * (size_t)C * seg_chunks());
  int64_t* dseg = (int64_t*)ctx->dmalloc(sizeof(int64_t) * (C + 1));
  MPSG_CUDA(cudaMemcpyAsync(dseg, segoff.data(), sizeof(int64_t) * (C + 1), cudaMemcpyHostToDevice, s));
  MPSG_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * std::max<int64_t>(n, 2), s));
  mv.run(psi.d, w);
  launch_sdot(psi.d, w, dseg, C, part, q, 1, s);
  launch_sdot(psi.d, psi.d, dseg, C, part, q + C, 1, s);
  std::vector<double> h(2 * (size_t)C);
  MPSG_CUDA(cudaMemcpyAsync(h.data(), q, sizeof(double) * 2 * C, cudaMemcpyDeviceToHost, s));
  ctx->sync();
  mv.check_error();
  ctx->dfree(w);
  ctx->dfree(part);
  ctx->dfree(dseg);
  if (st) {
    st->matvecs += 1;
    st->matvec_flops += mv.flops;
    st->matvec_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  std::vector<double> E(C, 0.0);
  for (int c = 0; c < C; ++c) E[c] = h[C + c] > 0 ? h[c] / h[C + c] : 0.0;
  return E;
}

// TSLanzcosEngine::simulate (src/lanzcos.hpp:165-278) for every chain of a direct sum at once: the
// same recurrence as the single-chain Lanczos with per-chain scalars, the energy test per chain, and
// a chain that has stopped riding along (its later vectors are never used).
SegLanczos lanczos_seg(Ctx* ctx, MatvecPlan& mv, const Tensor& th_init, Tensor& psi, const std::vector<int64_t>& segoff,
                       int itmax, double delta, bool testenergy, double tol_rel, int ndiag, double stall_rel,
                       LanczosStats* st) {
  const int C = (int)segoff.size() - 1;
  const int64_t n = th_init.nelem;
  MPSG_CHECK(C >= 1 && segoff.back() <= n && psi.nelem == n, "segmented Lanczos: bad segments");
  MPSG_CHECK(itmax >= 1 && itmax <= 1000, "itmax must be in [1, 1000]");
  auto t_start = std::chrono::steady_clock::now();
  cudaStream_t s = ctx->stream;
  const int na = itmax + 2;
  const size_t nsc = (size_t)C * na;
  double* dsc = (double*)ctx->dmalloc(sizeof(double) * nsc * 5);
  double *d_alpha = dsc, *d_beta = dsc + nsc, *d_norm2 = dsc + 2 * nsc, *d_E = dsc + 3 * nsc, *d_z = dsc + 4 * nsc;
  MPSG_CUDA(cudaMemsetAsync(dsc, 0, sizeof(double) * nsc * 5, s));
  double* part = (double*)ctx->dmalloc(sizeof(double) * (size_t)C * seg_chunks());
  int64_t* dseg = (int64_t*)ctx->dmalloc(sizeof(int64_t) * (C + 1));
  MPSG_CUDA(cudaMemcpyAsync(dseg, segoff.data(), sizeof(int64_t) * (C + 1), cudaMemcpyHostToDevice, s));
  int* dn = (int*)ctx->dmalloc(sizeof(int) * (size_t)C * (na + 1));  // n_of arrays, one per checkpoint
  std::vector<double*> V;
  double** dV = (double**)ctx->dmalloc(sizeof(double*) * (size_t)na);
  auto slot = [&](int j) -> double* {
    while ((int)V.size() <= j) {
      double* p = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(n, 2));
      V.push_back(p);
      MPSG_CUDA(cudaMemcpyAsync(dV + (V.size() - 1), &V.back(), sizeof(double*), cudaMemcpyHostToDevice, s));
      ctx->sync();
    }
    return V[j];
  };
  double* w = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(n, 2));
  MPSG_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * std::max<int64_t>(n, 2), s));
  MPSG_CUDA(cudaMemcpyAsync(slot(0), th_init.d, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  launch_sdot(V[0], V[0], dseg, C, part, d_norm2, na, s);
  std::vector<double> h(nsc * 4);
  std::vector<int> n_es(C, 0), hn((size_t)C * (na + 1), 0);
  std::vector<char> done(C, 0);
  std::vector<double> eold(C, 1e100), dE_prev(C, 1e100);
  int it = 0;
  auto any_active = [&]() { return std::find(done.begin(), done.end(), 0) != done.end(); };
  while (any_active()) {
    int ck = it;
    while (!((ck % ndiag == 0 && ck != 0) || ck >= itmax - 1)) ++ck;
    for (int j = it; j <= ck; ++j) {
      slot(j + 1);
      launch_sscale_by_norm(V[j], dseg, C, d_norm2 + j, na, delta, d_beta + j, s);
      mv.run(V[j], w);
      launch_sdot(w, V[j], dseg, C, part, d_alpha + j, na, s);
      if (testenergy && j % ndiag == 0 && j != 0) {
        int* dnj = dn + (size_t)C * (j / ndiag);
        int* hnj = hn.data() + (size_t)C * (j / ndiag);
        for (int c = 0; c < C; ++c) hnj[c] = done[c] ? 0 : j + 1;
        MPSG_CUDA(cudaMemcpyAsync(dnj, hnj, sizeof(int) * C, cudaMemcpyHostToDevice, s));
        launch_tri_lowest_seg(d_alpha, d_beta, dnj, C, j + 1, na, d_E + j / ndiag, na, nullptr, s);
      }
      launch_saxpy3(V[j + 1], w, V[j], j > 0 ? V[j - 1] : nullptr, d_alpha + j, d_beta + j, na, dseg, C, part,
                    d_norm2 + j + 1, s);
    }
    MPSG_CUDA(cudaMemcpyAsync(h.data(), dsc, sizeof(double) * nsc * 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    mv.check_error();
    if (st) {
      st->matvecs += ck - it + 1;
      st->matvec_flops += mv.flops * (ck - it + 1);
    }
    for (int c = 0; c < C; ++c) {
      if (done[c]) continue;
      const double* hnorm = h.data() + 2 * nsc + (size_t)c * na;
      const double* hE = h.data() + 3 * nsc + (size_t)c * na;
      for (int j = it; j <= ck; ++j) {
        const double k = std::sqrt(hnorm[j]);
        if (std::fabs(k) < delta) { n_es[c] = j; done[c] = 1; break; }
        n_es[c] = j + 1;
        if (testenergy && j % ndiag == 0 && j != 0) {
          const double E = hE[j / ndiag], dE = std::fabs(E - eold[c]);
          if (dE < std::max(delta, tol_rel * std::fabs(E))) { done[c] = 1; break; }
          if (stall_rel > 0 && dE < stall_rel * std::fabs(E) && dE > 0.5 * dE_prev[c]) { done[c] = 1; break; }
          dE_prev[c] = dE;
          eold[c] = E;
        }
        if (j + 1 >= itmax) { done[c] = 1; break; }
      }
    }
    it = ck + 1;
  }
  SegLanczos res;
  res.E0.assign(C, 0.0);
  res.iters = n_es;
  int nmax = 0;
  for (int c = 0; c < C; ++c) nmax = std::max(nmax, n_es[c]);
  if (nmax > 0) {
    int* dnf = dn + (size_t)C * na;
    MPSG_CUDA(cudaMemcpyAsync(dnf, n_es.data(), sizeof(int) * C, cudaMemcpyHostToDevice, s));
    launch_tri_lowest_seg(d_alpha, d_beta, dnf, C, nmax, na, d_E + na - 1, na, d_z, s);
    launch_scombine(psi.d, (const double* const*)dV, dnf, d_z, na, dseg, C, s);
    std::vector<double> e(nsc);
    MPSG_CUDA(cudaMemcpyAsync(e.data(), d_E, sizeof(double) * nsc, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    for (int c = 0; c < C; ++c) res.E0[c] = e[(size_t)c * na + na - 1];
  }
  for (double* p : V) ctx->dfree(p);
  ctx->dfree(w);
  ctx->dfree(dV);
  ctx->dfree(dn);
  ctx->dfree(dseg);
  ctx->dfree(part);
  ctx->dfree(dsc);
  ctx->sync();
  if (st) st->seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  return res;
}

}  // namespace

struct BatchEngine {
  Ctx* ctx = nullptr;
  std::shared_ptr<Ctx> keep;
  std::vector<Engine*> ch;  // not owned
  int prec = MPSG_PREC_FP64;
  int lanmax = 500;
  LanczosStats lst;
  int64_t global_steps = 0, chain_steps = 0, matvec_launches = 0;
  double split_seconds = 0, env_seconds = 0, wall = 0, device_seconds = 0, prepare_seconds = 0;

  // the (site, direction) sequence of DMRGengine::simulate with a fixed sweep count
  static std::vector<std::pair<int, int>> schedule(int N, int sweeps) {
    std::vector<std::pair<int, int>> s;
    for (int k = 0; k < sweeps; ++k) {
      for (int site = 0; site < N - 2; ++site) s.push_back({site, 1});
      for (int site = N - 2; site > 0; --site) s.push_back({site, -1});
    }
    s.push_back({0, -1});
    return s;
  }

  // one lockstep step: chain ids `act`, chain act[i] updates bond (site[i], site[i] + 1) in direction dir[i]
  void step(const std::vector<int>& act, const std::vector<int>& site, const std::vector<int>& dir, int chimax,
            bool doTrunc, double tr_weight, double delta, bool testenergy) {
    const int n = (int)act.size();
    std::vector<const Tensor *> Ls, Rs, A1s, A2s;
    std::vector<const MPO *> W1s, W2s;
    std::vector<uint32_t> offl(n), offm(n), offr(n), zero(n, 0u);
    uint32_t ol = 0, om = 0, orr = 0;
    const ItoKey& ik0 = ch[act[0]]->ik[site[0]];
    const ItoKey& ik1 = ch[act[0]]->ik[site[0] + 1];
    for (int i = 0; i < n; ++i) {
      Engine& e = *ch[act[i]];
      const int s = site[i];
      MPSG_CHECK(s >= 0 && s + 1 < e.N, "site out of range");
      MPSG_CHECK(e.L.count(s - 1) && e.R.count(s + 2), "environments missing");
      MPSG_CHECK(e.ik[s] == ik0 && e.ik[s + 1] == ik1, "batched chains need the same local charge map");
      MPSG_CHECK(e.mpo[s].Dr == e.mpo[s + 1].Dl, "MPO bond dimensions of neighbouring sites differ");
      Ls.push_back(e.L[s - 1].get());
      Rs.push_back(e.R[s + 2].get());
      A1s.push_back(e.mps[s].get());
      A2s.push_back(e.mps[s + 1].get());
      W1s.push_back(&e.mpo[s]);
      W2s.push_back(&e.mpo[s + 1]);
      offl[i] = ol;
      offm[i] = om;
      offr[i] = orr;
      ol += e.mpo[s].Dl;
      om += e.mpo[s].Dr;
      orr += e.mpo[s + 1].Dr;
    }
    TensorP Lt = direct_sum(ctx, Ls, offl, 1), Rt = direct_sum(ctx, Rs, offr, 1);
    TensorP A1t = direct_sum(ctx, A1s, zero, 1), A2t = direct_sum(ctx, A2s, zero, 1);
    const MPO W1t = mpo_direct_sum(W1s, offl, offm), W2t = mpo_direct_sum(W2s, offm, offr);
    // theta structure (as the single-chain doStep) and its closure under the matvec
    Layout s0;
    {
      std::map<Q, std::vector<int>> by_left;
      for (int j = 0; j < (int)A2t->b.size(); ++j) by_left[A2t->b[j].k.q0].push_back(j);
      for (auto& a : A1t->b) {
        auto it = by_left.find(a.k.q1);
        if (it == by_left.end()) continue;
        for (int j : it->second) {
          const Block& b = A2t->b[j];
          s0.add(K2(a.k.q0, b.k.q1, a.k.p0, b.k.p0), a.r, b.c);
        }
      }
      s0.finalize();
    }
    Layout sx = theta_closure(*Lt, *Rt, s0, W1t, W2t, ik0, ik1);
    TensorP th = theta_form(ctx, *A1t, *A2t, &sx);
    A1t.reset();
    A2t.reset();
    TensorP psi = make_tensor(ctx, 2, sx, true);
    std::vector<int64_t> segoff(n + 1, sx.nelem);
    {
      int c = 0;
      for (const Block& b : sx.b) {
        const int owner = (int)(b.k.q0 >> kChainShiftBits);
        while (c <= owner) segoff[c++] = b.off;
      }
      while (c < n) segoff[c++] = sx.nelem;
    }
    // Lanczos: FP64, a mixed precision, or AUTO (TF32X3, then the FP64 restart with the energy test
    // every iteration, as the single-chain AUTO)
    SegLanczos lr;
    if (prec == MPSG_PREC_FP64) {
      auto mv = build_matvec(ctx, *Lt, *Rt, sx, W1t, W2t, ik0, ik1, &sx, MPSG_PREC_FP64);
      const int64_t m0 = lst.matvecs;
      lr = lanczos_seg(ctx, *mv, *th, *psi, segoff, lanmax, delta, testenergy, 0.0, 5, 0.0, &lst);
      matvec_launches += (lst.matvecs - m0) * mv->launches_per_run();
    } else {
      const bool two_phase = prec == MPSG_PREC_AUTO || prec == MPSG_PREC_MIXED;
      const int lo = two_phase ? MPSG_PREC_TF32X3 : prec;
      auto mv = build_matvec(ctx, *Lt, *Rt, sx, W1t, W2t, ik0, ik1, &sx, lo);
      int64_t m0 = lst.matvecs;
      lr = lanczos_seg(ctx, *mv, *th, *psi, segoff, lanmax, delta, testenergy, prec_tol(lo), 5, prec_stall(lo), &lst);
      matvec_launches += (lst.matvecs - m0) * mv->launches_per_run();
      // the FP64 phase runs on the FP64 stage tables the tensor-core plan carries (no second plan)
      if (two_phase) mv->use_fp64();
      if (prec == MPSG_PREC_MIXED) {
        // per chain, the FP64 Rayleigh quotient of its mixed-precision ground state (one FP64 matvec
        // of the direct sum serves every chain), as the single-chain MIXED
        m0 = lst.matvecs;
        lr.E0 = rayleigh_quotient_seg(ctx, *mv, *psi, segoff, &lst);
        matvec_launches += (lst.matvecs - m0) * mv->launches_per_run();
      } else if (prec == MPSG_PREC_AUTO) {
        TensorP start = tensor_copy(*psi);
        m0 = lst.matvecs;
        SegLanczos r2 = lanczos_seg(ctx, *mv, *start, *psi, segoff, lanmax, delta, testenergy, 0.0, 1, 0.0, &lst);
        matvec_launches += (lst.matvecs - m0) * mv->launches_per_run();
        for (int i = 0; i < n; ++i) r2.iters[i] += lr.iters[i];
        lr = r2;
      }
    }
    th.reset();
    // split: every chain's sectors in one batch, truncation and lambda side per chain
    auto t0 = std::chrono::steady_clock::now();
    std::vector<Q> segq(n);
    std::vector<int> absorb(n);
    for (int i = 0; i < n; ++i) {
      segq[i] = chain_shift(i);
      absorb[i] = dir[i] > 0 ? 1 : -1;
    }
    SplitResult sp = split2(ctx, *psi, ik0, ik1, chimax, doTrunc, tr_weight, true, 1, &segq, &absorb);
    ctx->sync();
    auto t1 = std::chrono::steady_clock::now();
    split_seconds += std::chrono::duration<double>(t1 - t0).count();
    psi.reset();
    for (int i = 0; i < n; ++i) {
      Engine& e = *ch[act[i]];
      const int s = site[i];
      e.mps[s] = unsum(ctx, *sp.U, i, 0);
      e.mps[s + 1] = unsum(ctx, *sp.Vt, i, 0);
      e.lam[s] = unsum(ctx, *sp.lam, i, 0);
    }
    // environment updates, one direct sum per direction
    for (int d : {1, -1}) {
      std::vector<int> grp;
      for (int i = 0; i < n; ++i)
        if ((dir[i] > 0) == (d > 0)) grp.push_back(i);
      if (grp.empty()) continue;
      std::vector<const Tensor *> envs, As;
      std::vector<const MPO*> Ws;
      for (int i : grp) {
        Engine& e = *ch[act[i]];
        const int s = site[i];
        envs.push_back(d > 0 ? e.L[s - 1].get() : e.R[s + 2].get());
        As.push_back(d > 0 ? e.mps[s].get() : e.mps[s + 1].get());
        Ws.push_back(d > 0 ? &e.mpo[s] : &e.mpo[s + 1]);
      }
      auto out = env_batch(d, envs, As, Ws, d > 0 ? ik0 : ik1);
      for (size_t g = 0; g < grp.size(); ++g) {
        Engine& e = *ch[act[grp[g]]];
        const int s = site[grp[g]];
        if (d > 0) e.L[s] = out[g];
        else e.R[s + 1] = out[g];
      }
    }
    ctx->sync();
    env_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    for (int i = 0; i < n; ++i) {
      StepRec r{site[i], dir[i], lr.iters[i], sp.chi_seg[i], lr.E0[i], sp.tw_seg[i]};
      ch[act[i]]->steps.push_back(r);
    }
    ++global_steps;
    chain_steps += n;
  }

  // Environment updates of several chains at once: item g = (environment, site tensor, MPO tensor),
  // all in direction d (> 0: L, else R); returns the new environments in item order.
  std::vector<TensorP> env_batch(int d, const std::vector<const Tensor*>& envs, const std::vector<const Tensor*>& As,
                                 const std::vector<const MPO*>& Ws, const ItoKey& ik) {
    const size_t n = envs.size();
    std::vector<uint32_t> oin(n), oout(n), zg(n, 0u);
    uint32_t a = 0, b = 0;
    for (size_t g = 0; g < n; ++g) {
      oin[g] = a;  // channel of the incoming environment (left channel for d > 0, right otherwise)
      oout[g] = b;
      a += d > 0 ? Ws[g]->Dl : Ws[g]->Dr;
      b += d > 0 ? Ws[g]->Dr : Ws[g]->Dl;
    }
    TensorP Et = direct_sum(ctx, envs, oin, 1), At = direct_sum(ctx, As, zg, 1);
    const MPO Wt = d > 0 ? mpo_direct_sum(Ws, oin, oout) : mpo_direct_sum(Ws, oout, oin);
    TensorP out = env_update(ctx, *Et, *At, Wt, ik, d > 0 ? 1 : -1, nullptr);
    std::vector<TensorP> res;
    for (size_t g = 0; g < n; ++g) res.push_back(unsum(ctx, *out, (int)g, oout[g]));
    return res;
  }

  // Engine::prepare of every chain, batched: orthonormalize("rl") site by site counted from each
  // chain's right end (prepareMatrix per left-charge group, so the direct sum separates the chains),
  // then the right environments the same way.
  void prepare_all() {
    int K = 0;
    for (Engine* e : ch) K = std::max(K, e->N);
    for (int k = 0; k < K; ++k) {
      std::vector<int> act;
      for (size_t c = 0; c < ch.size(); ++c)
        if (ch[c]->N - 1 - k >= 0) act.push_back((int)c);
      std::vector<const Tensor *> b2, b1;
      std::vector<int> slot1;
      for (size_t i = 0; i < act.size(); ++i) {
        Engine& e = *ch[act[i]];
        const int s = e.N - 1 - k;
        b2.push_back(e.mps[s].get());
        if (s > 0) {
          b1.push_back(e.mps[s - 1].get());
          slot1.push_back((int)i);
        }
      }
      TensorP B2 = direct_sum(ctx, b2, {}, 1);
      TensorP B1 = b1.empty() ? nullptr : direct_sum(ctx, b1, {}, 1, &slot1);
      TensorP lamt;
      prepare_matrix_r(ctx, B1 ? &B1 : nullptr, B2, &lamt, 1e-16);
      for (size_t i = 0; i < act.size(); ++i) {
        Engine& e = *ch[act[i]];
        const int s = e.N - 1 - k;
        e.mps[s] = unsum(ctx, *B2, (int)i, 0);
        if (s > 0) e.mps[s - 1] = unsum(ctx, *B1, (int)i, 0);
        e.lam[s - 1] = unsum(ctx, *lamt, (int)i, 0);
      }
    }
    for (Engine* e : ch) {
      e->R.clear();
      e->R[e->N] = Engine::rmax(ctx, *e->mps[e->N - 1]);
      e->L.clear();
      e->L[-1] = Engine::lmin(ctx);
    }
    for (int k = 0;; ++k) {  // R[s] for s = N-1 .. 2, aligned at the right ends
      std::vector<int> act;
      for (size_t c = 0; c < ch.size(); ++c)
        if (ch[c]->N - 1 - k >= 2) act.push_back((int)c);
      if (act.empty()) break;
      std::vector<const Tensor *> envs, As;
      std::vector<const MPO*> Ws;
      for (int c : act) {
        Engine& e = *ch[c];
        const int s = e.N - 1 - k;
        envs.push_back(e.R[s + 1].get());
        As.push_back(e.mps[s].get());
        Ws.push_back(&e.mpo[s]);
        MPSG_CHECK(e.ik[s] == ch[act[0]]->ik[ch[act[0]]->N - 1 - k], "batched chains need the same local charge map");
      }
      const ItoKey& ik = ch[act[0]]->ik[ch[act[0]]->N - 1 - k];
      auto out = env_batch(-1, envs, As, Ws, ik);
      for (size_t i = 0; i < act.size(); ++i) ch[act[i]]->R[ch[act[i]]->N - 1 - k] = out[i];
    }
    ctx->sync();
  }

  // DMRGengine::simulate for every chain with `sweeps` sweeps (no early stop on EnConv), the final
  // doStep(0, -1) included; energies[c] = the last step's energy of chain c
  void simulate(int sweeps, int chimax, bool doTrunc, double tr_weight, double delta, bool testenergy,
                double* energies) {
    auto t0 = std::chrono::steady_clock::now();
    cudaEvent_t e0, e1;
    MPSG_CUDA(cudaEventCreate(&e0));
    MPSG_CUDA(cudaEventCreate(&e1));
    auto tp = std::chrono::steady_clock::now();
    prepare_all();
    prepare_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - tp).count();
    std::vector<std::vector<std::pair<int, int>>> sch;
    size_t longest = 0;
    for (Engine* e : ch) {
      sch.push_back(schedule(e->N, sweeps));
      longest = std::max(longest, sch.back().size());
    }
    MPSG_CUDA(cudaEventRecord(e0, ctx->stream));
    for (size_t g = 0; g < longest; ++g) {
      std::vector<int> act, site, dir;
      for (size_t c = 0; c < ch.size(); ++c)
        if (g < sch[c].size()) {
          act.push_back((int)c);
          site.push_back(sch[c][g].first);
          dir.push_back(sch[c][g].second);
        }
      step(act, site, dir, chimax, doTrunc, tr_weight, delta, testenergy);
    }
    MPSG_CUDA(cudaEventRecord(e1, ctx->stream));
    MPSG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    device_seconds += ms * 1e-3;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (size_t c = 0; c < ch.size(); ++c) energies[c] = ch[c]->steps.empty() ? 0.0 : ch[c]->steps.back().E;
    wall += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

}  // namespace mpsg

using namespace mpsg;

struct mpsg_batch_s {
  BatchEngine* b = nullptr;
};

extern "C" {

mpsg_status mpsg_batch_create(mpsg_ctx ctx, int32_t nchains, const mpsg_dmrg* chains, mpsg_batch* out) {
  API_BEGIN
  MPSG_CHECK(ctx && chains && out && nchains >= 1, "null argument or no chains");
  MPSG_CHECK(nchains < (1 << 20), "too many chains");
  std::unique_ptr<BatchEngine> b(new BatchEngine());
  b->ctx = C(ctx);
  b->keep = b->ctx->shared_from_this();
  for (int i = 0; i < nchains; ++i) {
    MPSG_CHECK(chains[i] && chains[i]->e, "null chain");
    MPSG_CHECK(chains[i]->e->ctx == b->ctx, "every chain must live on the batch's context");
    for (int j = 0; j < i; ++j) MPSG_CHECK(chains[j]->e != chains[i]->e, "a chain appears twice");
    b->ch.push_back(chains[i]->e);
  }
  *out = new mpsg_batch_s;
  (*out)->b = b.release();
  API_END
}

mpsg_status mpsg_batch_set_options(mpsg_batch b, mpsg_prec prec, int32_t lanmax) {
  API_BEGIN
  MPSG_CHECK(b && b->b, "null batch");
  MPSG_CHECK(prec >= MPSG_PREC_FP64 && prec <= MPSG_PREC_MIXED,
             "batched chains: precision must be FP64, TF32(X3), BF16(X3), AUTO or MIXED");
  MPSG_CHECK(lanmax >= 1 && lanmax <= 1000, "lanmax must be in [1, 1000]");
  b->b->prec = prec;
  b->b->lanmax = lanmax;
  API_END
}

mpsg_status mpsg_batch_simulate(mpsg_batch b, uint32_t sweeps, uint32_t chimax, int32_t doTrunc, double tr_weight,
                                double delta, int32_t testenergy, double* energies) {
  API_BEGIN
  MPSG_CHECK(b && b->b && energies, "null argument");
  MPSG_CHECK(sweeps >= 1, "sweeps < 1");
  b->b->simulate((int)sweeps, (int)chimax, doTrunc != 0, tr_weight, delta, testenergy != 0, energies);
  API_END
}

mpsg_status mpsg_batch_stats(mpsg_batch b, double* st) {
  API_BEGIN
  MPSG_CHECK(b && b->b && st, "null argument");
  const BatchEngine& x = *b->b;
  st[0] = (double)x.global_steps;
  st[1] = (double)x.chain_steps;
  st[2] = (double)x.lst.matvecs;
  st[3] = x.lst.matvec_flops;
  st[4] = (double)x.matvec_launches;
  st[5] = x.lst.seconds;
  st[6] = x.split_seconds;
  st[7] = x.env_seconds;
  st[8] = x.wall;
  st[9] = x.device_seconds;
  st[10] = x.prepare_seconds;
  API_END
}

void mpsg_batch_destroy(mpsg_batch b) {
  if (!b) return;
  try {
    delete b->b;
  } catch (...) {
  }
  delete b;
}

}  // extern "C"
