// applyMPO (src/MPSfunctions.hpp:2088-2346), compressTwoSite (src/MPSfunctions.hpp:2797-2940), compress
// (src/MPSfunctions.hpp:2349-2510) and compressSingleSite (src/MPSfunctions.hpp:2667-2792).
//
// applyMPO: the exact product W|psi>.  Each MPS block A(a, b; s_in) and each MPO element
// W[wl, wr](s_out <- s_in) = v give a piece v A of the "five-leg" block ((a, wl), (b, wr); s_out).
// New bond charges are propagated from the left: (a, wl) has the charge assigned on the previous bond
// (site 0: the left boundary charge), and (b, wr) gets charge(a, wl) + q(s_out) the first time it
// appears.  On a new bond every charge Q owns a coarse grid over the MPO channels: channel w holds the
// old sector (the pair (b, w) of charge Q) with the largest five-leg size seen for it (smaller pieces
// are zero-padded), channels without a piece have size 0; the new block (Q_l, Q_r; s_out) places the
// piece of channels (wl, wr) at the channels' offsets.  Host planning, device copies (pieces with one
// term copied with their factor, several terms summed by a block linear combination first).
//
// compressTwoSite, compress, compressSingleSite: variational fits of W|psi> (of psi for compress) at
// bond dimension <= chimax; see the functions.  The single-site update is contractSingle, the two-site
// matvec plan with a dummy second site.
#include <algorithm>
#include <cmath>

#include "engine.h"

namespace mpsg {

namespace {

struct PairKey {  // (old charge, MPO channel)
  Q q;
  uint32_t w;
  bool operator<(const PairKey& o) const { return q != o.q ? q < o.q : w < o.w; }
  bool operator==(const PairKey& o) const { return q == o.q && w == o.w; }
};
struct FiveKey {
  PairKey l, r;
  uint32_t s;
  bool operator<(const FiveKey& o) const {
    if (!(l == o.l)) return l < o.l;
    if (!(r == o.r)) return r < o.r;
    return s < o.s;
  }
};
struct Piece {  // sum of v_i * A_i (all of the same shape r x c)
  int r = 0, c = 0;
  std::vector<std::pair<const double*, double>> terms;
};

}  // namespace

std::vector<TensorP> apply_mpo(Ctx* ctx, const std::vector<const Tensor*>& mps, const std::vector<MPO>& W,
                               const std::vector<ItoKey>& ik) {
  const int N = (int)mps.size();
  MPSG_CHECK((int)W.size() == N && (int)ik.size() == N && N >= 1, "applyMPO: sizes differ");
  std::vector<TensorP> out;
  // left side of bond -1: the boundary charge of site 0's blocks with channel 0 ... Dl-1
  std::map<PairKey, Q> qleft;  // (old charge, channel) -> new charge
  std::map<Q, std::vector<int>> size_left;  // new charge -> size per left channel
  {
    MPSG_CHECK(!mps[0]->b.empty(), "applyMPO: empty site tensor");
    const Q q0 = mps[0]->b[0].k.q0;
    for (int w = 0; w < W[0].Dl; ++w) qleft[PairKey{q0, (uint32_t)w}] = q0;  // the reference's reset(ql)
    size_left[q0] = std::vector<int>(W[0].Dl, 1);
  }
  for (int s = 0; s < N; ++s) {
    const Tensor& A = *mps[s];
    const MPO& m = W[s];
    std::map<FiveKey, Piece> five;
    for (const MPOEntry& en : m.e)
      for (const OpEl& op : en.ops)
        for (const Block& b : A.b) {
          if (b.k.p0 != op.in) continue;
          FiveKey k{PairKey{b.k.q0, en.wl}, PairKey{b.k.q1, en.wr}, op.out};
          Piece& p = five[k];
          if (p.terms.empty()) {
            p.r = b.r;
            p.c = b.c;
          }
          MPSG_CHECK(p.r == b.r && p.c == b.c, "applyMPO: five-leg pieces of one key differ in shape");
          p.terms.push_back({A.d + b.off, op.v});
        }
    // right charges (first appearance, in key order) and the largest piece size per (charge, channel)
    std::map<PairKey, Q> qright;
    std::map<Q, std::vector<int>> size_right;
    std::vector<const std::pair<const FiveKey, Piece>*> kept;
    for (const auto& kv : five) {
      auto it = qleft.find(kv.first.l);
      if (it == qleft.end()) continue;  // no charge on the left: dropped (the reference erases them)
      MPSG_CHECK(kv.first.s < ik[s].size(), "applyMPO: operator index outside i_to_key");
      const Q qr = it->second + ik[s][kv.first.s];
      auto jt = qright.find(kv.first.r);
      if (jt == qright.end()) qright[kv.first.r] = qr;
      kept.push_back(&kv);
    }
    for (const auto* kv : kept) {
      const Q qr = qright.at(kv->first.r);
      auto& v = size_right[qr];
      if (v.empty()) v.assign(m.Dr, 0);
      v[kv->first.r.w] = std::max(v[kv->first.r.w], kv->second.c);
    }
    // new blocks (Q_l, Q_r; s_out): coarse grids
    struct NewBlock {
      int rows = 0, cols = 0;
      std::vector<std::pair<const std::pair<const FiveKey, Piece>*, std::pair<int, int>>> parts;  // (piece, (r0, c0))
    };
    std::map<BKey, NewBlock> nb;
    for (const auto* kv : kept) {
      const Q ql = qleft.at(kv->first.l), qr = qright.at(kv->first.r);
      const auto& sl = size_left.at(ql);
      const auto& sr = size_right.at(qr);
      MPSG_CHECK((int)sl.size() == m.Dl, "applyMPO: MPO bond dimensions of neighbouring sites differ");
      const BKey key = K1(ql, qr, kv->first.s);
      NewBlock& B = nb[key];
      if (B.parts.empty()) {
        for (int x : sl) B.rows += x;
        for (int x : sr) B.cols += x;
      }
      int r0 = 0, c0 = 0;
      for (uint32_t w = 0; w < kv->first.l.w; ++w) r0 += sl[w];
      for (uint32_t w = 0; w < kv->first.r.w; ++w) c0 += sr[w];
      MPSG_CHECK(kv->second.r <= sl[kv->first.l.w] && kv->second.c <= sr[kv->first.r.w],
                 "applyMPO: five-leg piece larger than its channel");
      B.parts.push_back({kv, {r0, c0}});
    }
    Layout lay;
    for (auto& kv : nb) lay.add(kv.first, kv.second.rows, kv.second.cols);
    lay.finalize();
    TensorP t = make_tensor(ctx, 1, lay, true);
    // pieces with several terms are summed into a scratch first
    int64_t scratch = 0;
    for (auto& kv : nb)
      for (auto& p : kv.second.parts)
        if (p.first->second.terms.size() > 1) scratch += (int64_t)p.first->second.r * p.first->second.c;
    double* dscr = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(scratch, 2));
    LincombPlan lp;
    std::vector<CopyOp> ops;
    int64_t so = 0;
    for (auto& kv : nb) {
      const Block& tb = t->b[t->find(kv.first)];
      for (auto& p : kv.second.parts) {
        const Piece& pc = p.first->second;
        double* dst = t->d + tb.off + p.second.first + (int64_t)p.second.second * tb.r;
        if (pc.terms.size() == 1) {
          ops.push_back(CopyOp{pc.terms[0].first, dst, nullptr, nullptr, pc.r, pc.c, pc.r, tb.r, 0, pc.terms[0].second});
        } else {
          lp.add(dscr + so, (int64_t)pc.r * pc.c, pc.terms);
          ops.push_back(CopyOp{dscr + so, dst, nullptr, nullptr, pc.r, pc.c, pc.r, tb.r, 0, 1.0});
          so += (int64_t)pc.r * pc.c;
        }
      }
    }
    lp.run(ctx);
    run_copyops(ctx, ops);
    ctx->sync();
    ctx->dfree(dscr);
    out.push_back(t);
    qleft = qright;
    size_left = size_right;
  }
  return out;
}

namespace {

std::vector<const Tensor*> cptrs(const std::vector<TensorP>& v) {
  std::vector<const Tensor*> o;
  for (auto& t : v) o.push_back(t.get());
  return o;
}

// truncate(mps, chimax, delta) (src/MPSfunctions.hpp:1705-1728) on a state whose lambdas are the bond
// Schmidt values: per bond DiagBlockMatrix::truncate(delta, chimax, false) (the split's weight rule),
// then dropDangling: columns of site s and rows of site s+1 beyond the kept count of their sector go.
void truncate_mps(Ctx* ctx, std::vector<TensorP>& mps, std::map<int, TensorP>& lam, int chimax, double delta) {
  const int N = (int)mps.size();
  if (chimax <= 0) return;  // truncate() with chimax 0 leaves the state as it is
  for (int site = 0; site + 1 < N; ++site) {
    const Tensor& l = *lam.at(site);
    std::vector<double> vals;  // the sectors' values back to back (the arena has padding between them)
    tensor_to_host(l, vals);
    const int nS = (int)vals.size();
    std::vector<int32_t> sec_of((size_t)std::max(nS, 1), 0);
    {
      int o = 0;
      for (int i = 0; i < (int)l.b.size(); ++i)
        for (int j = 0; j < l.b[i].r * l.b[i].c; ++j) sec_of[o++] = i;
    }
    int32_t* d = (int32_t*)ctx->dmalloc(sizeof(int32_t) * (3 * (size_t)std::max(nS, 1) + l.b.size() + 1) +
                                        sizeof(double) * ((size_t)std::max(nS, 1) + 8) + 64);
    int32_t* drank = d + std::max(nS, 1);
    int32_t* dcnt = drank + 2 * std::max(nS, 1);
    double* dout = (double*)(((uintptr_t)(dcnt + l.b.size() + 1) + 7) & ~(uintptr_t)7);
    double* dvals = dout + 4;
    MPSG_CUDA(cudaMemcpyAsync(d, sec_of.data(), sizeof(int32_t) * nS, cudaMemcpyHostToDevice, ctx->stream));
    if (nS) MPSG_CUDA(cudaMemcpyAsync(dvals, vals.data(), sizeof(double) * nS, cudaMemcpyHostToDevice, ctx->stream));
    launch_truncate(dvals, nS, d, (int)l.b.size(), chimax, 1, delta, drank, dcnt, dout, ctx->stream);
    std::vector<int32_t> cnt(l.b.size() + 1, 0);
    MPSG_CUDA(cudaMemcpyAsync(cnt.data(), dcnt, sizeof(int32_t) * l.b.size(), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    ctx->dfree(d);
    std::map<Q, int> keep;
    for (size_t i = 0; i < l.b.size(); ++i) keep[l.b[i].k.q0] = cnt[i];
    auto cut = [&](const Tensor& t, bool cols) {
      Layout lay;
      std::vector<std::pair<int, int>> src;
      for (int i = 0; i < (int)t.b.size(); ++i) {
        const Q q = cols ? t.b[i].k.q1 : t.b[i].k.q0;
        auto it = keep.find(q);
        const int k = it == keep.end() ? 0 : it->second;
        if (k <= 0) continue;
        lay.add(t.b[i].k, cols ? t.b[i].r : std::min(k, t.b[i].r), cols ? std::min(k, t.b[i].c) : t.b[i].c);
        src.push_back({i, 0});
      }
      lay.finalize();
      TensorP o = make_tensor(ctx, t.nphys, lay, false);
      std::vector<CopyOp> ops;
      for (auto& sp : src) {
        const Block& b = t.b[sp.first];
        const Block& nbk = o->b[o->find(b.k)];
        ops.push_back(CopyOp{t.d + b.off, o->d + nbk.off, nullptr, nullptr, nbk.r, nbk.c, b.r, nbk.r, 0, 1.0});
      }
      run_copyops(ctx, ops);
      return o;
    };
    mps[site] = cut(*mps[site], true);
    mps[site + 1] = cut(*mps[site + 1], false);
  }
  ctx->sync();
}

// prepareSite(mps, site, "l" / "r", true) (src/MPSTypes.hpp:586-621) without truncation; the last site
// ("l") and site 0 ("r") multiply into the boundary dummies, i.e. the norm is dropped.
TensorP prep_l(Ctx* ctx, std::vector<TensorP>& m, int site) {
  TensorP l;
  prepare_matrix_l(ctx, m[site], site + 1 < (int)m.size() ? &m[site + 1] : nullptr, &l, 0.0);
  return l;
}

TensorP prep_r(Ctx* ctx, std::vector<TensorP>& m, int site) {
  TensorP l;
  prepare_matrix_r(ctx, site > 0 ? &m[site - 1] : nullptr, m[site], &l, 0.0);
  return l;
}

void sweep_lr(Ctx* ctx, std::vector<TensorP>& m, std::map<int, TensorP>& lam) {
  const int N = (int)m.size();
  for (int site = 0; site + 1 < N; ++site) lam[site] = prep_l(ctx, m, site);
  for (int site = N - 1; site > 0; --site) lam[site - 1] = prep_r(ctx, m, site);
}

// contractSingle(out, BL, A, W, BR, itokey) (src/MPSfunctions.hpp:857-885): the two-site matvec plan
// with a dummy second site (identity on W's right channels, one local state of charge 0); the output
// holds every block the contraction reaches.
TensorP contract_single(Ctx* ctx, const Tensor& BL, const Tensor& BR, const Tensor& A, const MPO& W, const ItoKey& ik) {
  const MPO W2 = Engine::dummy_site_mpo(W.Dr);
  const ItoKey ikd(1, (Q)0);
  Layout s0;
  for (auto& b : A.b) s0.add(K2(b.k.q0, b.k.q1, b.k.p0, 0), b.r, b.c);
  s0.finalize();
  TensorP th = make_tensor(ctx, 2, s0, true);
  std::vector<CopyOp> ops;
  for (auto& b : A.b) {
    const Block& t = th->b[th->find(K2(b.k.q0, b.k.q1, b.k.p0, 0))];
    ops.push_back(CopyOp{A.d + b.off, th->d + t.off, nullptr, nullptr, b.r, b.c, b.r, t.r, 0, 1.0});
  }
  run_copyops(ctx, ops);
  auto mv = build_matvec(ctx, BL, BR, s0, W, W2, ik, ikd, nullptr, MPSG_PREC_FP64);
  TensorP o2 = make_tensor(ctx, 2, mv->out, true);
  mv->run(th->d, o2->d);
  Layout l1;
  for (auto& b : o2->b) l1.add(K1(b.k.q0, b.k.q1, b.k.p0), b.r, b.c);
  l1.finalize();
  TensorP o = make_tensor(ctx, 1, l1, false);
  ops.clear();
  for (auto& b : o2->b) {
    const Block& t = o->b[o->find(K1(b.k.q0, b.k.q1, b.k.p0))];
    ops.push_back(CopyOp{o2->d + b.off, o->d + t.off, nullptr, nullptr, b.r, b.c, b.r, t.r, 0, 1.0});
  }
  run_copyops(ctx, ops);
  ctx->sync();
  return o;
}

// The sweeps shared by compress and compressSingleSite (src/MPSfunctions.hpp:2397-2468, 2715-2777):
// environments <mps| W |comp> (mps lower, the fit upper), sites 0 .. N-2 right (contractSingle,
// prepareSite "l") and N-1 .. 1 left (contractSingle, prepareSite "r"); after each sweep
// conv = (n1^2 + n2^2 - 2 |<comp|mps>|) / n1^2; stop when conv grows, after maxstep sweeps or when
// |conv| < delta.  Leaves the environments in BL / BR.
void single_site_fit(Ctx* ctx, const std::vector<TensorP>& mps, std::vector<TensorP>& comp, const std::vector<MPO>& W,
                     const std::vector<ItoKey>& ik, double n1, int maxstep, double delta, std::map<int, TensorP>& BL,
                     std::map<int, TensorP>& BR) {
  const int N = (int)mps.size();
  BL[-1] = Engine::lmin(ctx);
  BR[N] = Engine::rmax(ctx, *mps[N - 1]);
  bool converged = maxstep == 0;
  if (!converged)
    for (int site = N - 1; site > 0; --site)
      BR[site] = env_update(ctx, *BR[site + 1], *mps[site], W[site], ik[site], -1, nullptr, comp[site].get());
  double conv_old = 1.0;
  int step = 1;
  while (!converged) {
    for (int site = 0; site < N - 1; ++site) {
      comp[site] = contract_single(ctx, *BL[site - 1], *BR[site + 1], *mps[site], W[site], ik[site]);
      prep_l(ctx, comp, site);
      BL[site] = env_update(ctx, *BL[site - 1], *mps[site], W[site], ik[site], 1, nullptr, comp[site].get());
    }
    for (int site = N - 1; site > 0; --site) {
      comp[site] = contract_single(ctx, *BL[site - 1], *BR[site + 1], *mps[site], W[site], ik[site]);
      prep_r(ctx, comp, site);
      BR[site] = env_update(ctx, *BR[site + 1], *mps[site], W[site], ik[site], -1, nullptr, comp[site].get());
    }
    const double n2 = std::sqrt(Engine::overlap(ctx, cptrs(comp), cptrs(comp), ik));
    const double conv =
        (n1 * n1 + n2 * n2 - 2 * std::fabs(Engine::overlap(ctx, cptrs(comp), cptrs(mps), ik))) / (n1 * n1);
    if (conv_old < conv) break;
    conv_old = conv;
    if (step >= maxstep || std::fabs(conv) < delta) converged = true;
    ++step;
  }
}

double conv_measure(Ctx* ctx, const std::vector<TensorP>& comp, const std::vector<TensorP>& mps,
                    const std::vector<ItoKey>& ik, double n1) {
  const double n2 = std::sqrt(Engine::overlap(ctx, cptrs(comp), cptrs(comp), ik));
  return (n1 * n1 + n2 * n2 - 2 * std::fabs(Engine::overlap(ctx, cptrs(comp), cptrs(mps), ik))) / (n1 * n1);
}

}  // namespace

// compressTwoSite(mps, mpo, chimax, maxstep, delta, doTrunc, tr_weight): the variational two-site fit
// of W|psi> at bond dimension <= chimax.  n1 = |W psi| from the exact product; the initial guess is W
// applied to psi truncated to chimax / D (D = the MPO's bond dimension at site 1) after a left and a
// right canonicalisation sweep, itself canonicalised; the right environments <psi| W |fit> (psi lower,
// the fit upper); then sweeps 0 .. N-3 right and N-2 .. 1 left, each update the two-site
// contractTwosite of psi's sites with the environments, split without normalisation (lambda into the
// right site going right, into the left site going left).  After each sweep conv = (n1^2 + n2^2 -
// 2 |<fit|psi>|) / n1^2 with n2 = |fit|, as the reference computes it (its overlap term is with psi,
// not W psi); the sweeps stop when conv grows, after maxstep sweeps or when |conv| < delta.  Returns
// conv and replaces mps by the fit.
double compress_two_site(Ctx* ctx, std::vector<TensorP>& mps, const std::vector<MPO>& W, const std::vector<ItoKey>& ik,
                         int chimax, int maxstep, double delta, bool doTrunc, double tr_weight) {
  const int N = (int)mps.size();
  MPSG_CHECK(N >= 3 && (int)W.size() == N && (int)ik.size() == N, "compress: sizes differ");
  double n1;
  {
    auto full = apply_mpo(ctx, cptrs(mps), W, ik);
    n1 = std::sqrt(Engine::overlap(ctx, cptrs(full), cptrs(full), ik));
  }
  std::vector<TensorP> tmps;
  for (auto& t : mps) tmps.push_back(tensor_copy(*t));
  std::map<int, TensorP> lam;
  sweep_lr(ctx, tmps, lam);
  const int chi = (int)std::floor((double)chimax / (double)W[1].Dr);
  truncate_mps(ctx, tmps, lam, chi, delta);
  std::vector<TensorP> comp = apply_mpo(ctx, cptrs(tmps), W, ik);
  tmps.clear();
  std::map<int, TensorP> lamc;
  sweep_lr(ctx, comp, lamc);
  std::map<int, TensorP> BL, BR;
  BL[-1] = Engine::lmin(ctx);
  BR[N] = Engine::rmax(ctx, *mps[N - 1]);
  bool converged = maxstep == 0;
  if (!converged)
    for (int site = N - 1; site > 1; --site)
      BR[site] = env_update(ctx, *BR[site + 1], *mps[site], W[site], ik[site], -1, nullptr, comp[site].get());
  auto fit = [&](int site) {
    TensorP in = theta_form(ctx, *mps[site], *mps[site + 1], nullptr);
    auto mv = build_matvec(ctx, *BL.at(site - 1), *BR.at(site + 2), layout_of(*in), W[site], W[site + 1], ik[site],
                           ik[site + 1], nullptr, MPSG_PREC_FP64);
    TensorP out = make_tensor(ctx, 2, mv->out, true);
    mv->run(in->d, out->d);
    return out;
  };
  double conv = 0, conv_old = 1.0;
  int step = 1;
  while (!converged) {
    for (int site = 0; site < N - 2; ++site) {
      TensorP out = fit(site);
      SplitResult sp = split2(ctx, *out, ik[site], ik[site + 1], chimax, doTrunc, tr_weight, false, 1);
      comp[site] = sp.U;
      comp[site + 1] = sp.Vt;
      BL[site] = env_update(ctx, *BL[site - 1], *mps[site], W[site], ik[site], 1, nullptr, comp[site].get());
    }
    for (int site = N - 2; site > 0; --site) {
      TensorP out = fit(site);
      SplitResult sp = split2(ctx, *out, ik[site], ik[site + 1], chimax, doTrunc, tr_weight, false, -1);
      comp[site] = sp.U;
      comp[site + 1] = sp.Vt;
      BR[site + 1] = env_update(ctx, *BR[site + 2], *mps[site + 1], W[site + 1], ik[site + 1], -1, nullptr,
                                comp[site + 1].get());
    }
    const double n2 = std::sqrt(Engine::overlap(ctx, cptrs(comp), cptrs(comp), ik));
    conv = (n1 * n1 + n2 * n2 - 2 * std::fabs(Engine::overlap(ctx, cptrs(comp), cptrs(mps), ik))) / (n1 * n1);
    if (conv_old < conv) break;
    conv_old = conv;
    if (step >= maxstep || std::fabs(conv) < delta) converged = true;
    ++step;
  }
  conv = conv_measure(ctx, comp, mps, ik, n1);
  mps = comp;
  return conv;
}

// compress(mps, chimax, maxstep, delta, verbose, normalize) (src/MPSfunctions.hpp:2349-2510): variational
// single-site compression of psi to bond dimension <= chimax.  psi is swept with prepareSite "l" over
// 0 .. Nmax-1 and "r" over Nmax-1 .. Nmin (Nmax = N-1, Nmin = 1; with normalize N and 0, which drops the
// norm into the boundary dummies); the initial guess is psi truncated to chimax with the lambdas of
// those sweeps, itself swept l and r; the fit sweeps with the identity MPO; then site 0 is fitted once
// more and the fit swept l and r.  conv = |fit - psi|^2 / |psi|^2.  Replaces mps by the fit.
// maxstep = 0 is rejected: the reference's last-site update then reads an environment it never built.
double compress(Ctx* ctx, std::vector<TensorP>& mps, const std::vector<ItoKey>& ik, int chimax, int maxstep,
                double delta, bool normalize) {
  const int N = (int)mps.size();
  MPSG_CHECK(N >= 3 && (int)ik.size() == N, "compress: sizes differ");
  MPSG_CHECK(maxstep >= 1, "compress: maxstep must be at least 1");
  const int nmin = normalize ? 0 : 1, nmax = normalize ? N : N - 1;
  std::map<int, TensorP> lam;
  for (int site = 0; site < nmax; ++site) lam[site] = prep_l(ctx, mps, site);
  for (int site = nmax - 1; site >= nmin; --site) lam[site - 1] = prep_r(ctx, mps, site);
  std::vector<TensorP> comp;
  for (auto& t : mps) comp.push_back(tensor_copy(*t));
  truncate_mps(ctx, comp, lam, chimax, delta);
  std::map<int, TensorP> lamc;
  sweep_lr(ctx, comp, lamc);
  const double n1 = std::sqrt(Engine::overlap(ctx, cptrs(mps), cptrs(mps), ik));
  std::vector<MPO> id;
  for (int s = 0; s < N; ++s) id.push_back(Engine::identity_mpo((int)ik[s].size()));
  std::map<int, TensorP> BL, BR;
  single_site_fit(ctx, mps, comp, id, ik, n1, maxstep, delta, BL, BR);
  comp[0] = contract_single(ctx, *BL[-1], *BR[1], *mps[0], id[0], ik[0]);
  sweep_lr(ctx, comp, lamc);
  const double conv = conv_measure(ctx, comp, mps, ik, n1);
  mps = comp;
  return conv;
}

// compressSingleSite(mps, mpo, chimax, maxstep, delta) (src/MPSfunctions.hpp:2667-2792): variational
// single-site fit of W|psi>.  n1 = |W psi| from the exact product; the initial guess is W applied to psi
// truncated to chimax / D (D = the MPO's right bond dimension at site 1) after an l and an r sweep,
// itself swept l and r; conv as compressTwoSite computes it (the overlap term with psi).  Replaces mps by
// the fit.
double compress_single_site(Ctx* ctx, std::vector<TensorP>& mps, const std::vector<MPO>& W,
                            const std::vector<ItoKey>& ik, int chimax, int maxstep, double delta) {
  const int N = (int)mps.size();
  MPSG_CHECK(N >= 3 && (int)W.size() == N && (int)ik.size() == N, "compress: sizes differ");
  double n1;
  {
    auto full = apply_mpo(ctx, cptrs(mps), W, ik);
    n1 = std::sqrt(Engine::overlap(ctx, cptrs(full), cptrs(full), ik));
  }
  std::vector<TensorP> tmps;
  for (auto& t : mps) tmps.push_back(tensor_copy(*t));
  std::map<int, TensorP> lam;
  sweep_lr(ctx, tmps, lam);
  truncate_mps(ctx, tmps, lam, (int)std::floor((double)chimax / (double)W[1].Dr), delta);
  std::vector<TensorP> comp = apply_mpo(ctx, cptrs(tmps), W, ik);
  tmps.clear();
  std::map<int, TensorP> lamc;
  sweep_lr(ctx, comp, lamc);
  std::map<int, TensorP> BL, BR;
  single_site_fit(ctx, mps, comp, W, ik, n1, maxstep, delta, BL, BR);
  const double conv = conv_measure(ctx, comp, mps, ik, n1);
  mps = comp;
  return conv;
}

}  // namespace mpsg

using namespace mpsg;

extern "C" {

static void sites_in(int32_t N, const mpsg_tensor* sites, const mpsg_mpo* W, const mpsg_itokey* ik,
                     std::vector<TensorP>& m, std::vector<MPO>& w, std::vector<ItoKey>& k) {
  for (int i = 0; i < N; ++i) {
    MPSG_CHECK(sites[i] && T(sites[i]).nphys == 1, "MPS site tensors must have one physical index");
    m.push_back(tensor_copy(T(sites[i])));
    w.push_back(mpo_from_c(&W[i]));
    k.push_back(itokey_from_c(&ik[i]));
  }
}

mpsg_status mpsg_apply_mpo(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* W, const mpsg_itokey* ik,
                           mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(ctx && sites && W && ik && out && N >= 1, "null argument");
  std::vector<TensorP> m;
  std::vector<MPO> w;
  std::vector<ItoKey> k;
  sites_in(N, sites, W, ik, m, w, k);
  std::vector<const Tensor*> p;
  for (auto& t : m) p.push_back(t.get());
  auto r = apply_mpo(C(ctx), p, w, k);
  for (int i = 0; i < N; ++i) out[i] = wrap(r[i]);
  API_END
}

mpsg_status mpsg_compress_two_site(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* W,
                                   const mpsg_itokey* ik, uint32_t chimax, uint32_t maxstep, double delta,
                                   int32_t doTrunc, double tr_weight, mpsg_tensor* out, double* conv) {
  API_BEGIN
  MPSG_CHECK(ctx && sites && W && ik && out && conv, "null argument");
  std::vector<TensorP> m;
  std::vector<MPO> w;
  std::vector<ItoKey> k;
  sites_in(N, sites, W, ik, m, w, k);
  *conv = compress_two_site(C(ctx), m, w, k, (int)chimax, (int)maxstep, delta, doTrunc != 0, tr_weight);
  for (int i = 0; i < N; ++i) out[i] = wrap(m[i]);
  API_END
}

mpsg_status mpsg_compress(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_itokey* ik, uint32_t chimax,
                          uint32_t maxstep, double delta, int32_t normalize, mpsg_tensor* out, double* conv) {
  API_BEGIN
  MPSG_CHECK(ctx && sites && ik && out && conv && N >= 1, "null argument");
  std::vector<TensorP> m;
  std::vector<ItoKey> k;
  for (int i = 0; i < N; ++i) {
    MPSG_CHECK(sites[i] && T(sites[i]).nphys == 1, "MPS site tensors must have one physical index");
    m.push_back(tensor_copy(T(sites[i])));
    k.push_back(itokey_from_c(&ik[i]));
  }
  *conv = compress(C(ctx), m, k, (int)chimax, (int)maxstep, delta, normalize != 0);
  for (int i = 0; i < N; ++i) out[i] = wrap(m[i]);
  API_END
}

mpsg_status mpsg_compress_single_site(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* W,
                                      const mpsg_itokey* ik, uint32_t chimax, uint32_t maxstep, double delta,
                                      mpsg_tensor* out, double* conv) {
  API_BEGIN
  MPSG_CHECK(ctx && sites && W && ik && out && conv && N >= 1, "null argument");
  std::vector<TensorP> m;
  std::vector<MPO> w;
  std::vector<ItoKey> k;
  sites_in(N, sites, W, ik, m, w, k);
  *conv = compress_single_site(C(ctx), m, w, k, (int)chimax, (int)maxstep, delta);
  for (int i = 0; i < N; ++i) out[i] = wrap(m[i]);
  API_END
}

}  // extern "C"
