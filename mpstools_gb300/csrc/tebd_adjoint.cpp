// Adjoint of the second-order TEBD evolution: the gradient of a time-evolved local observable
// O(T) = <psi(T)| O_c |psi(T)> with respect to one parameter theta_b per bond, where theta_b enters the
// bond Hamiltonian h_b (dh_b = d h_b / d theta_b is given by the caller).  The reference has no
// gradient; its TEBD (TEBDengine::simulate, src/container.hpp:1272-1406, with applyGate,
// src/MPSfunctions.hpp:1492-1548) is the forward map that is differentiated.
//
// With psi_T = L_K ... L_1 psi_0 (L_l = the gates G_b of layer l, disjoint bonds) and the gates treated
// as exact (truncation and renormalisation are not differentiated):
//
//   dO/dtheta_b = sum over layers l holding bond b of 2 Re <chi_l| B_b |psi_l>,
//   B_b = (dG_b / dtheta_b) G_b^H,  psi_l = L_l ... L_1 psi_0,  chi_l = L_{l+1}^H ... L_K^H O_c psi_T.
//
// dG_b follows from the eigen-decomposition h_b = V diag(E) V^T (Daleckii-Krein): B_b = V Psi V^T with
// Psi_kl = -i tau (V^T dh_b V)_kl exp(-i tau (E_k - E_l) / 2) sinc(tau (E_k - E_l) / 2).
//
// Host driver: the forward pass keeps the state every `every` layers (checkpoints); the backward pass
// walks the layers in reverse, recomputing the states of one checkpoint segment at a time from its
// checkpoint, evaluates the mixed two-site values <chi|B_b|psi> of the layer, then applies the adjoint
// gates G_b^H to chi (same truncation rule as the forward pass, no renormalisation: chi is linear in
// O_c psi_T).  chi starts as O_c psi_T brought back to Vidal form by identity gates sweeping right from
// the observable's site and then left, which keeps the truncation of the backward state meaningful.
//
// Mixed values on the GPU: with M_s = Gamma_s lambda_s for both states (one planar arena per state),
// the left environments E_L[s + 1](q') = sum M^chi_s(q, q')^H E_L[s](q) M^psi_s(q, q') and the right
// environments E_R[s](q) = sum M^psi_s(q, q') E_R[s + 1](q') M^chi_s(q, q')^H run as one grouped-GEMM
// descriptor set with one ranged launch per stage; then for all bonds of the layer at once:
// Theta^psi = M^psi_b M^psi_{b+1}, Phi = B_b Theta^psi (block linear combination),
// Y = E_L[b] Phi E_R[b + 2], Theta^chi = M^chi_b M^chi_{b+1}, value_b = sum Re <Theta^chi, Y>.
#include <algorithm>

#include "tebd.h"

namespace mpsg {
namespace {

struct State {
  std::vector<TensorP> G, lam;
};
State snapshot(const TebdEngine& e) { return State{e.G, e.lam}; }
void restore(TebdEngine& e, const State& s) {
  e.G = s.G;
  e.lam = s.lam;
}

CGate adjoint_gate(const CGate& g) {
  CGate a = g;
  const int D = g.d1 * g.d2;
  for (int x = 0; x < D; ++x)
    for (int y = 0; y < D; ++y) a.g[x + (size_t)y * D] = std::conj(g.g[y + (size_t)x * D]);
  return a;
}
CGate identity_gate(int d1, int d2) {
  CGate a;
  a.d1 = d1;
  a.d2 = d2;
  const int D = d1 * d2;
  a.g.assign((size_t)D * D, cplx(0, 0));
  for (int x = 0; x < D; ++x) a.g[x + (size_t)x * D] = cplx(1, 0);
  return a;
}

double sinc(double x) { return std::fabs(x) < 1e-4 ? 1.0 - x * x / 6.0 : std::sin(x) / x; }

int64_t round_up(int64_t n) { return (n + kAlign - 1) / kAlign * kAlign; }

// Segments of the complex product op(A) op(B) for the real and the imaginary plane of C.  A and B are
// planar (imaginary plane nA / nB elements after the real one); conj negates an imaginary plane.
void csegs(std::vector<GSegH>& sr, std::vector<GSegH>& si, int bA, int64_t offA, int64_t nA, int lda, int tA, bool cA,
           int bB, int64_t offB, int64_t nB, int ldb, int tB, bool cB, int K) {
  const double sa = cA ? -1.0 : 1.0, sb = cB ? -1.0 : 1.0;
  sr.push_back(GSegH{bA, bB, offA, offB, lda, ldb, K, tA, tB, 1.0});
  sr.push_back(GSegH{bA, bB, offA + nA, offB + nB, lda, ldb, K, tA, tB, -sa * sb});
  si.push_back(GSegH{bA, bB, offA, offB + nB, lda, ldb, K, tA, tB, sb});
  si.push_back(GSegH{bA, bB, offA + nA, offB, lda, ldb, K, tA, tB, sa});
}
void add_cproblem(GemmPlan& g, int bC, int64_t offC, int64_t nC, int M, int N, const std::vector<GSegH>& sr,
                  const std::vector<GSegH>& si) {
  g.add_problem(bC, offC, M, M, N, false, sr);
  g.add_problem(bC, offC + nC, M, M, N, false, si);
}

// Planar complex arena owned by the adjoint (freed on the context's stream).
struct Arena {
  Ctx* ctx = nullptr;
  int64_t nelem = 0;  // real plane length; the imaginary plane follows
  double* d = nullptr;
  void alloc(Ctx* c, int64_t n) {
    ctx = c;
    nelem = std::max<int64_t>(n, kAlign);
    d = (double*)c->dmalloc(sizeof(double) * 2 * nelem);
    MPSG_CUDA(cudaMemsetAsync(d, 0, sizeof(double) * 2 * nelem, c->stream));
  }
  Arena() {}
  Arena(const Arena&) = delete;
  ~Arena() {
    if (d) ctx->dfree(d);
  }
};

// M_s = Gamma_s lambda_s of every site (blocks whose right lambda exists) in one arena.
struct PackedMPS {
  std::vector<std::vector<Block>> b;  // per site; offsets into the arena
  std::vector<std::map<BKey, int>> idx;
  Arena a;
  const Block* find(int s, const BKey& k) const {
    auto it = idx[s].find(k);
    return it == idx[s].end() ? nullptr : &b[s][it->second];
  }
};
void pack_m(TebdEngine& e, const State& st, PackedMPS& P) {
  const int N = e.N;
  P.b.assign(N, {});
  P.idx.assign(N, {});
  int64_t off = 0;
  std::vector<std::vector<int>> src(N);
  for (int s = 0; s < N; ++s) {
    const Tensor& g = *st.G[s];
    for (int i = 0; i < (int)g.b.size(); ++i) {
      if (!e.lam_ptr(*st.lam[s + 1], g.b[i].k.q1, nullptr)) continue;
      Block x = g.b[i];
      x.off = off;
      off += round_up((int64_t)x.r * x.c);
      P.idx[s][x.k] = (int)P.b[s].size();
      P.b[s].push_back(x);
      src[s].push_back(i);
    }
  }
  P.a.alloc(e.ctx, off);
  std::vector<CopyOp> ops;
  for (int s = 0; s < N; ++s) {
    const Tensor& g = *st.G[s];
    for (size_t j = 0; j < P.b[s].size(); ++j) {
      const int i = src[s][j];
      const Block& x = P.b[s][j];
      const double* cs = e.lam_ptr(*st.lam[s + 1], x.k.q1, nullptr);
      ops.push_back(CopyOp{re(g, i), P.a.d + x.off, nullptr, cs, x.r, x.c, x.r, x.r, 0, 1.0});
      ops.push_back(CopyOp{im(g, i), P.a.d + P.a.nelem + x.off, nullptr, cs, x.r, x.c, x.r, x.r, 0, 1.0});
    }
  }
  run_copyops(e.ctx, ops);
}

struct EnvBlock {
  int r = 0, c = 0;
  int64_t off = 0;
};

// sum over bonds b of the layer starting at bond p of Re <chi| B_b |psi> (entry b of the result)
std::vector<double> layer_values(TebdEngine& e, const State& psi, const State& chi, int p, const std::vector<CGate>& B) {
  const int N = e.N;
  Ctx* ctx = e.ctx;
  std::vector<double> out(N - 1, 0.0);
  PackedMPS Pp, Pc;
  pack_m(e, psi, Pp);
  pack_m(e, chi, Pc);
  // ---- environment structure: L[s] (s = 0..N) rows chi, cols psi; R[s] rows psi, cols chi
  std::vector<std::map<Q, EnvBlock>> L(N + 1), R(N + 1);
  MPSG_CHECK(!psi.lam[0]->b.empty() && !psi.lam[N]->b.empty(), "TEBD state without boundary lambdas");
  const Q q0 = psi.lam[0]->b[0].k.q0, qN = psi.lam[N]->b[0].k.q0;
  L[0][q0] = EnvBlock{1, 1, 0};
  R[N][qN] = EnvBlock{1, 1, 0};
  for (int s = 0; s < N; ++s)
    for (const Block& x : Pp.b[s]) {
      const Block* y = Pc.find(s, x.k);
      if (!y || !L[s].count(x.k.q0)) continue;
      auto it = L[s + 1].find(x.k.q1);
      if (it == L[s + 1].end()) L[s + 1][x.k.q1] = EnvBlock{y->c, x.c, 0};
      else MPSG_CHECK(it->second.r == y->c && it->second.c == x.c, "inconsistent bond dimensions");
    }
  for (int s = N - 1; s >= 0; --s)
    for (const Block& x : Pp.b[s]) {
      const Block* y = Pc.find(s, x.k);
      if (!y || !R[s + 1].count(x.k.q1)) continue;
      auto it = R[s].find(x.k.q0);
      if (it == R[s].end()) R[s][x.k.q0] = EnvBlock{x.r, y->r, 0};
      else MPSG_CHECK(it->second.r == x.r && it->second.c == y->r, "inconsistent bond dimensions");
    }
  int64_t eoff = 0;
  for (auto* side : {&L, &R})
    for (auto& m : *side)
      for (auto& kv : m) {
        kv.second.off = eoff;
        eoff += round_up((int64_t)kv.second.r * kv.second.c);
      }
  Arena E;
  E.alloc(ctx, eoff);
  {
    static const double one = 1.0;
    MPSG_CUDA(cudaMemcpyAsync(E.d + L[0][q0].off, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    MPSG_CUDA(cudaMemcpyAsync(E.d + R[N][qN].off, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  }
  // ---- scratch T of stage 1 (left: chi rows x psi cols of M; right: psi rows x chi cols)
  struct TItem {
    int j;  // block of Pp.b[s]
    int64_t off;
    int r, c;
  };
  std::vector<std::vector<TItem>> TL(N), TR(N);
  int64_t toff = 0;
  for (int s = 0; s < N; ++s)
    for (int j = 0; j < (int)Pp.b[s].size(); ++j) {
      const Block& x = Pp.b[s][j];
      const Block* y = Pc.find(s, x.k);
      if (!y) continue;
      auto l = L[s].find(x.k.q0);
      if (l != L[s].end() && L[s + 1].count(x.k.q1)) {
        TL[s].push_back(TItem{j, toff, l->second.r, x.c});
        toff += round_up((int64_t)l->second.r * x.c);
      }
      auto r = R[s + 1].find(x.k.q1);
      if (r != R[s + 1].end() && R[s].count(x.k.q0)) {
        TR[s].push_back(TItem{j, toff, x.r, r->second.c});
        toff += round_up((int64_t)x.r * r->second.c);
      }
    }
  Arena T;
  T.alloc(ctx, toff);
  // ---- environment sweeps: step t = left site t and right site N-1-t; stage 1 then stage 2
  const int64_t nP = Pp.a.nelem, nC = Pc.a.nelem, nE = E.nelem, nT = T.nelem;
  GemmPlan env;
  std::vector<int> mark;
  for (int t = 0; t < N; ++t) {
    const int sl = t, sr = N - 1 - t;
    mark.push_back(env.nprob());
    for (const TItem& ti : TL[sl]) {  // T = E_L(q) M^psi
      const Block& x = Pp.b[sl][ti.j];
      const EnvBlock& el = L[sl].at(x.k.q0);
      MPSG_CHECK(el.c == x.r && el.r == ti.r && x.c == ti.c, "left environment and site tensor dimensions differ");
      std::vector<GSegH> a, b;
      csegs(a, b, 2, el.off, nE, el.r, 0, false, 0, x.off, nP, x.r, 0, false, el.c);
      add_cproblem(env, 3, ti.off, nT, ti.r, ti.c, a, b);
    }
    for (const TItem& ti : TR[sr]) {  // T = M^psi E_R(q')
      const Block& x = Pp.b[sr][ti.j];
      const EnvBlock& er = R[sr + 1].at(x.k.q1);
      MPSG_CHECK(er.r == x.c && x.r == ti.r && er.c == ti.c, "right environment and site tensor dimensions differ");
      std::vector<GSegH> a, b;
      csegs(a, b, 0, x.off, nP, x.r, 0, false, 2, er.off, nE, er.r, 0, false, x.c);
      add_cproblem(env, 3, ti.off, nT, ti.r, ti.c, a, b);
    }
    mark.push_back(env.nprob());
    {  // E_L[sl + 1](q') = sum M^chi^H T
      std::map<Q, std::pair<std::vector<GSegH>, std::vector<GSegH>>> acc;
      for (const TItem& ti : TL[sl]) {
        const Block& x = Pp.b[sl][ti.j];
        const Block* y = Pc.find(sl, x.k);
        const EnvBlock& eo = L[sl + 1].at(x.k.q1);
        MPSG_CHECK(ti.r == y->r && eo.r == y->c && eo.c == ti.c, "left environment update dimensions differ");
        auto& s2 = acc[x.k.q1];
        csegs(s2.first, s2.second, 1, y->off, nC, y->r, 1, true, 3, ti.off, nT, ti.r, 0, false, y->r);
      }
      for (auto& kv : acc) {
        const EnvBlock& eo = L[sl + 1].at(kv.first);
        add_cproblem(env, 2, eo.off, nE, eo.r, eo.c, kv.second.first, kv.second.second);
      }
    }
    {  // E_R[sr](q) = sum T M^chi^H
      std::map<Q, std::pair<std::vector<GSegH>, std::vector<GSegH>>> acc;
      for (const TItem& ti : TR[sr]) {
        const Block& x = Pp.b[sr][ti.j];
        const Block* y = Pc.find(sr, x.k);
        const EnvBlock& eo = R[sr].at(x.k.q0);
        MPSG_CHECK(ti.c == y->c && eo.r == ti.r && eo.c == y->r, "right environment update dimensions differ");
        auto& s2 = acc[x.k.q0];
        csegs(s2.first, s2.second, 3, ti.off, nT, ti.r, 0, false, 1, y->off, nC, y->r, 1, true, y->c);
      }
      for (auto& kv : acc) {
        const EnvBlock& eo = R[sr].at(kv.first);
        add_cproblem(env, 2, eo.off, nE, eo.r, eo.c, kv.second.first, kv.second.second);
      }
    }
  }
  mark.push_back(env.nprob());
  env.upload(ctx);
  {
    const double* bases[8] = {Pp.a.d, Pc.a.d, E.d, T.d, nullptr, nullptr, nullptr, nullptr};
    for (size_t m = 0; m + 1 < mark.size(); ++m) env.run_range(bases, mark[m], mark[m + 1]);
  }
  // ---- bonds of the layer
  struct TK {  // one Theta / Phi / Y block
    int b;
    BKey k;
    int r, c;
    int64_t off;
  };
  std::vector<TK> thp, thc;  // Theta^psi, Theta^chi
  std::map<std::pair<int, BKey>, int> thp_of, thc_of;
  GemmPlan gth;
  int64_t hoff = 0;
  auto theta_of = [&](const PackedMPS& P, int base, int64_t nPl, int b, std::vector<TK>& out,
                      std::map<std::pair<int, BKey>, int>& where,
                      std::map<BKey, std::pair<std::vector<GSegH>, std::vector<GSegH>>>& segs) {
    std::map<Q, std::vector<int>> byleft;
    for (int j = 0; j < (int)P.b[b + 1].size(); ++j) byleft[P.b[b + 1][j].k.q0].push_back(j);
    for (const Block& x : P.b[b]) {
      auto it = byleft.find(x.k.q1);
      if (it == byleft.end()) continue;
      for (int j : it->second) {
        const Block& y = P.b[b + 1][j];
        MPSG_CHECK(y.r == x.c, "neighbouring site tensors differ in bond dimension");
        const BKey k = K2(x.k.q0, y.k.q1, x.k.p0, y.k.p0);
        auto w = where.find({b, k});
        if (w == where.end()) {
          where[{b, k}] = (int)out.size();
          out.push_back(TK{b, k, x.r, y.c, 0});
        }
        auto& s2 = segs[k];
        csegs(s2.first, s2.second, base, x.off, nPl, x.r, 0, false, base, y.off, nPl, y.r, 0, false, x.c);
      }
    }
  };
  std::vector<std::map<BKey, std::pair<std::vector<GSegH>, std::vector<GSegH>>>> sp(N), sc(N);
  for (int b = p; b + 1 < N; b += 2) {
    theta_of(Pp, 0, nP, b, thp, thp_of, sp[b]);
    theta_of(Pc, 1, nC, b, thc, thc_of, sc[b]);
  }
  for (auto* v : {&thp, &thc})
    for (TK& t : *v) {
      t.off = hoff;
      hoff += round_up((int64_t)t.r * t.c);
    }
  Arena TH;
  TH.alloc(ctx, hoff);
  const int64_t nTH = TH.nelem;
  for (const TK& t : thp) {
    auto& s2 = sp[t.b].at(t.k);
    add_cproblem(gth, 4, t.off, nTH, t.r, t.c, s2.first, s2.second);
  }
  for (const TK& t : thc) {
    auto& s2 = sc[t.b].at(t.k);
    add_cproblem(gth, 4, t.off, nTH, t.r, t.c, s2.first, s2.second);
  }
  // Phi = B Theta^psi on the keys that meet Theta^chi and both environments
  std::vector<TK> phi;
  std::vector<std::vector<std::pair<int, cplx>>> phi_terms;
  for (int b = p; b + 1 < N; b += 2) {
    const CGate& g = B[b];
    std::map<BKey, int> made;
    for (const TK& t : thp) {
      if (t.b != b) continue;
      if (!L[b].count(t.k.q0) || !R[b + 2].count(t.k.q1)) continue;
      for (int o2 = 0; o2 < g.d2; ++o2)
        for (int o1 = 0; o1 < g.d1; ++o1) {
          const cplx gv = g.at(o1, o2, (int)t.k.p0, (int)t.k.p1);
          if (gv == cplx(0, 0)) continue;
          const BKey ko = K2(t.k.q0, t.k.q1, (uint32_t)o1, (uint32_t)o2);
          if (!thc_of.count({b, ko})) continue;
          auto it = made.find(ko);
          int id;
          if (it == made.end()) {
            id = (int)phi.size();
            made[ko] = id;
            phi.push_back(TK{b, ko, t.r, t.c, 0});
            phi_terms.emplace_back();
          } else {
            id = it->second;
            MPSG_CHECK(phi[id].r == t.r && phi[id].c == t.c, "two-site blocks of one charge pair differ in shape");
          }
          phi_terms[id].push_back({thp_of.at({b, t.k}), gv});
        }
    }
  }
  int64_t foff = 0, y1off = 0, yoff = 0;
  std::vector<int64_t> y1o(phi.size()), yo(phi.size());
  for (size_t i = 0; i < phi.size(); ++i) {
    TK& f = phi[i];
    f.off = foff;
    foff += round_up((int64_t)f.r * f.c);
    const EnvBlock& el = L[f.b].at(f.k.q0);
    const EnvBlock& er = R[f.b + 2].at(f.k.q1);
    y1o[i] = y1off;
    y1off += round_up((int64_t)el.r * f.c);
    yo[i] = yoff;
    yoff += round_up((int64_t)el.r * er.c);
  }
  Arena PHI, Y1, Y;
  PHI.alloc(ctx, foff);
  Y1.alloc(ctx, y1off);
  Y.alloc(ctx, yoff);
  gth.upload(ctx);
  {
    const double* bases[8] = {Pp.a.d, Pc.a.d, E.d, T.d, TH.d, PHI.d, Y1.d, Y.d};
    gth.run(bases);
  }
  if (!phi.empty()) {
    LincombPlan lp;
    for (size_t i = 0; i < phi.size(); ++i) {
      const TK& f = phi[i];
      const int64_t n = (int64_t)f.r * f.c;
      std::vector<std::pair<const double*, double>> tr, ti;
      for (auto& t : phi_terms[i]) {
        const TK& s = thp[t.first];
        const double* sr = TH.d + s.off;
        const double* si = TH.d + nTH + s.off;
        tr.push_back({sr, t.second.real()});
        tr.push_back({si, -t.second.imag()});
        ti.push_back({si, t.second.real()});
        ti.push_back({sr, t.second.imag()});
      }
      lp.add(PHI.d + f.off, n, tr);
      lp.add(PHI.d + PHI.nelem + f.off, n, ti);
    }
    lp.run(ctx);
    // Y1 = E_L Phi, Y = Y1 E_R
    GemmPlan g1, g2;
    for (size_t i = 0; i < phi.size(); ++i) {
      const TK& f = phi[i];
      const EnvBlock& el = L[f.b].at(f.k.q0);
      const EnvBlock& er = R[f.b + 2].at(f.k.q1);
      MPSG_CHECK(el.c == f.r && er.r == f.c, "environment and two-site block dimensions differ");
      std::vector<GSegH> a, b;
      csegs(a, b, 2, el.off, nE, el.r, 0, false, 5, f.off, PHI.nelem, f.r, 0, false, el.c);
      add_cproblem(g1, 6, y1o[i], Y1.nelem, el.r, f.c, a, b);
      std::vector<GSegH> a2, b2;
      csegs(a2, b2, 6, y1o[i], Y1.nelem, el.r, 0, false, 2, er.off, nE, er.r, 0, false, f.c);
      add_cproblem(g2, 7, yo[i], Y.nelem, el.r, er.c, a2, b2);
    }
    g1.upload(ctx);
    g2.upload(ctx);
    const double* bases[8] = {Pp.a.d, Pc.a.d, E.d, T.d, TH.d, PHI.d, Y1.d, Y.d};
    g1.run(bases);
    g2.run(bases);
    // value_b = sum Re <Theta^chi, Y>
    std::vector<CDotOp> ops;
    std::vector<int> bond_of;
    for (size_t i = 0; i < phi.size(); ++i) {
      const TK& f = phi[i];
      const TK& c = thc[thc_of.at({f.b, f.k})];
      const EnvBlock& el = L[f.b].at(f.k.q0);
      const EnvBlock& er = R[f.b + 2].at(f.k.q1);
      MPSG_CHECK(c.r == el.r && c.c == er.c, "two-site blocks of the two states differ in shape");
      ops.push_back(CDotOp{TH.d + c.off, TH.d + nTH + c.off, Y.d + yo[i], Y.d + Y.nelem + yo[i], (int64_t)c.r * c.c});
      bond_of.push_back(f.b);
    }
    CDotOp* d = (CDotOp*)ctx->dmalloc(sizeof(CDotOp) * ops.size() + sizeof(double) * ops.size());
    double* dout = (double*)(d + ops.size());
    MPSG_CUDA(cudaMemcpyAsync(d, ops.data(), sizeof(CDotOp) * ops.size(), cudaMemcpyHostToDevice, ctx->stream));
    launch_cdot_re(d, (int)ops.size(), dout, ctx->stream);
    std::vector<double> v(ops.size());
    MPSG_CUDA(cudaMemcpyAsync(v.data(), dout, sizeof(double) * ops.size(), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    ctx->dfree(d);
    for (size_t i = 0; i < v.size(); ++i) out[bond_of[i]] += v[i];
  }
  ctx->sync();
  return out;
}

}  // namespace

// B = (dG / dtheta) G^H for G = exp(-i tau h), h = V diag(E) V^T, dh = dh / dtheta (real symmetric).
CGate gate_tangent(const std::vector<double>& H, const std::vector<double>& dh, int d1, int d2, double tau) {
  const int D = d1 * d2;
  MPSG_CHECK((int)H.size() == D * D && (int)dh.size() == D * D, "bond matrices of the wrong size");
  std::vector<double> A = H, V, E;
  jacobi_sym(D, A, V, E);
  std::vector<double> T((size_t)D * D, 0.0), H1((size_t)D * D, 0.0);
  for (int k = 0; k < D; ++k)
    for (int j = 0; j < D; ++j) {
      double s = 0;
      for (int x = 0; x < D; ++x) s += V[x + (size_t)k * D] * dh[x + (size_t)j * D];
      T[k + (size_t)j * D] = s;
    }
  for (int k = 0; k < D; ++k)
    for (int l = 0; l < D; ++l) {
      double s = 0;
      for (int j = 0; j < D; ++j) s += T[k + (size_t)j * D] * V[j + (size_t)l * D];
      H1[k + (size_t)l * D] = s;
    }
  std::vector<cplx> P((size_t)D * D);
  for (int k = 0; k < D; ++k)
    for (int l = 0; l < D; ++l) {
      const double h = 0.5 * tau * (E[k] - E[l]);
      P[k + (size_t)l * D] = cplx(0.0, -tau) * H1[k + (size_t)l * D] * std::exp(cplx(0.0, -h)) * sinc(h);
    }
  CGate B;
  B.d1 = d1;
  B.d2 = d2;
  B.g.assign((size_t)D * D, cplx(0, 0));
  for (int x = 0; x < D; ++x)
    for (int y = 0; y < D; ++y) {
      cplx s(0, 0);
      for (int k = 0; k < D; ++k)
        for (int l = 0; l < D; ++l) s += V[x + (size_t)k * D] * P[k + (size_t)l * D] * V[y + (size_t)l * D];
      B.g[x + (size_t)y * D] = s;
    }
  return B;
}

std::pair<double, std::vector<double>> tebd_adjoint_second_order(TebdEngine& e, int steps, double dt, int chimax,
                                                                 bool doTrunc, double tr_weight, int obs_site,
                                                                 const std::vector<double>& obs,
                                                                 const std::vector<std::vector<double>>& dh, int every) {
  const int N = e.N;
  MPSG_CHECK(steps >= 1, "steps < 1");
  MPSG_CHECK(obs_site >= 0 && obs_site < N, "observable site out of range");
  MPSG_CHECK((int)dh.size() == N - 1, "one bond-Hamiltonian derivative per bond expected");
  auto t0 = std::chrono::steady_clock::now();
  const auto sched = TebdEngine::schedule(steps);
  const int nL = (int)sched.size();
  if (every <= 0) every = std::max(1, (int)std::ceil(std::sqrt((double)nL)));
  const auto full = e.make_gates(dt), half = e.make_gates(dt / 2);
  std::vector<CGate> Bf, Bh, Af, Ah;
  for (int b = 0; b + 1 < N; ++b) {
    const int d1 = (int)e.ik[b].size(), d2 = (int)e.ik[b + 1].size();
    const auto H = bond_hamiltonian(e.mpo[b], e.mpo[b + 1], b, N, d1, d2);
    Bf.push_back(gate_tangent(H, dh[b], d1, d2, dt));
    Bh.push_back(gate_tangent(H, dh[b], d1, d2, dt / 2));
    Af.push_back(adjoint_gate(full[b]));
    Ah.push_back(adjoint_gate(half[b]));
  }
  // forward pass with checkpoints
  std::vector<State> ckpt;
  for (int l = 0; l < nL; ++l) {
    if (l % every == 0) ckpt.push_back(snapshot(e));
    e.slice(sched[l].second ? half : full, sched[l].first, chimax, doTrunc, tr_weight, true);
  }
  const State fin = snapshot(e);
  const double value = e.measure_diag(obs_site, obs);
  // backward state chi = O psi_T in Vidal form
  TebdEngine chi;
  chi.ctx = e.ctx;
  chi.keep = e.keep;
  chi.N = N;
  chi.ik = e.ik;
  chi.mpo = e.mpo;
  chi.G = fin.G;
  chi.lam = fin.lam;
  {
    const Tensor& g = *fin.G[obs_site];
    Layout lay;
    std::vector<int> keepb;
    for (int i = 0; i < (int)g.b.size(); ++i) {
      MPSG_CHECK(g.b[i].k.p0 < obs.size(), "operator smaller than the local space");
      if (obs[g.b[i].k.p0] == 0.0) continue;
      lay.add(g.b[i].k, g.b[i].r, g.b[i].c);
      keepb.push_back(i);
    }
    TensorP o = make_ctensor(e.ctx, g.nphys, lay, false);
    std::vector<CopyOp> ops;
    for (int i : keepb) {
      const int j = o->find(g.b[i].k);
      const Block& b = g.b[i];
      const double w = obs[b.k.p0];
      ops.push_back(CopyOp{re(g, i), re(*o, j), nullptr, nullptr, b.r, b.c, b.r, b.r, 0, w});
      ops.push_back(CopyOp{im(g, i), im(*o, j), nullptr, nullptr, b.r, b.c, b.r, b.r, 0, w});
    }
    run_copyops(e.ctx, ops);
    chi.G[obs_site] = o;
    const int big = 1 << 30;
    for (int b = obs_site; b + 1 < N; ++b)
      chi.apply_gate(b, identity_gate((int)e.ik[b].size(), (int)e.ik[b + 1].size()), big, false, 0.0, false);
    for (int b = obs_site - 1; b >= 0; --b)
      chi.apply_gate(b, identity_gate((int)e.ik[b].size(), (int)e.ik[b + 1].size()), big, false, 0.0, false);
  }
  // backward pass
  std::vector<double> grad(N - 1, 0.0);
  std::vector<State> seg;
  int segk = -1;
  for (int l = nL - 1; l >= 0; --l) {
    const int k = l / every;
    if (k != segk) {
      seg.clear();
      restore(e, ckpt[k]);
      for (int m = k * every; m < std::min((k + 1) * every, nL); ++m) {
        e.slice(sched[m].second ? half : full, sched[m].first, chimax, doTrunc, tr_weight, true);
        seg.push_back(snapshot(e));
      }
      ckpt[k] = State();  // the segment's states are in `seg` now
      segk = k;
    }
    const std::vector<CGate>& B = sched[l].second ? Bh : Bf;
    const std::vector<double> v = layer_values(e, seg[l - k * every], snapshot(chi), sched[l].first, B);
    for (int b = 0; b + 1 < N; ++b) grad[b] += 2.0 * v[b];
    seg[l - k * every] = State();
    chi.slice(sched[l].second ? Ah : Af, sched[l].first, chimax, doTrunc, tr_weight, false);
  }
  restore(e, fin);
  e.ctx->sync();
  e.adjoint_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return {value, grad};
}

}  // namespace mpsg
