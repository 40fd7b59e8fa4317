// Host orchestration of the DMRG hot path: matvec / environment / theta plans, split with
// global truncation, right canonicalisation and the GPU Lanczos driver.
#include "host_ops.h"

#include <limits>
#include <mutex>
#include <queue>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <atomic>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <set>
#include <thread>
#include <tuple>

namespace mpsg {

static std::atomic<int64_t> g_split_fallbacks{0};
// MPSG_SPLIT_TIMING=1: split2 records events at its stage boundaries on the context's stream (after
// the worker streams have been joined) and prints the stage times to stderr
static thread_local std::vector<std::pair<const char*, cudaEvent_t>>* g_split_marks = nullptr;
static void split_mark(Ctx* ctx, const char* name) {
  if (!g_split_marks) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, ctx->stream);
  g_split_marks->push_back({name, e});
}
int64_t split_fallback_count() { return g_split_fallbacks.load(); }

static inline Q qat(const ItoKey& ik, uint32_t s) {
  MPSG_CHECK(s < ik.size(), "physical index outside itokey");
  return ik[s];
}

// ============================================================================ matvec
// Visits every term of the reference's doContraction loop (src/MPSfunctions.hpp:726-804):
// (L block i, W1 entry e1, W2 entry e2, op elements o1, o2, theta block, R block).
template <class F>
static void visit_matvec_terms(const Tensor& L, const Tensor& R, const Layout& th, const MPO& W1, const MPO& W2,
                               const ItoKey& ik0, const ItoKey& ik1, F&& f) {
  std::map<uint32_t, std::vector<int>> w2_by_wl;
  for (int e2 = 0; e2 < (int)W2.e.size(); ++e2) w2_by_wl[W2.e[e2].wl].push_back(e2);
  for (int i = 0; i < (int)L.b.size(); ++i) {
    const Block& lb = L.b[i];
    const Q a1 = lb.k.q0, a = lb.k.q1;
    for (int e1 = 0; e1 < (int)W1.e.size(); ++e1) {
      if (W1.e[e1].wl != lb.k.p0) continue;
      const uint32_t wm = W1.e[e1].wr;
      auto it2 = w2_by_wl.find(wm);
      if (it2 == w2_by_wl.end()) continue;
      for (int e2 : it2->second) {
        const uint32_t wr = W2.e[e2].wr;
        for (int o1 = 0; o1 < (int)W1.e[e1].ops.size(); ++o1) {
          const OpEl& op1 = W1.e[e1].ops[o1];
          for (int o2 = 0; o2 < (int)W2.e[e2].ops.size(); ++o2) {
            const OpEl& op2 = W2.e[e2].ops[o2];
            const Q b = a + qat(ik0, op1.out) + qat(ik1, op2.out);
            auto ti = th.idx.find(K2(a, b, op1.out, op2.out));
            if (ti == th.idx.end()) continue;
            const Q b1 = a1 + qat(ik0, op1.in) + qat(ik1, op2.in);
            const int rj = R.find(K1(b1, b, wr));
            if (rj < 0) continue;
            f(i, e1, o1, e2, o2, ti->second, rj, a1, a, b, b1, wm, op1, op2);
          }
        }
      }
    }
  }
}

Layout theta_closure(const Tensor& L, const Tensor& R, const Layout& th0, const MPO& W1, const MPO& W2,
                     const ItoKey& ik0, const ItoKey& ik1) {
  Layout cur = th0;
  cur.finalize();
  for (int iter = 0; iter < 64; ++iter) {
    std::map<BKey, std::pair<int, int>> add;
    visit_matvec_terms(L, R, cur, W1, W2, ik0, ik1,
                       [&](int i, int, int, int, int, int, int rj, Q a1, Q, Q, Q b1, uint32_t, const OpEl& op1,
                           const OpEl& op2) {
                         BKey k = K2(a1, b1, op1.in, op2.in);
                         if (!cur.idx.count(k)) add[k] = {L.b[i].r, R.b[rj].r};
                       });
    if (add.empty()) return cur;
    for (auto& x : add) cur.add(x.first, x.second.first, x.second.second);
    cur.finalize();
  }
  throw Err(1, "theta block closure did not terminate");
}

MatvecPlan::~MatvecPlan() {
  if (ctx) {
    ctx->dfree(dLt);
    ctx->dfree(dRt);
    ctx->dfree(dX);
    for (int i = 0; i < 4; ++i) ctx->dfree(dimg[i]);
    for (int i = 0; i < 2; ++i) {
      ctx->dfree(dprob[i]);
      ctx->dfree(dseg[i]);
      ctx->dfree(dtile[i]);
    }
    ctx->dfree(dconv_theta);
    ctx->dfree(derr);
  }
}

static TcBases tc_bases(MatvecPlan& P, const double* theta_in, double* theta_out) {
  TcBases B;
  for (int i = 0; i < 6; ++i) {
    B.img[i] = nullptr;
    B.lo_off[i] = 0;
    B.f64[i] = nullptr;
  }
  for (int i = 0; i < 4; ++i) {
    B.img[i] = P.dimg[i];
    B.lo_off[i] = P.img_hi[i];
  }
  B.f64[0] = const_cast<double*>(theta_in);
  B.f64[1] = theta_out;
  B.f64[2] = P.dLt;
  B.f64[3] = P.dRt;
  B.err = P.derr;
  return B;
}

void MatvecPlan::use_fp64() {
  if (!dX) dX = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(xa.nelem, 2));
  fp64 = true;
}

void MatvecPlan::run(const double* theta_in, double* theta_out) {
  if (prec == MPSG_PREC_FP64 || fp64) {
    const double* bases[8] = {dLt, theta_in, dX, dRt, theta_out, nullptr, nullptr, nullptr};
    stageA.run(bases);
    stageC.run(bases);
    return;
  }
  const TcBases B = tc_bases(*this, theta_in, theta_out);
  launch_tc_convert(kind, nprod == 3 ? 2 : 1, dconv_theta, nconv_theta, nimg_theta, B, ctx->stream);
  launch_tc_gemm(kind, nprod, dprob[0], dseg[0], dtile[0], ntile[0], B, nsm, ctx->stream, tgrid[0]);
  launch_tc_gemm(kind, nprod, dprob[1], dseg[1], dtile[1], ntile[1], B, nsm, ctx->stream, tgrid[1]);
}

void MatvecPlan::check_error() {
  if (!derr) return;
  int e = 0;
  MPSG_CUDA(cudaMemcpyAsync(&e, derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  ctx->sync();
  if (e) throw Err(5, "tensor-core matvec: a bounded device wait expired (code " + std::to_string(e) + ")");
}

// Tile-image arenas, conversion ops and tcgen05 work lists of the mixed-precision matvec.
template <class K>
static int64_t add_images(std::map<K, int64_t>& off, const K& key, int rows, int cols, int KC, int64_t& total) {
  auto it = off.find(key);
  if (it != off.end()) return it->second;
  const int64_t nimg = (int64_t)((rows + 127) / 128) * ((cols + KC - 1) / KC);
  off[key] = total;
  total += nimg * 16384;
  return off[key];
}

// ---- block schedules of the tcgen05 stages and their autotuner
static std::atomic<int64_t> g_tc_tuned{0}, g_tc_hits{0};
void tc_autotune_counts(int64_t* tuned, int64_t* cache_hits) {
  if (tuned) *tuned = g_tc_tuned.load();
  if (cache_hits) *cache_hits = g_tc_hits.load();
}
static std::atomic<int32_t> g_tc_last[2] = {{-1}, {-1}};
static std::mutex g_tc_ms_mu;
static float g_tc_ms[6] = {-1, -1, -1, -1, -1, -1};
void tc_last_schedules(int32_t* sched2, float* timing6) {
  sched2[0] = g_tc_last[0].load();
  sched2[1] = g_tc_last[1].load();
  if (timing6) {
    std::lock_guard<std::mutex> g(g_tc_ms_mu);
    for (int i = 0; i < 6; ++i) timing6[i] = g_tc_ms[i];
  }
}
const char* tc_schedule_name(int s) {
  return s == 0 ? "round_robin" : s == 1 ? "snake" : s == 2 ? "lpt" : "?";
}
constexpr int kTcSchedules = 3;
// Tile layout of schedule `sched` for `grid` persistent CTAs (CTA b runs positions b, b + grid, ...).
// tiles: (K chunks, tile), longest first.  A tile's estimated cost is its K chunks plus the fill and
// drain of the operand ring (about four chunks).
static std::vector<TcTile> tc_layout(const std::vector<std::pair<int, TcTile>>& tiles, int grid, int sched) {
  std::vector<TcTile> out;
  const int n = (int)tiles.size();
  if (sched == 0) {
    for (auto& t : tiles) out.push_back(t.second);
  } else if (sched == 1) {
    for (int r0 = 0; r0 < n; r0 += grid) {
      const int r1 = std::min(n, r0 + grid);
      const bool rev = ((r0 / grid) & 1) != 0;
      if (!rev || r1 - r0 < grid) {
        for (int i = r0; i < r1; ++i) out.push_back(tiles[i].second);
      } else {
        for (int i = r1 - 1; i >= r0; --i) out.push_back(tiles[i].second);
      }
    }
  } else {
    std::vector<std::vector<TcTile>> lists(grid);
    std::priority_queue<std::pair<int64_t, int>, std::vector<std::pair<int64_t, int>>, std::greater<>> load;
    for (int b = 0; b < grid; ++b) load.push({0, b});
    for (auto& t : tiles) {
      auto top = load.top();
      load.pop();
      lists[top.second].push_back(t.second);
      load.push({top.first + t.first + 4, top.second});
    }
    size_t len = 0;
    for (auto& l : lists) len = std::max(len, l.size());
    const TcTile pad{-1, 0, 0};
    for (size_t r = 0; r < len; ++r)
      for (int b = 0; b < grid; ++b) out.push_back(r < lists[b].size() ? lists[b][r] : pad);
  }
  return out;
}
// coarse signature of a stage: precision, stage, and the tile count / K chunks in ~20 % buckets
static uint64_t tc_signature(int kind, int nprod, int st, const std::vector<std::pair<int, TcTile>>& tiles) {
  auto bucket = [](double x) { return (uint64_t)std::lround(std::log(std::max(x, 1.0)) / std::log(1.2)); };
  int64_t ksum = 0;
  int kmax = 0;
  for (auto& t : tiles) {
    ksum += t.first;
    kmax = std::max(kmax, t.first);
  }
  return ((uint64_t)kind << 60) ^ ((uint64_t)nprod << 56) ^ ((uint64_t)st << 52) ^ (bucket((double)tiles.size()) << 36) ^
         (bucket((double)ksum) << 18) ^ bucket((double)kmax);
}
static bool tc_autotune_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("MPSG_TC_AUTOTUNE");
    return !(e && std::atoi(e) == 0);
  }();
  return on;
}
// MPSG_TC_SCHEDULE=0|1|2 fixes the block schedule (no timing); -1: the autotuner decides
static int tc_forced_schedule() {
  static const int v = [] {
    const char* e = std::getenv("MPSG_TC_SCHEDULE");
    const int x = e ? std::atoi(e) : -1;
    return (x >= 0 && x < kTcSchedules) ? x : -1;
  }();
  return v;
}

static void build_tc(MatvecPlan& P, Ctx* ctx, const Layout& th,
                     const std::map<K5, std::map<uint32_t, std::pair<K5, int>>>& xterms,
                     const std::map<BKey, std::set<std::pair<K5, K5>>>& oterms) {
  P.kind = (P.prec == MPSG_PREC_TF32 || P.prec == MPSG_PREC_TF32X3) ? 0 : 1;
  P.nprod = (P.prec == MPSG_PREC_TF32X3 || P.prec == MPSG_PREC_BF16X3) ? 3 : 1;
  const int KC = P.kind == 0 ? 32 : 64;
  const int ncomp = P.nprod == 3 ? 2 : 1;
  int dev = 0;
  MPSG_CUDA(cudaGetDevice(&dev));
  MPSG_CUDA(cudaDeviceGetAttribute(&P.nsm, cudaDevAttrMultiProcessorCount, dev));
  auto nkc = [&](int k) { return (k + KC - 1) / KC; };
  std::map<K5, int64_t> lt_img, rt_img, x_img;
  std::map<int, int64_t> th_img;
  int64_t tot[4] = {0, 0, 0, 0};
  std::vector<TcConv> conv_env, conv_th;
  int img_env = 0, img_th = 0;
  auto conv = [&](std::vector<TcConv>& v, int& img, int src_slot, int64_t src_off, int R, int K, int rs, int ks,
                  int dst_slot, int64_t dst_off) {
    TcConv c;
    c.src_off = src_off;
    c.dst_off = dst_off;
    c.R = R;
    c.K = K;
    c.rs = rs;
    c.ks = ks;
    c.nkc = nkc(K);
    c.img0 = img;
    c.scale = 1.0;
    c.src_slot = (int8_t)src_slot;
    c.dst_slot = (int8_t)dst_slot;
    img += ((R + 127) / 128) * c.nkc;
    v.push_back(c);
  };
  for (auto& x : P.lt.m) {  // A operand of stage A: rows a', K = a (column-major source)
    const int64_t o = add_images(lt_img, x.first, x.second.r, x.second.c, KC, tot[0]);
    conv(conv_env, img_env, 2, x.second.off, x.second.r, x.second.c, 1, x.second.r, 0, o);
  }
  for (auto& x : P.rt.m) {  // B operand of stage C: rows b', K = b (column-major source)
    const int64_t o = add_images(rt_img, x.first, x.second.r, x.second.c, KC, tot[3]);
    conv(conv_env, img_env, 3, x.second.off, x.second.r, x.second.c, 1, x.second.r, 3, o);
  }
  for (int i = 0; i < (int)th.b.size(); ++i) {  // B operand of stage A: rows b (columns of theta), K = a
    const Block& b = th.b[i];
    const int64_t o = add_images(th_img, i, b.c, b.r, KC, tot[1]);
    conv(conv_th, img_th, 0, b.off, b.c, b.r, b.r, 1, 1, o);
  }
  for (auto& x : P.xa.m) add_images(x_img, x.first, x.second.r, x.second.c, KC, tot[2]);
  for (int i = 0; i < 4; ++i) {
    P.img_hi[i] = std::max<int64_t>(tot[i], 16384);
    const size_t bytes = (size_t)P.img_hi[i] * ncomp;
    P.dimg[i] = (uint8_t*)ctx->dmalloc(bytes);
    MPSG_CUDA(cudaMemsetAsync(P.dimg[i], 0, bytes, ctx->stream));
  }
  P.derr = (int*)ctx->dmalloc(sizeof(int));
  MPSG_CUDA(cudaMemsetAsync(P.derr, 0, sizeof(int), ctx->stream));
  // work lists; the candidate block schedules of each stage
  std::vector<TcTile> cand[2][kTcSchedules];
  uint64_t sig[2] = {0, 0};
  for (int st = 0; st < 2; ++st) {
    std::vector<TcProb> probs;
    std::vector<TcSeg> segs;
    std::vector<std::pair<int, TcTile>> tiles;  // (K chunks, tile)
    auto add_prob = [&](TcProb p, const std::vector<TcSeg>& ss) {
      p.seg0 = (int32_t)segs.size();
      int work = 0;
      for (auto& s : ss) {
        segs.push_back(s);
        work += s.nkc;
      }
      p.seg1 = (int32_t)segs.size();
      const int pi = (int)probs.size();
      probs.push_back(p);
      for (int mt = 0; mt < (p.M + 127) / 128; ++mt)
        for (int nt = 0; nt < (p.N + 127) / 128; ++nt) tiles.push_back({work, TcTile{pi, mt, nt}});
    };
    if (st == 0) {
      for (auto& x : xterms) {
        const auto& XB = P.xa.at(x.first);
        TcProb p{};
        p.c_off = x_img.at(x.first);
        p.ldc = 0;
        p.M = XB.r;
        p.N = XB.c;
        p.c_nkc = nkc(XB.c);
        p.mode = 1;
        p.c_slot = 2;
        p.beta = 0;
        std::vector<TcSeg> ss;
        for (auto& s : x.second) {
          const auto& LB = P.lt.at(s.second.first);
          TcSeg g{};
          g.a_off = lt_img.at(s.second.first);
          g.b_off = th_img.at(s.second.second);
          g.nkc = nkc(LB.c);
          g.a_slot = 0;
          g.b_slot = 1;
          ss.push_back(g);
        }
        add_prob(p, ss);
      }
    } else {
      for (auto& o : oterms) {
        const Block& OB = P.out.b[P.out.idx.at(o.first)];
        TcProb p{};
        p.c_off = OB.off;
        p.ldc = OB.r;
        p.M = OB.r;
        p.N = OB.c;
        p.c_nkc = 0;
        p.mode = 0;
        p.c_slot = 1;
        p.beta = 0;
        std::vector<TcSeg> ss;
        for (auto& pr : o.second) {
          const auto& XB = P.xa.at(pr.first);
          TcSeg g{};
          g.a_off = x_img.at(pr.first);
          g.b_off = rt_img.at(pr.second);
          g.nkc = nkc(XB.c);
          g.a_slot = 2;
          g.b_slot = 3;
          ss.push_back(g);
        }
        add_prob(p, ss);
      }
    }
    std::stable_sort(tiles.begin(), tiles.end(),
                     [](const std::pair<int, TcTile>& a, const std::pair<int, TcTile>& b) { return a.first > b.first; });
    const int grid = std::max(1, std::min((int)tiles.size(), P.nsm));
    for (int c = 0; c < kTcSchedules; ++c) cand[st][c] = tc_layout(tiles, grid, c);
    sig[st] = tc_signature(P.kind, P.nprod, st, tiles);
    P.tgrid[st] = grid;
    P.dprob[st] = (TcProb*)ctx->dmalloc(sizeof(TcProb) * std::max<size_t>(probs.size(), 1));
    P.dseg[st] = (TcSeg*)ctx->dmalloc(sizeof(TcSeg) * std::max<size_t>(segs.size(), 1));
    if (!probs.empty())
      MPSG_CUDA(cudaMemcpyAsync(P.dprob[st], probs.data(), sizeof(TcProb) * probs.size(), cudaMemcpyHostToDevice, ctx->stream));
    if (!segs.empty())
      MPSG_CUDA(cudaMemcpyAsync(P.dseg[st], segs.data(), sizeof(TcSeg) * segs.size(), cudaMemcpyHostToDevice, ctx->stream));
  }
  P.nconv_theta = (int)conv_th.size();
  P.nimg_theta = img_th;
  P.dconv_theta = (TcConv*)ctx->dmalloc(sizeof(TcConv) * std::max<size_t>(conv_th.size(), 1));
  if (!conv_th.empty())
    MPSG_CUDA(cudaMemcpyAsync(P.dconv_theta, conv_th.data(), sizeof(TcConv) * conv_th.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
  // environments -> images, once per plan
  if (!conv_env.empty()) {
    TcConv* d = (TcConv*)ctx->dmalloc(sizeof(TcConv) * conv_env.size());
    MPSG_CUDA(cudaMemcpyAsync(d, conv_env.data(), sizeof(TcConv) * conv_env.size(), cudaMemcpyHostToDevice, ctx->stream));
    const TcBases B = tc_bases(P, nullptr, nullptr);
    launch_tc_convert(P.kind, ncomp, d, (int)conv_env.size(), img_env, B, ctx->stream);
    ctx->dfree(d);
  }
  // block schedule of each stage: from the cache, or timed (CUDA events, the plan's own images; stage
  // C into a scratch output) once per signature.  Every schedule computes every tile the same way,
  // so the choice never changes a result.
  static std::mutex mu;
  static std::map<uint64_t, int> best;
  for (int st = 0; st < 2; ++st) {
    int choice = tc_forced_schedule() >= 0 ? tc_forced_schedule() : 0;
    bool have = !tc_autotune_enabled() || tc_forced_schedule() >= 0 || cand[st][0].empty();
    if (!have) {
      std::lock_guard<std::mutex> g(mu);
      auto it = best.find(sig[st]);
      if (it != best.end()) {
        choice = it->second;
        have = true;
        g_tc_hits.fetch_add(1);
      }
    }
    if (!have) {
      double* scratch = st == 1 ? (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(P.out.nelem, 2)) : nullptr;
      std::vector<TcTile*> dev(kTcSchedules);
      for (int c = 0; c < kTcSchedules; ++c) {
        dev[c] = (TcTile*)ctx->dmalloc(sizeof(TcTile) * cand[st][c].size());
        MPSG_CUDA(cudaMemcpyAsync(dev[c], cand[st][c].data(), sizeof(TcTile) * cand[st][c].size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
      }
      const TcBases B = tc_bases(P, nullptr, scratch);
      cudaEvent_t e0, e1;
      MPSG_CUDA(cudaEventCreate(&e0));
      MPSG_CUDA(cudaEventCreate(&e1));
      float tbest = 1e30f;
      float tc_best[kTcSchedules];
      for (int c = 0; c < kTcSchedules; ++c) tc_best[c] = 1e30f;
      for (int rep = 0; rep < 3; ++rep)
        for (int c = 0; c < kTcSchedules; ++c) {
          MPSG_CUDA(cudaEventRecord(e0, ctx->stream));
          launch_tc_gemm(P.kind, P.nprod, P.dprob[st], P.dseg[st], dev[c], (int)cand[st][c].size(), B, P.nsm,
                         ctx->stream, P.tgrid[st]);
          MPSG_CUDA(cudaEventRecord(e1, ctx->stream));
          MPSG_CUDA(cudaEventSynchronize(e1));
          float ms = 0;
          MPSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
          if (rep > 0) tc_best[c] = std::min(tc_best[c], ms);
          if (rep > 0 && ms < tbest) {  // the first round warms up
            tbest = ms;
            choice = c;
          }
        }
      {
        std::lock_guard<std::mutex> g(g_tc_ms_mu);
        for (int c = 0; c < kTcSchedules; ++c) g_tc_ms[st * 3 + c] = tc_best[c];
        for (int c = 0; c < kTcSchedules && st == 0; ++c) g_tc_ms[3 + c] = -1.f;
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      for (auto* d : dev) ctx->dfree(d);
      if (scratch) ctx->dfree(scratch);
      P.check_error();
      std::lock_guard<std::mutex> g(mu);
      best[sig[st]] = choice;
      g_tc_tuned.fetch_add(1);
    }
    const std::vector<TcTile>& tl = cand[st][choice];
    P.tsched[st] = choice;
    g_tc_last[st].store(choice);
    P.ntile[st] = (int)tl.size();
    P.dtile[st] = (TcTile*)ctx->dmalloc(sizeof(TcTile) * std::max<size_t>(tl.size(), 1));
    if (!tl.empty())
      MPSG_CUDA(cudaMemcpyAsync(P.dtile[st], tl.data(), sizeof(TcTile) * tl.size(), cudaMemcpyHostToDevice, ctx->stream));
  }
}

std::unique_ptr<MatvecPlan> build_matvec(Ctx* ctx, const Tensor& L, const Tensor& R, const Layout& th, const MPO& W1,
                                         const MPO& W2, const ItoKey& ik0, const ItoKey& ik1,
                                         const Layout* out_layout, int prec) {
  MPSG_CHECK(prec >= MPSG_PREC_FP64 && prec <= MPSG_PREC_BF16X3, "unsupported matvec precision");
  std::unique_ptr<MatvecPlan> P(new MatvecPlan());
  P->ctx = ctx;
  P->keep = ctx->shared_from_this();
  P->prec = prec;
  std::map<K5, std::map<std::tuple<int, int, int>, double>> ltc, rtc;
  std::map<K5, std::map<uint32_t, std::pair<K5, int>>> xterms;
  std::map<BKey, std::set<std::pair<K5, K5>>> oterms;
  std::map<BKey, std::pair<int, int>> odims;
  std::set<std::tuple<int, int, int, int, int, int>> ypairs;  // F_B: distinct (L blk, theta blk, W pair)
  std::set<std::tuple<Q, Q, uint32_t, uint32_t, uint32_t>> yset;
  visit_matvec_terms(L, R, th, W1, W2, ik0, ik1,
                     [&](int i, int e1, int o1, int e2, int o2, int ti, int rj, Q a1, Q a, Q b, Q b1, uint32_t wm,
                         const OpEl& op1, const OpEl& op2) {
                       K5 lk{a1, a, wm, op1.in, op1.out};
                       ltc[lk][std::make_tuple(i, e1, o1)] = op1.v;
                       K5 rk{b1, b, wm, op2.in, op2.out};
                       rtc[rk][std::make_tuple(rj, e2, o2)] = op2.v;
                       K5 xk{a1, b, wm, op1.in, op2.out};
                       xterms[xk][op1.out] = std::make_pair(lk, ti);
                       BKey ok = K2(a1, b1, op1.in, op2.in);
                       oterms[ok].insert(std::make_pair(xk, rk));
                       odims[ok] = {L.b[i].r, R.b[rj].r};
                       const double ra1 = L.b[i].r, ca = L.b[i].c, cb = th.b[ti].c, rb1 = R.b[rj].r;
                       P->flops_ref += 2.0 * ra1 * ca * cb + 2.0 * ra1 * cb * rb1;
                       P->flops_factored += 2.0 * ra1 * cb;  // F_B term (W element pair on one X block)
                       yset.insert(std::make_tuple(a1, b, W2.e[e2].wr, op1.in, op2.in));
                     });
  // F_A: every (L block, theta block with left charge a) pair; F_C: every Y block with its R block
  {
    std::map<Q, std::vector<int>> thby;
    for (int t = 0; t < (int)th.b.size(); ++t) thby[th.b[t].k.q0].push_back(t);
    for (auto& lb : L.b) {
      auto it = thby.find(lb.k.q1);
      if (it == thby.end()) continue;
      for (int t : it->second) P->flops_factored += 2.0 * lb.r * lb.c * th.b[t].c;
    }
    for (auto& y : yset) {
      Q a1, b;
      uint32_t wr, s1p, s2p;
      std::tie(a1, b, wr, s1p, s2p) = y;
      const Q b1 = a1 + qat(ik0, s1p) + qat(ik1, s2p);
      const int rj = R.find(K1(b1, b, wr));
      int ra1 = 0;
      for (auto& lb : L.b)
        if (lb.k.q0 == a1) { ra1 = lb.r; break; }
      if (rj >= 0) P->flops_factored += 2.0 * ra1 * R.b[rj].c * R.b[rj].r;
    }
  }
  // arenas
  for (auto& x : ltc) {
    const Block& lb = L.b[std::get<0>(x.second.begin()->first)];
    P->lt.add(x.first, lb.r, lb.c);
  }
  for (auto& x : rtc) {
    const Block& rb = R.b[std::get<0>(x.second.begin()->first)];
    P->rt.add(x.first, rb.r, rb.c);
  }
  for (auto& x : xterms) {
    const auto& first = x.second.begin()->second;
    const int ra1 = P->lt.at(first.first).r;
    const int cb = th.b[first.second].c;
    P->xa.add(x.first, ra1, cb);
  }
  if (out_layout) {
    P->out = *out_layout;
    for (auto& o : oterms) MPSG_CHECK(P->out.idx.count(o.first), "matvec output block missing from output layout");
  } else {
    for (auto& o : odims) P->out.add(o.first, o.second.first, o.second.second);
    P->out.finalize();
  }
  P->dLt = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(P->lt.nelem, 2));
  P->dRt = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(P->rt.nelem, 2));
  if (prec == MPSG_PREC_FP64) P->dX = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(P->xa.nelem, 2));
  // combined environments
  for (auto& x : ltc) {
    std::vector<std::pair<const double*, double>> terms;
    for (auto& c : x.second) terms.push_back({L.ptr(std::get<0>(c.first)), c.second});
    const auto& B = P->lt.at(x.first);
    P->build_lt.add(P->dLt + B.off, (int64_t)B.r * B.c, terms);
  }
  for (auto& x : rtc) {
    std::vector<std::pair<const double*, double>> terms;
    for (auto& c : x.second) terms.push_back({R.ptr(std::get<0>(c.first)), c.second});
    const auto& B = P->rt.at(x.first);
    P->build_rt.add(P->dRt + B.off, (int64_t)B.r * B.c, terms);
  }
  P->build_lt.run(ctx);
  P->build_rt.run(ctx);
  // stage A: X = sum_s1 L~ theta
  for (auto& x : xterms) {
    const auto& XB = P->xa.at(x.first);
    std::vector<GSegH> segs;
    for (auto& s : x.second) {
      const auto& LB = P->lt.at(s.second.first);
      const Block& TB = th.b[s.second.second];
      MPSG_CHECK(LB.c == TB.r && LB.r == XB.r && TB.c == XB.c, "inconsistent block sizes in matvec (stage A)");
      segs.push_back(GSegH{0, 1, LB.off, TB.off, LB.r, TB.r, LB.c, 0, 0, 1.0});
    }
    P->stageA.add_problem(2, XB.off, XB.r, XB.r, XB.c, false, segs);
  }
  // stage C: out = sum X R~^T
  for (auto& o : oterms) {
    const Block& OB = P->out.b[P->out.idx.at(o.first)];
    std::vector<GSegH> segs;
    for (auto& pr : o.second) {
      const auto& XB = P->xa.at(pr.first);
      const auto& RB = P->rt.at(pr.second);
      MPSG_CHECK(XB.c == RB.c && XB.r == OB.r && RB.r == OB.c, "inconsistent block sizes in matvec (stage C)");
      segs.push_back(GSegH{2, 3, XB.off, RB.off, XB.r, RB.r, XB.c, 0, 1, 1.0});
    }
    P->stageC.add_problem(4, OB.off, OB.r, OB.r, OB.c, false, segs);
  }
  P->stageA.upload(ctx);
  P->stageC.upload(ctx);
  P->flops = P->stageA.flops + P->stageC.flops;
  int64_t nl = 0, nr = 0, nt = 0;
  for (auto& b : L.b) nl += (int64_t)b.r * b.c;
  for (auto& b : R.b) nr += (int64_t)b.r * b.c;
  for (auto& b : th.b) nt += (int64_t)b.r * b.c;
  P->bytes_alg = 8 * (nl + nr + 2 * nt);
  if (prec != MPSG_PREC_FP64) build_tc(*P, ctx, th, xterms, oterms);
  return P;
}

// ============================================================================ environment update
EnvPlan::~EnvPlan() {
  if (ctx) {
    ctx->dfree(dCt);
    ctx->dfree(dT);
  }
}
void EnvPlan::run(const double* A, double* out_d, const double* Aup) {
  const double* bases[8] = {dCt, A, dT, out_d, Aup ? Aup : A, nullptr, nullptr, nullptr};
  if (tc1) {
    tc1->run(bases);
    tc2->run(bases);
    return;
  }
  st1.run(bases);
  st2.run(bases);
}

// ---- a GemmPlan stage on the tensor cores
void TcStage::build(Ctx* c, const GemmPlan& g, int prec) {
  ctx = c;
  kind = (prec == MPSG_PREC_TF32 || prec == MPSG_PREC_TF32X3) ? 0 : 1;
  nprod = (prec == MPSG_PREC_TF32X3 || prec == MPSG_PREC_BF16X3) ? 3 : 1;
  const int KC = kind == 0 ? 32 : 64;
  const int ncomp = nprod == 3 ? 2 : 1;
  int dev = 0;
  MPSG_CUDA(cudaGetDevice(&dev));
  MPSG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  auto nkc_of = [&](int K) { return (K + KC - 1) / KC; };
  // operand images keyed by (slot, offset, rows, K, row stride, K stride, scale)
  std::map<std::tuple<int, int64_t, int, int, int, int, double>, int64_t> imgs;
  std::vector<TcConv> conv;
  int64_t tot = 0;
  int nimg_tot = 0;
  auto image = [&](int slot, int64_t off, int rows, int K, int rs, int ks, double scale) {
    const auto key = std::make_tuple(slot, off, rows, K, rs, ks, scale);
    auto it = imgs.find(key);
    if (it != imgs.end()) return it->second;
    const int nkc = nkc_of(K);
    const int64_t n = (int64_t)((rows + 127) / 128) * nkc;
    TcConv cv{};
    cv.src_off = off;
    cv.dst_off = tot;
    cv.R = rows;
    cv.K = K;
    cv.rs = rs;
    cv.ks = ks;
    cv.nkc = nkc;
    cv.img0 = nimg_tot;
    cv.scale = scale;
    cv.src_slot = (int8_t)slot;
    cv.dst_slot = 0;
    conv.push_back(cv);
    imgs[key] = tot;
    tot += n * 16384;
    nimg_tot += (int)n;
    return imgs[key];
  };
  std::vector<TcProb> probs;
  std::vector<TcSeg> segs;
  std::vector<std::pair<int, TcTile>> tiles;
  for (const GProbH& p : g.hprob) {
    TcProb q{};
    q.c_off = p.offC;
    q.ldc = p.ldc;
    q.M = p.M;
    q.N = p.N;
    q.seg0 = (int32_t)segs.size();
    q.c_nkc = 0;
    q.mode = 0;
    q.c_slot = (int8_t)p.baseC;
    q.beta = (int8_t)p.beta;
    int work = 0;
    for (int si = p.seg0; si < p.seg1; ++si) {
      const GSegH& h = g.hseg[si];
      // A operand: op(A) is M x K; image rows = M.  B operand: op(B) is K x N; image rows = N.
      const int64_t ao = image(h.baseA, h.offA, p.M, h.K, h.tA ? h.lda : 1, h.tA ? 1 : h.lda, h.alpha);
      const int64_t bo = image(h.baseB, h.offB, p.N, h.K, h.tB ? 1 : h.ldb, h.tB ? h.ldb : 1, 1.0);
      TcSeg sg{};
      sg.a_off = ao;
      sg.b_off = bo;
      sg.nkc = nkc_of(h.K);
      sg.a_slot = 0;
      sg.b_slot = 0;
      segs.push_back(sg);
      work += sg.nkc;
    }
    q.seg1 = (int32_t)segs.size();
    const int pi = (int)probs.size();
    probs.push_back(q);
    for (int mt = 0; mt < (p.M + 127) / 128; ++mt)
      for (int nt = 0; nt < (p.N + 127) / 128; ++nt) tiles.push_back({work, TcTile{pi, mt, nt}});
  }
  std::stable_sort(tiles.begin(), tiles.end(),
                   [](const std::pair<int, TcTile>& a, const std::pair<int, TcTile>& b) { return a.first > b.first; });
  grid = std::max(1, std::min((int)tiles.size(), nsm));
  const std::vector<TcTile> tl = tc_layout(tiles, grid, 1);  // snake over longest-K-first
  img_hi = std::max<int64_t>(tot, 16384);
  dimg = (uint8_t*)ctx->dmalloc((size_t)img_hi * ncomp);
  nconv = (int)conv.size();
  nimg = nimg_tot;
  ntile = (int)tl.size();
  dconv = (TcConv*)ctx->dmalloc(sizeof(TcConv) * std::max<size_t>(conv.size(), 1));
  dprob = (TcProb*)ctx->dmalloc(sizeof(TcProb) * std::max<size_t>(probs.size(), 1));
  dseg = (TcSeg*)ctx->dmalloc(sizeof(TcSeg) * std::max<size_t>(segs.size(), 1));
  dtile = (TcTile*)ctx->dmalloc(sizeof(TcTile) * std::max<size_t>(tl.size(), 1));
  derr = (int*)ctx->dmalloc(sizeof(int));
  cudaStream_t st = ctx->stream;
  MPSG_CUDA(cudaMemsetAsync(derr, 0, sizeof(int), st));
  if (!conv.empty()) MPSG_CUDA(cudaMemcpyAsync(dconv, conv.data(), sizeof(TcConv) * conv.size(), cudaMemcpyHostToDevice, st));
  if (!probs.empty()) MPSG_CUDA(cudaMemcpyAsync(dprob, probs.data(), sizeof(TcProb) * probs.size(), cudaMemcpyHostToDevice, st));
  if (!segs.empty()) MPSG_CUDA(cudaMemcpyAsync(dseg, segs.data(), sizeof(TcSeg) * segs.size(), cudaMemcpyHostToDevice, st));
  if (!tl.empty()) MPSG_CUDA(cudaMemcpyAsync(dtile, tl.data(), sizeof(TcTile) * tl.size(), cudaMemcpyHostToDevice, st));
}
void TcStage::run(const double* const* bases) {
  if (ntile == 0) return;
  TcBases B;
  for (int i = 0; i < 6; ++i) {
    B.img[i] = nullptr;
    B.lo_off[i] = 0;
    B.f64[i] = const_cast<double*>(bases[i]);
  }
  B.img[0] = dimg;
  B.lo_off[0] = img_hi;
  B.err = derr;
  launch_tc_convert(kind, nprod == 3 ? 2 : 1, dconv, nconv, nimg, B, ctx->stream);
  launch_tc_gemm(kind, nprod, dprob, dseg, dtile, ntile, B, nsm, ctx->stream, grid);
}
TcStage::~TcStage() {
  if (!ctx) return;
  for (void* p : {(void*)dimg, (void*)dconv, (void*)dprob, (void*)dseg, (void*)dtile, (void*)derr}) ctx->dfree(p);
}

std::unique_ptr<EnvPlan> build_env(Ctx* ctx, const Tensor& BL, const Tensor& A, const MPO& W, const ItoKey& ik,
                                   int direction, const Tensor* Aup, int prec) {
  const Tensor& U = Aup ? *Aup : A;  // upper tensor (add_out_sub, src/MPSfunctions.hpp:360-434)
  MPSG_CHECK(prec >= MPSG_PREC_FP64 && prec <= MPSG_PREC_BF16X3, "unsupported environment-update precision");
  std::unique_ptr<EnvPlan> P(new EnvPlan());
  P->ctx = ctx;
  P->keep = ctx->shared_from_this();
  P->prec = prec;
  const bool left = direction > 0;
  std::map<std::pair<uint32_t, Q>, std::vector<int>> envby;  // (w, lower charge) -> env blocks
  for (int i = 0; i < (int)BL.b.size(); ++i) envby[{BL.b[i].k.p0, BL.b[i].k.q1}].push_back(i);
  std::map<K5, std::map<std::tuple<int, int, int>, double>> ctc;
  std::map<K5, std::map<uint32_t, std::pair<K5, int>>> tterms;          // T key -> so -> (Ct key, A block)
  std::map<BKey, std::map<std::pair<uint32_t, Q>, std::pair<int, K5>>> oterms;  // out -> (si, charge) -> (A blk, T key)
  for (int j = 0; j < (int)A.b.size(); ++j) {
    const Block& ad = A.b[j];
    const Q a = ad.k.q0, b = ad.k.q1;
    const uint32_t so = ad.k.p0;
    for (int e = 0; e < (int)W.e.size(); ++e) {
      const MPOEntry& en = W.e[e];
      for (int o = 0; o < (int)en.ops.size(); ++o) {
        const OpEl& op = en.ops[o];
        if (op.out != so) continue;
        const uint32_t si = op.in;
        if (left) {
          // add_out_sub_2, direction > 0: key_b = (p - q(out), p; out) with p = b
          MPSG_CHECK(b == a + qat(ik, so), "MPS block violates charge conservation");
          auto it = envby.find({en.wl, a});
          if (it == envby.end()) continue;
          for (int i : it->second) {
            const Q a1 = BL.b[i].k.q0;
            const Q b1 = a1 + qat(ik, si);
            const int au = U.find(K1(a1, b1, si));
            if (au < 0) continue;
            K5 ck{a1, a, en.wr, si, so};
            ctc[ck][std::make_tuple(i, e, o)] = op.v;
            K5 tk{a1, b, en.wr, si, 0};
            tterms[tk][so] = std::make_pair(ck, j);
            oterms[K1(b1, b, en.wr)][{si, a1}] = std::make_pair(au, tk);
          }
        } else {
          // direction <= 0: key_b = (p, p + q(out); out) with p = a
          auto it = envby.find({en.wr, b});
          if (it == envby.end()) continue;
          for (int i : it->second) {
            const Q b1 = BL.b[i].k.q0;
            const Q a1 = b1 - qat(ik, si);
            const int au = U.find(K1(a1, b1, si));
            if (au < 0) continue;
            K5 ck{b1, b, en.wl, si, so};
            ctc[ck][std::make_tuple(i, e, o)] = op.v;
            K5 tk{a, b1, en.wl, si, 0};
            tterms[tk][so] = std::make_pair(ck, j);
            oterms[K1(a1, a, en.wl)][{si, b1}] = std::make_pair(au, tk);
          }
        }
      }
    }
  }
  for (auto& x : ctc) {
    const Block& eb = BL.b[std::get<0>(x.second.begin()->first)];
    P->ct.add(x.first, eb.r, eb.c);
  }
  for (auto& x : tterms) {
    const auto& f = x.second.begin()->second;
    const Block& ab = A.b[f.second];
    const auto& CB = P->ct.at(f.first);
    if (left) P->tt.add(x.first, CB.r, ab.c);   // (chi_a' x chi_b)
    else P->tt.add(x.first, ab.r, CB.r);        // (chi_a x chi_b')
  }
  for (auto& o : oterms) {
    const auto& f = o.second.begin()->second;
    const Block& au = U.b[f.first];
    const auto& TB = P->tt.at(f.second);
    if (left) P->out.add(o.first, au.c, TB.c);  // (chi_b' x chi_b)
    else P->out.add(o.first, au.r, TB.r);       // (chi_a' x chi_a)
  }
  P->out.finalize();
  P->dCt = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(P->ct.nelem, 2));
  P->dT = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(P->tt.nelem, 2));
  for (auto& x : ctc) {
    std::vector<std::pair<const double*, double>> terms;
    for (auto& c : x.second) terms.push_back({BL.ptr(std::get<0>(c.first)), c.second});
    const auto& B = P->ct.at(x.first);
    P->build_ct.add(P->dCt + B.off, (int64_t)B.r * B.c, terms);
  }
  P->build_ct.run(ctx);
  // bases: 0 = Ct, 1 = A (lower), 2 = T, 3 = out, 4 = upper tensor
  for (auto& x : tterms) {
    const auto& TB = P->tt.at(x.first);
    std::vector<GSegH> segs;
    for (auto& s : x.second) {
      const auto& CB = P->ct.at(s.second.first);
      const Block& ab = A.b[s.second.second];
      if (left) {  // T(a',b) += Ct(a',a) A(a,b)
        MPSG_CHECK(CB.c == ab.r && CB.r == TB.r && ab.c == TB.c, "inconsistent block sizes (env, stage 1)");
        segs.push_back(GSegH{0, 1, CB.off, ab.off, CB.r, ab.r, CB.c, 0, 0, 1.0});
      } else {     // T(a,b') += A(a,b) Ct(b',b)^T
        MPSG_CHECK(ab.c == CB.c && ab.r == TB.r && CB.r == TB.c, "inconsistent block sizes (env, stage 1)");
        segs.push_back(GSegH{1, 0, ab.off, CB.off, ab.r, CB.r, ab.c, 0, 1, 1.0});
      }
    }
    P->st1.add_problem(2, TB.off, TB.r, TB.r, TB.c, false, segs);
  }
  for (auto& o : oterms) {
    const Block& OB = P->out.b[P->out.idx.at(o.first)];
    std::vector<GSegH> segs;
    for (auto& s : o.second) {
      const Block& au = U.b[s.second.first];
      const auto& TB = P->tt.at(s.second.second);
      if (left) {  // out(b',b) += Aup(a',b')^T T(a',b)
        MPSG_CHECK(au.r == TB.r && au.c == OB.r && TB.c == OB.c, "inconsistent block sizes (env, stage 2)");
        segs.push_back(GSegH{4, 2, au.off, TB.off, au.r, TB.r, au.r, 1, 0, 1.0});
      } else {     // out(a',a) += Aup(a',b') T(a,b')^T
        MPSG_CHECK(au.c == TB.c && au.r == OB.r && TB.r == OB.c, "inconsistent block sizes (env, stage 2)");
        segs.push_back(GSegH{4, 2, au.off, TB.off, au.r, TB.r, au.c, 0, 1, 1.0});
      }
    }
    P->st2.add_problem(3, OB.off, OB.r, OB.r, OB.c, false, segs);
  }
  P->st1.upload(ctx);
  P->st2.upload(ctx);
  P->flops = P->st1.flops + P->st2.flops;
  if (prec != MPSG_PREC_FP64) {
    P->tc1.reset(new TcStage());
    P->tc1->build(ctx, P->st1, prec);
    P->tc2.reset(new TcStage());
    P->tc2->build(ctx, P->st2, prec);
  }
  return P;
}

TensorP env_update(Ctx* ctx, const Tensor& BL, const Tensor& A, const MPO& W, const ItoKey& ik, int direction,
                   double* flops_out, const Tensor* Aup, int prec) {
  auto P = build_env(ctx, BL, A, W, ik, direction, Aup, prec);
  TensorP out = make_tensor(ctx, 1, P->out, true);
  P->run(A.d, out->d, Aup ? Aup->d : nullptr);
  if (P->tc1) {  // bounded device waits of the tensor-core stages
    int e1 = 0, e2 = 0;
    MPSG_CUDA(cudaMemcpyAsync(&e1, P->tc1->derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MPSG_CUDA(cudaMemcpyAsync(&e2, P->tc2->derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    if (e1 || e2) throw Err(5, "tensor-core environment update: a bounded device wait expired");
  }
  if (flops_out) *flops_out += P->flops;
  return out;
}

// ============================================================================ theta formation
TensorP theta_form(Ctx* ctx, const Tensor& A1, const Tensor& A2, const Layout* layout) {
  std::map<Q, std::vector<int>> by_left;
  for (int j = 0; j < (int)A2.b.size(); ++j) by_left[A2.b[j].k.q0].push_back(j);
  std::vector<std::tuple<BKey, int, int>> prods;
  Layout lay;
  for (int i = 0; i < (int)A1.b.size(); ++i) {
    auto it = by_left.find(A1.b[i].k.q1);
    if (it == by_left.end()) continue;
    for (int j : it->second) {
      BKey k = K2(A1.b[i].k.q0, A2.b[j].k.q1, A1.b[i].k.p0, A2.b[j].k.p0);
      prods.emplace_back(k, i, j);
      if (!layout) lay.add(k, A1.b[i].r, A2.b[j].c);
    }
  }
  if (layout) lay = *layout;
  else lay.finalize();
  TensorP th = make_tensor(ctx, 2, lay, true);
  GemmPlan g;
  for (auto& p : prods) {
    const int o = th->find(std::get<0>(p));
    MPSG_CHECK(o >= 0, "theta block missing from layout");
    const Block& a = A1.b[std::get<1>(p)];
    const Block& b = A2.b[std::get<2>(p)];
    MPSG_CHECK(a.c == b.r, "bond dimension mismatch between A1 and A2");
    g.add_problem(2, th->b[o].off, a.r, a.r, b.c, false, {GSegH{0, 1, a.off, b.off, a.r, b.r, a.c, 0, 0, 1.0}});
  }
  g.upload(ctx);
  const double* bases[8] = {A1.d, A2.d, th->d, nullptr, nullptr, nullptr, nullptr, nullptr};
  g.run(bases);
  ctx->sync();
  return th;
}

// ============================================================================ batched SVD (cuSOLVER gesvdj)
// Sector matrices (m x n) are stored as ms x ns with ms >= ns (transposed when m < n).  After the
// SVD, Q (m x k) carries the left vectors and P (n x k) the right vectors (columns of P = rows of Vt);
// FixPhase is applied so that the first abs-max entry of every Vt row is positive.
struct SvdBatch {
  struct Sec {
    int m, n, ms, ns, k;
    bool trans;
    int64_t offM, offU, offV, offS;
  };
  std::vector<Sec> s;
  std::vector<int> kr;  // resolved singular pairs per sector (density routes; empty: all k)
  int kcols(size_t i) const { return kr.empty() ? s[i].k : kr[i]; }
  Ctx* ctx = nullptr;
  double *dM = nullptr, *dU = nullptr, *dV = nullptr, *dS = nullptr;
  int* dinfo = nullptr;
  int64_t nS = 0;
  std::function<void(cudaEvent_t)> on_bidiag;  // see split2
  // complex mode of the bidiagonal route (the TEBD split): zM holds the complex sector matrices at the
  // offsets of dM; the real bidiagonal, its values and the real U_B, V_B come out as in the real mode,
  // U = Q [U_B; 0] and V = P V_B are written to zUo / zVo (per sector: pointer, leading dimension);
  // no FixPhase, no Jacobi fallback (zfailed is set instead)
  double2* zM = nullptr;
  std::vector<std::pair<double2*, int>> zUo, zVo;
  bool zfailed = false;
  explicit SvdBatch(Ctx* c) : ctx(c) {}
  ~SvdBatch() {
    bidiag_free();
    ctx->dfree(dM);
    ctx->dfree(dU);
    ctx->dfree(dV);
    ctx->dfree(dS);
    ctx->dfree(dinfo);
  }
  void plan(const std::vector<std::pair<int, int>>& mn) {
    int64_t oM = 0, oU = 0, oV = 0, oS = 0;
    auto al = [](int64_t x) { return (x + kAlign - 1) / kAlign * kAlign; };
    for (auto& d : mn) {
      Sec x;
      x.m = d.first;
      x.n = d.second;
      x.trans = x.m < x.n;
      x.ms = std::max(x.m, x.n);
      x.ns = std::min(x.m, x.n);
      x.k = x.ns;
      x.offM = oM; oM += al((int64_t)x.ms * x.ns);
      x.offU = oU; oU += al((int64_t)x.ms * x.k);
      x.offV = oV; oV += al((int64_t)x.ns * x.k);
      x.offS = oS; oS += x.k;
      s.push_back(x);
    }
    nS = oS;
    dM = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oM, 2));
    dU = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oU, 2));
    dV = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oV, 2));
    dS = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oS, 2));
    dinfo = (int*)ctx->dmalloc(sizeof(int) * std::max<size_t>(s.size(), 1));
    MPSG_CUDA(cudaMemsetAsync(dM, 0, sizeof(double) * std::max<int64_t>(oM, 2), ctx->stream));
  }
  // destination of logical element (r, c) of sector i's m x n matrix
  CopyOp gather_op(int i, const double* src, int rows, int cols, int r0, int c0) const {
    const Sec& x = s[i];
    CopyOp o;
    o.src = src;
    o.rs = nullptr;
    o.cs = nullptr;
    o.scale = 1.0;
    o.lds = rows;
    o.ldd = x.ms;
    if (!x.trans) {
      o.dst = dM + x.offM + r0 + (int64_t)c0 * x.ms;
      o.rows = rows;
      o.cols = cols;
      o.trans = 0;
    } else {
      o.dst = dM + x.offM + c0 + (int64_t)r0 * x.ms;
      o.rows = cols;
      o.cols = rows;
      o.trans = 1;
    }
    return o;
  }
  double* Qp(int i, int* ld) const {
    const Sec& x = s[i];
    if (!x.trans) { *ld = x.ms; return dU + x.offU; }
    *ld = x.ns; return dV + x.offV;
  }
  double* Pp(int i, int* ld) const {
    const Sec& x = s[i];
    if (!x.trans) { *ld = x.ns; return dV + x.offV; }
    *ld = x.ms; return dU + x.offU;
  }
  // Density-matrix route: G = Mst^T Mst (grouped FP64 GEMM), eigenpairs of G (FP64), Vst = eigenvectors
  // in descending order, Ust = Mst Vst with unit columns, s_j = |Mst v_j|.  The Gram matrix squares the
  // condition number: eigenvalues below 32 n eps lambda_max are not resolved and their pairs are dropped
  // (s_j = 0); above that floor u_i . u_j ~ n eps lambda_max / (s_i s_j), which CholeskyQR removes
  // (orthonormalize_left), so the kept left vectors are orthonormal to rounding.
  // Batched density-matrix route: sectors are grouped by size class (next power of two >= ns, at
  // least 32); each G_i = Mst_i^T Mst_i is written into the top-left corner of its class slot and the
  // padding diagonal is set to -1, so the padded eigenvalues sort below the (non-negative) spectrum.
  // One cusolverDnXsyevBatched call per class.
  void run_gram() {
    cusolverDnHandle_t h = ctx->svd_handle();
    std::map<int, std::vector<int>> cls;  // class size -> sectors
    for (size_t i = 0; i < s.size(); ++i) {
      if (s[i].k == 0) continue;
      int c = 32;
      while (c < s[i].ns) c <<= 1;
      cls[c].push_back((int)i);
    }
    std::vector<int64_t> slot_off(s.size(), 0), lam_off(s.size(), 0), cls_of(s.size(), 0);
    int64_t oB = 0, oW = 0;
    for (auto& c : cls)
      for (int i : c.second) {
        slot_off[i] = oB;
        lam_off[i] = oW;
        cls_of[i] = c.first;
        oB += (int64_t)c.first * c.first;
        oW += c.first;
      }
    double* dB = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oB, 2));
    double* dWv = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oW, 2));
    int* dinf = (int*)ctx->dmalloc(sizeof(int) * (s.size() + 1));
    MPSG_CUDA(cudaMemsetAsync(dB, 0, sizeof(double) * std::max<int64_t>(oB, 2), ctx->stream));
    {  // G_i into the class slots, padding diagonal -1
      GemmPlan g;
      std::vector<double*> pads;
      std::vector<GramPad> pd;
      for (size_t i = 0; i < s.size(); ++i) {
        const Sec& x = s[i];
        if (x.k == 0) continue;
        g.add_problem(2, slot_off[i], (int)cls_of[i], x.ns, x.ns, false,
                      {GSegH{0, 0, x.offM, x.offM, x.ms, x.ms, x.ms, 1, 0, 1.0}});
        pd.push_back(GramPad{dB + slot_off[i], (int32_t)cls_of[i], x.ns});
      }
      g.upload(ctx);
      const double* bases[8] = {dM, nullptr, dB, nullptr, nullptr, nullptr, nullptr, nullptr};
      g.run(bases);
      if (!pd.empty()) {
        GramPad* d = (GramPad*)ctx->dmalloc(sizeof(GramPad) * pd.size());
        MPSG_CUDA(cudaMemcpyAsync(d, pd.data(), sizeof(GramPad) * pd.size(), cudaMemcpyHostToDevice, ctx->stream));
        launch_gram_pad(d, (int)pd.size(), ctx->stream);
        ctx->dfree(d);
      }
    }
    int ib = 0;
    for (auto& c : cls) {
      const int64_t n = c.first, batch = (int64_t)c.second.size();
      double* A = dB + slot_off[c.second[0]];
      double* W = dWv + lam_off[c.second[0]];
      size_t wd = 0, wh = 0;
      if (cusolverDnXsyevBatched_bufferSize(h, ctx->solver_params(), CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                            CUDA_R_64F, A, n, CUDA_R_64F, W, CUDA_R_64F, &wd, &wh, batch) !=
          CUSOLVER_STATUS_SUCCESS)
        throw Err(3, "syevBatched_bufferSize failed");
      void* dwork = ctx->dmalloc(wd + 16);
      std::vector<char> hwork(wh + 16);
      if (cusolverDnXsyevBatched(h, ctx->solver_params(), CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F,
                                 A, n, CUDA_R_64F, W, CUDA_R_64F, dwork, wd, hwork.data(), wh, dinf + ib, batch) !=
          CUSOLVER_STATUS_SUCCESS)
        throw Err(3, "syevBatched failed");
      ctx->sync();  // host workspace must outlive the call
      ctx->dfree(dwork);
      ib += (int)batch;
    }
    {
      std::vector<int> inf(ib + 1, 0);
      MPSG_CUDA(cudaMemcpyAsync(inf.data(), dinf, sizeof(int) * (ib + 1), cudaMemcpyDeviceToHost, ctx->stream));
      ctx->sync();
      for (int i = 0; i < ib; ++i)
        if (inf[i] != 0) throw Err(3, "batched eigensolver failed (info=" + std::to_string(inf[i]) + ")");
      MPSG_CUDA(cudaMemsetAsync(dinfo, 0, sizeof(int) * std::max<size_t>(s.size(), 1), ctx->stream));
    }
    std::vector<GramPost> post;
    for (size_t i = 0; i < s.size(); ++i) {
      const Sec& x = s[i];
      if (x.k == 0) continue;
      const int64_t nc = cls_of[i], pad = nc - x.ns;
      (void)pad;
      post.push_back(GramPost{dB + slot_off[i], dWv + lam_off[i], dV + x.offV, dS + x.offS, x.ns, (int32_t)nc,
                              (int32_t)nc});
    }
    if (!post.empty()) {
      GramPost* d = (GramPost*)ctx->dmalloc(sizeof(GramPost) * post.size());
      MPSG_CUDA(cudaMemcpyAsync(d, post.data(), sizeof(GramPost) * post.size(), cudaMemcpyHostToDevice, ctx->stream));
      launch_gram_post(d, (int)post.size(), ctx->stream);
      ctx->dfree(d);
    }
    left_vectors();
    orthonormalize_left();
    ctx->dfree(dB);
    ctx->dfree(dWv);
    ctx->dfree(dinf);
    fixphase();
  }

  // Density-matrix route on the library's own batched eigensolver (eig_f64.cu): Gram matrices by the
  // grouped FP64 GEMM, cluster-parallel Householder tridiagonalisation, bisection and inverse
  // iteration for the eigenpairs above the resolution floor, reflector back-transformation,
  // CholeskyQR of the eigenvector matrix (inverse iteration leaves ~eps lambda_max / gap between
  // close eigenvalues), then the left vectors as in the other density routes.  Sectors wider than the
  // cluster kernel's limit use run_gram.
  void run_gram_custom() {
    std::vector<int> idx;
    int nmax = 0;
    for (size_t i = 0; i < s.size(); ++i)
      if (s[i].k > 0) {
        idx.push_back((int)i);
        nmax = std::max(nmax, s[i].ns);
      }
    if (idx.empty()) return;
    MPSG_CHECK(nmax <= sytrd_max_n() && nmax <= 512, "density split: sector too wide");
    cudaStream_t st = ctx->stream;
    MPSG_CUDA(cudaMemsetAsync(dinfo, 0, sizeof(int) * std::max<size_t>(s.size(), 1), st));  // no solver status
    std::vector<int64_t> offG(s.size(), 0);
    int64_t oG = 0;
    for (int i : idx) {
      offG[i] = oG;
      oG += ((int64_t)s[i].ns * s[i].ns + kAlign - 1) / kAlign * kAlign;
    }
    double* dG = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oG, 2));
    // per sector: d (n), e (n), e^2 (n), tau (n), W (n), meta (4)
    double* dT = (double*)ctx->dmalloc(sizeof(double) * (size_t)(5 * nS + 4 * (int64_t)idx.size() + 2));
    double *dd = dT, *de = dT + nS, *de2 = dT + 2 * nS, *dtau = dT + 3 * nS, *dW = dT + 4 * nS,
           *dmeta = dT + 5 * nS;
    {
      GemmPlan g;
      for (int i : idx)
        g.add_problem(2, offG[i], s[i].ns, s[i].ns, s[i].ns, false,
                      {GSegH{0, 0, s[i].offM, s[i].offM, s[i].ms, s[i].ms, s[i].ms, 1, 0, 1.0}});
      g.upload(ctx);
      const double* bases[8] = {dM, nullptr, dG, nullptr, nullptr, nullptr, nullptr, nullptr};
      g.run(bases);
      std::vector<GramScaleOp> so;
      for (int i : idx) so.push_back(GramScaleOp{dG + offG[i], s[i].ns, s[i].ns});
      GramScaleOp* d = (GramScaleOp*)ctx->dmalloc(sizeof(GramScaleOp) * so.size());
      MPSG_CUDA(cudaMemcpyAsync(d, so.data(), sizeof(GramScaleOp) * so.size(), cudaMemcpyHostToDevice, st));
      launch_gram_scale(d, (int)so.size(), st);
      ctx->dfree(d);
    }
    // 1. tridiagonalisation, one launch per cluster size
    {
      std::map<int, std::vector<SytrdOp>> byCL;
      std::map<int, int> nmaxCL;
      for (int i : idx) {
        const int CL = sytrd_cluster_size(s[i].ns);
        byCL[CL].push_back(SytrdOp{dG + offG[i], dd + s[i].offS, de + s[i].offS, dtau + s[i].offS, s[i].ns, s[i].ns});
        nmaxCL[CL] = std::max(nmaxCL[CL], s[i].ns);
      }
      // the cluster sizes are independent launches: one worker stream each, largest clusters first
      std::vector<std::pair<int, SytrdOp*>> bufs;
      for (auto it = byCL.rbegin(); it != byCL.rend(); ++it) {
        SytrdOp* d = (SytrdOp*)ctx->dmalloc(sizeof(SytrdOp) * it->second.size());
        MPSG_CUDA(cudaMemcpyAsync(d, it->second.data(), sizeof(SytrdOp) * it->second.size(), cudaMemcpyHostToDevice, st));
        bufs.push_back({it->first, d});
      }
      const int nw = std::min<int>((int)bufs.size(), ctx->nworkers());
      ctx->fork(nw);
      for (size_t j = 0; j < bufs.size(); ++j)
        launch_sytrd(bufs[j].second, (int)byCL[bufs[j].first].size(), bufs[j].first, nmaxCL[bufs[j].first],
                     ctx->wstreams[j % nw]);
      ctx->join(nw);
      for (auto& b : bufs) ctx->dfree(b.second);
    }
    // 2./3. eigenvalues and eigenvectors of T, written in descending order into V's columns
    std::vector<TriOp> tops;
    std::vector<int> op_of, k_of;
    std::vector<int64_t> soff;
    int64_t scratch = 0;
    for (size_t t = 0; t < idx.size(); ++t) {
      const Sec& x = s[idx[t]];
      tops.push_back(TriOp{dd + x.offS, de + x.offS, de2 + x.offS, dW + x.offS, dV + x.offV, dmeta + 4 * t,
                           32.0 * x.ns * DBL_EPSILON, x.ns, x.ns});
      for (int k = 0; k < x.ns; ++k) {
        op_of.push_back((int)t);
        k_of.push_back(k);
        soff.push_back(scratch);
        scratch += 5 * (int64_t)x.ns;
      }
    }
    const int nthreads = (int)op_of.size();
    TriOp* dtops = (TriOp*)ctx->dmalloc(sizeof(TriOp) * tops.size());
    int* dmap = (int*)ctx->dmalloc(sizeof(int) * 2 * (size_t)nthreads);
    int64_t* dsoff = (int64_t*)ctx->dmalloc(sizeof(int64_t) * (size_t)nthreads);
    double* dscr = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(scratch, 2));
    MPSG_CUDA(cudaMemcpyAsync(dtops, tops.data(), sizeof(TriOp) * tops.size(), cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(dmap, op_of.data(), sizeof(int) * nthreads, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(dmap + nthreads, k_of.data(), sizeof(int) * nthreads, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(dsoff, soff.data(), sizeof(int64_t) * nthreads, cudaMemcpyHostToDevice, st));
    launch_tri_bounds(dtops, (int)tops.size(), st);
    launch_tri_bisect(dtops, dmap, dmap + nthreads, nthreads, 0.0, st);
    launch_tri_invit(dtops, dmap, dmap + nthreads, nthreads, 1e-12, dscr, dsoff, st);
    {  // resolved eigenpairs per sector (W is descending, -1 below the floor)
      int* dcnt = (int*)ctx->dmalloc(sizeof(int) * idx.size());
      launch_count_nonneg(dtops, (int)tops.size(), dcnt, st);
      std::vector<int> cnt(idx.size());
      MPSG_CUDA(cudaMemcpyAsync(cnt.data(), dcnt, sizeof(int) * cnt.size(), cudaMemcpyDeviceToHost, st));
      ctx->sync();
      ctx->dfree(dcnt);
      kr.assign(s.size(), 0);
      for (size_t t = 0; t < idx.size(); ++t) kr[idx[t]] = cnt[t];
    }
    // 4. back-transformation V = Q Z, blocks of 8 columns
    {
      std::vector<OrmtrOp> oo;
      for (int i : idx)
        for (int c0 = 0; c0 < kr[i]; c0 += 8)
          oo.push_back(OrmtrOp{dG + offG[i], dtau + s[i].offS, dW + s[i].offS, dV + s[i].offV, s[i].ns, s[i].ns,
                               s[i].ns, c0, std::min(c0 + 8, kr[i])});
      OrmtrOp* d = (OrmtrOp*)ctx->dmalloc(sizeof(OrmtrOp) * oo.size());
      MPSG_CUDA(cudaMemcpyAsync(d, oo.data(), sizeof(OrmtrOp) * oo.size(), cudaMemcpyHostToDevice, st));
      launch_ormtr(d, (int)oo.size(), nmax, st);
      ctx->dfree(d);
    }
    // 5. S = sqrt(W); the eigenvector matrix re-orthonormalised (CholeskyQR, two passes)
    {
      std::vector<EigPostOp> po;
      for (int i : idx) po.push_back(EigPostOp{dW + s[i].offS, dS + s[i].offS, s[i].ns});
      EigPostOp* d = (EigPostOp*)ctx->dmalloc(sizeof(EigPostOp) * po.size());
      MPSG_CUDA(cudaMemcpyAsync(d, po.data(), sizeof(EigPostOp) * po.size(), cudaMemcpyHostToDevice, st));
      launch_eig_post(d, (int)po.size(), st);
      ctx->dfree(d);
    }
    ctx->dfree(dscr);  // stream-ordered: released after the kernels above
    ctx->dfree(dsoff);
    ctx->dfree(dmap);
    ctx->dfree(dtops);
    ctx->dfree(dT);
    ctx->dfree(dG);
    std::vector<int> failed;
    cholqr(false, 2, &failed);
    left_vectors();
    orthonormalize_left(&failed);
    fixphase();
    if (!failed.empty()) {
      // singular vectors too dependent for CholeskyQR: these sectors are redone exactly
      std::sort(failed.begin(), failed.end());
      failed.erase(std::unique(failed.begin(), failed.end()), failed.end());
      g_split_fallbacks.fetch_add((int64_t)failed.size());
      if (std::getenv("MPSG_VERBOSE"))
        for (int i : failed)
          std::fprintf(stderr, "libmpsg: CholeskyQR failed in sector %d (%d x %d); redone on the Jacobi route\n", i,
                       s[i].ms, s[i].ns);
      for (int i : failed) kr[i] = s[i].k;
      run_jacobi(&failed);
    }
  }

  // Density-matrix route with one cuSOLVER syevd per sector, sectors spread over worker threads
  // that each own a stream and a solver handle (largest sectors first), so the solver's per-call
  // latency overlaps across sectors.
  void run_gram_mt() {
    const int nw = ctx->nworkers();
    int64_t oG = 0;
    std::vector<int64_t> offG(s.size());
    std::vector<int> order;
    for (size_t i = 0; i < s.size(); ++i) {
      offG[i] = oG;
      oG += ((int64_t)s[i].ns * s[i].ns + kAlign - 1) / kAlign * kAlign;
      if (s[i].k > 0) order.push_back((int)i);
    }
    std::sort(order.begin(), order.end(), [&](int a, int b) { return s[a].ns > s[b].ns; });
    double* dG = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oG, 2));
    double* dL = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(nS, 2));
    {
      GemmPlan g;
      for (int i : order)
        g.add_problem(2, offG[i], s[i].ns, s[i].ns, s[i].ns, false,
                      {GSegH{0, 0, s[i].offM, s[i].offM, s[i].ms, s[i].ms, s[i].ms, 1, 0, 1.0}});
      g.upload(ctx);
      const double* bases[8] = {dM, nullptr, dG, nullptr, nullptr, nullptr, nullptr, nullptr};
      g.run(bases);
    }
    cudaEvent_t ready;
    MPSG_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    MPSG_CUDA(cudaEventRecord(ready, ctx->stream));
    ctx->sync();  // G complete before the workers allocate workspaces on their streams
    std::vector<std::vector<int>> part(nw);
    for (size_t t = 0; t < order.size(); ++t) part[t % nw].push_back(order[t]);
    std::vector<std::string> errs(nw);
    std::vector<std::thread> th;
    for (int w = 0; w < nw; ++w) {
      if (part[w].empty()) continue;
      th.emplace_back([&, w]() {
        try {
          cudaStream_t st = ctx->wstreams[w];
          cusolverDnHandle_t h = ctx->whandles[w];
          MPSG_CUDA(cudaSetDevice(ctx->device));
          int lwork = 0;
          for (int i : part[w]) {
            int lw = 0;
            if (cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, s[i].ns, dG + offG[i],
                                            s[i].ns, dL + s[i].offS, &lw) != CUSOLVER_STATUS_SUCCESS)
              throw Err(3, "syevd_bufferSize failed");
            lwork = std::max(lwork, lw);
          }
          double* work = nullptr;
          MPSG_CUDA(cudaMallocAsync(&work, sizeof(double) * std::max(lwork, 2), st));
          for (int i : part[w])
            if (cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, s[i].ns, dG + offG[i], s[i].ns,
                                 dL + s[i].offS, work, lwork, dinfo + i) != CUSOLVER_STATUS_SUCCESS)
              throw Err(3, "syevd failed");
          MPSG_CUDA(cudaFreeAsync(work, st));
          MPSG_CUDA(cudaStreamSynchronize(st));
        } catch (const std::exception& e) {
          errs[w] = e.what();
        }
      });
    }
    for (auto& t : th) t.join();
    cudaEventDestroy(ready);
    for (auto& e : errs)
      if (!e.empty()) throw Err(3, e);
    std::vector<GramPost> post;
    for (int i : order)
      post.push_back(GramPost{dG + offG[i], dL + s[i].offS, dV + s[i].offV, dS + s[i].offS, s[i].ns, s[i].ns,
                              s[i].ns});
    if (!post.empty()) {
      GramPost* d = (GramPost*)ctx->dmalloc(sizeof(GramPost) * post.size());
      MPSG_CUDA(cudaMemcpyAsync(d, post.data(), sizeof(GramPost) * post.size(), cudaMemcpyHostToDevice, ctx->stream));
      launch_gram_post(d, (int)post.size(), ctx->stream);
      ctx->dfree(d);
    }
    left_vectors();
    orthonormalize_left();
    ctx->dfree(dG);
    ctx->dfree(dL);
    fixphase();
  }

  // density-matrix route with one cuSOLVER syevd per sector (kept for comparison)
  void run_gram_seq() {
    cusolverDnHandle_t h = ctx->svd_handle();
    int64_t oG = 0;
    std::vector<int64_t> offG(s.size());
    for (size_t i = 0; i < s.size(); ++i) {
      offG[i] = oG;
      oG += ((int64_t)s[i].ns * s[i].ns + kAlign - 1) / kAlign * kAlign;
    }
    double* dG = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oG, 2));
    double* dL = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(nS, 2));
    {  // G_i = Mst_i^T Mst_i
      GemmPlan g;
      for (size_t i = 0; i < s.size(); ++i) {
        const Sec& x = s[i];
        if (x.k == 0) continue;
        g.add_problem(2, offG[i], x.ns, x.ns, x.ns, false, {GSegH{0, 0, x.offM, x.offM, x.ms, x.ms, x.ms, 1, 0, 1.0}});
      }
      g.upload(ctx);
      const double* bases[8] = {dM, nullptr, dG, nullptr, nullptr, nullptr, nullptr, nullptr};
      g.run(bases);
    }
    int lwork = 0;
    for (size_t i = 0; i < s.size(); ++i) {
      if (s[i].k == 0) continue;
      int lw = 0;
      if (cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, s[i].ns, dG + offG[i], s[i].ns,
                                      dL + s[i].offS, &lw) != CUSOLVER_STATUS_SUCCESS)
        throw Err(3, "syevd_bufferSize failed");
      lwork = std::max(lwork, lw);
    }
    double* work = (double*)ctx->dmalloc(sizeof(double) * std::max(lwork, 2));
    for (size_t i = 0; i < s.size(); ++i) {
      if (s[i].k == 0) continue;
      if (cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, s[i].ns, dG + offG[i], s[i].ns,
                           dL + s[i].offS, work, lwork, dinfo + i) != CUSOLVER_STATUS_SUCCESS)
        throw Err(3, "syevd failed");
    }
    ctx->dfree(work);
    // s, 1/s and Vst (eigenvectors in descending order)
    std::vector<GramPost> post;
    for (size_t i = 0; i < s.size(); ++i) {
      if (s[i].k == 0) continue;
      post.push_back(
          GramPost{dG + offG[i], dL + s[i].offS, dV + s[i].offV, dS + s[i].offS, s[i].ns, s[i].ns, s[i].ns});
    }
    if (!post.empty()) {
      GramPost* d = (GramPost*)ctx->dmalloc(sizeof(GramPost) * post.size());
      MPSG_CUDA(cudaMemcpyAsync(d, post.data(), sizeof(GramPost) * post.size(), cudaMemcpyHostToDevice, ctx->stream));
      launch_gram_post(d, (int)post.size(), ctx->stream);
      ctx->dfree(d);
    }
    left_vectors();
    orthonormalize_left();
    ctx->dfree(dG);
    ctx->dfree(dL);
    fixphase();
  }

  // Ust = Mst Vst with unit columns; s_j = |Mst v_j| (columns whose eigenvalue was below the Gram
  // route's resolution keep s_j = 0 and a zero column).
  void left_vectors() {
    GemmPlan g;
    std::vector<ColNorm> cn;
    for (size_t i = 0; i < s.size(); ++i) {
      const Sec& x = s[i];
      if (x.k == 0) continue;
      if (kcols(i) > 0)
        g.add_problem(2, x.offU, x.ms, x.ms, kcols(i), false,
                      {GSegH{0, 1, x.offM, x.offV, x.ms, x.ns, x.ns, 0, 0, 1.0}});
      cn.push_back(ColNorm{dU + x.offU, dS + x.offS, x.ms, x.k, x.ms});  // clears the unresolved columns
    }
    g.upload(ctx);
    const double* bases[8] = {dM, dV, dU, nullptr, nullptr, nullptr, nullptr, nullptr};
    g.run(bases);
    if (!cn.empty()) {
      ColNorm* d = (ColNorm*)ctx->dmalloc(sizeof(ColNorm) * cn.size());
      MPSG_CUDA(cudaMemcpyAsync(d, cn.data(), sizeof(ColNorm) * cn.size(), cudaMemcpyHostToDevice, ctx->stream));
      launch_colnorm(d, (int)cn.size(), ctx->stream);
      ctx->dfree(d);
    }
  }

  // CholeskyQR of every sector's matrix X (columns in descending s order), in place: C = X^T X by the
  // grouped FP64 GEMM (zero columns get C_jj = 1 and stay zero), C = R^T R by the cluster Cholesky
  // kernel, X <- X R^-1 by blocked forward substitution.  left: X = Ust (ms x ns) and s_j is
  // multiplied by R_jj of the first pass (the norm of y_j after removing its components along the
  // larger pairs); otherwise X = Vst (ns x ns).  Each pass leaves X orthonormal to ~eps cond(X)^2.
  // failed (optional): sectors whose Cholesky met a non-positive pivot are appended instead of throwing
  // ub_rows: the left matrix holds U_B (ns rows, zero below): only its first ns rows are processed
  struct CholSide {
    bool left, scale_s, ub_rows;
  };
  void cholqr(bool left, int passes, std::vector<int>* failed = nullptr, bool scale_s = true, bool ub_rows = false) {
    cholqr_sides({CholSide{left, scale_s, ub_rows}}, passes, failed);
  }
  // CholeskyQR of several sides (U and / or V of every sector) in the same launches: the Gram
  // matrices in one grouped GEMM, the Cholesky factorisations in one launch per cluster size, the
  // blocked substitution in one GEMM + one substitution launch per 64-column block.
  void cholqr_sides(const std::vector<CholSide>& sides, int passes, std::vector<int>* failed) {
    struct Prob {
      int i;  // sector
      const CholSide* sd;
      int base;  // operand slot of X: 0 = dU, 3 = dV
      int64_t offX, offC, offR;
      int ldx, rows, kc;
    };
    std::vector<Prob> ps;
    int kmax = 0;
    int64_t oC = 0, oR = 0;
    for (const CholSide& sd : sides)
      for (size_t i = 0; i < s.size(); ++i) {
        const int kc = kcols(i);
        if (kc <= 0) continue;
        Prob p;
        p.i = (int)i;
        p.sd = &sd;
        p.base = sd.left ? 0 : 3;
        p.offX = sd.left ? s[i].offU : s[i].offV;
        p.ldx = sd.left ? s[i].ms : s[i].ns;
        p.rows = sd.left && !sd.ub_rows ? s[i].ms : s[i].ns;
        p.kc = kc;
        p.offC = oC;
        oC += ((int64_t)kc * kc + kAlign - 1) / kAlign * kAlign;
        p.offR = oR;
        oR += kc;
        ps.push_back(p);
        kmax = std::max(kmax, kc);
      }
    if (ps.empty()) return;
    MPSG_CHECK(kmax <= chol_max_k(), "CholeskyQR: sector wider than the cluster kernel's limit");
    cudaStream_t st = ctx->stream;
    double* dC = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oC, 2));
    double* dR = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oR, 2));  // 1 / R_jj
    int* dinf = (int*)ctx->dmalloc(sizeof(int) * ps.size());
    MPSG_CUDA(cudaMemsetAsync(dinf, 0, sizeof(int) * ps.size(), st));
    // Gram matrices C = X^T X, lower triangle only (all the Cholesky reads): per 64-column block j0,
    // rows j0.. of C
    GemmPlan g;
    for (const Prob& p : ps)
      for (int j0 = 0; j0 < p.kc; j0 += 64) {
        const int bw = std::min(64, p.kc - j0);
        const int64_t xo = p.offX + (int64_t)j0 * p.ldx;
        g.add_problem(2, p.offC + j0 + (int64_t)j0 * p.kc, p.kc, p.kc - j0, bw, false,
                      {GSegH{p.base, p.base, xo, xo, p.ldx, p.ldx, p.rows, 1, 0, 1.0}});
      }
    g.upload(ctx);
    std::vector<CholOp> zd;
    std::map<int, std::vector<CholQROp>> byCL[2];
    std::map<int, int> kmaxCL;
    for (size_t t = 0; t < ps.size(); ++t) {
      const Prob& p = ps[t];
      zd.push_back(CholOp{dC + p.offC, nullptr, p.kc, p.kc});
      const int CL = chol_cluster_size(p.kc);
      for (int pass = 0; pass < 2; ++pass)
        byCL[pass][CL].push_back(CholQROp{dC + p.offC, dR + p.offR,
                                          (pass == 0 && p.sd->left && p.sd->scale_s) ? dS + s[p.i].offS : nullptr,
                                          dinf + t, p.kc, p.kc});
      kmaxCL[CL] = std::max(kmaxCL[CL], p.kc);
    }
    // X <- X R^-1 by 64-column blocks: X_b -= X_<b R_<b,b (grouped GEMM), then X_b <- X_b R_bb^-1
    // (row-parallel substitution over 64 columns)
    constexpr int kTB = 64;
    const int nblk = (kmax + kTB - 1) / kTB;
    std::vector<std::unique_ptr<GemmPlan>> upd(nblk);
    std::vector<std::vector<TrsmRowsOp>> tr(nblk);
    for (int b = 0; b < nblk; ++b) {
      upd[b].reset(new GemmPlan());
      for (const Prob& p : ps) {
        const int c0 = b * kTB, kc = p.kc;
        if (c0 >= kc) continue;
        const int bw = std::min(kTB, kc - c0);
        double* X = p.base == 0 ? dU : dV;
        if (b > 0)
          upd[b]->add_problem(p.base, p.offX + (int64_t)c0 * p.ldx, p.ldx, p.rows, bw, true,
                              {GSegH{p.base, 1, p.offX, p.offC + (int64_t)c0 * kc, p.ldx, kc, c0, 0, 0, -1.0}});
        for (int r0 = 0; r0 < p.rows; r0 += 32)
          tr[b].push_back(TrsmRowsOp{X + p.offX + (int64_t)c0 * p.ldx, dC + p.offC + c0 + (int64_t)c0 * kc,
                                     dR + p.offR + c0, bw, p.ldx, kc, r0, std::min(r0 + 32, p.rows)});
      }
      upd[b]->upload(ctx);
    }
    size_t bytes = sizeof(CholOp) * zd.size() + 16;
    for (int b = 0; b < nblk; ++b) bytes += sizeof(TrsmRowsOp) * tr[b].size() + 16;
    for (int pass = 0; pass < 2; ++pass)
      for (auto& c : byCL[pass]) bytes += sizeof(CholQROp) * c.second.size() + 16;
    char* dops = (char*)ctx->dmalloc(bytes + 64);
    std::vector<char> hops(bytes + 64);
    size_t off = 0;
    auto put = [&](const void* p, size_t n) {
      std::memcpy(hops.data() + off, p, n);
      char* d = dops + off;
      off += (n + 15) / 16 * 16;
      return d;
    };
    CholOp* dzd = (CholOp*)put(zd.data(), sizeof(CholOp) * zd.size());
    std::vector<TrsmRowsOp*> dtr(nblk);
    for (int b = 0; b < nblk; ++b) dtr[b] = (TrsmRowsOp*)put(tr[b].data(), sizeof(TrsmRowsOp) * tr[b].size());
    std::map<int, CholQROp*> dch[2];
    for (int pass = 0; pass < 2; ++pass)
      for (auto& c : byCL[pass]) dch[pass][c.first] = (CholQROp*)put(c.second.data(), sizeof(CholQROp) * c.second.size());
    MPSG_CHECK(off <= bytes + 64, "CholeskyQR descriptor overflow");
    MPSG_CUDA(cudaMemcpyAsync(dops, hops.data(), off, cudaMemcpyHostToDevice, st));
    const double* bases[8] = {dU, dC, dC, dV, nullptr, nullptr, nullptr, nullptr};
    for (int pass = 0; pass < passes; ++pass) {
      split_mark(ctx, "CholeskyQR setup");
      g.run(bases);
      launch_chol_unit_zero_diag(dzd, (int)zd.size(), st);
      split_mark(ctx, "Gram matrices");
      const int which = pass == 0 ? 0 : 1;
      {  // cluster sizes concurrently on worker streams, largest first
        const int nw = std::min<int>((int)byCL[which].size(), ctx->nworkers());
        ctx->fork(nw);
        int j = 0;
        for (auto it = byCL[which].rbegin(); it != byCL[which].rend(); ++it, ++j)
          launch_chol(dch[which][it->first], (int)it->second.size(), it->first, kmaxCL[it->first],
                      ctx->wstreams[j % nw]);
        ctx->join(nw);
      }
      split_mark(ctx, "Cholesky");
      // X <- X R^-1 by blocked forward substitution: an explicit inverse of R (one GEMM) was measured
      // to lose orthonormality where kept values cluster (R ill-conditioned: error ~eps cond(R)^2),
      // which moved MIXED DMRG energies by 3e-10 relative
      for (int b = 0; b < nblk; ++b) {
        if (b > 0) upd[b]->run(bases);
        launch_trsm_rows(dtr[b], (int)tr[b].size(), kTB, st);
      }
    }
    std::vector<int> inf(ps.size(), 0);
    MPSG_CUDA(cudaMemcpyAsync(inf.data(), dinf, sizeof(int) * inf.size(), cudaMemcpyDeviceToHost, st));
    ctx->sync();
    ctx->dfree(dops);
    ctx->dfree(dinf);
    ctx->dfree(dR);
    ctx->dfree(dC);
    for (size_t t = 0; t < ps.size(); ++t)
      if (inf[t] != 0) {
        const Prob& p = ps[t];
        if (failed) {
          failed->push_back(p.i);
          continue;
        }
        const Sec& x = s[p.i];
        throw Err(3, std::string("CholeskyQR of ") + (p.sd->left ? "U" : "V") +
                         ": the Gram matrix of the singular vectors is not positive definite (sector " +
                         std::to_string(p.i) + " of " + std::to_string(s.size()) + ", " + std::to_string(x.ms) +
                         " x " + std::to_string(x.ns) + ", " + std::to_string(kcols(p.i)) +
                         " resolved columns, column " + std::to_string(inf[t] - 1) + ")");
      }
  }
  void orthonormalize_left(std::vector<int>* failed = nullptr) { cholqr(true, 1, failed); }

  void run(int method) {
    int nmax = 0;
    for (auto& x : s) nmax = std::max(nmax, x.k > 0 ? x.ns : 0);
    if (method >= 1 && method <= 3 && nmax > 512) method = 0;  // the density routes cover widths <= 512
    if (method == 4 && !bidiag_fits()) method = 0;
    if (method == 1) run_gram();
    else if (method == 2) run_gram_mt();
    else if (method == 3) run_gram_custom();
    else if (method == 4) run_bidiag_all();
    else run_jacobi();
  }

  // ---------------------------------------------------------------- bidiagonal route (svd_bidiag.cu)
  // Exact route on the library's own kernels: Householder bidiagonalisation of every sector on a
  // thread-block cluster, singular values by bisection on the Golub-Kahan tridiagonal, restricted to
  // the values at or above the truncation cut of each segment; singular vectors only for the values
  // the truncation keeps (inverse iteration, CholeskyQR of U_B and V_B, reflector back-transformation).
  struct Bidiag {
    double *d = nullptr, *e = nullptr, *tq = nullptr, *tp = nullptr, *Pr = nullptr, *b = nullptr, *b2 = nullptr,
           *meta = nullptr, *Z = nullptr, *xlo = nullptr, *Mcopy = nullptr;
    double2 *tqz = nullptr, *tpz = nullptr, *Prz = nullptr;  // complex mode
    int32_t *kcomp = nullptr, *seg = nullptr, *kept = nullptr, *opseg = nullptr;
    GkOp* ops_d = nullptr;
    std::vector<GkOp> ops;
    std::vector<int> idx;  // sector of each op
    std::vector<int64_t> offPr, offB;
  } bd;
  bool bidiag_fits() const {  // the cluster bidiagonalisation (shared- or global-memory variant)
    for (auto& x : s)
      if (x.k > 0 && (zM ? zgebrd_cluster_size(x.ms, x.ns) : gebrd_cluster_size(x.ms, x.ns)) == 0) return false;
    return true;
  }
  void bidiag_free() {
    for (double* p : {bd.d, bd.e, bd.tq, bd.tp, bd.Pr, bd.b, bd.b2, bd.meta, bd.Z, bd.xlo, bd.Mcopy}) ctx->dfree(p);
    for (double2* p : {bd.tqz, bd.tpz, bd.Prz}) ctx->dfree(p);
    ctx->dfree(bd.kcomp);  // kept and seg live in the same allocation
    ctx->dfree(bd.ops_d);
    bd = Bidiag();
  }
  // Singular values at or above each segment's cut into dS (descending, 0 past the computed ones).
  // seg_first[c] = first sector of segment c (size nseg + 1, ascending); chimax: values kept per
  // segment at most; floor_abs: values below it are never kept (the reference drops <= 1e-15).
  void bidiag_values(const std::vector<int>& seg_first, int chimax, double floor_abs) {
    cudaStream_t st = ctx->stream;
    MPSG_CUDA(cudaMemsetAsync(dinfo, 0, sizeof(int) * std::max<size_t>(s.size(), 1), st));
    MPSG_CUDA(cudaMemsetAsync(dS, 0, sizeof(double) * std::max<int64_t>(nS, 2), st));
    bd.idx.clear();
    int64_t oPr = 0, oB = 0;
    for (size_t i = 0; i < s.size(); ++i) {
      bd.offPr.push_back(oPr);
      bd.offB.push_back(oB);
      if (s[i].k == 0) continue;
      bd.idx.push_back((int)i);
      oPr += ((int64_t)s[i].ns * s[i].ns + kAlign - 1) / kAlign * kAlign;
      oB += 2 * (int64_t)s[i].ns;
    }
    const int nop = (int)bd.idx.size();
    if (nop == 0) return;
    auto alloc = [&](int64_t n) { return (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(n, 2)); };
    bd.d = alloc(nS);
    bd.e = alloc(nS);
    bd.tq = alloc(nS);
    bd.tp = alloc(nS);
    bd.Pr = alloc(oPr);
    bd.b = alloc(oB);
    bd.b2 = alloc(oB);
    bd.meta = alloc(4 * (int64_t)nop);
    const int nseg = (int)seg_first.size() - 1;
    bd.xlo = (double*)ctx->dmalloc(gk_cut_state_bytes() * std::max(nseg, 1));  // per-segment cut state
    // the sector matrices, kept for sectors whose vectors have to be redone on the Jacobi route (the
    // bidiagonalisation overwrites them with its reflectors)
    const int64_t nM = s.empty() || zM ? 0 : s.back().offM + (int64_t)s.back().ms * s.back().ns;
    bd.Mcopy = alloc(nM);
    if (nM) MPSG_CUDA(cudaMemcpyAsync(bd.Mcopy, dM, sizeof(double) * nM, cudaMemcpyDeviceToDevice, st));
    bd.kcomp = (int32_t*)ctx->dmalloc(sizeof(int32_t) * (size_t)nop * 3 + sizeof(int32_t) * (nseg + 1));
    bd.kept = bd.kcomp + nop;
    bd.opseg = bd.kept + nop;
    bd.seg = bd.opseg + nop;
    // 1. bidiagonalisation, one launch per cluster size on worker streams (largest clusters first);
    //    the largest global-memory sectors on two clusters each, in a launch of their own
    if (zM) {  // complex sectors: real bidiagonal, complex reflectors (shared-memory clusters only)
      auto zalloc = [&](int64_t n) { return (double2*)ctx->dmalloc(sizeof(double2) * std::max<int64_t>(n, 2)); };
      bd.tqz = zalloc(nS);
      bd.tpz = zalloc(nS);
      bd.Prz = zalloc(oPr);
      MPSG_CUDA(cudaMemsetAsync(bd.tpz, 0, sizeof(double2) * std::max<int64_t>(nS, 2), st));
      std::map<int, std::vector<ZGebrdOp>> byCL;
      std::map<int, size_t> smem;
      for (int i : bd.idx) {
        const Sec& x = s[i];
        const int CL = zgebrd_cluster_size(x.ms, x.ns);
        MPSG_CHECK(CL > 0, "complex bidiagonalisation: sector too large for the cluster");
        byCL[CL].push_back(ZGebrdOp{zM + x.offM, bd.d + x.offS, bd.e + x.offS, bd.tqz + x.offS, bd.tpz + x.offS,
                                    bd.Prz + bd.offPr[i], x.ms, x.ns, x.ms});
        smem[CL] = std::max(smem[CL], zgebrd_smem(x.ms, x.ns, CL));
      }
      std::vector<std::pair<int, ZGebrdOp*>> bufs;
      for (auto it = byCL.rbegin(); it != byCL.rend(); ++it) {
        ZGebrdOp* dp = (ZGebrdOp*)ctx->dmalloc(sizeof(ZGebrdOp) * it->second.size());
        MPSG_CUDA(cudaMemcpyAsync(dp, it->second.data(), sizeof(ZGebrdOp) * it->second.size(), cudaMemcpyHostToDevice, st));
        bufs.push_back({it->first, dp});
      }
      const int nw = std::min<int>((int)bufs.size(), ctx->nworkers());
      ctx->fork(nw);
      for (size_t j = 0; j < bufs.size(); ++j)
        launch_zgebrd(bufs[j].second, (int)byCL[bufs[j].first].size(), bufs[j].first, smem[bufs[j].first],
                      ctx->wstreams[j % nw]);
      ctx->join(nw);
      for (auto& b : bufs) ctx->dfree(b.second);
    } else {
      std::map<int, std::vector<GebrdOp>> byCL;
      std::map<int, size_t> smem;  // per cluster-size code, the largest of its sectors' needs
      std::vector<GebrdOp> mc;
      std::vector<int> mc_sec;
      size_t mc_smem = 0;
      for (int i : bd.idx) {
        const Sec& x = s[i];
        const GebrdOp op{dM + x.offM, bd.d + x.offS, bd.e + x.offS, bd.tq + x.offS, bd.tp + x.offS,
                         bd.Pr + bd.offPr[i], x.ms, x.ns, x.ms};
        if (gebrd_mc_clusters(x.ms, x.ns) == 2 && (int)mc.size() < gebrd_mc_capacity()) {
          mc.push_back(op);
          mc_sec.push_back(i);
          mc_smem = std::max(mc_smem, gebrd_mc_smem(x.ms, x.ns, 2));
          continue;
        }
        const int CL = gebrd_cluster_size(x.ms, x.ns);
        byCL[CL].push_back(op);
        smem[CL] = std::max(smem[CL], gebrd_smem(x.ms, x.ns, CL));
      }
      // two-cluster sectors: exchange buffers, barrier counters (zero) and the error flag
      double* mcbuf = nullptr;
      unsigned* mcctr = nullptr;
      if (!mc.empty()) {
        size_t nxg = 0;
        for (auto& op : mc) nxg += gebrd_mc_xg_doubles(op.m, 2);
        mcbuf = (double*)ctx->dmalloc(sizeof(double) * nxg + sizeof(unsigned) * (mc.size() + 1) + 16);
        mcctr = (unsigned*)(mcbuf + nxg);
        MPSG_CUDA(cudaMemsetAsync(mcctr, 0, sizeof(unsigned) * (mc.size() + 1), st));
        size_t o = 0;
        for (size_t t = 0; t < mc.size(); ++t) {
          mc[t].xg = mcbuf + o;
          o += gebrd_mc_xg_doubles(mc[t].m, 2);
          mc[t].ctr = mcctr + t;
          mc[t].err = (int*)(mcctr + mc.size());
        }
      }
      std::vector<std::pair<int, GebrdOp*>> bufs;
      if (!mc.empty()) bufs.push_back({-2, nullptr});
      for (auto it = byCL.rbegin(); it != byCL.rend(); ++it) bufs.push_back({it->first, nullptr});
      for (auto& b : bufs) {
        const std::vector<GebrdOp>& v = b.first == -2 ? mc : byCL[b.first];
        b.second = (GebrdOp*)ctx->dmalloc(sizeof(GebrdOp) * v.size());
        MPSG_CUDA(cudaMemcpyAsync(b.second, v.data(), sizeof(GebrdOp) * v.size(), cudaMemcpyHostToDevice, st));
      }
      const int nw = std::min<int>((int)bufs.size(), ctx->nworkers());
      ctx->fork(nw);
      for (size_t j = 0; j < bufs.size(); ++j) {
        if (bufs[j].first == -2) launch_gebrd_mc(bufs[j].second, (int)mc.size(), 2, mc_smem, ctx->wstreams[j % nw]);
        else
          launch_gebrd(bufs[j].second, (int)byCL[bufs[j].first].size(), bufs[j].first, smem[bufs[j].first],
                       ctx->wstreams[j % nw]);
      }
      if (on_bidiag) on_bidiag(ctx->fork_event);  // ready together with the launches above
      ctx->join(nw);
      if (!mc.empty()) {
        // a two-cluster sector whose barrier wait expired is redone on one cluster from the copy
        int err = 0;
        MPSG_CUDA(cudaMemcpyAsync(&err, mcctr + mc.size(), sizeof(int), cudaMemcpyDeviceToHost, st));
        ctx->sync();
        if (err) {
          g_split_fallbacks.fetch_add((int64_t)mc.size());
          if (std::getenv("MPSG_VERBOSE"))
            std::fprintf(stderr, "libmpsg: two-cluster bidiagonalisation timed out; redone on one cluster\n");
          std::map<int, std::vector<GebrdOp>> re;
          std::map<int, size_t> resm;
          for (size_t t = 0; t < mc.size(); ++t) {
            const Sec& x = s[mc_sec[t]];
            MPSG_CUDA(cudaMemcpyAsync(dM + x.offM, bd.Mcopy + x.offM, sizeof(double) * (size_t)x.ms * x.ns,
                                      cudaMemcpyDeviceToDevice, st));
            const int CL = gebrd_cluster_size(x.ms, x.ns);
            GebrdOp op = mc[t];
            op.xg = nullptr;
            op.ctr = nullptr;
            op.err = nullptr;
            re[CL].push_back(op);
            resm[CL] = std::max(resm[CL], gebrd_smem(x.ms, x.ns, CL));
          }
          for (auto& kv : re) {
            GebrdOp* dp = (GebrdOp*)ctx->dmalloc(sizeof(GebrdOp) * kv.second.size());
            MPSG_CUDA(cudaMemcpyAsync(dp, kv.second.data(), sizeof(GebrdOp) * kv.second.size(), cudaMemcpyHostToDevice,
                                      st));
            launch_gebrd(dp, (int)kv.second.size(), kv.first, resm[kv.first], st);
            ctx->dfree(dp);
          }
        }
        ctx->dfree(mcbuf);
      }
      for (auto& b : bufs) ctx->dfree(b.second);
    }
    split_mark(ctx, "bidiagonalisation");
    // 2.-4. Golub-Kahan matrices, the cut of each segment, the singular values above it
    std::vector<int32_t> segop(nseg + 1, 0);
    {
      int t = 0;
      for (int c = 0; c <= nseg; ++c) {
        while (t < nop && bd.idx[t] < seg_first[c]) ++t;
        segop[c] = t;
      }
      segop[nseg] = nop;
    }
    std::vector<int32_t> seg_of_op(nop, 0);
    for (int c = 0; c < nseg; ++c)
      for (int t = segop[c]; t < segop[c + 1]; ++t) seg_of_op[t] = c;
    bd.ops.clear();
    std::vector<int32_t> op_of, k_of;
    for (int t = 0; t < nop; ++t) {
      const Sec& x = s[bd.idx[t]];
      GkOp g;
      g.d = bd.d + x.offS;
      g.e = bd.e + x.offS;
      g.b = bd.b + bd.offB[bd.idx[t]];
      g.b2 = bd.b2 + bd.offB[bd.idx[t]];
      g.S = dS + x.offS;
      g.Z = nullptr;
      g.meta = bd.meta + 4 * t;
      g.xlo = gk_cut_xlo(bd.xlo, seg_of_op[t]);
      g.kcomp = bd.kcomp + t;
      g.n = x.ns;
      g.ldz = 2 * x.ns;
      bd.ops.push_back(g);
      for (int k = 0; k < x.ns; ++k) {
        op_of.push_back(t);
        k_of.push_back(k);
      }
    }
    const int nth = (int)op_of.size();
    bd.ops_d = (GkOp*)ctx->dmalloc(sizeof(GkOp) * nop);
    int32_t* dmap = (int32_t*)ctx->dmalloc(sizeof(int32_t) * 2 * (size_t)nth);
    MPSG_CUDA(cudaMemcpyAsync(bd.ops_d, bd.ops.data(), sizeof(GkOp) * nop, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(bd.seg, segop.data(), sizeof(int32_t) * (nseg + 1), cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(bd.opseg, seg_of_op.data(), sizeof(int32_t) * nop, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(dmap, op_of.data(), sizeof(int32_t) * nth, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(dmap + nth, k_of.data(), sizeof(int32_t) * nth, cudaMemcpyHostToDevice, st));
    launch_gk_setup(bd.ops_d, nop, st);
    launch_gk_cut(bd.ops_d, bd.seg, bd.opseg, nop, nseg, chimax, floor_abs, bd.xlo, st);
    launch_gk_bisect(bd.ops_d, dmap, dmap + nth, nth, st);
    ctx->dfree(dmap);
    split_mark(ctx, "cut + bisection");
  }
  // Singular vectors of the kept values (kept[i] per sector, from the truncation): U (ms x kept) and
  // V (ns x kept) in dU / dV, FixPhase applied.  Sectors whose vectors CholeskyQR cannot
  // orthonormalise are redone on the exact Jacobi route.
  void bidiag_vectors(const std::vector<int32_t>& kept) {
    cudaStream_t st = ctx->stream;
    const int nop = (int)bd.idx.size();
    kr.assign(s.size(), 0);
    for (int i : bd.idx) kr[i] = kept[i];
    if (nop == 0) return;
    std::vector<int32_t> kk(nop);
    int64_t oZ = 0;
    std::vector<int64_t> offZ(nop);
    std::vector<int32_t> op_of, k_of;
    int lenmax = 0, nmax2 = 2;
    for (int t = 0; t < nop; ++t) {
      const Sec& x = s[bd.idx[t]];
      kk[t] = kept[bd.idx[t]];
      offZ[t] = oZ;
      oZ += 2 * (int64_t)x.ns * kk[t];
      for (int k = 0; k < kk[t]; ++k) {
        op_of.push_back(t);
        k_of.push_back(k);
      }
      lenmax = std::max(lenmax, x.ms);
      if (kk[t] > 0) nmax2 = std::max(nmax2, 2 * x.ns);
    }
    const int nth = (int)op_of.size();
    if (nth == 0) return;
    bd.Z = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oZ, 2));
    for (int t = 0; t < nop; ++t) bd.ops[t].Z = bd.Z + offZ[t];
    double* dscr = (double*)ctx->dmalloc(sizeof(double) * 6 * (size_t)nmax2 * nth);
    int32_t* dmap = (int32_t*)ctx->dmalloc(sizeof(int32_t) * 2 * (size_t)nth);
    MPSG_CUDA(cudaMemcpyAsync(bd.ops_d, bd.ops.data(), sizeof(GkOp) * nop, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(bd.kept, kk.data(), sizeof(int32_t) * nop, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(dmap, op_of.data(), sizeof(int32_t) * nth, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(dmap + nth, k_of.data(), sizeof(int32_t) * nth, cudaMemcpyHostToDevice, st));
    // 5./6. eigenvectors of T for the kept values, split into U_B (first ns rows of U) and V_B
    split_mark(ctx, "truncation");
    launch_gk_invit(bd.ops_d, dmap, dmap + nth, bd.kept, nth, nmax2, dscr, st);
    split_mark(ctx, "inverse iteration");
    {
      std::vector<GkVecOp> vo;
      for (int t = 0; t < nop; ++t) {
        const Sec& x = s[bd.idx[t]];
        for (int k = 0; k < kk[t]; ++k)
          vo.push_back(GkVecOp{bd.Z + offZ[t], dU + x.offU, dV + x.offV, x.ns, x.ms, 2 * x.ns, x.ms, x.ns, k});
      }
      GkVecOp* dv = (GkVecOp*)ctx->dmalloc(sizeof(GkVecOp) * vo.size());
      MPSG_CUDA(cudaMemcpyAsync(dv, vo.data(), sizeof(GkVecOp) * vo.size(), cudaMemcpyHostToDevice, st));
      launch_gk_vectors(dv, (int)vo.size(), st);
      ctx->dfree(dv);
    }
    ctx->dfree(dscr);
    ctx->dfree(dmap);
    // orthonormal to rounding: inverse iteration leaves ~eps ||T|| / gap between close values (far
    // below one for values bisection tells apart, which the groups above cover), so one CholeskyQR pass
    // (error ~eps cond^2) suffices; U_B's rows past ns are zero and are left out
    std::vector<int> failed;
    for (int i : bd.idx)  // more kept vectors than the cluster Cholesky takes: the Jacobi route below
      if (kr[i] > chol_max_k()) {
        failed.push_back(i);
        kr[i] = 0;
      }
    split_mark(ctx, "vectors of T");
    cholqr_sides({CholSide{true, false, true}, CholSide{false, false, false}}, 1, &failed);
    split_mark(ctx, "CholeskyQR");
    // 7. U = Q [U_B; 0], V = P V_B
    if (zM) {  // complex reflectors into the caller's complex outputs
      std::vector<ZReflOp> ro;
      const int cb = zapply_refl_cols_per_block(lenmax);
      for (int i : bd.idx) {
        const Sec& x = s[i];
        for (int c0 = 0; c0 < kr[i]; c0 += cb) {
          const int c1 = std::min(c0 + cb, kr[i]);
          ro.push_back(ZReflOp{zM + x.offM, bd.tqz + x.offS, dU + x.offU, zUo[i].first, x.ms, x.ns, 0, x.ms, x.ms,
                               zUo[i].second, x.ns, c0, c1});
          ro.push_back(ZReflOp{bd.Prz + bd.offPr[i], bd.tpz + x.offS, dV + x.offV, zVo[i].first, x.ns, x.ns - 1, 1,
                               x.ns, x.ns, zVo[i].second, x.ns, c0, c1});
        }
      }
      if (!ro.empty()) {
        ZReflOp* dr = (ZReflOp*)ctx->dmalloc(sizeof(ZReflOp) * ro.size());
        MPSG_CUDA(cudaMemcpyAsync(dr, ro.data(), sizeof(ZReflOp) * ro.size(), cudaMemcpyHostToDevice, st));
        launch_zapply_refl(dr, (int)ro.size(), lenmax, st);
        ctx->dfree(dr);
      }
      zfailed = !failed.empty();
      bidiag_free();
      return;
    }
    {
      std::vector<ReflOp> ro;
      for (int i : bd.idx) {
        const Sec& x = s[i];
        const int cb = apply_refl_cols_per_block(lenmax);
        for (int c0 = 0; c0 < kr[i]; c0 += cb) {
          const int c1 = std::min(c0 + cb, kr[i]);
          ro.push_back(ReflOp{dM + x.offM, bd.tq + x.offS, dU + x.offU, x.ms, x.ns, 0, x.ms, x.ms, c0, c1});
          ro.push_back(ReflOp{bd.Pr + bd.offPr[i], bd.tp + x.offS, dV + x.offV, x.ns, x.ns - 1, 1, x.ns, x.ns, c0, c1});
        }
      }
      if (!ro.empty()) {
        ReflOp* dr = (ReflOp*)ctx->dmalloc(sizeof(ReflOp) * ro.size());
        MPSG_CUDA(cudaMemcpyAsync(dr, ro.data(), sizeof(ReflOp) * ro.size(), cudaMemcpyHostToDevice, st));
        launch_apply_refl(dr, (int)ro.size(), lenmax, st);
        ctx->dfree(dr);
      }
    }
    split_mark(ctx, "back-transformation");
    fixphase();
    if (!failed.empty()) {
      std::sort(failed.begin(), failed.end());
      failed.erase(std::unique(failed.begin(), failed.end()), failed.end());
      g_split_fallbacks.fetch_add((int64_t)failed.size());
      if (std::getenv("MPSG_VERBOSE"))
        for (int i : failed)
          std::fprintf(stderr, "libmpsg: bidiagonal SVD vectors of sector %d (%d x %d) redone on the Jacobi route\n", i,
                       s[i].ms, s[i].ns);
      for (int i : failed) {  // the sector matrix back from the copy, all its columns from gesvdj
        MPSG_CUDA(cudaMemcpyAsync(dM + s[i].offM, bd.Mcopy + s[i].offM, sizeof(double) * (size_t)s[i].ms * s[i].ns,
                                  cudaMemcpyDeviceToDevice, st));
        kr[i] = s[i].k;
      }
      run_jacobi(&failed);
    }
    bidiag_free();
  }
  // the whole SVD on the bidiagonal route without truncation: every value >= 1e-16 with its vectors
  void run_bidiag_all() {
    std::vector<int> seg_first = {0, (int)s.size()};
    bidiag_values(seg_first, INT32_MAX, 1e-16);
    std::vector<int32_t> kc(bd.idx.size());
    if (!kc.empty())
      MPSG_CUDA(cudaMemcpyAsync(kc.data(), bd.kcomp, sizeof(int32_t) * kc.size(), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    std::vector<int32_t> kept(s.size(), 0);
    for (size_t t = 0; t < bd.idx.size(); ++t) kept[bd.idx[t]] = kc[t];
    bidiag_vectors(kept);
  }

  // only (optional): the sectors to decompose (the others keep their factors)
  void run_jacobi(const std::vector<int>* only = nullptr) {
    cusolverDnHandle_t h = ctx->svd_handle();
    std::vector<char> sel(s.size(), only ? 0 : 1);
    if (only)
      for (int i : *only) sel[i] = 1;
    int lwork = 0;
    for (size_t i = 0; i < s.size(); ++i) {
      const Sec& x = s[i];
      if (x.k == 0 || !sel[i]) continue;
      int lw = 0;
      cusolverStatus_t st = cusolverDnDgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, x.ms, x.ns, dM + x.offM, x.ms,
                                                         dS + x.offS, dU + x.offU, x.ms, dV + x.offV, x.ns, &lw,
                                                         ctx->svdp);
      if (st != CUSOLVER_STATUS_SUCCESS) throw Err(3, "gesvdj_bufferSize failed");
      lwork = std::max(lwork, lw);
    }
    double* work = (double*)ctx->dmalloc(sizeof(double) * std::max(lwork, 2));
    for (size_t i = 0; i < s.size(); ++i) {
      const Sec& x = s[i];
      if (x.k == 0 || !sel[i]) continue;
      cusolverStatus_t st = cusolverDnDgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, x.ms, x.ns, dM + x.offM, x.ms,
                                              dS + x.offS, dU + x.offU, x.ms, dV + x.offV, x.ns, work, lwork,
                                              dinfo + i, ctx->svdp);
      if (st != CUSOLVER_STATUS_SUCCESS) throw Err(3, "gesvdj failed");
    }
    ctx->dfree(work);
    fixphase();
  }
  void fixphase() {
    std::vector<PhaseOp> ph;
    int maxk = 0;
    for (size_t i = 0; i < s.size(); ++i) {
      if (s[i].k == 0) continue;
      PhaseOp p;
      int lq, lp;
      p.Qm = Qp((int)i, &lq);
      p.Pm = Pp((int)i, &lp);
      p.m = s[i].m;
      p.n = s[i].n;
      p.k = kcols(i);
      p.ldq = lq;
      p.ldp = lp;
      ph.push_back(p);
      maxk = std::max(maxk, kcols(i));
    }
    if (!ph.empty()) {
      PhaseOp* d = (PhaseOp*)ctx->dmalloc(sizeof(PhaseOp) * ph.size());
      MPSG_CUDA(cudaMemcpyAsync(d, ph.data(), sizeof(PhaseOp) * ph.size(), cudaMemcpyHostToDevice, ctx->stream));
      launch_fixphase(d, (int)ph.size(), maxk, ctx->stream);
      ctx->dfree(d);
    }
  }
  void check_info() {
    std::vector<int> info(s.size());
    if (s.empty()) return;
    MPSG_CUDA(cudaMemcpyAsync(info.data(), dinfo, sizeof(int) * s.size(), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    for (size_t i = 0; i < s.size(); ++i)
      if (s[i].k > 0 && info[i] != 0)
        throw Err(3, "SVD solver did not converge (info=" + std::to_string(info[i]) + ")");
  }
};

// ============================================================================ split
bool zsvd_bidiag(Ctx* ctx, const std::vector<ZSvdSec>& secs, double2* zM, double* dS) {
  if (secs.empty()) return true;
  SvdBatch sv(ctx);
  std::vector<std::pair<int, int>> mn;
  for (auto& z : secs) {
    MPSG_CHECK(z.ms >= z.ns, "complex SVD: sectors are stored tall");
    mn.push_back({z.ms, z.ns});
  }
  sv.plan(mn);
  sv.zM = zM;
  for (size_t i = 0; i < secs.size(); ++i) {
    sv.s[i].offM = secs[i].offM;  // the caller's layout of the complex matrices
    sv.zUo.push_back({secs[i].U, secs[i].ldu});
    sv.zVo.push_back({secs[i].V, secs[i].ldv});
    if (secs[i].ns > 0) {
      MPSG_CUDA(cudaMemsetAsync(secs[i].U, 0, sizeof(double2) * (size_t)secs[i].ldu * secs[i].ns, ctx->stream));
      MPSG_CUDA(cudaMemsetAsync(secs[i].V, 0, sizeof(double2) * (size_t)secs[i].ldv * secs[i].ns, ctx->stream));
    }
  }
  if (!sv.bidiag_fits()) {
    g_split_fallbacks.fetch_add(1);
    return false;
  }
  sv.run_bidiag_all();
  if (sv.zfailed) {
    g_split_fallbacks.fetch_add(1);
    return false;
  }
  if (sv.nS) MPSG_CUDA(cudaMemcpyAsync(dS, sv.dS, sizeof(double) * sv.nS, cudaMemcpyDeviceToDevice, ctx->stream));
  ctx->sync();
  return true;
}

static SplitResult split2_impl(Ctx* ctx, const Tensor& th, const ItoKey& ik0, const ItoKey& ik1, int chimax,
                               bool doTrunc, double tr_weight, bool normalize, int absorb, const std::vector<Q>* seg_q0,
                               const std::vector<int>* seg_absorb, const std::function<void(cudaEvent_t)>& on_bidiag) {
  struct SecInfo {
    std::map<uint32_t, std::pair<int, int>> rx, ry;  // index -> (start, size)
    std::vector<int> blocks;
  };
  std::map<Q, SecInfo> secs;
  for (int i = 0; i < (int)th.b.size(); ++i) {
    const Block& b = th.b[i];
    const Q qc = b.k.q0 + qat(ik0, b.k.p0);
    SecInfo& s = secs[qc];
    s.blocks.push_back(i);
    s.rx[b.k.p0] = {0, b.r};
    s.ry[b.k.p1] = {0, b.c};
  }
  std::vector<Q> qcs;
  std::vector<std::pair<int, int>> mn;
  for (auto& x : secs) {
    int st = 0;
    for (auto& r : x.second.rx) { r.second.first = st; st += r.second.second; }
    int m = st;
    st = 0;
    for (auto& r : x.second.ry) { r.second.first = st; st += r.second.second; }
    qcs.push_back(x.first);
    mn.push_back({m, st});
  }
  if (!chimax && doTrunc) chimax = 100;
  if (!chimax && !doTrunc) chimax = 200;
  SvdBatch sv(ctx);
  sv.on_bidiag = on_bidiag;
  sv.plan(mn);
  std::vector<CopyOp> gops;
  for (size_t si = 0; si < qcs.size(); ++si) {
    SecInfo& s = secs[qcs[si]];
    for (int bi : s.blocks) {
      const Block& b = th.b[bi];
      gops.push_back(sv.gather_op((int)si, th.d + b.off, b.r, b.c, s.rx.at(b.k.p0).first, s.ry.at(b.k.p1).first));
    }
  }
  run_copyops(ctx, gops);
  // global truncation; with segments (a direct sum of independent chains, chain c holding the
  // centre charges in [seg_q0[c], seg_q0[c + 1])) one truncation per chain over its own sectors
  const int nseg = seg_q0 ? (int)seg_q0->size() : 1;
  std::vector<int> seg_of_sec(qcs.size(), 0), s0(nseg + 1, (int)qcs.size());
  if (seg_q0) {
    for (size_t si = 0; si < qcs.size(); ++si) {
      const int c = (int)(std::upper_bound(seg_q0->begin(), seg_q0->end(), qcs[si]) - seg_q0->begin()) - 1;
      MPSG_CHECK(c >= 0, "centre charge below the first segment");
      MPSG_CHECK(si == 0 || c >= seg_of_sec[si - 1], "segments out of charge order");
      seg_of_sec[si] = c;
    }
  }
  for (int si = (int)qcs.size() - 1; si >= 0; --si) s0[seg_of_sec[si]] = si;
  for (int c = nseg - 1; c >= 0; --c) s0[c] = std::min(s0[c], s0[c + 1]);
  // the bidiagonal route computes only the values at or above each segment's truncation cut here, and
  // the singular vectors of the kept ones after the truncation; every other route decomposes fully
  const bool bidiag = ctx->svd_method == 4 && sv.bidiag_fits() && !sv.s.empty();
  split_mark(ctx, "gather");
  // truncate(tr_weight, chimax) measures the discarded weight against the norm of ALL values
  // (src/BlockTensor.hpp:90-108), so with doTrunc every value above the floor is computed (no
  // chimax cut); truncate(chimax) needs only the values above the top-chimax cut
  if (bidiag) sv.bidiag_values(s0, doTrunc ? std::numeric_limits<int>::max() : chimax, 1e-15);
  else sv.run(ctx->svd_method == 4 ? 0 : ctx->svd_method);
  std::vector<int32_t> sec_of(sv.nS);
  for (size_t si = 0; si < qcs.size(); ++si)
    for (int j = 0; j < sv.s[si].k; ++j) sec_of[sv.s[si].offS + j] = (int32_t)si - s0[seg_of_sec[si]];
  const int nS = (int)sv.nS;
  int32_t* dsec = (int32_t*)ctx->dmalloc(sizeof(int32_t) * std::max(nS, 1) * 3 + sizeof(int32_t) * (qcs.size() + 1) +
                                         sizeof(double) * 3 * (nseg + 1));
  int32_t* drank = dsec + std::max(nS, 1);
  int32_t* dcnt = drank + 2 * std::max(nS, 1);
  double* dout3 = (double*)(((uintptr_t)(dcnt + qcs.size() + 1) + 7) & ~(uintptr_t)7);
  if (nS) MPSG_CUDA(cudaMemcpyAsync(dsec, sec_of.data(), sizeof(int32_t) * nS, cudaMemcpyHostToDevice, ctx->stream));
  MPSG_CUDA(cudaMemsetAsync(dout3, 0, sizeof(double) * 3 * nseg, ctx->stream));
  for (int c = 0; c < nseg; ++c) {
    const int a = s0[c], b = s0[c + 1];
    if (a >= b) continue;
    const int v0 = (int)sv.s[a].offS, v1 = (int)(sv.s[b - 1].offS + sv.s[b - 1].k);
    launch_truncate(sv.dS + v0, v1 - v0, dsec + v0, b - a, chimax, doTrunc ? 1 : 0, tr_weight, drank + 2 * v0,
                    dcnt + a, dout3 + 3 * c, ctx->stream);
  }
  std::vector<int32_t> counts(qcs.size() + 1);
  std::vector<double> out3(3 * nseg);
  MPSG_CUDA(cudaMemcpyAsync(counts.data(), dcnt, sizeof(int32_t) * qcs.size(), cudaMemcpyDeviceToHost, ctx->stream));
  MPSG_CUDA(cudaMemcpyAsync(out3.data(), dout3, sizeof(double) * 3 * nseg, cudaMemcpyDeviceToHost, ctx->stream));
  sv.check_info();  // syncs
  std::vector<double> inv_norm_seg(nseg, 1.0);
  SplitResult R;
  R.tw_seg.resize(nseg);
  R.chi_seg.resize(nseg);
  for (int c = 0; c < nseg; ++c) {
    R.tw_seg[c] = out3[3 * c];
    R.chi_seg[c] = (int)out3[3 * c + 1];
    if (normalize) inv_norm_seg[c] = out3[3 * c + 2];
  }
  const double tw = R.tw_seg[0];
  const int chi = R.chi_seg[0];
  ctx->dfree(dsec);
  if (bidiag) {
    std::vector<int32_t> kept(qcs.size());
    for (size_t si = 0; si < qcs.size(); ++si) kept[si] = std::max(counts[si], 0);
    sv.bidiag_vectors(kept);
  }
  split_mark(ctx, "FixPhase");
  // result layouts (dropDangling: sectors without kept values vanish, blocks cut to the kept count)
  Layout lu, lv, ll;
  for (size_t si = 0; si < qcs.size(); ++si) {
    const int c = counts[si];
    if (c <= 0) continue;
    const Q qc = qcs[si];
    SecInfo& s = secs[qc];
    for (auto& r : s.rx) lu.add(K1(qc - qat(ik0, r.first), qc, r.first), r.second.second, c);
    for (auto& r : s.ry) lv.add(K1(qc, qc + qat(ik1, r.first), r.first), c, r.second.second);
    ll.add(K1(qc, qc, 0), c, 1);
  }
  lu.finalize();
  lv.finalize();
  ll.finalize();
  R.U = make_tensor(ctx, 1, lu, false);
  R.Vt = make_tensor(ctx, 1, lv, false);
  R.lam = make_tensor(ctx, 0, ll, true);
  R.tw = tw;
  R.chi = chi;
  std::vector<CopyOp> ops;
  for (size_t si = 0; si < qcs.size(); ++si) {
    const int c = counts[si];
    if (c <= 0) continue;
    const Q qc = qcs[si];
    SecInfo& s = secs[qc];
    const double inv_norm = inv_norm_seg[seg_of_sec[si]];
    const int ab = seg_absorb ? seg_absorb->at(seg_of_sec[si]) : absorb;
    int ldq, ldp;
    double* Qm = sv.Qp((int)si, &ldq);
    double* Pm = sv.Pp((int)si, &ldp);
    const double* Sv = sv.dS + sv.s[si].offS;
    for (auto& r : s.rx) {
      const int ob = R.U->find(K1(qc - qat(ik0, r.first), qc, r.first));
      CopyOp o;
      o.src = Qm + r.second.first;
      o.dst = R.U->d + R.U->b[ob].off;
      o.rs = nullptr;
      o.cs = ab < 0 ? Sv : nullptr;
      o.rows = r.second.second;
      o.cols = c;
      o.lds = ldq;
      o.ldd = r.second.second;
      o.trans = 0;
      o.scale = ab < 0 ? inv_norm : 1.0;
      ops.push_back(o);
    }
    for (auto& r : s.ry) {
      const int ob = R.Vt->find(K1(qc, qc + qat(ik1, r.first), r.first));
      CopyOp o;
      o.src = Pm + r.second.first;
      o.dst = R.Vt->d + R.Vt->b[ob].off;
      o.rs = ab > 0 ? Sv : nullptr;
      o.cs = nullptr;
      o.rows = c;
      o.cols = r.second.second;
      o.lds = ldp;
      o.ldd = c;
      o.trans = 1;
      o.scale = ab > 0 ? inv_norm : 1.0;
      ops.push_back(o);
    }
    const int ol = R.lam->find(K1(qc, qc, 0));
    CopyOp o;
    o.src = Sv;
    o.dst = R.lam->d + R.lam->b[ol].off;
    o.rs = nullptr;
    o.cs = nullptr;
    o.rows = c;
    o.cols = 1;
    o.lds = c;
    o.ldd = c;
    o.trans = 0;
    o.scale = inv_norm;
    ops.push_back(o);
  }
  run_copyops(ctx, ops);
  return R;
}

SplitResult split2(Ctx* ctx, const Tensor& th, const ItoKey& ik0, const ItoKey& ik1, int chimax, bool doTrunc,
                   double tr_weight, bool normalize, int absorb, const std::vector<Q>* seg_q0,
                   const std::vector<int>* seg_absorb, const std::function<void(cudaEvent_t)>& on_bidiag) {
  static const bool timing = std::getenv("MPSG_SPLIT_TIMING") != nullptr;
  if (!timing || g_split_marks)
    return split2_impl(ctx, th, ik0, ik1, chimax, doTrunc, tr_weight, normalize, absorb, seg_q0, seg_absorb, on_bidiag);
  std::vector<std::pair<const char*, cudaEvent_t>> marks;
  g_split_marks = &marks;
  split_mark(ctx, "start");
  SplitResult r;
  try {
    r = split2_impl(ctx, th, ik0, ik1, chimax, doTrunc, tr_weight, normalize, absorb, seg_q0, seg_absorb, on_bidiag);
  } catch (...) {
    g_split_marks = nullptr;
    for (auto& m : marks) cudaEventDestroy(m.second);
    throw;
  }
  split_mark(ctx, "scatter");
  g_split_marks = nullptr;
  ctx->sync();
  std::string line = "libmpsg: split stages (ms):";
  for (size_t k = 1; k < marks.size(); ++k) {
    float ms = 0;
    cudaEventElapsedTime(&ms, marks[k - 1].second, marks[k].second);
    char buf[96];
    std::snprintf(buf, sizeof(buf), " %s %.2f", marks[k].first, ms);
    line += buf;
  }
  std::fprintf(stderr, "%s\n", line.c_str());
  for (auto& m : marks) cudaEventDestroy(m.second);
  return r;
}

// ============================================================================ right canonicalisation
void prepare_matrix_r(Ctx* ctx, TensorP* BL1, TensorP& BL2, TensorP* lam_out, double delta) {
  std::map<Q, std::vector<int>> groups;  // left charge -> blocks (key order)
  for (int i = 0; i < (int)BL2->b.size(); ++i) groups[BL2->b[i].k.q0].push_back(i);
  std::vector<Q> keys;
  std::vector<std::pair<int, int>> mn;
  std::vector<std::vector<int>> coloff;
  for (auto& g : groups) {
    int rows = BL2->b[g.second[0]].r, cols = 0;
    std::vector<int> co;
    for (int i : g.second) {
      MPSG_CHECK(BL2->b[i].r == rows, "row mismatch inside a charge group");
      co.push_back(cols);
      cols += BL2->b[i].c;
    }
    keys.push_back(g.first);
    mn.push_back({rows, cols});
    coloff.push_back(co);
  }
  SvdBatch sv(ctx);
  sv.plan(mn);
  std::vector<CopyOp> gops;
  for (size_t gi = 0; gi < keys.size(); ++gi) {
    const auto& bl = groups[keys[gi]];
    for (size_t t = 0; t < bl.size(); ++t) {
      const Block& b = BL2->b[bl[t]];
      gops.push_back(sv.gather_op((int)gi, BL2->d + b.off, b.r, b.c, 0, coloff[gi][t]));
    }
  }
  run_copyops(ctx, gops);
  sv.run(ctx->svd_method);
  sv.check_info();
  std::vector<double> S(std::max<int64_t>(sv.nS, 1));
  if (sv.nS) MPSG_CUDA(cudaMemcpyAsync(S.data(), sv.dS, sizeof(double) * sv.nS, cudaMemcpyDeviceToHost, ctx->stream));
  ctx->sync();
  std::vector<int> keep(keys.size());
  for (size_t gi = 0; gi < keys.size(); ++gi) {
    int l = 0;
    while (l < sv.s[gi].k && std::fabs(S[sv.s[gi].offS + l]) > delta) ++l;  // cut(D, delta)
    keep[gi] = l;
  }
  // new BL2 (Vd rows), lambdas
  Layout l2, ll;
  for (size_t gi = 0; gi < keys.size(); ++gi) {
    if (!keep[gi]) continue;
    for (int i : groups[keys[gi]]) l2.add(BL2->b[i].k, keep[gi], BL2->b[i].c);
    ll.add(K1(keys[gi], keys[gi], 0), keep[gi], 1);
  }
  l2.finalize();
  ll.finalize();
  TensorP nb2 = make_tensor(ctx, 1, l2, false);
  TensorP lam = make_tensor(ctx, 0, ll, false);
  std::vector<CopyOp> ops;
  // U*D per group, into a scratch for the BL1 products
  KeyedArena<Q> qd;
  for (size_t gi = 0; gi < keys.size(); ++gi)
    if (keep[gi]) qd.add(keys[gi], sv.s[gi].m, keep[gi]);
  double* dQD = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(qd.nelem, 2));
  for (size_t gi = 0; gi < keys.size(); ++gi) {
    const int l = keep[gi];
    if (!l) continue;
    int ldq, ldp;
    double* Qm = sv.Qp((int)gi, &ldq);
    double* Pm = sv.Pp((int)gi, &ldp);
    const double* Sv = sv.dS + sv.s[gi].offS;
    const auto& bl = groups[keys[gi]];
    for (size_t t = 0; t < bl.size(); ++t) {
      const Block& ob = nb2->b[nb2->find(BL2->b[bl[t]].k)];
      ops.push_back(CopyOp{Pm + coloff[gi][t], nb2->d + ob.off, nullptr, nullptr, l, ob.c, ldp, l, 1, 1.0});
    }
    const Block& lb = lam->b[lam->find(K1(keys[gi], keys[gi], 0))];
    ops.push_back(CopyOp{Sv, lam->d + lb.off, nullptr, nullptr, l, 1, l, l, 0, 1.0});
    const auto& Bq = qd.at(keys[gi]);
    ops.push_back(CopyOp{Qm, dQD + Bq.off, nullptr, Sv, sv.s[gi].m, l, ldq, sv.s[gi].m, 0, 1.0});
  }
  run_copyops(ctx, ops);
  if (BL1 && *BL1) {
    Tensor& b1 = **BL1;
    Layout l1;
    std::vector<std::pair<int, int>> src;  // (old block, group) ; group -1 = copy unchanged
    std::map<Q, int> gidx;
    for (size_t gi = 0; gi < keys.size(); ++gi) gidx[keys[gi]] = (int)gi;
    for (int i = 0; i < (int)b1.b.size(); ++i) {
      auto it = gidx.find(b1.b[i].k.q1);
      if (it == gidx.end()) {
        l1.add(b1.b[i].k, b1.b[i].r, b1.b[i].c);
        src.push_back({i, -1});
      } else if (keep[it->second]) {
        l1.add(b1.b[i].k, b1.b[i].r, keep[it->second]);
        src.push_back({i, it->second});
      }
    }
    l1.finalize();
    TensorP nb1 = make_tensor(ctx, 1, l1, true);
    GemmPlan g;
    std::vector<CopyOp> cps;
    for (auto& p : src) {
      const Block& ob = b1.b[p.first];
      const Block& nb = nb1->b[nb1->find(ob.k)];
      if (p.second < 0) {
        cps.push_back(CopyOp{b1.d + ob.off, nb1->d + nb.off, nullptr, nullptr, ob.r, ob.c, ob.r, ob.r, 0, 1.0});
      } else {
        const auto& Bq = qd.at(keys[p.second]);
        MPSG_CHECK(ob.c == Bq.r, "bond dimension mismatch in prepareMatrix");
        g.add_problem(2, nb.off, nb.r, nb.r, nb.c, false, {GSegH{0, 1, ob.off, Bq.off, ob.r, Bq.r, ob.c, 0, 0, 1.0}});
      }
    }
    g.upload(ctx);
    const double* bases[8] = {b1.d, dQD, nb1->d, nullptr, nullptr, nullptr, nullptr, nullptr};
    g.run(bases);
    run_copyops(ctx, cps);
    ctx->sync();
    *BL1 = nb1;
  }
  ctx->dfree(dQD);
  BL2 = nb2;
  if (lam_out) *lam_out = lam;
}

// ============================================================================ left canonicalisation
// prepareMatrix(BL1, lambda, BL2, "l", multiply=true, truncate, delta) (src/MPSfunctions.hpp:21-142,
// dir "l"): per right charge q the blocks (a, q; s) of BL1 stacked by rows form M_q = U D Vd; BL1
// becomes U (left-orthonormal), lambda(q) = D, and D Vd multiplies the blocks (q, b; s) of BL2 from
// the left (BL2 may be null at the right edge).  Singular values <= delta are dropped (delta = 0
// keeps every nonzero one).
void prepare_matrix_l(Ctx* ctx, TensorP& BL1, TensorP* BL2, TensorP* lam_out, double delta) {
  std::map<Q, std::vector<int>> groups;  // right charge -> blocks (key order)
  for (int i = 0; i < (int)BL1->b.size(); ++i) groups[BL1->b[i].k.q1].push_back(i);
  std::vector<Q> keys;
  std::vector<std::pair<int, int>> mn;
  std::vector<std::vector<int>> rowoff;
  for (auto& g : groups) {
    int rows = 0;
    const int cols = BL1->b[g.second[0]].c;
    std::vector<int> ro;
    for (int i : g.second) {
      MPSG_CHECK(BL1->b[i].c == cols, "column mismatch inside a charge group");
      ro.push_back(rows);
      rows += BL1->b[i].r;
    }
    keys.push_back(g.first);
    mn.push_back({rows, cols});
    rowoff.push_back(ro);
  }
  SvdBatch sv(ctx);
  sv.plan(mn);
  std::vector<CopyOp> gops;
  for (size_t gi = 0; gi < keys.size(); ++gi) {
    const auto& bl = groups[keys[gi]];
    for (size_t t = 0; t < bl.size(); ++t) {
      const Block& b = BL1->b[bl[t]];
      gops.push_back(sv.gather_op((int)gi, BL1->d + b.off, b.r, b.c, rowoff[gi][t], 0));
    }
  }
  run_copyops(ctx, gops);
  sv.run(ctx->svd_method);
  sv.check_info();
  std::vector<double> S(std::max<int64_t>(sv.nS, 1));
  if (sv.nS) MPSG_CUDA(cudaMemcpyAsync(S.data(), sv.dS, sizeof(double) * sv.nS, cudaMemcpyDeviceToHost, ctx->stream));
  ctx->sync();
  std::vector<int> keep(keys.size());
  for (size_t gi = 0; gi < keys.size(); ++gi) {
    int l = 0;
    while (l < sv.s[gi].k && std::fabs(S[sv.s[gi].offS + l]) > delta) ++l;
    keep[gi] = l;
  }
  Layout l1, ll;
  for (size_t gi = 0; gi < keys.size(); ++gi) {
    if (!keep[gi]) continue;
    for (int i : groups[keys[gi]]) l1.add(BL1->b[i].k, BL1->b[i].r, keep[gi]);
    ll.add(K1(keys[gi], keys[gi], 0), keep[gi], 1);
  }
  l1.finalize();
  ll.finalize();
  TensorP nb1 = make_tensor(ctx, 1, l1, false);
  TensorP lam = make_tensor(ctx, 0, ll, false);
  std::vector<CopyOp> ops;
  KeyedArena<Q> dv;  // D Vd per group (keep x cols)
  for (size_t gi = 0; gi < keys.size(); ++gi)
    if (keep[gi]) dv.add(keys[gi], keep[gi], sv.s[gi].n);
  double* dDV = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(dv.nelem, 2));
  for (size_t gi = 0; gi < keys.size(); ++gi) {
    const int l = keep[gi];
    if (!l) continue;
    int ldq, ldp;
    double* Qm = sv.Qp((int)gi, &ldq);
    double* Pm = sv.Pp((int)gi, &ldp);
    const double* Sv = sv.dS + sv.s[gi].offS;
    const auto& bl = groups[keys[gi]];
    for (size_t t = 0; t < bl.size(); ++t) {
      const Block& ob = nb1->b[nb1->find(BL1->b[bl[t]].k)];
      ops.push_back(CopyOp{Qm + rowoff[gi][t], nb1->d + ob.off, nullptr, nullptr, ob.r, l, ldq, ob.r, 0, 1.0});
    }
    const Block& lb = lam->b[lam->find(K1(keys[gi], keys[gi], 0))];
    ops.push_back(CopyOp{Sv, lam->d + lb.off, nullptr, nullptr, l, 1, l, l, 0, 1.0});
    const auto& Bq = dv.at(keys[gi]);
    ops.push_back(CopyOp{Pm, dDV + Bq.off, Sv, nullptr, l, sv.s[gi].n, ldp, l, 1, 1.0});  // D Vd = D P^T
  }
  run_copyops(ctx, ops);
  if (BL2 && *BL2) {
    Tensor& b2 = **BL2;
    Layout l2;
    std::vector<std::pair<int, int>> src;  // (old block, group); group -1 = copy unchanged
    std::map<Q, int> gidx;
    for (size_t gi = 0; gi < keys.size(); ++gi) gidx[keys[gi]] = (int)gi;
    for (int i = 0; i < (int)b2.b.size(); ++i) {
      auto it = gidx.find(b2.b[i].k.q0);
      if (it == gidx.end()) {
        l2.add(b2.b[i].k, b2.b[i].r, b2.b[i].c);
        src.push_back({i, -1});
      } else if (keep[it->second]) {
        l2.add(b2.b[i].k, keep[it->second], b2.b[i].c);
        src.push_back({i, it->second});
      }
    }
    l2.finalize();
    TensorP nb2 = make_tensor(ctx, 1, l2, true);
    GemmPlan g;
    std::vector<CopyOp> cps;
    for (auto& p : src) {
      const Block& ob = b2.b[p.first];
      const Block& nb = nb2->b[nb2->find(ob.k)];
      if (p.second < 0) {
        cps.push_back(CopyOp{b2.d + ob.off, nb2->d + nb.off, nullptr, nullptr, ob.r, ob.c, ob.r, ob.r, 0, 1.0});
      } else {
        const auto& Bq = dv.at(keys[p.second]);
        MPSG_CHECK(ob.r == Bq.c, "bond dimension mismatch in prepareMatrix");
        g.add_problem(2, nb.off, nb.r, nb.r, nb.c, false, {GSegH{1, 0, Bq.off, ob.off, Bq.r, ob.r, ob.r, 0, 0, 1.0}});
      }
    }
    g.upload(ctx);
    const double* bases[8] = {b2.d, dDV, nb2->d, nullptr, nullptr, nullptr, nullptr, nullptr};
    g.run(bases);
    run_copyops(ctx, cps);
    ctx->sync();
    *BL2 = nb2;
  }
  ctx->dfree(dDV);
  BL1 = nb1;
  if (lam_out) *lam_out = lam;
}

// ============================================================================ Lanczos
LanczosResult lanczos(Ctx* ctx, MatvecPlan& mv, const Tensor& th_init, Tensor& psi, int itmax, double delta,
                      bool testenergy, bool reorth, LanczosStats* st, double tol_rel, int ndiag, double stall_rel,
                      const double* proj) {
  MPSG_CHECK(ndiag >= 1, "ndiag must be >= 1");
  auto t_start = std::chrono::steady_clock::now();
  const int64_t n = th_init.nelem;
  MPSG_CHECK(psi.nelem == n, "Lanczos state layout mismatch");
  MPSG_CHECK(itmax >= 1 && itmax <= 1000, "itmax must be in [1, 1000]");
  cudaStream_t s = ctx->stream;
  // device scalars: alpha[itmax+1], beta[itmax+1], norm2[itmax+2], E[itmax/5+2], z[itmax+1], coef[itmax+1]
  const int na = itmax + 2;
  double* dsc = (double*)ctx->dmalloc(sizeof(double) * (size_t)na * 6);
  double *d_alpha = dsc, *d_beta = dsc + na, *d_norm2 = dsc + 2 * na, *d_E = dsc + 3 * na, *d_z = dsc + 4 * na,
         *d_coef = dsc + 5 * na;
  MPSG_CUDA(cudaMemsetAsync(dsc, 0, sizeof(double) * (size_t)na * 6, s));
  double* d_proj = reorth ? (double*)ctx->dmalloc(sizeof(double) * 64 * (size_t)na) : nullptr;
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
  // projected Lanczos (TSLanzcosEngine::simulate with a state, src/lanzcos.hpp:282-400): the start
  // vector and every new Krylov vector lose their component along `proj`
  double* d_ph = nullptr;
  double** d_pp = nullptr;
  if (proj) {
    d_ph = (double*)ctx->dmalloc(sizeof(double) * (std::max<int64_t>(n, 2) + 2 + 64));
    d_pp = (double**)ctx->dmalloc(sizeof(double*));
    MPSG_CUDA(cudaMemcpyAsync(d_ph, proj, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    double* d_pn = d_ph + std::max<int64_t>(n, 2);
    launch_dot(d_ph, d_ph, n, ctx->part, d_pn, s);
    launch_scale_by_norm(d_ph, n, d_pn, 0.0, nullptr, s);  // unit vector (a zero state projects nothing)
    MPSG_CUDA(cudaMemcpyAsync(d_pp, &d_ph, sizeof(double*), cudaMemcpyHostToDevice, s));
    ctx->sync();
  }
  auto project_out = [&](double* x) {
    if (!proj) return;
    double* d_pc = d_ph + std::max<int64_t>(n, 2) + 1;
    double* d_pparts = d_pc + 1;
    launch_project((const double* const*)d_pp, 1, x, n, d_pparts, d_pc, s);
    launch_combine(x, (const double* const*)d_pp, 1, d_pc, n, 1, s);
  };
  project_out(V[0]);
  launch_dot(V[0], V[0], n, ctx->part, d_norm2, s);
  cudaEvent_t e0, e1;
  MPSG_CUDA(cudaEventCreate(&e0));
  MPSG_CUDA(cudaEventCreate(&e1));
  std::vector<double> ha(na), hb(na), hn(na), hE(na);
  int it = 0, n_es = 0;
  double eold = 1e100, dE_prev = 1e100;
  bool done = false;
  float mv_ms_total = 0;
  // Batches after the first hold ndiag iterations each and end on an energy checkpoint: they are
  // captured once as a CUDA graph (iteration index on the device, matvec on fixed buffers) and the
  // graph is replayed for every later batch.  Projected and reorthogonalised runs stay launch by launch.
  bool graphs = !proj && !reorth && !std::getenv("MPSG_NO_LANCZOS_GRAPH");
  cudaGraphExec_t gexec = nullptr;
  size_t gnodes = 0;
  int* d_j = nullptr;
  double* xin = nullptr;
  while (!done) {
    // batch up to the next energy checkpoint (it % ndiag == 0, it != 0) or itmax-1
    int ck = it;
    while (!((ck % ndiag == 0 && ck != 0) || ck >= itmax - 1)) ++ck;
    if (graphs && it > 0 && ck - it + 1 == ndiag && ck % ndiag == 0 && !gexec) {
      slot(ck + 1);
      d_j = (int*)ctx->dmalloc(sizeof(int) * 4);
      xin = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(n, 2));
      lz_prepare_attributes(itmax);
      cudaGraph_t g = nullptr;
      const int64_t launched0 = kernel_launch_count() + tc_launch_count();  // captured, not run
      cudaError_t ce = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
      if (ce == cudaSuccess) {
        for (int u = 0; u < ndiag; ++u) {
          launch_lz_pre(dV, d_j, d_norm2, delta, d_beta, xin, n, s);
          mv.run(xin, w);
          launch_lz_post(dV, d_j, w, xin, d_alpha, d_beta, d_norm2, d_E, ndiag, testenergy && u == ndiag - 1, itmax,
                         n, ctx->part, s);
        }
        ce = cudaStreamEndCapture(s, &g);
      }
      count_graph_launches(launched0 - (kernel_launch_count() + tc_launch_count()));
      if (ce == cudaSuccess && g && cudaGraphGetNodes(g, nullptr, &gnodes) == cudaSuccess &&
          cudaGraphInstantiate(&gexec, g, 0) == cudaSuccess) {
      } else {  // capture not possible on this stream: the launch-by-launch path
        cudaGetLastError();
        gexec = nullptr;
        graphs = false;
        if (std::getenv("MPSG_VERBOSE")) std::fprintf(stderr, "libmpsg: Lanczos graph capture failed (%s)\n", cudaGetErrorString(ce));
      }
      if (g) cudaGraphDestroy(g);
    }
    if (gexec && it > 0 && ck - it + 1 == ndiag && ck % ndiag == 0) {
      slot(ck + 1);  // the batch's Krylov vectors exist (and are in the device table) before the graph runs
      int* hj = reinterpret_cast<int*>(ctx->hscal + 4095);  // pinned, past the scalars read back below
      hj[0] = it;
      MPSG_CUDA(cudaMemcpyAsync(d_j, hj, sizeof(int), cudaMemcpyHostToDevice, s));
      MPSG_CUDA(cudaEventRecord(e0, s));
      MPSG_CUDA(cudaGraphLaunch(gexec, s));
      count_graph_launches((int64_t)gnodes);
    } else {
    MPSG_CUDA(cudaEventRecord(e0, s));
    for (int j = it; j <= ck; ++j) {
      slot(j + 1);
      launch_scale_by_norm(V[j], n, d_norm2 + j, delta, d_beta + j, s);
      mv.run(V[j], w);
      launch_dot(w, V[j], n, ctx->part, d_alpha + j, s);
      if (testenergy && j % ndiag == 0 && j != 0)
        launch_tri_lowest(d_alpha, d_beta, j + 1, d_E + j / ndiag, nullptr, s);
      launch_axpy3(V[j + 1], w, V[j], j > 0 ? V[j - 1] : nullptr, d_alpha + j, d_beta + j, n, ctx->part,
                   d_norm2 + j + 1, s);
      if (proj) {
        project_out(V[j + 1]);
        launch_dot(V[j + 1], V[j + 1], n, ctx->part, d_norm2 + j + 1, s);
      }
      if (reorth) {
        for (int pass = 0; pass < 2; ++pass) {
          launch_project((const double* const*)dV, j + 1, V[j + 1], n, d_proj, d_coef, s);
          launch_combine(V[j + 1], (const double* const*)dV, j + 1, d_coef, n, 1, s);
        }
        launch_dot(V[j + 1], V[j + 1], n, ctx->part, d_norm2 + j + 1, s);
      }
    }
    }
    MPSG_CUDA(cudaEventRecord(e1, s));
    MPSG_CUDA(cudaMemcpyAsync(ctx->hscal, dsc, sizeof(double) * (size_t)na * 4, cudaMemcpyDeviceToHost, s));
    ctx->sync();
    mv.check_error();
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    mv_ms_total += ms;
    std::memcpy(ha.data(), ctx->hscal, sizeof(double) * na);
    std::memcpy(hb.data(), ctx->hscal + na, sizeof(double) * na);
    std::memcpy(hn.data(), ctx->hscal + 2 * na, sizeof(double) * na);
    std::memcpy(hE.data(), ctx->hscal + 3 * na, sizeof(double) * na);
    if (st) {
      st->matvecs += ck - it + 1;
      st->matvec_flops += mv.flops * (ck - it + 1);
    }
    for (int j = it; j <= ck; ++j) {
      const double k = std::sqrt(hn[j]);
      if (std::fabs(k) < delta) { n_es = j; done = true; break; }
      n_es = j + 1;
      if (testenergy && j % ndiag == 0 && j != 0) {
        const double E = hE[j / ndiag], dE = std::fabs(E - eold);
        if (dE < std::max(delta, tol_rel * std::fabs(E))) { done = true; break; }
        // stall: below the stall level and no longer shrinking (noise floor of a low-precision matvec)
        if (stall_rel > 0 && dE < stall_rel * std::fabs(E) && dE > 0.5 * dE_prev) { done = true; break; }
        dE_prev = dE;
        eold = E;
      }
      if (j + 1 >= itmax) { done = true; break; }
    }
    it = ck + 1;
  }
  if (st) st->matvec_seconds += mv_ms_total * 1e-3;
  LanczosResult res;
  res.n = n_es;
  res.iterations = n_es;
  if (n_es > 0) {
    launch_tri_lowest(d_alpha, d_beta, n_es, d_E + na - 1, d_z, s);
    launch_combine(psi.d, (const double* const*)dV, n_es, d_z, n, 0, s);
    MPSG_CUDA(cudaMemcpyAsync(ctx->hscal, d_E + na - 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    ctx->sync();
    res.E0 = ctx->hscal[0];
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (gexec) cudaGraphExecDestroy(gexec);
  ctx->dfree(d_j);
  ctx->dfree(xin);
  for (double* p : V) ctx->dfree(p);
  ctx->dfree(w);
  ctx->dfree(dV);
  ctx->dfree(dsc);
  if (d_proj) ctx->dfree(d_proj);
  if (d_ph) ctx->dfree(d_ph);
  if (d_pp) ctx->dfree(d_pp);
  ctx->sync();
  if (st) st->seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  return res;
}

// Relative energy-change floor of the Lanczos energy test per matvec precision (FP32 accumulation
// bounds the hi/lo modes; single-product modes are limited by the 10 / 7 bit operands).
double prec_tol(int prec) {
  switch (prec) {
    case MPSG_PREC_TF32X3: return 1e-11;
    case MPSG_PREC_BF16X3: return 1e-9;
    case MPSG_PREC_TF32: return 1e-7;
    case MPSG_PREC_BF16: return 1e-6;
    default: return 0.0;
  }
}
double prec_stall(int prec) {
  switch (prec) {
    case MPSG_PREC_TF32X3: return 1e-9;
    case MPSG_PREC_BF16X3: return 1e-7;
    case MPSG_PREC_TF32: return 1e-5;
    case MPSG_PREC_BF16: return 1e-4;
    default: return 0.0;
  }
}

double rayleigh_quotient(Ctx* ctx, MatvecPlan& mv, const Tensor& psi, LanczosStats* st) {
  const int64_t n = psi.nelem;
  cudaStream_t s = ctx->stream;
  double* w = (double*)ctx->dmalloc(sizeof(double) * (std::max<int64_t>(n, 2) + 2));
  double* d_q = w + std::max<int64_t>(n, 2);
  MPSG_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * std::max<int64_t>(n, 2), s));
  auto t0 = std::chrono::steady_clock::now();
  mv.run(psi.d, w);
  launch_dot(psi.d, w, n, ctx->part, d_q, s);
  launch_dot(psi.d, psi.d, n, ctx->part, d_q + 1, s);
  double q[2] = {0, 0};
  MPSG_CUDA(cudaMemcpyAsync(q, d_q, sizeof(q), cudaMemcpyDeviceToHost, s));
  ctx->sync();
  ctx->dfree(w);
  if (st) {
    st->matvecs += 1;
    st->matvec_flops += mv.flops;
    st->matvec_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  MPSG_CHECK(q[1] > 0, "Rayleigh quotient of a zero state");
  return q[0] / q[1];
}

void EnergyJob::prepare(Ctx* c, std::unique_ptr<MatvecPlan> plan, const Tensor& state, LanczosStats* s) {
  release();
  ctx = c;
  mv = std::move(plan);
  st = s;
  psi = &state;
  launched = false;
  nw = std::max<int64_t>(state.nelem, 2);
  buf = (double*)ctx->dmalloc(sizeof(double) * (nw + kRedBlocks + 64 + 2));
  MPSG_CUDA(cudaMemsetAsync(buf, 0, sizeof(double) * nw, ctx->stream));
  for (auto& e : ev) MPSG_CUDA(cudaEventCreate(&e));
  MPSG_CUDA(cudaEventRecord(ev[2], ctx->stream));  // psi, the plan's FP64 tables, buf
}

void EnergyJob::launch(cudaEvent_t after) {
  MPSG_CHECK(pending() && !launched, "energy job not prepared");
  launched = true;
  double* w = buf;
  double* part = buf + nw;
  double* dq = part + kRedBlocks + 64;
  cudaStream_t side = ctx->side_stream();
  MPSG_CUDA(cudaStreamWaitEvent(side, ev[2], 0));
  if (after) MPSG_CUDA(cudaStreamWaitEvent(side, after, 0));
  cudaStream_t main = ctx->stream;
  ctx->stream = side;  // the plan launches on ctx->stream
  try {
    MPSG_CUDA(cudaEventRecord(ev[0], side));
    mv->run(psi->d, w);
    MPSG_CUDA(cudaEventRecord(ev[1], side));
    launch_dot(psi->d, w, psi->nelem, part, dq, side);
    launch_dot(psi->d, psi->d, psi->nelem, part, dq + 1, side);
    MPSG_CUDA(cudaEventRecord(ev[2], side));
  } catch (...) {
    ctx->stream = main;
    throw;
  }
  ctx->stream = main;
}

double EnergyJob::finish() {
  MPSG_CHECK(pending(), "energy job not started");
  if (!launched) launch(nullptr);
  MPSG_CUDA(cudaEventSynchronize(ev[2]));
  float ms = 0;
  MPSG_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
  double q[2] = {0, 0};
  cudaStream_t side = ctx->side_stream();
  MPSG_CUDA(cudaMemcpyAsync(q, buf + nw + kRedBlocks + 64, sizeof(q), cudaMemcpyDeviceToHost, side));
  MPSG_CUDA(cudaStreamSynchronize(side));
  if (st) {
    st->matvecs += 1;
    st->matvec_flops += mv->flops;
    st->matvec_seconds += ms * 1e-3;
  }
  release();
  MPSG_CHECK(q[1] > 0, "Rayleigh quotient of a zero state");
  return q[0] / q[1];
}

void EnergyJob::release() {
  if (!ctx) return;
  cudaStreamSynchronize(ctx->side_stream());
  for (auto& e : ev)
    if (e) {
      cudaEventDestroy(e);
      e = nullptr;
    }
  ctx->dfree(buf);
  buf = nullptr;
  mv.reset();
  ctx = nullptr;
}

LanczosResult lanczos_prec(Ctx* ctx, const Tensor& L, const Tensor& R, const Layout& sx, const MPO& W1, const MPO& W2,
                           const ItoKey& ik0, const ItoKey& ik1, const Tensor& th_init, Tensor& psi, int itmax,
                           double delta, bool testenergy, bool reorth, int prec, LanczosStats* st, const double* proj,
                           EnergyJob* energy) {
  if (prec == MPSG_PREC_FP64) {
    auto mv = build_matvec(ctx, L, R, sx, W1, W2, ik0, ik1, &sx, MPSG_PREC_FP64);
    return lanczos(ctx, *mv, th_init, psi, itmax, delta, testenergy, reorth, st, 0.0, 5, 0.0, proj);
  }
  const int lo = (prec == MPSG_PREC_AUTO || prec == MPSG_PREC_MIXED) ? MPSG_PREC_TF32X3 : prec;
  LanczosResult r;
  auto mv = build_matvec(ctx, L, R, sx, W1, W2, ik0, ik1, &sx, lo);
  r = lanczos(ctx, *mv, th_init, psi, itmax, delta, testenergy, reorth, st, prec_tol(lo), 5, prec_stall(lo), proj);
  if (prec == MPSG_PREC_MIXED) {
    // the energy measured in FP64: the Rayleigh quotient of the mixed-precision ground state.  The
    // tensor-core matvec scales H by a systematic factor (FP32 accumulation rounds towards zero; at
    // chi = 2048 about 1 - 5e-6), which shifts the Ritz value but not the eigenvector.
    mv->use_fp64();
    if (energy) {
      energy->prepare(ctx, std::move(mv), psi, st);
      r.E0 = std::numeric_limits<double>::quiet_NaN();
    } else {
      r.E0 = rayleigh_quotient(ctx, *mv, psi, st);
    }
    return r;
  }
  if (prec != MPSG_PREC_AUTO) return r;
  // FP64 finish: the reference's Lanczos restarted from the mixed-precision ground state, energy test
  // every iteration, so the final energy carries the same convergence criterion as the FP64 path
  mv->use_fp64();
  TensorP start = tensor_copy(psi);
  LanczosResult r2 = lanczos(ctx, *mv, *start, psi, itmax, delta, testenergy, reorth, st, 0.0, 1, 0.0, proj);
  r2.iterations += r.iterations;
  return r2;
}

}  // namespace mpsg
