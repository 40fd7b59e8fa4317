// C ABI of libmpsg (include/mpsg.h) and the DMRG engine (DMRGengine::simulate / doStep).
#include <chrono>
#include <cmath>
#include <cstring>

#include "capi_types.h"

using namespace mpsg;

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
  std::vector<StepRec> steps;
  LanczosStats lst;
  double env_seconds = 0, split_seconds = 0, env_flops = 0, wall = 0;

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

  StepRec do_step_impl(int site, int dir, int chimax, bool doTrunc, double tr_weight, double delta,
                       bool testenergy) {
    MPSG_CHECK(site >= 0 && site + 1 < N, "site out of range");
    MPSG_CHECK(L.count(site - 1) && R.count(site + 2), "environments missing (call prepare first)");
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
    Layout sx = theta_closure(Le, Re, s0, mpo[site], mpo[site + 1], ik[site], ik[site + 1]);
    TensorP th = theta_form(ctx, *mps[site], *mps[site + 1], &sx);
    TensorP psi = make_tensor(ctx, 2, sx, true);
    LanczosResult lr = lanczos_prec(ctx, Le, Re, sx, mpo[site], mpo[site + 1], ik[site], ik[site + 1], *th, *psi,
                                    lanmax, delta, testenergy, reorth, (int)prec, &lst);
    th.reset();
    auto t0 = std::chrono::steady_clock::now();
    SplitResult sp = split2(ctx, *psi, ik[site], ik[site + 1], chimax, doTrunc, tr_weight, true, dir > 0 ? 1 : -1);
    ctx->sync();
    auto t1 = std::chrono::steady_clock::now();
    split_seconds += std::chrono::duration<double>(t1 - t0).count();
    psi.reset();
    mps[site] = sp.U;
    mps[site + 1] = sp.Vt;
    lam[site] = sp.lam;
    if (dir > 0) L[site] = env_update(ctx, *L[site - 1], *mps[site], mpo[site], ik[site], 1, &env_flops);
    else R[site + 1] = env_update(ctx, *R[site + 2], *mps[site + 1], mpo[site + 1], ik[site + 1], -1, &env_flops);
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
  Engine* e = nullptr;
};
struct mpsg_matvec_plan_s {
  std::unique_ptr<MatvecPlan> p;
};

// ============================================================================ error plumbing

extern "C" {

const char* mpsg_last_error(void) { return g_last_error.c_str(); }

mpsg_status mpsg_ctx_create(int32_t device, mpsg_ctx* out) {
  API_BEGIN
  MPSG_CHECK(out, "null output");
  mpsg_ctx c = new mpsg_ctx_s;
  try {
    c->c = std::make_shared<Ctx>(device);
  } catch (...) {
    delete c;
    throw;
  }
  *out = c;
  API_END
}
void mpsg_ctx_destroy(mpsg_ctx ctx) {
  if (!ctx) return;
  try {
    ctx->c.reset();  // the Ctx lives on while tensors, plans or engines still use it
  } catch (...) {
  }
  delete ctx;
}
mpsg_status mpsg_ctx_set_stream(mpsg_ctx ctx, void* stream) {
  API_BEGIN
  Ctx* c = C(ctx);
  c->sync();
  c->stream = stream ? (cudaStream_t)stream : c->own;
  API_END
}
mpsg_status mpsg_ctx_sync(mpsg_ctx ctx) {
  API_BEGIN
  C(ctx)->sync();
  API_END
}
int64_t mpsg_ctx_kernel_launches(mpsg_ctx) { return kernel_launch_count() + tc_launch_count() + eig_launch_count() + tebd_launch_count(); }
mpsg_status mpsg_ctx_set_svd_method(mpsg_ctx ctx, int32_t method) {
  API_BEGIN
  MPSG_CHECK(method >= 0 && method <= 3,
             "svd method must be 0 (Jacobi SVD), 1 (density matrix, cuSOLVER batched), 2 (density matrix, "
             "cuSOLVER concurrent) or 3 (density matrix, own batched eigensolver)");
  C(ctx)->svd_method = method;
  API_END
}

mpsg_status mpsg_tensor_create(mpsg_ctx ctx, int32_t nphys, int32_t nblocks, const uint64_t* q, const uint32_t* p,
                               const int32_t* rows, const int32_t* cols, const double* host_data,
                               mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(out, "null output");
  MPSG_CHECK(nblocks == 0 || (q && rows && cols && (nphys == 0 || p)), "null structure arrays");
  *out = wrap(tensor_from_host(C(ctx), nphys, nblocks, q, p, rows, cols, host_data));
  API_END
}
mpsg_status mpsg_tensor_shape(mpsg_tensor t, int32_t* nphys, int32_t* nblocks, int64_t* nelem) {
  API_BEGIN
  const Tensor& x = T(t);
  if (nphys) *nphys = x.nphys;
  if (nblocks) *nblocks = (int32_t)x.b.size();
  if (nelem) {
    int64_t s = 0;
    for (auto& b : x.b) s += (int64_t)b.r * b.c;
    *nelem = s;
  }
  API_END
}
mpsg_status mpsg_tensor_export(mpsg_tensor t, uint64_t* q, uint32_t* p, int32_t* rows, int32_t* cols,
                               double* host_data) {
  API_BEGIN
  const Tensor& x = T(t);
  for (size_t i = 0; i < x.b.size(); ++i) {
    if (q) {
      q[2 * i] = x.b[i].k.q0;
      q[2 * i + 1] = x.b[i].k.q1;
    }
    if (p && x.nphys >= 1) p[x.nphys * i] = x.b[i].k.p0;
    if (p && x.nphys >= 2) p[x.nphys * i + 1] = x.b[i].k.p1;
    if (rows) rows[i] = x.b[i].r;
    if (cols) cols[i] = x.b[i].c;
  }
  if (host_data) {
    std::vector<double> h;
    tensor_to_host(x, h);
    if (!h.empty()) std::memcpy(host_data, h.data(), sizeof(double) * h.size());
  }
  API_END
}
mpsg_status mpsg_tensor_device_view(mpsg_tensor t, double** dptr, int64_t* offsets) {
  API_BEGIN
  const Tensor& x = T(t);
  if (dptr) *dptr = x.d;
  if (offsets)
    for (size_t i = 0; i < x.b.size(); ++i) offsets[i] = x.b[i].off;
  API_END
}
void mpsg_tensor_destroy(mpsg_tensor t) {
  if (!t) return;
  try {
    t->t.reset();
  } catch (...) {
  }
  delete t;
}

static void check_prec(mpsg_prec prec) {  // FP64 only (environment update, split)
  MPSG_CHECK(prec == MPSG_PREC_FP64, "only MPSG_PREC_FP64 is available for this entry point");
}
static void check_matvec_prec(mpsg_prec prec) {
  MPSG_CHECK(prec >= MPSG_PREC_FP64 && prec <= MPSG_PREC_BF16X3, "matvec precision must be FP64, TF32(X3) or BF16(X3)");
}
static void check_lanczos_prec(mpsg_prec prec) {
  MPSG_CHECK(prec >= MPSG_PREC_FP64 && prec <= MPSG_PREC_AUTO, "unknown precision mode");
}

mpsg_status mpsg_contract_twosite(mpsg_ctx ctx, mpsg_tensor L, mpsg_tensor R, mpsg_tensor theta, const mpsg_mpo* Wl,
                                  const mpsg_mpo* Wr, const mpsg_itokey* ikl, const mpsg_itokey* ikr, mpsg_prec prec,
                                  mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(out, "null output");
  check_matvec_prec(prec);
  Ctx* c = C(ctx);
  const Tensor& th = T(theta);
  MPSG_CHECK(th.nphys == 2 && T(L).nphys == 1 && T(R).nphys == 1, "tensor kinds do not match");
  Layout lin = layout_of(th);
  auto P = build_matvec(c, T(L), T(R), lin, mpo_from_c(Wl), mpo_from_c(Wr), itokey_from_c(ikl), itokey_from_c(ikr),
                        nullptr, prec);
  TensorP o = make_tensor(c, 2, P->out, true);
  P->run(th.d, o->d);
  P->check_error();
  c->sync();
  *out = wrap(o);
  API_END
}

mpsg_status mpsg_add_contraction_layer(mpsg_ctx ctx, mpsg_tensor BL, mpsg_tensor A, const mpsg_mpo* W,
                                       const mpsg_itokey* ik, int32_t direction, mpsg_prec prec, mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(out, "null output");
  check_prec(prec);
  Ctx* c = C(ctx);
  MPSG_CHECK(T(A).b.size() > 0, "Error in addContractionLayer: A is empty.");
  TensorP o = env_update(c, T(BL), T(A), mpo_from_c(W), itokey_from_c(ik), direction, nullptr);
  c->sync();
  *out = wrap(o);
  API_END
}

mpsg_status mpsg_add_contraction_layer2(mpsg_ctx ctx, mpsg_tensor BL, mpsg_tensor A, mpsg_tensor Ap,
                                        const mpsg_mpo* W, const mpsg_itokey* ik, int32_t direction, mpsg_prec prec,
                                        mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(out, "null output");
  check_prec(prec);
  Ctx* c = C(ctx);
  MPSG_CHECK(T(A).b.size() > 0, "Error in addContractionLayer: A is empty.");
  MPSG_CHECK(T(Ap).b.size() > 0, "Error in addContractionLayer: Ap is empty.");
  TensorP o = env_update(c, T(BL), T(A), mpo_from_c(W), itokey_from_c(ik), direction, nullptr, &T(Ap));
  c->sync();
  *out = wrap(o);
  API_END
}

mpsg_status mpsg_overlap(mpsg_ctx ctx, int32_t N, const mpsg_tensor* a, const mpsg_tensor* b, const mpsg_itokey* ik,
                         double* out) {
  API_BEGIN
  MPSG_CHECK(N >= 1 && a && b && ik && out, "null argument or N < 1");
  std::vector<const Tensor*> ta, tb;
  std::vector<ItoKey> k;
  for (int s = 0; s < N; ++s) {
    MPSG_CHECK(a[s] && b[s], "null site tensor");
    ta.push_back(&T(a[s]));
    tb.push_back(&T(b[s]));
    k.push_back(itokey_from_c(&ik[s]));
  }
  *out = mpsg::Engine::overlap(C(ctx), ta, tb, k);
  API_END
}

mpsg_status mpsg_mpo_measure(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* W,
                             const mpsg_itokey* ik, double* out) {
  API_BEGIN
  MPSG_CHECK(N >= 1 && sites && W && ik && out, "null argument or N < 1");
  std::vector<const Tensor*> ts;
  std::vector<MPO> w;
  std::vector<ItoKey> k;
  for (int s = 0; s < N; ++s) {
    MPSG_CHECK(sites[s], "null site tensor");
    MPSG_CHECK(T(sites[s]).b.size() > 0, "Error in addContractionLayer: A is empty.");
    ts.push_back(&T(sites[s]));
    w.push_back(mpo_from_c(&W[s]));
    k.push_back(itokey_from_c(&ik[s]));
  }
  *out = mpsg::Engine::mpo_expectation(C(ctx), ts, w, k);
  API_END
}

mpsg_status mpsg_theta(mpsg_ctx ctx, mpsg_tensor A1, mpsg_tensor A2, mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(out, "null output");
  *out = wrap(theta_form(C(ctx), T(A1), T(A2), nullptr));
  API_END
}

mpsg_status mpsg_split2(mpsg_ctx ctx, mpsg_tensor theta, const mpsg_itokey* ikl, const mpsg_itokey* ikr,
                        uint32_t chimax, int32_t doTrunc, double tr_weight, int32_t normalize, mpsg_tensor* U,
                        mpsg_tensor* Vt, mpsg_tensor* lambda, double* tw, uint32_t* chi) {
  API_BEGIN
  MPSG_CHECK(U && Vt && lambda, "null output");
  Ctx* c = C(ctx);
  SplitResult r = split2(c, T(theta), itokey_from_c(ikl), itokey_from_c(ikr), (int)chimax, doTrunc != 0, tr_weight,
                         normalize != 0, 0);
  c->sync();
  *U = wrap(r.U);
  *Vt = wrap(r.Vt);
  *lambda = wrap(r.lam);
  if (tw) *tw = r.tw;
  if (chi) *chi = (uint32_t)r.chi;
  API_END
}

mpsg_status mpsg_lanczos2(mpsg_ctx ctx, mpsg_tensor L, mpsg_tensor R, mpsg_tensor mpsl, mpsg_tensor mpsr,
                          const mpsg_mpo* Wl, const mpsg_mpo* Wr, const mpsg_itokey* ikl, const mpsg_itokey* ikr,
                          int32_t itmax, double delta, int32_t testenergy, mpsg_prec prec, int32_t reorth,
                          mpsg_tensor* state, double* E0, int32_t* iterations) {
  API_BEGIN
  MPSG_CHECK(state, "null output");
  check_lanczos_prec(prec);
  Ctx* c = C(ctx);
  MPO w1 = mpo_from_c(Wl), w2 = mpo_from_c(Wr);
  ItoKey k0 = itokey_from_c(ikl), k1 = itokey_from_c(ikr);
  TensorP th0 = theta_form(c, T(mpsl), T(mpsr), nullptr);
  Layout sx = theta_closure(T(L), T(R), layout_of(*th0), w1, w2, k0, k1);
  TensorP th = theta_form(c, T(mpsl), T(mpsr), &sx);
  TensorP psi = make_tensor(c, 2, sx, true);
  LanczosResult r = lanczos_prec(c, T(L), T(R), sx, w1, w2, k0, k1, *th, *psi, itmax, delta, testenergy != 0,
                                 reorth != 0, (int)prec, nullptr);
  c->sync();
  *state = wrap(psi);
  if (E0) *E0 = r.E0;
  if (iterations) *iterations = r.iterations;
  API_END
}

mpsg_status mpsg_dmrg_create(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* mpos,
                             const mpsg_itokey* itokeys, mpsg_dmrg* out) {
  API_BEGIN
  MPSG_CHECK(out && sites && mpos && itokeys, "null argument");
  MPSG_CHECK(N >= 3, "DMRG needs at least 3 sites");
  Engine* e = new Engine();
  e->ctx = C(ctx);
  e->keep = e->ctx->shared_from_this();
  e->N = N;
  try {
    for (int i = 0; i < N; ++i) {
      MPSG_CHECK(T(sites[i]).nphys == 1, "MPS site tensors must have one physical index");
      e->mps.push_back(tensor_copy(T(sites[i])));
      e->mpo.push_back(mpo_from_c(&mpos[i]));
      e->ik.push_back(itokey_from_c(&itokeys[i]));
    }
  } catch (...) {
    delete e;
    throw;
  }
  mpsg_dmrg d = new mpsg_dmrg_s;
  d->e = e;
  *out = d;
  API_END
}
mpsg_status mpsg_dmrg_set_options(mpsg_dmrg e, mpsg_prec prec, int32_t reorth, int32_t lanmax) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  check_lanczos_prec(prec);
  MPSG_CHECK(lanmax >= 1 && lanmax <= 1000, "lanmax must be in [1, 1000]");
  e->e->prec = prec;
  e->e->reorth = reorth != 0;
  e->e->lanmax = lanmax;
  API_END
}
mpsg_status mpsg_dmrg_simulate(mpsg_dmrg e, uint32_t maxsteps, double EnConv, uint32_t chimax, int32_t doTrunc,
                               double tr_weight, double delta, int32_t testenergy, double* E) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  MPSG_CHECK(EnConv > 0, "EnConv must be > 0");
  const double r = e->e->simulate((int)maxsteps, EnConv, (int)chimax, doTrunc != 0, tr_weight, delta, testenergy != 0);
  if (E) *E = r;
  API_END
}
mpsg_status mpsg_dmrg_prepare(mpsg_dmrg e) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  e->e->prepare();
  API_END
}
mpsg_status mpsg_dmrg_do_step(mpsg_dmrg e, int32_t site, int32_t dir, uint32_t chimax, int32_t doTrunc,
                              double tr_weight, double delta, int32_t testenergy, double* E) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  StepRec r = e->e->do_step(site, dir, (int)chimax, doTrunc != 0, tr_weight, delta, testenergy != 0);
  if (E) *E = r.E;
  API_END
}
int32_t mpsg_dmrg_nsteps(mpsg_dmrg e) { return (e && e->e) ? (int32_t)e->e->steps.size() : 0; }
mpsg_status mpsg_dmrg_steps(mpsg_dmrg e, int32_t* site, int32_t* dir, int32_t* iters, int32_t* chi, double* E,
                            double* tw) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  auto& s = e->e->steps;
  for (size_t i = 0; i < s.size(); ++i) {
    if (site) site[i] = s[i].site;
    if (dir) dir[i] = s[i].dir;
    if (iters) iters[i] = s[i].iters;
    if (chi) chi[i] = s[i].chi;
    if (E) E[i] = s[i].E;
    if (tw) tw[i] = s[i].tw;
  }
  API_END
}
mpsg_status mpsg_dmrg_stats(mpsg_dmrg e, double* st) {
  API_BEGIN
  MPSG_CHECK(e && e->e && st, "null argument");
  Engine& g = *e->e;
  st[0] = (double)g.lst.matvecs;
  st[1] = g.lst.matvec_flops;
  st[2] = g.lst.matvec_seconds;
  st[3] = g.env_seconds;
  st[4] = g.split_seconds;
  st[5] = g.lst.seconds;
  st[6] = g.env_flops;
  st[7] = g.wall;
  st[8] = g.step_device_seconds;
  st[9] = (double)g.nstep_calls;
  API_END
}
mpsg_status mpsg_dmrg_build_environments(mpsg_dmrg e, int32_t center) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  e->e->build_environments(center);
  API_END
}
mpsg_status mpsg_dmrg_env(mpsg_dmrg e, int32_t which, int32_t site, mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(e && e->e && out, "null argument");
  auto& m = which ? e->e->R : e->e->L;
  auto it = m.find(site);
  MPSG_CHECK(it != m.end() && it->second, "environment not available");
  *out = wrap(tensor_copy(*it->second));
  e->e->ctx->sync();
  API_END
}

mpsg_status mpsg_matvec2_plan_create(mpsg_ctx ctx, mpsg_tensor L, mpsg_tensor R, mpsg_tensor theta_layout,
                                     const mpsg_mpo* Wl, const mpsg_mpo* Wr, const mpsg_itokey* ikl,
                                     const mpsg_itokey* ikr, mpsg_prec prec, mpsg_matvec_plan* out) {
  API_BEGIN
  MPSG_CHECK(out, "null output");
  check_matvec_prec(prec);
  Ctx* c = C(ctx);
  const Tensor& th = T(theta_layout);
  MPSG_CHECK(th.nphys == 2, "theta_layout must be a two-site tensor");
  Layout lay = layout_of(th);
  auto P = build_matvec(c, T(L), T(R), lay, mpo_from_c(Wl), mpo_from_c(Wr), itokey_from_c(ikl), itokey_from_c(ikr),
                        &lay, prec);
  mpsg_matvec_plan p = new mpsg_matvec_plan_s;
  p->p = std::move(P);
  *out = p;
  API_END
}
mpsg_status mpsg_matvec2_plan_execute(mpsg_matvec_plan plan, const double* theta_in, double* theta_out) {
  API_BEGIN
  MPSG_CHECK(plan && plan->p, "null plan");
  MPSG_CHECK(theta_in && theta_out && theta_in != theta_out, "matvec needs distinct input and output arenas");
  plan->p->run(theta_in, theta_out);
  MPSG_CUDA(cudaGetLastError());
  API_END
}
mpsg_status mpsg_matvec2_plan_execute_noalloc(mpsg_matvec_plan plan, const double* theta_in, double* theta_out) {
  API_BEGIN
  MPSG_CHECK(plan && plan->p, "null plan");
  MPSG_CHECK(theta_in && theta_out && theta_in != theta_out, "matvec needs distinct input and output arenas");
  matvec_noalloc(*plan->p, theta_in, theta_out);
  API_END
}
mpsg_status mpsg_matvec2_plan_info(mpsg_matvec_plan plan, double* info) {
  API_BEGIN
  MPSG_CHECK(plan && plan->p && info, "null argument");
  info[0] = plan->p->flops;
  info[1] = plan->p->flops_ref;
  info[2] = (double)plan->p->bytes_alg;
  info[3] = (double)plan->p->launches_per_run();
  API_END
}
void mpsg_matvec2_plan_destroy(mpsg_matvec_plan plan) {
  if (!plan) return;
  try {
    plan->p.reset();
  } catch (...) {
  }
  delete plan;
}
mpsg_status mpsg_theta_closure(mpsg_ctx ctx, mpsg_tensor L, mpsg_tensor R, mpsg_tensor theta, const mpsg_mpo* Wl,
                               const mpsg_mpo* Wr, const mpsg_itokey* ikl, const mpsg_itokey* ikr,
                               mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(out, "null output");
  Ctx* c = C(ctx);
  const Tensor& th = T(theta);
  Layout sx = theta_closure(T(L), T(R), layout_of(th), mpo_from_c(Wl), mpo_from_c(Wr), itokey_from_c(ikl),
                            itokey_from_c(ikr));
  TensorP o = make_tensor(c, 2, sx, true);
  std::vector<CopyOp> ops;
  for (auto& b : th.b) {
    const Block& nb = o->b[o->find(b.k)];
    ops.push_back(CopyOp{th.d + b.off, o->d + nb.off, nullptr, nullptr, b.r, b.c, b.r, b.r, 0, 1.0});
  }
  run_copyops(c, ops);
  c->sync();
  *out = wrap(o);
  API_END
}
mpsg_status mpsg_dmrg_site(mpsg_dmrg e, int32_t site, mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(e && e->e && out, "null argument");
  MPSG_CHECK(site >= 0 && site < e->e->N, "site out of range");
  *out = wrap(tensor_copy(*e->e->mps[site]));
  e->e->ctx->sync();
  API_END
}
mpsg_status mpsg_dmrg_lambda(mpsg_dmrg e, int32_t bond, mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(e && e->e && out, "null argument");
  auto it = e->e->lam.find(bond);
  MPSG_CHECK(it != e->e->lam.end() && it->second, "no lambda stored for this bond");
  *out = wrap(tensor_copy(*it->second));
  e->e->ctx->sync();
  API_END
}
mpsg_status mpsg_dmrg_measure_energy(mpsg_dmrg e, double* E) {
  API_BEGIN
  MPSG_CHECK(e && e->e && E, "null argument");
  *E = e->e->measure_energy();
  API_END
}
mpsg_status mpsg_dmrg_measure_mpo(mpsg_dmrg e, const mpsg_mpo* W, double* out) {
  API_BEGIN
  MPSG_CHECK(e && e->e && W && out, "null argument");
  std::vector<MPO> w;
  for (int s = 0; s < e->e->N; ++s) w.push_back(mpo_from_c(&W[s]));
  *out = e->e->measure(w);
  API_END
}
void mpsg_dmrg_destroy(mpsg_dmrg e) {
  if (!e) return;
  try {
    delete e->e;
  } catch (...) {
  }
  delete e;
}

}  // extern "C"
