// C ABI of libmpsg (include/mpsg.h) and the DMRG engine (DMRGengine::simulate / doStep).
#include <chrono>
#include <cmath>
#include <cstring>

#include "capi_types.h"
#include "engine.h"

using namespace mpsg;

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
    // place the no-allocation matvec's scratch array now (module load, symbol address), so that
    // mpsg_matvec2_plan_execute_noalloc itself allocates nothing
    noalloc_scratch_address(device);
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
mpsg_status mpsg_ctx_trim(mpsg_ctx ctx) {
  API_BEGIN
  Ctx* c = C(ctx);
  c->sync();
  if (c->side) MPSG_CUDA(cudaStreamSynchronize(c->side));
  cudaMemPool_t pool;
  MPSG_CUDA(cudaDeviceGetDefaultMemPool(&pool, c->device));
  MPSG_CUDA(cudaMemPoolTrimTo(pool, 0));
  API_END
}
void mpsg_tc_autotune_info(int64_t* tuned, int64_t* cache_hits, int32_t* last_schedule2, float* last_timing6) {
  tc_autotune_counts(tuned, cache_hits);
  if (last_schedule2) tc_last_schedules(last_schedule2, last_timing6);
  else if (last_timing6) {
    int32_t tmp[2];
    tc_last_schedules(tmp, last_timing6);
  }
}
int64_t mpsg_ctx_kernel_launches(mpsg_ctx) {
  return kernel_launch_count() + tc_launch_count() + eig_launch_count() + tebd_launch_count() + batch_launch_count() +
         bidiag_launch_count();
}
int64_t mpsg_split_fallbacks(void) { return split_fallback_count(); }
mpsg_status mpsg_ctx_set_svd_method(mpsg_ctx ctx, int32_t method) {
  API_BEGIN
  MPSG_CHECK(method >= 0 && method <= 4,
             "svd method must be 0 (Jacobi SVD), 1 (density matrix, cuSOLVER batched), 2 (density matrix, "
             "cuSOLVER concurrent), 3 (density matrix, own batched eigensolver) or 4 (own bidiagonal SVD)");
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
  if (host_data) tensor_pack_to_host(x, host_data);
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
// environment updates: FP64 or a tensor-core precision (AUTO and MIXED are Lanczos modes)
static void check_env_prec(mpsg_prec prec) {
  MPSG_CHECK(prec >= MPSG_PREC_FP64 && prec <= MPSG_PREC_BF16X3,
             "the environment update takes MPSG_PREC_FP64, TF32, TF32X3, BF16 or BF16X3");
}
static void check_matvec_prec(mpsg_prec prec) {
  MPSG_CHECK(prec >= MPSG_PREC_FP64 && prec <= MPSG_PREC_BF16X3, "matvec precision must be FP64, TF32(X3) or BF16(X3)");
}
static void check_lanczos_prec(mpsg_prec prec) {
  MPSG_CHECK(prec >= MPSG_PREC_FP64 && prec <= MPSG_PREC_MIXED, "unknown precision mode");
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
  check_env_prec(prec);
  Ctx* c = C(ctx);
  MPSG_CHECK(T(A).b.size() > 0, "Error in addContractionLayer: A is empty.");
  TensorP o = env_update(c, T(BL), T(A), mpo_from_c(W), itokey_from_c(ik), direction, nullptr, nullptr, (int)prec);
  c->sync();
  *out = wrap(o);
  API_END
}

mpsg_status mpsg_add_contraction_layer2(mpsg_ctx ctx, mpsg_tensor BL, mpsg_tensor A, mpsg_tensor Ap,
                                        const mpsg_mpo* W, const mpsg_itokey* ik, int32_t direction, mpsg_prec prec,
                                        mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(out, "null output");
  check_env_prec(prec);
  Ctx* c = C(ctx);
  MPSG_CHECK(T(A).b.size() > 0, "Error in addContractionLayer: A is empty.");
  MPSG_CHECK(T(Ap).b.size() > 0, "Error in addContractionLayer: Ap is empty.");
  TensorP o = env_update(c, T(BL), T(A), mpo_from_c(W), itokey_from_c(ik), direction, nullptr, &T(Ap), (int)prec);
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
mpsg_status mpsg_dmrg_excited_simulate(mpsg_dmrg e, const mpsg_tensor* target, double delta_ortho, uint32_t maxsteps,
                                       double EnConv, uint32_t chimax, int32_t doTrunc, double tr_weight, double delta,
                                       int32_t testenergy, int32_t leaveoutlast, double* E) {
  API_BEGIN
  MPSG_CHECK(e && e->e && target && E, "null argument");
  MPSG_CHECK(EnConv > 0, "EnConv must be > 0");
  (void)delta_ortho;  // the reference's only use of it is commented out (src/lanzcos.hpp:349)
  std::vector<TensorP> tgt;
  for (int i = 0; i < e->e->N; ++i) {
    MPSG_CHECK(target[i], "null target tensor");
    MPSG_CHECK(T(target[i]).nphys == 1, "target site tensors must have one physical index");
    tgt.push_back(tensor_copy(T(target[i])));
  }
  *E = e->e->excited_simulate(tgt, (int)maxsteps, EnConv, (int)chimax, doTrunc != 0, tr_weight, delta,
                              testenergy != 0, leaveoutlast != 0);
  API_END
}
mpsg_status mpsg_dmrg_ss_simulate(mpsg_dmrg e, uint32_t maxsteps, double EnConv, double delta, int32_t testenergy,
                                  double* E) {
  API_BEGIN
  MPSG_CHECK(e && e->e && E, "null argument");
  MPSG_CHECK(EnConv > 0, "EnConv must be > 0");
  *E = e->e->ss_simulate((int)maxsteps, EnConv, delta, testenergy != 0);
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
mpsg_status mpsg_dmrg_set_env_prec(mpsg_dmrg e, mpsg_prec prec) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  check_env_prec(prec);
  e->e->env_prec = prec;
  API_END
}
mpsg_status mpsg_dmrg_get_options(mpsg_dmrg e, int32_t* prec, int32_t* reorth, int32_t* lanmax) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  if (prec) *prec = (int32_t)e->e->prec;
  if (reorth) *reorth = e->e->reorth ? 1 : 0;
  if (lanmax) *lanmax = e->e->lanmax;
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
mpsg_status mpsg_dmrg_stats_ext(mpsg_dmrg e, double* st, int32_t n) {
  API_BEGIN
  MPSG_CHECK(e && e->e && st && n >= 0, "null argument");
  Engine& g = *e->e;
  const double v[12] = {(double)g.lst.matvecs, g.lst.matvec_flops, g.lst.matvec_seconds, g.env_seconds,
                        g.split_seconds, g.lst.seconds, g.env_flops, g.wall, g.step_device_seconds,
                        (double)g.nstep_calls, g.prep_seconds, g.lanczos_call_seconds};
  for (int i = 0; i < n && i < 12; ++i) st[i] = v[i];
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
