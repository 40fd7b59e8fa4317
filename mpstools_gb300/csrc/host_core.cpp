// Host core of libmpsg: context, device memory, block-sparse tensors, MPO terms and the
// grouped-GEMM / linear-combination plans that the contractions are built from.
#include <cstdio>
#include "host_core.h"

#include <algorithm>
#include <cstring>

namespace mpsg {

thread_local std::string g_last_error;

// ============================================================================ context
// The library's streams are created at the highest priority, so that kernels queued on the
// lowest-priority side stream (Ctx::side_stream) only take SMs the main work leaves idle.
static int stream_priority(bool highest) {
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return highest ? greatest : least;
}

Ctx::Ctx(int dev) : device(dev) {
  MPSG_CUDA(cudaSetDevice(dev));
  MPSG_CUDA(cudaStreamCreateWithPriority(&own, cudaStreamNonBlocking, stream_priority(true)));
  stream = own;
  cudaMemPool_t pool;
  MPSG_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
  uint64_t thr = UINT64_MAX;
  MPSG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  part = (double*)dmalloc(sizeof(double) * (kRedBlocks + 64));
  MPSG_CUDA(cudaMallocHost(&hscal, sizeof(double) * 4096));
}
Ctx::~Ctx() {
  if (solver) cusolverDnDestroy(solver);
  if (svdp) cusolverDnDestroyGesvdjInfo(svdp);
  if (params) cusolverDnDestroyParams(params);
  for (auto h : whandles) cusolverDnDestroy(h);
  for (auto h : wblas) cublasDestroy(h);
  if (blas) cublasDestroy(blas);
  for (auto s : wstreams) cudaStreamDestroy(s);
  if (side) {
    cudaStreamSynchronize(side);
    cudaStreamDestroy(side);
  }
  for (auto e : wevents) cudaEventDestroy(e);
  if (fork_event) cudaEventDestroy(fork_event);
  if (part) cudaFreeAsync(part, stream);
  cudaStreamSynchronize(stream);
  if (hscal) cudaFreeHost(hscal);
  if (own) cudaStreamDestroy(own);
}
void* Ctx::dmalloc(size_t bytes) {
  if (bytes == 0) bytes = 16;
  void* p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes, stream);
  if (e != cudaSuccess) throw Err(4, std::string("device allocation of ") + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
  return p;
}
void Ctx::dfree(void* p) {
  if (!p) return;
  const cudaError_t e = cudaFreeAsync(p, stream);
  if (e != cudaSuccess) {  // a library bug: report it here instead of at the next unrelated status check
    cudaGetLastError();
    std::fprintf(stderr, "libmpsg: cudaFreeAsync failed: %s\n", cudaGetErrorString(e));
  }
}
cusolverDnHandle_t Ctx::svd_handle() {
  if (!solver) {
    if (cusolverDnCreate(&solver) != CUSOLVER_STATUS_SUCCESS) throw Err(3, "cusolverDnCreate failed");
    cusolverDnSetStream(solver, stream);
    if (cusolverDnCreateGesvdjInfo(&svdp) != CUSOLVER_STATUS_SUCCESS) throw Err(3, "cusolverDnCreateGesvdjInfo failed");
    cusolverDnXgesvdjSetSortEig(svdp, 1);
  }
  cusolverDnSetStream(solver, stream);
  return solver;
}
cublasHandle_t Ctx::blas_handle() {
  if (!blas && cublasCreate(&blas) != CUBLAS_STATUS_SUCCESS) throw Err(3, "cublasCreate failed");
  cublasSetStream(blas, stream);
  return blas;
}
cusolverDnParams_t Ctx::solver_params() {
  if (!params && cusolverDnCreateParams(&params) != CUSOLVER_STATUS_SUCCESS) throw Err(3, "cusolverDnCreateParams failed");
  return params;
}
int Ctx::nworkers() {
  constexpr int kWorkers = 8;
  while ((int)wstreams.size() < kWorkers) {
    cudaStream_t s;
    MPSG_CUDA(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, stream_priority(true)));
    cusolverDnHandle_t h;
    if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS) throw Err(3, "cusolverDnCreate failed");
    cusolverDnSetStream(h, s);
    cublasHandle_t b;
    if (cublasCreate(&b) != CUBLAS_STATUS_SUCCESS) throw Err(3, "cublasCreate failed");
    cublasSetStream(b, s);
    wstreams.push_back(s);
    whandles.push_back(h);
    wblas.push_back(b);
  }
  return kWorkers;
}
cudaStream_t Ctx::side_stream() {
  if (!side) MPSG_CUDA(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, stream_priority(false)));
  return side;
}
void Ctx::fork(int n) {
  MPSG_CHECK(n >= 0 && n <= nworkers(), "fork: more streams than workers");
  if (!fork_event) MPSG_CUDA(cudaEventCreateWithFlags(&fork_event, cudaEventDisableTiming));
  MPSG_CUDA(cudaEventRecord(fork_event, stream));
  for (int i = 0; i < n; ++i) MPSG_CUDA(cudaStreamWaitEvent(wstreams[i], fork_event, 0));
}
void Ctx::join(int n) {
  while ((int)wevents.size() < n) {
    cudaEvent_t e;
    MPSG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    wevents.push_back(e);
  }
  for (int i = 0; i < n; ++i) {
    MPSG_CUDA(cudaEventRecord(wevents[i], wstreams[i]));
    MPSG_CUDA(cudaStreamWaitEvent(stream, wevents[i], 0));
  }
}
void Ctx::sync() { MPSG_CUDA(cudaStreamSynchronize(stream)); }

// ============================================================================ layouts and tensors
void Layout::finalize() {
  std::sort(b.begin(), b.end(), [](const Block& x, const Block& y) { return x.k < y.k; });
  idx.clear();
  int64_t off = 0;
  for (size_t i = 0; i < b.size(); ++i) {
    if (i && b[i].k == b[i - 1].k) throw Err(1, "duplicate block key");
    b[i].off = off;
    off += ((int64_t)b[i].r * b[i].c + kAlign - 1) / kAlign * kAlign;
    idx[b[i].k] = (int)i;
  }
  nelem = off;
}

Tensor::~Tensor() {
  if (d && ctx) ctx->dfree(d);
}

TensorP make_tensor(Ctx* ctx, int nphys, const Layout& lay, bool zero) {
  TensorP t = std::make_shared<Tensor>();
  t->ctx = ctx;
  t->keep = ctx->shared_from_this();
  t->nphys = nphys;
  t->b = lay.b;
  t->idx = lay.idx;
  t->nelem = lay.nelem;
  t->d = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(t->nelem, 2));
  if (zero) MPSG_CUDA(cudaMemsetAsync(t->d, 0, sizeof(double) * std::max<int64_t>(t->nelem, 2), ctx->stream));
  return t;
}

Layout layout_of(const Tensor& t) {
  Layout l;
  l.b = t.b;
  l.idx = t.idx;
  l.nelem = t.nelem;
  return l;
}

TensorP tensor_from_host(Ctx* ctx, int nphys, int n, const uint64_t* q, const uint32_t* p, const int32_t* rows,
                         const int32_t* cols, const double* data) {
  MPSG_CHECK(nphys >= 0 && nphys <= 2, "nphys must be 0, 1 or 2");
  MPSG_CHECK(n >= 0, "nblocks < 0");
  Layout lay;
  std::vector<int64_t> src_off(n);
  int64_t so = 0;
  for (int i = 0; i < n; ++i) {
    MPSG_CHECK(rows[i] >= 0 && cols[i] >= 0, "negative block size");
    BKey k;
    k.q0 = q[2 * i];
    k.q1 = q[2 * i + 1];
    if (nphys >= 1) k.p0 = p[nphys * i];
    if (nphys >= 2) k.p1 = p[nphys * i + 1];
    lay.add(k, rows[i], cols[i]);
    src_off[i] = so;
    so += (int64_t)rows[i] * cols[i];
  }
  // keep the caller's order to find sources after sorting
  std::map<BKey, int64_t> srcpos;
  for (int i = 0; i < n; ++i) srcpos[lay.b[i].k] = src_off[i];
  lay.finalize();
  TensorP t = make_tensor(ctx, nphys, lay, true);
  if (data && n && so > 0) {
    // the caller's packed buffer goes up in one copy (DMA straight from it when the caller pinned it)
    // and a gather kernel places the blocks at their aligned arena offsets
    double* stage = (double*)ctx->dmalloc(sizeof(double) * (size_t)so);
    MPSG_CUDA(cudaMemcpyAsync(stage, data, sizeof(double) * (size_t)so, cudaMemcpyHostToDevice, ctx->stream));
    std::vector<CopyOp> ops;
    for (auto& b : t->b) {
      if (!b.r || !b.c) continue;
      ops.push_back(CopyOp{stage + srcpos[b.k], t->d + b.off, nullptr, nullptr, b.r, b.c, b.r, b.r, 0, 1.0});
    }
    run_copyops(ctx, ops);
    ctx->dfree(stage);
    ctx->sync();
  }
  return t;
}

void tensor_pack_to_host(const Tensor& t, double* dst) {
  int64_t total = 0;
  for (auto& b : t.b) total += (int64_t)b.r * b.c;
  if (total == 0) return;
  Ctx* ctx = t.ctx;
  double* stage = (double*)ctx->dmalloc(sizeof(double) * (size_t)total);
  std::vector<CopyOp> ops;
  int64_t o = 0;
  for (auto& b : t.b) {
    if (b.r && b.c) ops.push_back(CopyOp{t.d + b.off, stage + o, nullptr, nullptr, b.r, b.c, b.r, b.r, 0, 1.0});
    o += (int64_t)b.r * b.c;
  }
  run_copyops(ctx, ops);
  MPSG_CUDA(cudaMemcpyAsync(dst, stage, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost, ctx->stream));
  ctx->dfree(stage);
  ctx->sync();
}

void tensor_to_host(const Tensor& t, std::vector<double>& packed) {
  int64_t total = 0;
  for (auto& b : t.b) total += (int64_t)b.r * b.c;
  packed.assign((size_t)total, 0.0);
  tensor_pack_to_host(t, packed.data());
}

TensorP tensor_copy(const Tensor& t) {
  TensorP c = make_tensor(t.ctx, t.nphys, layout_of(t), false);
  MPSG_CUDA(cudaMemcpyAsync(c->d, t.d, sizeof(double) * std::max<int64_t>(t.nelem, 2), cudaMemcpyDeviceToDevice, t.ctx->stream));
  return c;
}

// ============================================================================ MPO
MPO mpo_from_c(const mpsg_mpo* w) {
  MPSG_CHECK(w != nullptr, "null MPO");
  MPO m;
  m.Dl = w->Dl;
  m.Dr = w->Dr;
  std::map<std::pair<uint32_t, uint32_t>, std::map<std::pair<uint32_t, uint32_t>, double>> tmp;
  for (int i = 0; i < w->nterms; ++i) tmp[{w->wl[i], w->wr[i]}][{w->in[i], w->out[i]}] = w->value[i];
  for (auto& e : tmp) {
    MPOEntry en;
    en.wl = e.first.first;
    en.wr = e.first.second;
    for (auto& o : e.second) en.ops.push_back(OpEl{o.first.second, o.first.first, o.second});
    m.e.push_back(en);
  }
  return m;
}
ItoKey itokey_from_c(const mpsg_itokey* ik) {
  MPSG_CHECK(ik != nullptr && ik->d > 0, "bad itokey");
  return ItoKey(ik->charge, ik->charge + ik->d);
}

// ============================================================================ grouped GEMM plan
void GemmPlan::add_problem(int baseC, int64_t offC, int ldc, int M, int N, bool accumulate,
                           const std::vector<GSegH>& segs) {
  GProbH p;
  p.baseC = baseC;
  p.offC = offC;
  p.ldc = ldc;
  p.M = M;
  p.N = N;
  p.beta = accumulate ? 1 : 0;
  p.seg0 = (int)hseg.size();
  for (auto& s : segs) {
    hseg.push_back(s);
    flops += 2.0 * (double)M * N * s.K;
  }
  p.seg1 = (int)hseg.size();
  hprob.push_back(p);
}
void GemmPlan::upload(Ctx* ctx) {
  this->ctx = ctx;
  keep = ctx->shared_from_this();
  std::vector<GTile> tiles;
  prob_tile0.assign(hprob.size() + 1, 0);
  for (size_t i = 0; i < hprob.size(); ++i) {
    prob_tile0[i] = (int)tiles.size();
    // 64 x 64 tiles, the last of each row / column trimmed to the block edge in steps of 16
    for (int m0 = 0; m0 < hprob[i].M; m0 += 64)
      for (int n0 = 0; n0 < hprob[i].N; n0 += 64) {
        const int mi = std::min(4, (hprob[i].M - m0 + 15) / 16), nj = std::min(4, (hprob[i].N - n0 + 15) / 16);
        tiles.push_back(GTile{(int32_t)i, m0, n0, (int8_t)mi, (int8_t)nj});
      }
  }
  ntiles = (int)tiles.size();
  prob_tile0[hprob.size()] = ntiles;
  std::vector<GProb> p(hprob.size());
  std::vector<GSeg> s(hseg.size());
  for (size_t i = 0; i < hprob.size(); ++i) {
    const GProbH& h = hprob[i];
    p[i].offC = h.offC;
    p[i].ldc = h.ldc;
    p[i].M = h.M;
    p[i].N = h.N;
    p[i].seg0 = h.seg0;
    p[i].seg1 = h.seg1;
    p[i].baseC = (int8_t)h.baseC;
    p[i].beta = (int8_t)h.beta;
  }
  for (size_t i = 0; i < hseg.size(); ++i) {
    const GSegH& h = hseg[i];
    s[i].offA = h.offA;
    s[i].offB = h.offB;
    s[i].lda = h.lda;
    s[i].ldb = h.ldb;
    s[i].K = h.K;
    s[i].baseA = (int8_t)h.baseA;
    s[i].baseB = (int8_t)h.baseB;
    s[i].tA = (int8_t)h.tA;
    s[i].tB = (int8_t)h.tB;
    s[i].alpha = h.alpha;
  }
  dprob = (GProb*)ctx->dmalloc(sizeof(GProb) * std::max<size_t>(p.size(), 1));
  dseg = (GSeg*)ctx->dmalloc(sizeof(GSeg) * std::max<size_t>(s.size(), 1));
  dtile = (GTile*)ctx->dmalloc(sizeof(GTile) * std::max<size_t>(tiles.size(), 1));
  if (!tiles.empty())
    MPSG_CUDA(cudaMemcpyAsync(dtile, tiles.data(), sizeof(GTile) * tiles.size(), cudaMemcpyHostToDevice, ctx->stream));
  if (!p.empty()) MPSG_CUDA(cudaMemcpyAsync(dprob, p.data(), sizeof(GProb) * p.size(), cudaMemcpyHostToDevice, ctx->stream));
  if (!s.empty()) MPSG_CUDA(cudaMemcpyAsync(dseg, s.data(), sizeof(GSeg) * s.size(), cudaMemcpyHostToDevice, ctx->stream));
}
void GemmPlan::run(const double* const* bases) {
  if (hprob.empty()) return;
  Bases b;
  for (int i = 0; i < 8; ++i) b.p[i] = bases[i];
  launch_gemm_f64(dprob, dseg, dtile, ntiles, b, ctx->stream);
}
void GemmPlan::run_range(const double* const* bases, int p0, int p1) {
  MPSG_CHECK(p0 >= 0 && p0 <= p1 && p1 <= (int)hprob.size(), "GEMM problem range outside the plan");
  const int t0 = prob_tile0[p0], t1 = prob_tile0[p1];
  if (t1 <= t0) return;
  Bases b;
  for (int i = 0; i < 8; ++i) b.p[i] = bases[i];
  launch_gemm_f64(dprob, dseg, dtile + t0, t1 - t0, b, ctx->stream);
}
GemmPlan::~GemmPlan() {
  if (ctx) {
    ctx->dfree(dprob);
    ctx->dfree(dseg);
    ctx->dfree(dtile);
  }
}

// ============================================================================ linear combination plan
void LincombPlan::add(double* dst, int64_t n, const std::vector<std::pair<const double*, double>>& terms) {
  LCOut o;
  o.dst = dst;
  o.n = n;
  o.t0 = (int32_t)hterm.size();
  for (auto& t : terms) hterm.push_back(LCTerm{t.first, t.second});
  o.t1 = (int32_t)hterm.size();
  hout.push_back(o);
  maxn = std::max(maxn, n);
}
void LincombPlan::run(Ctx* ctx) {
  if (hout.empty()) return;
  LCOut* dout = (LCOut*)ctx->dmalloc(sizeof(LCOut) * hout.size());
  LCTerm* dterm = (LCTerm*)ctx->dmalloc(sizeof(LCTerm) * std::max<size_t>(hterm.size(), 1));
  MPSG_CUDA(cudaMemcpyAsync(dout, hout.data(), sizeof(LCOut) * hout.size(), cudaMemcpyHostToDevice, ctx->stream));
  if (!hterm.empty())
    MPSG_CUDA(cudaMemcpyAsync(dterm, hterm.data(), sizeof(LCTerm) * hterm.size(), cudaMemcpyHostToDevice, ctx->stream));
  launch_lincomb(dout, dterm, (int)hout.size(), maxn, ctx->stream);
  ctx->dfree(dout);
  ctx->dfree(dterm);
}

void run_copyops(Ctx* ctx, const std::vector<CopyOp>& ops) {
  if (ops.empty()) return;
  CopyOp* d = (CopyOp*)ctx->dmalloc(sizeof(CopyOp) * ops.size());
  MPSG_CUDA(cudaMemcpyAsync(d, ops.data(), sizeof(CopyOp) * ops.size(), cudaMemcpyHostToDevice, ctx->stream));
  launch_copyops(d, (int)ops.size(), ctx->stream);
  ctx->dfree(d);
}

}  // namespace mpsg
