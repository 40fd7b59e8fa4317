// TEBD engine on the GPU (complex FP64 Vidal form): shared by the forward evolution (tebd.cpp) and the
// adjoint (tebd_adjoint.cpp).
//
// TEBD on the GPU: two-site gates exp(-i dt h_b) (MPO::getNNGate, src/MPOTypes.hpp:1090-1209),
// applyGate on the Vidal form lambda Gamma lambda Gamma lambda (src/MPSfunctions.hpp:1492-1548),
// time slices over even / odd bonds (TEBDengine::doTimeSlice, src/container.hpp:1195-1233) and the
// second-order Trotter schedule (TEBDengine::simulate, src/container.hpp:1325-1395).
//
// Complex block tensors are planar Tensors: the arena holds the real parts of all blocks, then the
// imaginary parts at offset nelem.  Complex products run on the grouped FP64 GEMM as four real
// products, the gate is a complex linear combination of blocks (k_lincomb), and the split takes, per
// charge sector, the library's bidiagonal SVD for complex matrices (svd method 4: complex Householder
// bidiagonalisation to a real bidiagonal, the real Golub-Kahan stages, complex back-transformation;
// zsvd_bidiag), cuSOLVER's one-sided Jacobi SVD (zgesvdj, method 0 and the fallback) or the density
// route, with the complex FixPhase.
#pragma once
#include <cfloat>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>

#include "capi_types.h"

namespace mpsg {

typedef std::complex<double> cplx;

inline Q qat_(const ItoKey& ik, uint32_t s) {
  MPSG_CHECK(s < ik.size(), "physical index outside i_to_key");
  return ik[s];
}

// planar complex tensor: TensorP whose arena is 2 * nelem (re plane, im plane)
inline TensorP make_ctensor(Ctx* ctx, int nphys, Layout lay, bool zero) {
  lay.finalize();
  TensorP t = std::make_shared<Tensor>();
  t->ctx = ctx;
  t->keep = ctx->shared_from_this();
  t->nphys = nphys;
  t->b = lay.b;
  t->idx = lay.idx;
  t->nelem = lay.nelem;
  const size_t bytes = sizeof(double) * std::max<int64_t>(2 * t->nelem, 2);
  t->d = (double*)ctx->dmalloc(bytes);
  if (zero) MPSG_CUDA(cudaMemsetAsync(t->d, 0, bytes, ctx->stream));
  return t;
}
inline double* re(const Tensor& t, int i) { return t.d + t.b[i].off; }
inline double* im(const Tensor& t, int i) { return t.d + t.nelem + t.b[i].off; }

// ---------------------------------------------------------------- direct sums of independent bonds
// Part i's charges are shifted by i << 32; shifting keeps each part's key order and puts part i
// after part i - 1, so a direct sum is the concatenation of the parts' planes.
inline Layout shifted_layout(const std::vector<const Tensor*>& parts) {
  Layout lay;
  for (size_t i = 0; i < parts.size(); ++i)
    for (const Block& b : parts[i]->b) {
      MPSG_CHECK(b.k.q0 < ((Q)1 << 32) && b.k.q1 < ((Q)1 << 32), "charge too large for a bond direct sum");
      BKey k = b.k;
      k.q0 += (Q)i << 32;
      k.q1 += (Q)i << 32;
      lay.add(k, b.r, b.c);
    }
  return lay;
}
// planes = 2 for planar complex tensors, 1 for real ones
inline TensorP bond_sum(Ctx* ctx, const std::vector<const Tensor*>& parts, int nphys, int planes) {
  Layout lay = shifted_layout(parts);
  TensorP t;
  if (planes == 2) {
    t = make_ctensor(ctx, nphys, lay, false);
  } else {
    lay.finalize();
    t = make_tensor(ctx, nphys, lay, false);
  }
  int64_t pre = 0;
  size_t j = 0;
  for (const Tensor* p : parts) {
    for (const Block& b : p->b) MPSG_CHECK(t->b[j++].off == pre + b.off, "bond direct sum is not a concatenation");
    MPSG_CHECK(pre + p->nelem <= t->nelem, "bond direct sum smaller than its parts");
    for (int pl = 0; pl < planes; ++pl)
      if (p->nelem > 0)
        MPSG_CUDA(cudaMemcpyAsync(t->d + pl * t->nelem + pre, p->d + pl * p->nelem, sizeof(double) * p->nelem,
                                  cudaMemcpyDeviceToDevice, ctx->stream));
    pre += p->nelem;
  }
  return t;
}
inline TensorP bond_part(Ctx* ctx, const Tensor& t, int i, int planes) {
  Layout lay;
  int j0 = -1, j1 = -1;
  for (int j = 0; j < (int)t.b.size(); ++j) {
    const Block& b = t.b[j];
    if ((b.k.q0 >> 32) != (Q)i) continue;
    if (j0 < 0) j0 = j;
    j1 = j + 1;
    BKey k = b.k;
    k.q0 -= (Q)i << 32;
    k.q1 -= (Q)i << 32;
    lay.add(k, b.r, b.c);
  }
  TensorP o;
  if (planes == 2) {
    o = make_ctensor(ctx, t.nphys, lay, false);
  } else {
    lay.finalize();
    o = make_tensor(ctx, t.nphys, lay, false);
  }
  if (j0 >= 0) {
    const int64_t off0 = t.b[j0].off;
    for (int j = j0; j < j1; ++j) MPSG_CHECK(o->b[j - j0].off == t.b[j].off - off0, "bond part is not contiguous");
    MPSG_CHECK(off0 + o->nelem <= t.nelem, "bond part outside the direct sum");
    for (int pl = 0; pl < planes; ++pl)
      if (o->nelem > 0)
        MPSG_CUDA(cudaMemcpyAsync(o->d + pl * o->nelem, t.d + pl * t.nelem + off0, sizeof(double) * o->nelem,
                                  cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return o;
}

// ---------------------------------------------------------------- gate (host)
// Dense (d1 d2) x (d1 d2) gate, index o1 + d1*o2, column-major.
struct CGate {
  int d1 = 0, d2 = 0;
  std::vector<cplx> g;
  cplx at(int o1, int o2, int i1, int i2) const {
    const int D = d1 * d2;
    return g[(size_t)(o1 + d1 * o2) + (size_t)(i1 + d1 * i2) * D];
  }
};

// Eigen-decomposition of a small real symmetric matrix (column-major n x n) by cyclic Jacobi rotations:
// A = V diag(E) V^T.  A is overwritten.
void jacobi_sym(int n, std::vector<double>& A, std::vector<double>& V, std::vector<double>& E);

// Bond Hamiltonian h_b of bond (site1, site1 + 1) from the two MPO tensors, as a real (d1 d2) x (d1 d2)
// column-major matrix in the gate index o1 + d1 * o2; entries below 1e-14 set to zero.
std::vector<double> bond_hamiltonian(const MPO& m1, const MPO& m2, int site1, int N, int d1, int d2);

// G = exp(-(dt_im + i dt_re) h_b) (MPO::getNNGate).
CGate nn_gate(const MPO& m1, const MPO& m2, int site1, int N, double dt_re, double dt_im, int d1, int d2);

// ---------------------------------------------------------------- engine
struct TebdEngine {
  Ctx* ctx = nullptr;
  std::shared_ptr<Ctx> keep;
  int N = 0;
  std::vector<ItoKey> ik;
  std::vector<MPO> mpo;
  std::vector<TensorP> G;    // Gamma[s], planar complex, nphys 1
  std::vector<TensorP> lam;  // lam[b + 1] = lambda of bond b (b = -1 .. N-1), real, blocks (q, q) n x 1
  double seconds = 0, split_seconds = 0, adjoint_seconds = 0;
  int64_t zsvd_fallbacks = 0;  // splits the bidiagonal route handed to zgesvdj
  int64_t gates = 0;
  // Layer batching: when seg_gates is set, the engine holds a direct sum of independent bonds (bond i's
  // charges shifted by i << 32), block (q0, ...) uses the gate seg_gates[q0 >> 32], and truncation and
  // normalisation run per bond; seg_tw / seg_chi receive the per-bond results.
  std::vector<const CGate*> seg_gates;
  std::vector<double> seg_tw;
  std::vector<int> seg_chi;
  bool batch_layers = true;  // slice(): one split per layer (direct sum over its bonds)

  const double* lam_ptr(const Tensor& l, Q q, int* n) const {
    const int i = l.find(K1(q, q, 0));
    if (i < 0) return nullptr;
    if (n) *n = l.b[i].r;
    return l.d + l.b[i].off;
  }
  TensorP recip(const Tensor& l) {
    TensorP t = make_tensor(ctx, 0, layout_of(l), false);
    launch_recip(t->d, l.d, l.nelem, ctx->stream);
    return t;
  }
  // block max |x|^2 of every block (one sync)
  std::vector<double> block_max2(const Tensor& t) {
    std::vector<double> out(t.b.size(), 0.0);
    if (t.b.empty()) return out;
    std::vector<CBlockOp> ops;
    for (size_t i = 0; i < t.b.size(); ++i)
      ops.push_back(CBlockOp{re(t, (int)i), im(t, (int)i), (int64_t)t.b[i].r * t.b[i].c});
    CBlockOp* d = (CBlockOp*)ctx->dmalloc(sizeof(CBlockOp) * ops.size() + sizeof(double) * ops.size());
    double* dout = (double*)(d + ops.size());
    MPSG_CUDA(cudaMemcpyAsync(d, ops.data(), sizeof(CBlockOp) * ops.size(), cudaMemcpyHostToDevice, ctx->stream));
    launch_cblock_max2(d, (int)ops.size(), dout, ctx->stream);
    MPSG_CUDA(cudaMemcpyAsync(out.data(), dout, sizeof(double) * ops.size(), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    ctx->dfree(d);
    return out;
  }
  // planar copy of the blocks `keep` of t with row / column scale arrays from rs_of / cs_of
  template <class RS, class CS>
  TensorP scaled_copy(const Tensor& t, const std::vector<int>& keepb, RS rs_of, CS cs_of) {
    Layout lay;
    for (int i : keepb) lay.add(t.b[i].k, t.b[i].r, t.b[i].c);
    TensorP o = make_ctensor(ctx, t.nphys, lay, false);
    std::vector<CopyOp> ops;
    for (int i : keepb) {
      const int j = o->find(t.b[i].k);
      const Block& b = t.b[i];
      for (int pl = 0; pl < 2; ++pl)
        ops.push_back(CopyOp{pl ? im(t, i) : re(t, i), pl ? im(*o, j) : re(*o, j), rs_of(b), cs_of(b), b.r, b.c, b.r,
                             b.r, 0, 1.0});
    }
    run_copyops(ctx, ops);
    return o;
  }

  void init_product(const std::vector<int>& local) {
    G.clear();
    lam.clear();
    auto unit_lam = [&](Q q) {
      Layout l;
      l.add(K1(q, q, 0), 1, 1);
      l.finalize();
      double one = 1.0;
      uint64_t qq[2] = {q, q};
      uint32_t p[1] = {0};
      int32_t r[1] = {1}, c[1] = {1};
      return tensor_from_host(ctx, 0, 1, qq, p, r, c, &one);
    };
    Q q = 0;
    lam.push_back(unit_lam(q));
    for (int s = 0; s < N; ++s) {
      MPSG_CHECK(local[s] >= 0 && local[s] < (int)ik[s].size(), "local state index outside i_to_key");
      const Q q1 = q + qat_(ik[s], (uint32_t)local[s]);
      Layout l;
      l.add(K1(q, q1, (uint32_t)local[s]), 1, 1);
      TensorP g = make_ctensor(ctx, 1, l, true);
      const double one = 1.0;
      MPSG_CUDA(cudaMemcpyAsync(g->d, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
      ctx->sync();
      G.push_back(g);
      lam.push_back(unit_lam(q1));
      q = q1;
    }
  }

  // one centre-charge sector of the split: rows (s1 ranges) x columns (s2 ranges); M stored tall
  // (M^H for a wide sector) in the interleaved complex arena
  struct Sec {
    std::map<uint32_t, std::pair<int, int>> rx, ry;
    std::vector<int> blocks;
    int m = 0, n = 0, k = 0;
    int64_t offM = 0, offU = 0, offV = 0, offS = 0;
  };

  // Density-matrix SVD of every sector (the exact route is cuSOLVER zgesvdj): G = A^H A of the stored
  // tall matrix A (ms x ns) by cuBLAS zgemm into slots of power-of-two size classes (padding diagonal
  // -1), cuSOLVER's batched Hermitian eigensolver per class, the eigenvectors ranked descending
  // (eigenvalues below 32 ns eps lambda_max unresolved: zero), then y_j = A v_j, s_j = |y_j|, u_j =
  // y_j / s_j.  A singular value s carries an absolute error ~ eps s_max^2 / s (the Gram matrix's
  // resolution); the u_j are orthonormal to ~eps s_max / s.
  void density_svd(std::map<Q, Sec>& secs, double2* dM, double2* dU, double2* dV, double* dS) {
    cusolverDnHandle_t h = ctx->svd_handle();
    cublasHandle_t bh = ctx->blas_handle();
    std::map<int, std::vector<Sec*>> cls;
    for (auto& x : secs) {
      Sec& s = x.second;
      if (s.k == 0) continue;
      int c = 32;
      while (c < std::min(s.m, s.n)) c <<= 1;
      cls[c].push_back(&s);
    }
    int64_t oB = 0, oW = 0, nsec = 0;
    for (auto& c : cls) {
      oB += (int64_t)c.first * c.first * (int64_t)c.second.size();
      oW += (int64_t)c.first * (int64_t)c.second.size();
      nsec += (int64_t)c.second.size();
    }
    double2* dB = (double2*)ctx->dmalloc(sizeof(double2) * std::max<int64_t>(oB, 2));
    double* dWv = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oW, 2));
    int* dinf = (int*)ctx->dmalloc(sizeof(int) * (size_t)(nsec + 1));
    MPSG_CUDA(cudaMemsetAsync(dB, 0, sizeof(double2) * std::max<int64_t>(oB, 2), ctx->stream));
    MPSG_CUDA(cudaMemsetAsync(dinf, 0, sizeof(int) * (size_t)(nsec + 1), ctx->stream));
    const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
    struct Slot {
      Sec* s;
      double2* B;
      double* W;
      int nc;
    };
    std::vector<Slot> slots;
    std::vector<CGramPad> pads;
    {
      int64_t b = 0, w = 0;
      for (auto& c : cls)
        for (Sec* s : c.second) {
          slots.push_back(Slot{s, dB + b, dWv + w, c.first});
          b += (int64_t)c.first * c.first;
          w += c.first;
        }
    }
    for (Slot& sl : slots) {
      Sec& s = *sl.s;
      const bool tall = s.m >= s.n;
      const int ms = tall ? s.m : s.n, ns = tall ? s.n : s.m;
      if (cublasZgemm(bh, CUBLAS_OP_C, CUBLAS_OP_N, ns, ns, ms, &one, (const cuDoubleComplex*)(dM + s.offM), ms,
                      (const cuDoubleComplex*)(dM + s.offM), ms, &zero, (cuDoubleComplex*)sl.B, sl.nc) !=
          CUBLAS_STATUS_SUCCESS)
        throw Err(3, "zgemm (Gram matrix) failed");
      pads.push_back(CGramPad{sl.B, sl.nc, ns});
    }
    {
      CGramPad* d = (CGramPad*)ctx->dmalloc(sizeof(CGramPad) * pads.size());
      MPSG_CUDA(cudaMemcpyAsync(d, pads.data(), sizeof(CGramPad) * pads.size(), cudaMemcpyHostToDevice, ctx->stream));
      launch_cgram_pad(d, (int)pads.size(), ctx->stream);
      ctx->dfree(d);
    }
    int ib = 0;
    size_t first = 0;
    for (auto& c : cls) {
      const int64_t n = c.first, batch = (int64_t)c.second.size();
      double2* A = slots[first].B;
      double* W = slots[first].W;
      size_t wd = 0, wh = 0;
      if (cusolverDnXsyevBatched_bufferSize(h, ctx->solver_params(), CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                            CUDA_C_64F, A, n, CUDA_R_64F, W, CUDA_C_64F, &wd, &wh, batch) !=
          CUSOLVER_STATUS_SUCCESS)
        throw Err(3, "complex syevBatched_bufferSize failed");
      void* dwork = ctx->dmalloc(wd + 16);
      std::vector<char> hwork(wh + 16);
      if (cusolverDnXsyevBatched(h, ctx->solver_params(), CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                 CUDA_C_64F, A, n, CUDA_R_64F, W, CUDA_C_64F, dwork, wd, hwork.data(), wh, dinf + ib,
                                 batch) != CUSOLVER_STATUS_SUCCESS)
        throw Err(3, "complex syevBatched failed");
      ctx->sync();  // the host workspace must outlive the call
      ctx->dfree(dwork);
      ib += (int)batch;
      first += (size_t)batch;
    }
    {
      std::vector<int> inf(ib + 1, 0);
      MPSG_CUDA(cudaMemcpyAsync(inf.data(), dinf, sizeof(int) * (ib + 1), cudaMemcpyDeviceToHost, ctx->stream));
      ctx->sync();
      for (int i = 0; i < ib; ++i)
        if (inf[i] != 0) throw Err(3, "batched Hermitian eigensolver failed (info=" + std::to_string(inf[i]) + ")");
    }
    std::vector<CGramPost> post;
    std::vector<CColNorm> cn;
    for (Slot& sl : slots) {
      Sec& s = *sl.s;
      const bool tall = s.m >= s.n;
      const int ms = tall ? s.m : s.n, ns = tall ? s.n : s.m;
      double2* uo = tall ? dU + s.offU : dV + s.offV;  // left vectors of the stored matrix
      double2* vo = tall ? dV + s.offV : dU + s.offU;  // right vectors of the stored matrix
      post.push_back(CGramPost{sl.B, sl.W, vo, dS + s.offS, ns, sl.nc});
      cn.push_back(CColNorm{uo, dS + s.offS, ms, s.k, ms});
    }
    {
      CGramPost* d = (CGramPost*)ctx->dmalloc(sizeof(CGramPost) * post.size());
      MPSG_CUDA(cudaMemcpyAsync(d, post.data(), sizeof(CGramPost) * post.size(), cudaMemcpyHostToDevice, ctx->stream));
      launch_cgram_post(d, (int)post.size(), ctx->stream);
      ctx->dfree(d);
    }
    for (Slot& sl : slots) {  // y = A V
      Sec& s = *sl.s;
      const bool tall = s.m >= s.n;
      const int ms = tall ? s.m : s.n, ns = tall ? s.n : s.m;
      double2* uo = tall ? dU + s.offU : dV + s.offV;
      const double2* vo = tall ? dV + s.offV : dU + s.offU;
      if (cublasZgemm(bh, CUBLAS_OP_N, CUBLAS_OP_N, ms, s.k, ns, &one, (const cuDoubleComplex*)(dM + s.offM), ms,
                      (const cuDoubleComplex*)vo, ns, &zero, (cuDoubleComplex*)uo, ms) != CUBLAS_STATUS_SUCCESS)
        throw Err(3, "zgemm (left vectors) failed");
    }
    {
      CColNorm* d = (CColNorm*)ctx->dmalloc(sizeof(CColNorm) * cn.size());
      MPSG_CUDA(cudaMemcpyAsync(d, cn.data(), sizeof(CColNorm) * cn.size(), cudaMemcpyHostToDevice, ctx->stream));
      launch_ccolnorm(d, (int)cn.size(), ctx->stream);
      ctx->dfree(d);
    }
    ctx->dfree(dinf);
    ctx->dfree(dWv);
    ctx->dfree(dB);
  }

  // applyGate on bond (site, site+1); returns (truncated weight, kept count)
  std::pair<double, int> apply_gate(int site, const CGate& gate, int chimax, bool doTrunc, double tr_weight,
                                    bool normalize) {
    const Tensor &Gl = *G[site], &Gr = *G[site + 1];
    const Tensor &ll = *lam[site], &lc = *lam[site + 1], &lr = *lam[site + 2];
    // Ml = lambda_l Gamma_l lambda_c, Mr = Gamma_r lambda_r (blocks without lambdas dropped)
    std::vector<int> kl, kr;
    for (int i = 0; i < (int)Gl.b.size(); ++i)
      if (lam_ptr(ll, Gl.b[i].k.q0, nullptr) && lam_ptr(lc, Gl.b[i].k.q1, nullptr)) kl.push_back(i);
    for (int i = 0; i < (int)Gr.b.size(); ++i)
      if (lam_ptr(lr, Gr.b[i].k.q1, nullptr)) kr.push_back(i);
    TensorP Ml = scaled_copy(Gl, kl, [&](const Block& b) { return lam_ptr(ll, b.k.q0, nullptr); },
                             [&](const Block& b) { return lam_ptr(lc, b.k.q1, nullptr); });
    TensorP Mr = scaled_copy(Gr, kr, [&](const Block&) { return (const double*)nullptr; },
                             [&](const Block& b) { return lam_ptr(lr, b.k.q1, nullptr); });
    // theta(a, b; s1, s2) = Ml(a, c; s1) Mr(c, b; s2), complex as four real products
    std::map<BKey, std::vector<std::pair<int, int>>> tp;
    std::map<BKey, std::pair<int, int>> tdim;
    std::map<Q, std::vector<int>> byleft;
    for (int j = 0; j < (int)Mr->b.size(); ++j) byleft[Mr->b[j].k.q0].push_back(j);
    for (int i = 0; i < (int)Ml->b.size(); ++i) {
      auto it = byleft.find(Ml->b[i].k.q1);
      if (it == byleft.end()) continue;
      for (int j : it->second) {
        BKey k = K2(Ml->b[i].k.q0, Mr->b[j].k.q1, Ml->b[i].k.p0, Mr->b[j].k.p0);
        tp[k].push_back({i, j});
        tdim[k] = {Ml->b[i].r, Mr->b[j].c};
      }
    }
    Layout lt;
    for (auto& x : tdim) lt.add(x.first, x.second.first, x.second.second);
    TensorP th = make_ctensor(ctx, 2, lt, false);
    {
      GemmPlan g;
      const int64_t pl = Ml->nelem, pr = Mr->nelem, pt = th->nelem;
      for (auto& x : tp) {
        const Block& tb = th->b[th->find(x.first)];
        std::vector<GSegH> sre, sim;
        for (auto& pr_ : x.second) {
          const Block& a = Ml->b[pr_.first];
          const Block& b = Mr->b[pr_.second];
          sre.push_back(GSegH{0, 1, a.off, b.off, a.r, b.r, a.c, 0, 0, 1.0});
          sre.push_back(GSegH{0, 1, a.off + pl, b.off + pr, a.r, b.r, a.c, 0, 0, -1.0});
          sim.push_back(GSegH{0, 1, a.off, b.off + pr, a.r, b.r, a.c, 0, 0, 1.0});
          sim.push_back(GSegH{0, 1, a.off + pl, b.off, a.r, b.r, a.c, 0, 0, 1.0});
        }
        g.add_problem(2, tb.off, tb.r, tb.r, tb.c, false, sre);
        g.add_problem(2, tb.off + pt, tb.r, tb.r, tb.c, false, sim);
      }
      g.upload(ctx);
      const double* bases[8] = {Ml->d, Mr->d, th->d, nullptr, nullptr, nullptr, nullptr, nullptr};
      g.run(bases);
    }
    // theta'(a, b; o1, o2) = sum_{i1, i2} G[(o1, o2), (i1, i2)] theta(a, b; i1, i2)
    std::map<BKey, std::vector<std::pair<int, cplx>>> gt;
    for (int i = 0; i < (int)th->b.size(); ++i) {
      const Block& b = th->b[i];
      const CGate& gb = seg_gates.empty() ? gate : *seg_gates.at((size_t)(b.k.q0 >> 32));
      for (int o2 = 0; o2 < gb.d2; ++o2)
        for (int o1 = 0; o1 < gb.d1; ++o1) {
          const cplx gv = gb.at(o1, o2, (int)b.k.p0, (int)b.k.p1);
          if (gv == cplx(0, 0)) continue;
          gt[K2(b.k.q0, b.k.q1, (uint32_t)o1, (uint32_t)o2)].push_back({i, gv});
        }
    }
    Layout lg;
    for (auto& x : gt) lg.add(x.first, th->b[x.second[0].first].r, th->b[x.second[0].first].c);
    TensorP tg = make_ctensor(ctx, 2, lg, false);
    {
      LincombPlan lp;
      for (auto& x : gt) {
        const int o = tg->find(x.first);
        const int64_t n = (int64_t)tg->b[o].r * tg->b[o].c;
        std::vector<std::pair<const double*, double>> tr, ti;
        for (auto& t : x.second) {
          tr.push_back({re(*th, t.first), t.second.real()});
          tr.push_back({im(*th, t.first), -t.second.imag()});
          ti.push_back({im(*th, t.first), t.second.real()});
          ti.push_back({re(*th, t.first), t.second.imag()});
        }
        lp.add(re(*tg, o), n, tr);
        lp.add(im(*tg, o), n, ti);
      }
      lp.run(ctx);
    }
    th.reset();
    Ml.reset();
    Mr.reset();
    // theta.squeeze(1e-15)
    std::vector<int> kt;
    {
      auto mx = block_max2(*tg);
      for (int i = 0; i < (int)tg->b.size(); ++i)
        if (mx[i] > 1e-30) kt.push_back(i);
    }
    auto t0 = std::chrono::steady_clock::now();
    // split by centre charge
    const ItoKey &ik0 = ik[site], &ik1 = ik[site + 1];
    std::map<Q, Sec> secs;
    for (int i : kt) {
      const Block& b = tg->b[i];
      Sec& s = secs[b.k.q0 + qat_(ik0, b.k.p0)];
      s.blocks.push_back(i);
      s.rx[b.k.p0] = {0, b.r};
      s.ry[b.k.p1] = {0, b.c};
    }
    std::vector<Q> qcs;
    int64_t oM = 0, oU = 0, oV = 0, oS = 0;
    for (auto& x : secs) {
      Sec& s = x.second;
      for (auto& r : s.rx) { r.second.first = s.m; s.m += r.second.second; }
      for (auto& r : s.ry) { r.second.first = s.n; s.n += r.second.second; }
      s.k = std::min(s.m, s.n);
      s.offM = oM; oM += (int64_t)s.m * s.n;
      s.offU = oU; oU += (int64_t)s.m * s.k;
      s.offV = oV; oV += (int64_t)s.n * s.k;
      s.offS = oS; oS += s.k;
      qcs.push_back(x.first);
    }
    double2* dM = (double2*)ctx->dmalloc(sizeof(double2) * std::max<int64_t>(oM + oU + oV, 2));
    double2* dU = dM + oM;
    double2* dV = dU + oU;
    double* dS = (double*)ctx->dmalloc(sizeof(double) * std::max<int64_t>(oS, 2));
    int* dinfo = (int*)ctx->dmalloc(sizeof(int) * std::max<size_t>(qcs.size(), 1));
    MPSG_CUDA(cudaMemsetAsync(dinfo, 0, sizeof(int) * std::max<size_t>(qcs.size(), 1), ctx->stream));
    std::vector<CGatherOp> go;
    {
      for (auto& x : secs) {
        Sec& s = x.second;
        for (int i : s.blocks) {
          const Block& b = tg->b[i];
          const int r0 = s.rx.at(b.k.p0).first, c0 = s.ry.at(b.k.p1).first;
          if (s.m >= s.n)  // M (m x n)
            go.push_back(CGatherOp{re(*tg, i), im(*tg, i), dM + s.offM + r0 + (int64_t)c0 * s.m, b.r, b.c, b.r, s.m, 0});
          else  // wide: M^H (n x m) = V S U^H
            go.push_back(CGatherOp{re(*tg, i), im(*tg, i), dM + s.offM + c0 + (int64_t)r0 * s.n, b.r, b.c, b.r, s.n, 1});
        }
      }
    }
    auto gather = [&]() {
      if (go.empty()) return;
      CGatherOp* d = (CGatherOp*)ctx->dmalloc(sizeof(CGatherOp) * go.size());
      MPSG_CUDA(cudaMemcpyAsync(d, go.data(), sizeof(CGatherOp) * go.size(), cudaMemcpyHostToDevice, ctx->stream));
      launch_cgather(d, (int)go.size(), ctx->stream);
      ctx->dfree(d);
    };
    gather();
    // svd method 4 (default): the library's own bidiagonal route for complex sectors (real bidiagonal,
    // complex reflectors); sectors beyond its cluster kernel or whose vectors would need the Jacobi
    // route send the whole split to cuSOLVER zgesvdj (the sector matrices gathered again)
    bool svd_done = false;
    if (ctx->svd_method == 4) {
      std::vector<ZSvdSec> zs;
      for (auto& x : secs) {
        Sec& sc = x.second;
        const bool tall = sc.m >= sc.n;
        const int ms = tall ? sc.m : sc.n, ns = tall ? sc.n : sc.m;
        zs.push_back(ZSvdSec{ms, ns, sc.offM, tall ? dU + sc.offU : dV + sc.offV, tall ? dV + sc.offV : dU + sc.offU,
                             ms, ns});
      }
      svd_done = zsvd_bidiag(ctx, zs, dM, dS);
      if (!svd_done) {
        ++zsvd_fallbacks;
        gather();
      }
    }
    if (svd_done) {
    } else if (ctx->svd_method != 0 && ctx->svd_method != 4) {
      density_svd(secs, dM, dU, dV, dS);
    } else {
      cusolverDnHandle_t h = ctx->svd_handle();
      int lwork = 0;
      for (auto& x : secs) {
        Sec& s = x.second;
        if (s.k == 0) continue;
        int lw = 0;
        const bool tall = s.m >= s.n;
        const int ms = tall ? s.m : s.n, ns = tall ? s.n : s.m;
        cuDoubleComplex* uo = (cuDoubleComplex*)(tall ? dU + s.offU : dV + s.offV);
        cuDoubleComplex* vo = (cuDoubleComplex*)(tall ? dV + s.offV : dU + s.offU);
        if (cusolverDnZgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, ms, ns, (cuDoubleComplex*)(dM + s.offM), ms,
                                         dS + s.offS, uo, ms, vo, ns, &lw, ctx->svdp) != CUSOLVER_STATUS_SUCCESS)
          throw Err(3, "zgesvdj_bufferSize failed");
        lwork = std::max(lwork, lw);
      }
      cuDoubleComplex* work = (cuDoubleComplex*)ctx->dmalloc(sizeof(cuDoubleComplex) * std::max(lwork, 2));
      int si = 0;
      for (auto& x : secs) {
        Sec& s = x.second;
        const bool tall = s.m >= s.n;
        const int ms = tall ? s.m : s.n, ns = tall ? s.n : s.m;
        cuDoubleComplex* uo = (cuDoubleComplex*)(tall ? dU + s.offU : dV + s.offV);
        cuDoubleComplex* vo = (cuDoubleComplex*)(tall ? dV + s.offV : dU + s.offU);
        if (s.k > 0 && cusolverDnZgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, ms, ns, (cuDoubleComplex*)(dM + s.offM), ms,
                                         dS + s.offS, uo, ms, vo, ns, work, lwork, dinfo + si,
                                         ctx->svdp) != CUSOLVER_STATUS_SUCCESS)
          throw Err(3, "zgesvdj failed");
        ++si;
      }
      ctx->dfree(work);
    }
    {
      std::vector<CPhaseOp> ph;
      for (auto& x : secs) {
        Sec& s = x.second;
        if (s.k > 0) ph.push_back(CPhaseOp{dU + s.offU, dV + s.offV, s.m, s.n, s.k, s.m, s.n});
      }
      if (!ph.empty()) {
        CPhaseOp* d = (CPhaseOp*)ctx->dmalloc(sizeof(CPhaseOp) * ph.size());
        MPSG_CUDA(cudaMemcpyAsync(d, ph.data(), sizeof(CPhaseOp) * ph.size(), cudaMemcpyHostToDevice, ctx->stream));
        launch_cfixphase(d, (int)ph.size(), ctx->stream);
        ctx->dfree(d);
      }
    }
    // global truncation (DiagBlockMatrix::truncate, same rank rule as the real split)
    if (!chimax && doTrunc) chimax = 100;
    if (!chimax && !doTrunc) chimax = 200;
    // sectors of one bond are contiguous (centre charges ascend, bond i in [i << 32, (i + 1) << 32))
    const int nseg = seg_gates.empty() ? 1 : (int)seg_gates.size();
    std::vector<int> seg_of_sec(qcs.size(), 0), s0(nseg + 1, (int)qcs.size());
    if (!seg_gates.empty())
      for (size_t si = 0; si < qcs.size(); ++si) {
        seg_of_sec[si] = (int)(qcs[si] >> 32);
        MPSG_CHECK(seg_of_sec[si] < nseg, "centre charge outside the bonds of the layer");
      }
    for (int si = (int)qcs.size() - 1; si >= 0; --si) s0[seg_of_sec[si]] = si;
    for (int c = nseg - 1; c >= 0; --c) s0[c] = std::min(s0[c], s0[c + 1]);
    std::vector<int64_t> offS_of(qcs.size() + 1, oS);
    std::vector<int32_t> sec_of(oS);
    {
      int si = 0;
      for (auto& x : secs) {
        offS_of[si] = x.second.offS;
        for (int j = 0; j < x.second.k; ++j) sec_of[x.second.offS + j] = si - s0[seg_of_sec[si]];
        ++si;
      }
    }
    const int nS = (int)oS;
    int32_t* dsec = (int32_t*)ctx->dmalloc(sizeof(int32_t) * (std::max(nS, 1) * 3 + qcs.size() + 1) +
                                           sizeof(double) * 3 * (nseg + 1));
    int32_t* drank = dsec + std::max(nS, 1);
    int32_t* dcnt = drank + 2 * std::max(nS, 1);
    double* dout3 = (double*)(((uintptr_t)(dcnt + qcs.size() + 1) + 7) & ~(uintptr_t)7);
    if (nS) MPSG_CUDA(cudaMemcpyAsync(dsec, sec_of.data(), sizeof(int32_t) * nS, cudaMemcpyHostToDevice, ctx->stream));
    MPSG_CUDA(cudaMemsetAsync(dout3, 0, sizeof(double) * 3 * nseg, ctx->stream));
    for (int c = 0; c < nseg; ++c) {
      const int a = s0[c], b = s0[c + 1];
      if (a >= b) continue;
      const int64_t v0 = offS_of[a], v1 = offS_of[b];
      launch_truncate(dS + v0, (int)(v1 - v0), dsec + v0, b - a, chimax, doTrunc ? 1 : 0, tr_weight, drank + 2 * v0,
                      dcnt + a, dout3 + 3 * c, ctx->stream);
    }
    std::vector<int32_t> counts(qcs.size() + 1, 0);
    std::vector<int> info(qcs.size() + 1, 0);
    std::vector<double> out3(3 * nseg, 0.0);
    if (!qcs.empty()) {
      MPSG_CUDA(cudaMemcpyAsync(counts.data(), dcnt, sizeof(int32_t) * qcs.size(), cudaMemcpyDeviceToHost, ctx->stream));
      MPSG_CUDA(cudaMemcpyAsync(info.data(), dinfo, sizeof(int) * qcs.size(), cudaMemcpyDeviceToHost, ctx->stream));
    }
    MPSG_CUDA(cudaMemcpyAsync(out3.data(), dout3, sizeof(double) * 3 * nseg, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    for (size_t i = 0; i < qcs.size(); ++i)
      if (info[i] < 0) throw Err(3, "zgesvdj: invalid argument (info=" + std::to_string(info[i]) + ")");
    seg_tw.assign(nseg, 0.0);
    seg_chi.assign(nseg, 0);
    std::vector<double> inv_norm_seg(nseg, 1.0);
    for (int c = 0; c < nseg; ++c) {
      seg_tw[c] = out3[3 * c];
      seg_chi[c] = (int)out3[3 * c + 1];
      if (normalize) inv_norm_seg[c] = out3[3 * c + 2];
    }
    const double tw = seg_tw[0];
    const int chi = seg_chi[0];
    ctx->dfree(dsec);
    // U, Vt and lambda (dropDangling: sectors without kept values vanish)
    Layout lu, lv, ll2;
    {
      int si = 0;
      for (auto& x : secs) {
        const int c = counts[si++];
        if (c <= 0) continue;
        const Q qc = x.first;
        for (auto& r : x.second.rx) lu.add(K1(qc - qat_(ik0, r.first), qc, r.first), r.second.second, c);
        for (auto& r : x.second.ry) lv.add(K1(qc, qc + qat_(ik1, r.first), r.first), c, r.second.second);
        ll2.add(K1(qc, qc, 0), c, 1);
      }
    }
    ll2.finalize();
    TensorP U = make_ctensor(ctx, 1, lu, false), Vt = make_ctensor(ctx, 1, lv, false);
    TensorP lnew = make_tensor(ctx, 0, ll2, true);
    {
      std::vector<CScatterOp> so;
      std::vector<CopyOp> lo;
      int si = 0;
      for (auto& x : secs) {
        const int c = counts[si++];
        if (c <= 0) continue;
        const Q qc = x.first;
        const Sec& s = x.second;
        for (auto& r : s.rx) {
          const int ob = U->find(K1(qc - qat_(ik0, r.first), qc, r.first));
          so.push_back(CScatterOp{dU + s.offU + r.second.first, re(*U, ob), im(*U, ob), nullptr, nullptr,
                                  r.second.second, c, s.m, r.second.second, 0});
        }
        for (auto& r : s.ry) {
          const int ob = Vt->find(K1(qc, qc + qat_(ik1, r.first), r.first));
          so.push_back(CScatterOp{dV + s.offV + r.second.first, re(*Vt, ob), im(*Vt, ob), nullptr, nullptr, c,
                                  r.second.second, s.n, c, 1});
        }
        const int ol = lnew->find(K1(qc, qc, 0));
        lo.push_back(CopyOp{dS + s.offS, lnew->d + lnew->b[ol].off, nullptr, nullptr, c, 1, c, c, 0,
                            inv_norm_seg[seg_of_sec[si - 1]]});
      }
      if (!so.empty()) {
        CScatterOp* d = (CScatterOp*)ctx->dmalloc(sizeof(CScatterOp) * so.size());
        MPSG_CUDA(cudaMemcpyAsync(d, so.data(), sizeof(CScatterOp) * so.size(), cudaMemcpyHostToDevice, ctx->stream));
        launch_cscatter(d, (int)so.size(), ctx->stream);
        ctx->dfree(d);
      }
      run_copyops(ctx, lo);
    }
    ctx->dfree(dinfo);
    ctx->dfree(dS);
    ctx->dfree(dM);
    tg.reset();
    // mps[0].squeeze(1e-15), mps[1].squeeze(1e-15); Gamma_l = lambda_l^-1 U, Gamma_r = Vt lambda_r^-1
    TensorP il = recip(ll), ir = recip(lr);
    std::vector<int> ku, kv;
    {
      auto mu = block_max2(*U), mv = block_max2(*Vt);
      for (int i = 0; i < (int)U->b.size(); ++i)
        if (mu[i] > 1e-30 && lam_ptr(*il, U->b[i].k.q0, nullptr)) ku.push_back(i);
      for (int i = 0; i < (int)Vt->b.size(); ++i)
        if (mv[i] > 1e-30 && lam_ptr(*ir, Vt->b[i].k.q1, nullptr)) kv.push_back(i);
    }
    TensorP ngl = scaled_copy(*U, ku, [&](const Block& b) { return lam_ptr(*il, b.k.q0, nullptr); },
                              [&](const Block&) { return (const double*)nullptr; });
    TensorP ngr = scaled_copy(*Vt, kv, [&](const Block&) { return (const double*)nullptr; },
                              [&](const Block& b) { return lam_ptr(*ir, b.k.q1, nullptr); });
    ctx->sync();
    G[site] = ngl;
    G[site + 1] = ngr;
    lam[site + 1] = lnew;
    split_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    ++gates;
    return {tw, chi};
  }

  // doTimeSlice: the gates of one parity.  The bonds of a slice are disjoint, so with batch_layers
  // they are applied at once to the direct sum of the bonds (one theta formation, one split, one
  // scatter for the whole slice; gate, truncation and normalisation per bond).
  void slice(const std::vector<CGate>& gates_, int start, int chimax, bool doTrunc, double tr_weight, bool normalize) {
    std::vector<int> sites;
    for (int site = start; site < N - 1; site += 2) sites.push_back(site);
    bool uniform = true;
    for (int s : sites) uniform = uniform && ik[s] == ik[sites[0]] && ik[s + 1] == ik[sites[0] + 1];
    if (!batch_layers || sites.size() < 2 || !uniform) {
      for (int site : sites) apply_gate(site, gates_[site], chimax, doTrunc, tr_weight, normalize);
      return;
    }
    std::vector<const Tensor *> gl, gr, ll, lc, lr;
    for (int s : sites) {
      gl.push_back(G[s].get());
      gr.push_back(G[s + 1].get());
      ll.push_back(lam[s].get());
      lc.push_back(lam[s + 1].get());
      lr.push_back(lam[s + 2].get());
    }
    TebdEngine t;
    t.ctx = ctx;
    t.keep = keep;
    t.N = 2;
    t.ik = {ik[sites[0]], ik[sites[0] + 1]};
    t.G = {bond_sum(ctx, gl, 1, 2), bond_sum(ctx, gr, 1, 2)};
    t.lam = {bond_sum(ctx, ll, 0, 1), bond_sum(ctx, lc, 0, 1), bond_sum(ctx, lr, 0, 1)};
    for (int s : sites) t.seg_gates.push_back(&gates_[s]);
    t.apply_gate(0, gates_[sites[0]], chimax, doTrunc, tr_weight, normalize);
    for (size_t i = 0; i < sites.size(); ++i) {
      const int s = sites[i];
      G[s] = bond_part(ctx, *t.G[0], (int)i, 2);
      G[s + 1] = bond_part(ctx, *t.G[1], (int)i, 2);
      lam[s + 1] = bond_part(ctx, *t.lam[1], (int)i, 1);
    }
    split_seconds += t.split_seconds;
    gates += (int64_t)sites.size();
  }
  std::vector<CGate> make_gates(double dt) const {
    std::vector<CGate> g;
    for (int s = 0; s + 1 < N; ++s)
      g.push_back(nn_gate(mpo[s], mpo[s + 1], s, N, dt, 0.0, (int)ik[s].size(), (int)ik[s + 1].size()));
    return g;
  }
  // Layers of the second-order schedule, in order: (first bond, 1 for a half step dt/2): a half step
  // on the odd bonds, then per step the even bonds and the odd bonds, the last odd layer a half step.
  static std::vector<std::pair<int, int>> schedule(int steps) {
    std::vector<std::pair<int, int>> s{{1, 1}};
    for (int step = 1; step <= steps; ++step) {
      s.push_back({0, 0});
      s.push_back({1, step < steps ? 0 : 1});
    }
    return s;
  }
  void second_order(int steps, double dt, int chimax, bool doTrunc, double tr_weight, bool normalize) {
    auto t0 = std::chrono::steady_clock::now();
    const auto full = make_gates(dt), half = make_gates(dt / 2);
    for (auto& l : schedule(steps)) slice(l.second ? half : full, l.first, chimax, doTrunc, tr_weight, normalize);
    ctx->sync();
    seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  // SparseLocalOperator::measure for a diagonal operator on lambda(site-1) Gamma(site) lambda(site)
  double measure_diag(int site, const std::vector<double>& op) {
    const Tensor& g = *G[site];
    std::vector<CMeasureOp> ops;
    for (int i = 0; i < (int)g.b.size(); ++i) {
      const double* l0 = lam_ptr(*lam[site], g.b[i].k.q0, nullptr);
      const double* l1 = lam_ptr(*lam[site + 1], g.b[i].k.q1, nullptr);
      if (!l0 || !l1) continue;
      MPSG_CHECK(g.b[i].k.p0 < op.size(), "operator smaller than the local space");
      ops.push_back(CMeasureOp{re(g, i), im(g, i), l0, l1, g.b[i].r, g.b[i].c, op[g.b[i].k.p0]});
    }
    if (ops.empty()) return 0.0;
    CMeasureOp* d = (CMeasureOp*)ctx->dmalloc(sizeof(CMeasureOp) * ops.size() + sizeof(double) * ops.size());
    double* dout = (double*)(d + ops.size());
    MPSG_CUDA(cudaMemcpyAsync(d, ops.data(), sizeof(CMeasureOp) * ops.size(), cudaMemcpyHostToDevice, ctx->stream));
    launch_cmeasure(d, (int)ops.size(), dout, ctx->stream);
    std::vector<double> out(ops.size());
    MPSG_CUDA(cudaMemcpyAsync(out.data(), dout, sizeof(double) * ops.size(), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    ctx->dfree(d);
    double s = 0;
    for (double v : out) s += v;
    return s;
  }
};

// (dG/dtheta) G^H for G = exp(-i tau h) with dh/dtheta = dh (tebd_adjoint.cpp).
CGate gate_tangent(const std::vector<double>& H, const std::vector<double>& dh, int d1, int d2, double tau);

// Second-order evolution of e with the gradient of <O_obs_site> at the end with respect to one
// parameter per bond (dh[b] = d h_b / d theta_b); returns (value, gradient) (tebd_adjoint.cpp).
std::pair<double, std::vector<double>> tebd_adjoint_second_order(TebdEngine& e, int steps, double dt, int chimax,
                                                                 bool doTrunc, double tr_weight, int obs_site,
                                                                 const std::vector<double>& obs,
                                                                 const std::vector<std::vector<double>>& dh, int every);

}  // namespace mpsg
