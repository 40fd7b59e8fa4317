// TEBD on the GPU: two-site gates exp(-i dt h_b) (MPO::getNNGate, src/MPOTypes.hpp:1090-1209),
// applyGate on the Vidal form lambda Gamma lambda Gamma lambda (src/MPSfunctions.hpp:1492-1548),
// time slices over even / odd bonds (TEBDengine::doTimeSlice, src/container.hpp:1195-1233) and the
// second-order Trotter schedule (TEBDengine::simulate, src/container.hpp:1325-1395).
//
// Complex block tensors are planar Tensors: the arena holds the real parts of all blocks, then the
// imaginary parts at offset nelem.  Complex products run on the grouped FP64 GEMM as four real
// products, the gate is a complex linear combination of blocks (k_lincomb), and the split takes a
// one-sided Jacobi SVD per charge sector (cuSOLVER zgesvdj) with the complex FixPhase.
#include "tebd.h"

namespace mpsg {

// Eigen-decomposition of a small real symmetric matrix by cyclic Jacobi rotations.
void jacobi_sym(int n, std::vector<double>& A, std::vector<double>& V, std::vector<double>& E) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i + (size_t)i * n] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[p + (size_t)q * n] * A[p + (size_t)q * n];
    if (off < 1e-32) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p + (size_t)q * n];
        if (std::fabs(apq) < 1e-300) continue;
        const double th = 0.5 * (A[q + (size_t)q * n] - A[p + (size_t)p * n]) / apq;
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double a = A[k + (size_t)p * n], b = A[k + (size_t)q * n];
          A[k + (size_t)p * n] = c * a - s * b;
          A[k + (size_t)q * n] = s * a + c * b;
        }
        for (int k = 0; k < n; ++k) {
          const double a = A[p + (size_t)k * n], b = A[q + (size_t)k * n];
          A[p + (size_t)k * n] = c * a - s * b;
          A[q + (size_t)k * n] = s * a + c * b;
        }
        for (int k = 0; k < n; ++k) {
          const double a = V[k + (size_t)p * n], b = V[k + (size_t)q * n];
          V[k + (size_t)p * n] = c * a - s * b;
          V[k + (size_t)q * n] = s * a + c * b;
        }
      }
  }
  E.resize(n);
  for (int i = 0; i < n; ++i) E[i] = A[i + (size_t)i * n];
}

// h_b = sum_i W1[row, i] (x) W2[i, 0]: on a bulk bond row = Dl-1 and the two on-site channels (i = 0
// for site1, i = Dr-1 for site2) count one half; at the chain ends the end site's channel counts
// fully (row 0 of the left boundary tensor).
std::vector<double> bond_hamiltonian(const MPO& m1, const MPO& m2, int site1, int N, int d1, int d2) {
  const int site2 = site1 + 1, D = d1 * d2;
  std::vector<double> H((size_t)D * D, 0.0);
  auto add = [&](uint32_t r1, uint32_t c1, uint32_t r2, uint32_t c2, double w1, double w2) {
    const MPOEntry *a = nullptr, *b = nullptr;
    for (auto& e : m1.e)
      if (e.wl == r1 && e.wr == c1) a = &e;
    for (auto& e : m2.e)
      if (e.wl == r2 && e.wr == c2) b = &e;
    if (!a || !b) return;
    for (auto& x : a->ops)
      for (auto& y : b->ops) {
        const int o = (int)x.out + d1 * (int)y.out, in = (int)x.in + d1 * (int)y.in;
        H[o + (size_t)in * D] += x.v * w1 * y.v * w2;
      }
  };
  const uint32_t lend = (uint32_t)m1.Dl - 1, last = (uint32_t)m1.Dr - 1;
  for (uint32_t i = 0; i <= last; ++i) {
    if (site1 == 0 && site2 != N - 1) add(0, i, i, 0, 1.0, i == last && i != 0 ? 0.5 : 1.0);
    if (site2 == N - 1 && site1 != 0) add(lend, i, i, 0, i == 0 ? 0.5 : 1.0, 1.0);
    if (site2 != N - 1 && site1 != 0) add(lend, i, i, 0, i == 0 ? 0.5 : 1.0, i == last ? 0.5 : 1.0);
  }
  for (auto& h : H)
    if (std::fabs(h) < 1e-14) h = 0.0;
  return H;
}

// G = exp(-(dt_im + i dt_re) h_b) by the eigenvectors of h_b (real symmetric for the real MPOs here);
// entries below 1e-15 set to zero.
CGate nn_gate(const MPO& m1, const MPO& m2, int site1, int N, double dt_re, double dt_im, int d1, int d2) {
  const int D = d1 * d2;
  const std::vector<double> H = bond_hamiltonian(m1, m2, site1, N, d1, d2);
  std::vector<double> A = H, V, E;
  jacobi_sym(D, A, V, E);
  CGate G;
  G.d1 = d1;
  G.d2 = d2;
  G.g.assign((size_t)D * D, cplx(0, 0));
  for (int x = 0; x < D; ++x)
    for (int y = 0; y < D; ++y) {
      cplx s(0, 0);
      for (int k = 0; k < D; ++k) s += V[x + (size_t)k * D] * std::exp(-cplx(dt_im, dt_re) * E[k]) * V[y + (size_t)k * D];
      G.g[x + (size_t)y * D] = std::abs(s) < 1e-15 ? cplx(0, 0) : s;
    }
  return G;
}

}  // namespace mpsg

using namespace mpsg;

struct mpsg_tebd_s {
  TebdEngine* e = nullptr;
};

extern "C" {

mpsg_status mpsg_tebd_create(mpsg_ctx ctx, int32_t N, const int32_t* local_state, const mpsg_mpo* W,
                             const mpsg_itokey* ik, mpsg_tebd* out) {
  API_BEGIN
  MPSG_CHECK(out && local_state && W && ik && N >= 2, "null argument or N < 2");
  Ctx* c = C(ctx);
  std::unique_ptr<TebdEngine> e(new TebdEngine());
  e->ctx = c;
  e->keep = c->shared_from_this();
  e->N = N;
  for (int s = 0; s < N; ++s) {
    e->mpo.push_back(mpo_from_c(&W[s]));
    e->ik.push_back(itokey_from_c(&ik[s]));
  }
  e->init_product(std::vector<int>(local_state, local_state + N));
  *out = new mpsg_tebd_s;
  (*out)->e = e.release();
  API_END
}

mpsg_status mpsg_tebd_second_order(mpsg_tebd e, int32_t steps, double dt, uint32_t chimax, int32_t doTrunc,
                                   double tr_weight, int32_t normalize) {
  API_BEGIN
  MPSG_CHECK(e && e->e && steps >= 1, "null engine or steps < 1");
  e->e->second_order(steps, dt, (int)chimax, doTrunc != 0, tr_weight, normalize != 0);
  API_END
}

mpsg_status mpsg_tebd_measure_diag(mpsg_tebd e, int32_t site, const double* op_diag, int32_t d, double* out) {
  API_BEGIN
  MPSG_CHECK(e && e->e && op_diag && out, "null argument");
  MPSG_CHECK(site >= 0 && site < e->e->N, "site out of range");
  *out = e->e->measure_diag(site, std::vector<double>(op_diag, op_diag + d));
  API_END
}

mpsg_status mpsg_tebd_lambda(mpsg_tebd e, int32_t bond, mpsg_tensor* out) {
  API_BEGIN
  MPSG_CHECK(e && e->e && out, "null argument");
  MPSG_CHECK(bond >= -1 && bond < e->e->N, "bond out of range");
  *out = wrap(tensor_copy(*e->e->lam[bond + 1]));
  API_END
}

mpsg_status mpsg_tebd_gamma_shape(mpsg_tebd e, int32_t site, int32_t* nblocks, int64_t* nelem) {
  API_BEGIN
  MPSG_CHECK(e && e->e && nblocks && nelem, "null argument");
  MPSG_CHECK(site >= 0 && site < e->e->N, "site out of range");
  const Tensor& g = *e->e->G[site];
  *nblocks = (int32_t)g.b.size();
  int64_t n = 0;
  for (auto& b : g.b) n += (int64_t)b.r * b.c;
  *nelem = n;
  API_END
}

mpsg_status mpsg_tebd_gamma_export(mpsg_tebd e, int32_t site, uint64_t* q, uint32_t* p, int32_t* rows,
                                   int32_t* cols, double* data_interleaved) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  MPSG_CHECK(site >= 0 && site < e->e->N, "site out of range");
  const Tensor& g = *e->e->G[site];
  std::vector<double> h((size_t)std::max<int64_t>(2 * g.nelem, 2));
  MPSG_CUDA(cudaMemcpyAsync(h.data(), g.d, sizeof(double) * 2 * g.nelem, cudaMemcpyDeviceToHost, g.ctx->stream));
  g.ctx->sync();
  size_t o = 0;
  for (size_t i = 0; i < g.b.size(); ++i) {
    const Block& b = g.b[i];
    q[2 * i] = b.k.q0;
    q[2 * i + 1] = b.k.q1;
    p[i] = b.k.p0;
    rows[i] = b.r;
    cols[i] = b.c;
    if (data_interleaved)
      for (int64_t x = 0; x < (int64_t)b.r * b.c; ++x) {
        data_interleaved[o++] = h[b.off + x];
        data_interleaved[o++] = h[g.nelem + b.off + x];
      }
  }
  API_END
}

mpsg_status mpsg_tebd_stats(mpsg_tebd e, double* seconds, double* split_seconds, int64_t* gates) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  if (seconds) *seconds = e->e->seconds;
  if (split_seconds) *split_seconds = e->e->split_seconds;
  if (gates) *gates = e->e->gates;
  API_END
}

mpsg_status mpsg_nn_gate(const mpsg_mpo* W1, const mpsg_mpo* W2, int32_t site1, int32_t N, double dt_re, double dt_im,
                         int32_t d1, int32_t d2, double* out_interleaved) {
  API_BEGIN
  MPSG_CHECK(W1 && W2 && out_interleaved && d1 > 0 && d2 > 0, "null argument");
  CGate g = nn_gate(mpo_from_c(W1), mpo_from_c(W2), site1, N, dt_re, dt_im, d1, d2);
  for (size_t i = 0; i < g.g.size(); ++i) {
    out_interleaved[2 * i] = g.g[i].real();
    out_interleaved[2 * i + 1] = g.g[i].imag();
  }
  API_END
}

mpsg_status mpsg_bond_hamiltonian(const mpsg_mpo* W1, const mpsg_mpo* W2, int32_t site1, int32_t N, int32_t d1,
                                  int32_t d2, double* out) {
  API_BEGIN
  MPSG_CHECK(W1 && W2 && out && d1 > 0 && d2 > 0, "null argument");
  const auto H = bond_hamiltonian(mpo_from_c(W1), mpo_from_c(W2), site1, N, d1, d2);
  std::memcpy(out, H.data(), sizeof(double) * H.size());
  API_END
}

mpsg_status mpsg_nn_gate_tangent(const mpsg_mpo* W1, const mpsg_mpo* W2, int32_t site1, int32_t N, double dt,
                                 const double* dh, int32_t d1, int32_t d2, double* out_interleaved) {
  API_BEGIN
  MPSG_CHECK(W1 && W2 && dh && out_interleaved && d1 > 0 && d2 > 0, "null argument");
  const int D = d1 * d2;
  const auto H = bond_hamiltonian(mpo_from_c(W1), mpo_from_c(W2), site1, N, d1, d2);
  const CGate B = gate_tangent(H, std::vector<double>(dh, dh + (size_t)D * D), d1, d2, dt);
  for (size_t i = 0; i < B.g.size(); ++i) {
    out_interleaved[2 * i] = B.g[i].real();
    out_interleaved[2 * i + 1] = B.g[i].imag();
  }
  API_END
}

mpsg_status mpsg_tebd_adjoint_second_order(mpsg_tebd e, int32_t steps, double dt, uint32_t chimax, int32_t doTrunc,
                                           double tr_weight, int32_t obs_site, const double* obs_diag, int32_t d,
                                           const double* dh, int32_t checkpoint_every, double* value, double* grad) {
  API_BEGIN
  MPSG_CHECK(e && e->e && obs_diag && dh && value && grad && d > 0, "null argument");
  TebdEngine& t = *e->e;
  MPSG_CHECK(steps >= 1, "steps < 1");
  MPSG_CHECK(obs_site >= 0 && obs_site < t.N, "observable site out of range");
  std::vector<std::vector<double>> dhv;
  size_t off = 0;
  for (int b = 0; b + 1 < t.N; ++b) {
    const size_t D = t.ik[b].size() * t.ik[b + 1].size();
    dhv.emplace_back(dh + off, dh + off + D * D);
    off += D * D;
  }
  auto r = tebd_adjoint_second_order(t, steps, dt, (int)chimax, doTrunc != 0, tr_weight, obs_site,
                                     std::vector<double>(obs_diag, obs_diag + d), dhv, checkpoint_every);
  *value = r.first;
  std::copy(r.second.begin(), r.second.end(), grad);
  API_END
}

mpsg_status mpsg_tebd_set_batch_layers(mpsg_tebd e, int32_t batch_layers) {
  API_BEGIN
  MPSG_CHECK(e && e->e, "null engine");
  e->e->batch_layers = batch_layers != 0;
  API_END
}

mpsg_status mpsg_tebd_adjoint_seconds(mpsg_tebd e, double* seconds) {
  API_BEGIN
  MPSG_CHECK(e && e->e && seconds, "null argument");
  *seconds = e->e->adjoint_seconds;
  API_END
}

void mpsg_tebd_destroy(mpsg_tebd e) {
  if (!e) return;
  try {
    delete e->e;
  } catch (...) {
  }
  delete e;
}

}  // extern "C"
