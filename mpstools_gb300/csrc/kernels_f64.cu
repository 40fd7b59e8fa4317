// FP64 kernels of libmpsg (sm_103a): grouped block GEMM, block linear combinations,
// gather/scatter copies, FixPhase, Lanczos vector operations, the tridiagonal
// lowest-eigenpair solver and the global singular-value truncation.
#include <cuda_runtime.h>
#include <atomic>
#include <cfloat>
#include <climits>
#include "mpsg_internal.h"

namespace mpsg {

static std::atomic<int64_t> g_launches{0};
int64_t kernel_launch_count() { return g_launches.load(); }
#define LAUNCHED() g_launches.fetch_add(1)

// ============================================================================ grouped DGEMM
// One CTA computes an mh x nh tile of one problem, accumulating every segment (product term) of the
// problem; FP64 FMA on CUDA cores.  Tiles are 64 x 64 inside a block and trimmed at its edges to
// the next multiple of 16 (mh, nh in {16, 32, 48, 64}): the executed FMAs then exceed the
// algorithmic ones by at most 15 rows / columns per block instead of 63 (on the chi = 2048 centre
// bond's sector sizes 1.20x instead of 1.53x).  256 threads as 16 x 16: thread (tx, ty) owns rows
// tx + 16 i, i < MI = mh / 16, and columns ty + 16 j, j < NJ = nh / 16; each tile shape is its own
// compiled loop (no predicated-off FMAs).
constexpr int GM = 64, GN = 64, GK = 16;

template <int MI, int NJ>
__device__ __forceinline__ void gemm_tile(const GProb& P, const GTile& t, const GSeg* __restrict__ seg,
                                          const Bases& bases, double (*As)[GM + 1], double (*Bs)[GN + 1]) {
  constexpr int TM = 16 * MI, TN = 16 * NJ;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  double acc[MI][NJ];
#pragma unroll
  for (int i = 0; i < MI; ++i)
#pragma unroll
    for (int j = 0; j < NJ; ++j) acc[i][j] = 0.0;

  for (int s = P.seg0; s < P.seg1; ++s) {
    const GSeg S = seg[s];
    const double* __restrict__ Ap = bases.p[S.baseA] + S.offA;
    const double* __restrict__ Bp = bases.p[S.baseB] + S.offB;
    for (int k0 = 0; k0 < S.K; k0 += GK) {
#pragma unroll
      for (int r = 0; r < (TM * GK + 255) / 256; ++r) {
        const int e = tid + r * 256;
        if ((TM * GK) % 256 == 0 || e < TM * GK) {
          int m, k;
          if (!S.tA) { m = e % TM; k = e / TM; } else { k = e % GK; m = e / GK; }
          const int gm = t.m0 + m, gk = k0 + k;
          double v = 0.0;
          if (gm < P.M && gk < S.K)
            v = S.tA ? Ap[gk + (int64_t)gm * S.lda] : Ap[gm + (int64_t)gk * S.lda];
          As[k][m] = v * S.alpha;
        }
      }
#pragma unroll
      for (int r = 0; r < (TN * GK + 255) / 256; ++r) {
        const int e = tid + r * 256;
        if ((TN * GK) % 256 == 0 || e < TN * GK) {
          int n, k;
          if (!S.tB) { k = e % GK; n = e / GK; } else { n = e % TN; k = e / TN; }
          const int gn = t.n0 + n, gk = k0 + k;
          double v = 0.0;
          if (gn < P.N && gk < S.K)
            v = S.tB ? Bp[gn + (int64_t)gk * S.ldb] : Bp[gk + (int64_t)gn * S.ldb];
          Bs[k][n] = v;
        }
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < GK; ++k) {
        double a[MI], b[NJ];
#pragma unroll
        for (int i = 0; i < MI; ++i) a[i] = As[k][tx + 16 * i];
#pragma unroll
        for (int j = 0; j < NJ; ++j) b[j] = Bs[k][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < MI; ++i)
#pragma unroll
          for (int j = 0; j < NJ; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int gn = t.n0 + ty + 16 * j;
    if (gn >= P.N) continue;
#pragma unroll
    for (int i = 0; i < MI; ++i) {
      const int gm = t.m0 + tx + 16 * i;
      if (gm >= P.M) continue;
      double* c = const_cast<double*>(bases.p[P.baseC]) + P.offC + gm + (int64_t)gn * P.ldc;
      *c = P.beta ? (*c + acc[i][j]) : acc[i][j];
    }
  }
}

__global__ void __launch_bounds__(256) k_gemm_f64(const GProb* __restrict__ prob, const GSeg* __restrict__ seg,
                                                  const GTile* __restrict__ tile, const Bases bases) {
  __shared__ double As[GK][GM + 1];
  __shared__ double Bs[GK][GN + 1];
  const GTile t = tile[blockIdx.x];
  const GProb P = prob[t.prob];
#define MPSG_GEMM_SHAPE(I, J) \
  case (I - 1) * 4 + (J - 1): gemm_tile<I, J>(P, t, seg, bases, As, Bs); break;
  switch ((t.mi - 1) * 4 + (t.nj - 1)) {
    MPSG_GEMM_SHAPE(1, 1) MPSG_GEMM_SHAPE(1, 2) MPSG_GEMM_SHAPE(1, 3) MPSG_GEMM_SHAPE(1, 4)
    MPSG_GEMM_SHAPE(2, 1) MPSG_GEMM_SHAPE(2, 2) MPSG_GEMM_SHAPE(2, 3) MPSG_GEMM_SHAPE(2, 4)
    MPSG_GEMM_SHAPE(3, 1) MPSG_GEMM_SHAPE(3, 2) MPSG_GEMM_SHAPE(3, 3) MPSG_GEMM_SHAPE(3, 4)
    MPSG_GEMM_SHAPE(4, 1) MPSG_GEMM_SHAPE(4, 2) MPSG_GEMM_SHAPE(4, 3) MPSG_GEMM_SHAPE(4, 4)
    default: break;
  }
#undef MPSG_GEMM_SHAPE
}

void launch_gemm_f64(const GProb* prob, const GSeg* seg, const GTile* tile, int ntiles, const Bases& bases,
                     cudaStream_t s) {
  if (ntiles <= 0) return;
  // (FP64 tensor-core variants with mma.sync m8n8k4 measured slower on this GPU: 7.05 ms per chi=2048
  // matvec with 64 x 64 tiles on 8 warps, 6.97 ms with 32 x 32 warp tiles and double-buffered slices,
  // against 6.0 ms for this FMA kernel)
  k_gemm_f64<<<ntiles, 256, 0, s>>>(prob, seg, tile, bases);
  LAUNCHED();
}

// ============================================================================ block linear combination
__global__ void k_lincomb(const LCOut* __restrict__ outs, const LCTerm* __restrict__ terms) {
  const LCOut o = outs[blockIdx.x];
  for (int64_t i = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; i < o.n; i += (int64_t)gridDim.y * blockDim.x) {
    double s = 0.0;
    for (int t = o.t0; t < o.t1; ++t) s = fma(terms[t].coef, terms[t].src[i], s);
    o.dst[i] = s;
  }
}
void launch_lincomb(const LCOut* outs, const LCTerm* terms, int nout, int64_t maxn, cudaStream_t s) {
  if (nout <= 0) return;
  int chunks = (int)std::min<int64_t>((maxn + 255) / 256, 64);
  if (chunks < 1) chunks = 1;
  k_lincomb<<<dim3(nout, chunks), 256, 0, s>>>(outs, terms);
  LAUNCHED();
}

// ============================================================================ strided block copies
__global__ void k_copy(const CopyOp* __restrict__ ops) {
  const CopyOp o = ops[blockIdx.x];
  const int64_t tot = (int64_t)o.rows * o.cols;
  for (int64_t e = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.y * blockDim.x) {
    const int i = (int)(e % o.rows), j = (int)(e / o.rows);
    double v = o.trans ? o.src[j + (int64_t)i * o.lds] : o.src[i + (int64_t)j * o.lds];
    v *= o.scale;
    if (o.rs) v *= o.rs[i];
    if (o.cs) v *= o.cs[j];
    o.dst[i + (int64_t)j * o.ldd] = v;
  }
}
void launch_copyops(const CopyOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_copy<<<dim3(nops, 16), 256, 0, s>>>(ops);
  LAUNCHED();
}

// ============================================================================ FixPhase
// For singular index i the sign of the first abs-max entry of P(:,i) (a row of Vt) is made
// positive; the same sign multiplies Q(:,i) (blas/helperfunctions.hpp:36-51).
__global__ void k_fixphase(const PhaseOp* __restrict__ ops) {
  const PhaseOp o = ops[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = blockIdx.y * 8 + warp; i < o.k; i += gridDim.y * 8) {
    double* p = o.Pm + (int64_t)i * o.ldp;
    double best = 0.0;
    int bi = INT_MAX;
    for (int j = lane; j < o.n; j += 32) {
      const double a = fabs(p[j]);
      if (a > best) { best = a; bi = j; }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, off);
      const int oi = __shfl_down_sync(0xffffffffu, bi, off);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    bi = __shfl_sync(0xffffffffu, bi, 0);
    best = __shfl_sync(0xffffffffu, best, 0);
    if (best == 0.0) bi = 0;
    const double sgn = (o.n > 0 && p[bi] > 0) ? 1.0 : -1.0;
    __syncwarp();
    if (sgn < 0) {
      for (int j = lane; j < o.n; j += 32) p[j] = -p[j];
      double* q = o.Qm + (int64_t)i * o.ldq;
      for (int j = lane; j < o.m; j += 32) q[j] = -q[j];
    }
  }
}
void launch_fixphase(const PhaseOp* ops, int nops, int maxk, cudaStream_t s) {
  if (nops <= 0 || maxk <= 0) return;
  int gy = (maxk + 7) / 8;
  if (gy > 64) gy = 64;
  k_fixphase<<<dim3(nops, gy), 256, 0, s>>>(ops);
  LAUNCHED();
}

// ============================================================================ density-matrix SVD post-processing
// s_i = sqrt(lambda_(i)) for the i-th largest eigenvalue, V(:, i) = its eigenvector
// The eigenpairs come from an nc x nc slot whose padding eigenvalues are -1; the n eigenvalues
// >= -0.5 are the sector's, in any order.  They are ranked descending (ties by index) without
// relying on the solver's ordering.  Eigenvalues at or below the eigensolver's noise level
// (32 n eps lambda_max) are not resolved by the Gram route and are reported as exact zeros, so
// truncation never keeps their vectors.
__global__ void k_gram_post(const GramPost* __restrict__ ops) {
  const GramPost o = ops[blockIdx.x];
  const int n = o.n, nc = o.nc;
  __shared__ double lmax_s;
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int j = 0; j < nc; ++j) m = fmax(m, o.lam[j]);
    lmax_s = m;
  }
  __syncthreads();
  const double floor_l = 32.0 * n * DBL_EPSILON * lmax_s;
  for (int j = threadIdx.x; j < nc; j += blockDim.x) {
    const double lj = o.lam[j];
    if (!(lj > -0.5)) continue;  // padding
    int rank = 0;
    for (int l = 0; l < nc; ++l) {
      const double ll = o.lam[l];
      rank += (ll > -0.5) && (ll > lj || (ll == lj && l < j));
    }
    if (rank >= n) continue;  // defensive: more than n non-padding eigenvalues
    const double sv = lj > floor_l ? sqrt(lj) : 0.0;
    o.S[rank] = sv;
    const double* w = o.W + (int64_t)j * o.ldw;
    double* v = o.V + (int64_t)rank * n;
    for (int r = 0; r < n; ++r) v[r] = w[r];
  }
}
void launch_gram_post(const GramPost* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_gram_post<<<nops, 256, 0, s>>>(ops);
  LAUNCHED();
}
// Left vectors of the density-matrix route: y_j = M v_j has norm s_j (the singular value the pair
// (u_j, v_j) actually carries, free of the Gram eigenvalue's absolute error), u_j = y_j / s_j is unit
// length; unresolved columns (S already 0) are cleared so truncation never keeps them.
// One block per sector, one warp per column at a time.
__global__ void k_colnorm(const ColNorm* __restrict__ ops) {
  const ColNorm o = ops[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int j = warp; j < o.k; j += nwarp) {
    double* u = o.U + (int64_t)j * o.ldu;
    if (o.S[j] == 0.0) {
      for (int r = lane; r < o.m; r += 32) u[r] = 0.0;
      continue;
    }
    double acc = 0.0;
    for (int r = lane; r < o.m; r += 32) acc = fma(u[r], u[r], acc);
    for (int off = 16; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    const double nrm = sqrt(acc);
    const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
    for (int r = lane; r < o.m; r += 32) u[r] *= inv;
    __syncwarp();
    if (lane == 0) o.S[j] = nrm;
  }
}
void launch_colnorm(const ColNorm* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_colnorm<<<nops, 256, 0, s>>>(ops);
  LAUNCHED();
}
__global__ void k_chol_unit_zero_diag(const CholOp* __restrict__ ops) {
  const CholOp o = ops[blockIdx.x];
  for (int j = threadIdx.x; j < o.n; j += blockDim.x) {
    double* c = o.C + j + (int64_t)j * o.ld;
    if (*c == 0.0) *c = 1.0;
  }
}
void launch_chol_unit_zero_diag(const CholOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_chol_unit_zero_diag<<<nops, 128, 0, s>>>(ops);
  LAUNCHED();
}
__global__ void k_chol_scale_s(const CholOp* __restrict__ ops) {
  const CholOp o = ops[blockIdx.x];
  for (int j = threadIdx.x; j < o.n; j += blockDim.x) o.S[j] *= fabs(o.C[j + (int64_t)j * o.ld]);
}
void launch_chol_scale_s(const CholOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_chol_scale_s<<<nops, 128, 0, s>>>(ops);
  LAUNCHED();
}
__global__ void k_gram_pad(const GramPad* __restrict__ ops) {
  const GramPad o = ops[blockIdx.x];
  for (int i = o.n + threadIdx.x; i < o.nc; i += blockDim.x) o.A[i + (int64_t)i * o.nc] = -1.0;
}
void launch_gram_pad(const GramPad* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_gram_pad<<<nops, 128, 0, s>>>(ops);
  LAUNCHED();
}

// ============================================================================ reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}
__device__ double block_sum(double v) {  // blockDim.x == 256
  __shared__ double sh[8];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < 8 ? sh[threadIdx.x] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

__global__ void k_dot_part(const double* __restrict__ x, const double* __restrict__ y, int64_t n, double* part) {
  double s = 0.0;
  const int64_t n2 = n >> 1;
  const double2* x2 = reinterpret_cast<const double2*>(x);
  const double2* y2 = reinterpret_cast<const double2*>(y);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = x2[i], b = y2[i];
    s = fma(a.x, b.x, s);
    s = fma(a.y, b.y, s);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) s = fma(x[n - 1], y[n - 1], s);
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void k_sum_parts(const double* part, int np, double* out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  s = block_sum(s);
  if (threadIdx.x == 0) *out = s;
}
void launch_dot(const double* x, const double* y, int64_t n, double* part, double* out, cudaStream_t s) {
  k_dot_part<<<kRedBlocks, 256, 0, s>>>(x, y, n, part);
  k_sum_parts<<<1, 256, 0, s>>>(part, kRedBlocks, out);
  g_launches.fetch_add(2);
}

__global__ void k_scale_by_norm(double* x, int64_t n, const double* norm2, double delta, double* beta_out) {
  const double k = sqrt(*norm2);
  const double sc = (k < delta) ? 0.0 : 1.0 / k;
  if (beta_out && blockIdx.x == 0 && threadIdx.x == 0) *beta_out = k;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= sc;
}
void launch_scale_by_norm(double* x, int64_t n, const double* norm2, double delta, double* beta_out,
                          cudaStream_t s) {
  k_scale_by_norm<<<kRedBlocks, 256, 0, s>>>(x, n, norm2, delta, beta_out);
  LAUNCHED();
}

// out = (v*(-alpha) + w) + vprev*(-beta), and the squared norm of out
__global__ void k_axpy3(double* __restrict__ out, const double* __restrict__ w, const double* __restrict__ v,
                        const double* __restrict__ vp, const double* alpha, const double* beta, int64_t n,
                        double* part) {
  const double a = -(*alpha);
  const double b = vp ? -(*beta) : 0.0;
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double o = v[i] * a + w[i];
    if (vp) o = o + vp[i] * b;
    out[i] = o;
    s = fma(o, o, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}
void launch_axpy3(double* out, const double* w, const double* v, const double* vprev, const double* alpha,
                  const double* beta, int64_t n, double* part, double* norm2_out, cudaStream_t s) {
  k_axpy3<<<kRedBlocks, 256, 0, s>>>(out, w, v, vprev, alpha, beta, n, part);
  k_sum_parts<<<1, 256, 0, s>>>(part, kRedBlocks, norm2_out);
  g_launches.fetch_add(2);
}

// y = (or -=) sum_j c[j] * V_j, V given as a device array of vector pointers
__global__ void k_combine(double* y, const double* const* __restrict__ V, int nv, const double* __restrict__ c,
                          int64_t n, int subtract) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < nv; ++j) s = fma(V[j][i], c[j], s);
    y[i] = subtract ? (y[i] - s) : s;
  }
}
void launch_combine(double* y, const double* const* V, int nv, const double* c, int64_t n, int subtract,
                    cudaStream_t s) {
  k_combine<<<kRedBlocks, 256, 0, s>>>(y, V, nv, c, n, subtract);
  LAUNCHED();
}

constexpr int kProjChunks = 64;
__global__ void k_project_part(const double* const* __restrict__ V, const double* __restrict__ x, int64_t n,
                               double* part) {
  const int j = blockIdx.y;
  const double* v = V[j];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s = fma(v[i], x[i], s);
  s = block_sum(s);
  if (threadIdx.x == 0) part[(int64_t)j * kProjChunks + blockIdx.x] = s;
}
__global__ void k_project_sum(const double* part, double* c) {
  const int j = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < kProjChunks; i += blockDim.x) s += part[(int64_t)j * kProjChunks + i];
  s = block_sum(s);
  if (threadIdx.x == 0) c[j] = s;
}
void launch_project(const double* const* V, int nv, const double* x, int64_t n, double* part_nv, double* c,
                    cudaStream_t s) {
  if (nv <= 0) return;
  k_project_part<<<dim3(kProjChunks, nv), 256, 0, s>>>(V, x, n, part_nv);
  k_project_sum<<<nv, 256, 0, s>>>(part_nv, c);
  g_launches.fetch_add(2);
}

__global__ void k_fill(double* x, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}
void launch_fill(double* x, int64_t n, double v, cudaStream_t s) {
  if (n <= 0) return;
  k_fill<<<kRedBlocks, 256, 0, s>>>(x, n, v);
  LAUNCHED();
}

// ============================================================================ tridiagonal eigensolver
// Lowest eigenvalue of T (diag a[0..n), offdiag b[1..n)) by Sturm-count multisection in one warp,
// eigenvector by inverse iteration with a pivoted tridiagonal LU (one thread).
// Number of eigenvalues of the tridiagonal (diagonal a[0..n), off-diagonal squares b2[i] coupling
// i-1 and i) below x: sign changes of the characteristic-polynomial sequence p_i = (a_i - x) p_{i-1}
// - b2_i p_{i-2}, kept in range by exact power-of-two rescaling (no division: FP64 division is a
// long instruction sequence on this GPU).  A zero p_i counts as a sign change (the ratio form's
// -pivmin rule).
__device__ int sturm_count_nodiv(const double* a, const double* b2, int n, double x) {
  int c = 0;
  double p0 = 1.0, p1 = a[0] - x;
  if (p1 == 0.0) p1 = -DBL_MIN;
  c += p1 < 0.0;
  for (int i = 1; i < n; ++i) {
    double p2 = fma(a[i] - x, p1, -b2[i] * p0);
    if (p2 == 0.0) p2 = p1 > 0.0 ? -DBL_MIN : DBL_MIN;
    c += (p2 < 0.0) != (p1 < 0.0);
    p0 = p1;
    p1 = p2;
    const double m = fabs(p1);
    if (m > 0x1p+400) { p0 *= 0x1p-400; p1 *= 0x1p-400; }
    else if (m < 0x1p-400) { p0 *= 0x1p+400; p1 *= 0x1p+400; }
  }
  return c;
}

__device__ void tri_lowest_dev(const double* __restrict__ a_g, const double* __restrict__ b, int n, double* E0,
                               double* z) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x;
  double* a = sm + 6 * n;   // diagonal and squared off-diagonal, staged for the Sturm counts
  double* b2 = sm + 7 * n;
  for (int i = lane; i < n; i += 32) {
    a[i] = a_g[i];
    b2[i] = i > 0 ? b[i] * b[i] : 0.0;
  }
  __syncwarp();
  // Gershgorin interval
  double lo = DBL_MAX, hi = -DBL_MAX, bmax = 0.0;
  for (int i = lane; i < n; i += 32) {
    const double r = (i > 0 ? fabs(b[i]) : 0.0) + (i + 1 < n ? fabs(b[i + 1]) : 0.0);
    lo = fmin(lo, a[i] - r);
    hi = fmax(hi, a[i] + r);
    if (i > 0) bmax = fmax(bmax, b[i] * b[i]);
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, off));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, off));
    bmax = fmax(bmax, __shfl_xor_sync(0xffffffffu, bmax, off));
  }
  const double pivmin = fmax(DBL_MIN, DBL_MIN * bmax);
  const double tnorm = fmax(fabs(lo), fabs(hi));
  lo -= 2.0 * DBL_EPSILON * tnorm + pivmin;
  hi += 2.0 * DBL_EPSILON * tnorm + pivmin;
  for (int round = 0; round < 80; ++round) {
    if (hi - lo <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + pivmin) break;
    const double x = lo + (hi - lo) * (double)(lane + 1) / 33.0;
    const int c = sturm_count_nodiv(a, b2, n, x);
    const unsigned ball = __ballot_sync(0xffffffffu, c >= 1);
    const double xprev = __shfl_up_sync(0xffffffffu, x, 1);
    if (ball == 0) {
      lo = __shfl_sync(0xffffffffu, x, 31);
    } else {
      const int l = __ffs(ball) - 1;
      const double nhi = __shfl_sync(0xffffffffu, x, l);
      const double nlo = (l == 0) ? lo : __shfl_sync(0xffffffffu, xprev, l);
      lo = nlo;
      hi = nhi;
    }
  }
  const double lam = 0.5 * (lo + hi);
  if (lane == 0) *E0 = lam;
  if (!z || lane != 0) return;
  // inverse iteration: (T - lam) x = rhs, LU with partial pivoting (dgttrf/dgtts2 scheme)
  double* dl = sm;
  double* d = sm + n;
  double* du = sm + 2 * n;
  double* du2 = sm + 3 * n;
  double* x = sm + 4 * n;
  int* piv = reinterpret_cast<int*>(sm + 5 * n);
  const double tiny = DBL_EPSILON * fmax(tnorm, DBL_MIN);
  for (int i = 0; i < n; ++i) {
    d[i] = a[i] - lam;
    dl[i] = (i + 1 < n) ? b[i + 1] : 0.0;
    du[i] = (i + 1 < n) ? b[i + 1] : 0.0;
    du2[i] = 0.0;
    piv[i] = i;
    x[i] = 1.0;
  }
  for (int i = 0; i < n - 1; ++i) {
    if (fabs(d[i]) >= fabs(dl[i])) {
      if (d[i] == 0.0) d[i] = tiny;
      const double f = dl[i] / d[i];
      dl[i] = f;
      d[i + 1] -= f * du[i];
      du2[i] = 0.0;
    } else {
      const double f = d[i] / dl[i];
      d[i] = dl[i];
      dl[i] = f;
      const double tmp = du[i];
      du[i] = d[i + 1];
      d[i + 1] = tmp - f * d[i + 1];
      if (i < n - 2) {
        du2[i] = du[i + 1];
        du[i + 1] = -f * du[i + 1];
      }
      piv[i] = i + 1;
    }
  }
  if (d[n - 1] == 0.0) d[n - 1] = tiny;
  for (int i = 0; i < n; ++i) d[i] = 1.0 / d[i];  // reciprocal pivots: the solves only multiply
  for (int it = 0; it < 3; ++it) {
    // forward: apply L^{-1} P
    for (int i = 0; i < n - 1; ++i) {
      if (piv[i] == i) {
        x[i + 1] -= dl[i] * x[i];
      } else {
        const double t = x[i];
        x[i] = x[i + 1];
        x[i + 1] = t - dl[i] * x[i];
      }
    }
    // backward: U x = y
    x[n - 1] *= d[n - 1];
    if (n > 1) x[n - 2] = (x[n - 2] - du[n - 2] * x[n - 1]) * d[n - 2];
    for (int i = n - 3; i >= 0; --i) x[i] = (x[i] - du[i] * x[i + 1] - du2[i] * x[i + 2]) * d[i];
    double nrm = 0.0, amax = 0.0;
    int imax = 0;
    for (int i = 0; i < n; ++i) {
      nrm += x[i] * x[i];
      if (fabs(x[i]) > amax) { amax = fabs(x[i]); imax = i; }
    }
    const double s = (x[imax] < 0 ? -1.0 : 1.0) / sqrt(nrm);
    for (int i = 0; i < n; ++i) x[i] *= s;
  }
  for (int i = 0; i < n; ++i) z[i] = x[i];
}
__global__ void k_tri_lowest(const double* __restrict__ a_g, const double* __restrict__ b, int n, double* E0,
                             double* z) {
  tri_lowest_dev(a_g, b, n, E0, z);
}
void launch_tri_lowest(const double* alpha, const double* beta, int n, double* E0, double* z, cudaStream_t s) {
  if (n <= 0) return;
  const size_t sh = (size_t)n * 8 * sizeof(double) + 16;
  k_tri_lowest<<<1, 32, sh, s>>>(alpha, beta, n, E0, z);
  LAUNCHED();
}
// ============================================================================ graph-replayed Lanczos
// The Lanczos iterations between two energy checkpoints are captured once as a CUDA graph and replayed
// for every later batch: the iteration index j lives on the device (*jp), the kernels below read it
// and address the Krylov vectors through the device table V; the matvec works on fixed buffers (xin
// holds the normalised V[j]).  The arithmetic is that of the launch-by-launch kernels above.
__global__ void k_lz_scale(double* const* __restrict__ V, const int* __restrict__ jp, const double* __restrict__ norm2,
                           double delta, double* beta, double* __restrict__ xin, int64_t n) {
  const int j = *jp;
  double* x = V[j];
  const double k = sqrt(norm2[j]);
  const double sc = (k < delta) ? 0.0 : 1.0 / k;
  if (blockIdx.x == 0 && threadIdx.x == 0) beta[j] = k;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i] * sc;
    x[i] = v;
    xin[i] = v;
  }
}
// base[*jp + offset] = sum of the block partials; incr: then *jp += 1
__global__ void k_lz_sum(const double* part, int np, double* base, int* jp, int offset, int incr) {
  const int j = *jp;
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  s = block_sum(s);
  if (threadIdx.x == 0) {
    base[j + offset] = s;
    if (incr) *jp = j + 1;
  }
}
__global__ void k_lz_axpy3(double* const* __restrict__ V, const int* __restrict__ jp, const double* __restrict__ w,
                           const double* __restrict__ v, const double* alpha, const double* beta, int64_t n,
                           double* part) {
  const int j = *jp;
  double* __restrict__ out = V[j + 1];
  const double* __restrict__ vp = j > 0 ? V[j - 1] : nullptr;
  const double a = -alpha[j];
  const double b = vp ? -beta[j] : 0.0;
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double o = v[i] * a + w[i];
    if (vp) o = o + vp[i] * b;
    out[i] = o;
    s = fma(o, o, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void k_lz_tri_lowest(const double* __restrict__ a_g, const double* __restrict__ b, const int* jp, int ndiag,
                                double* E) {
  const int j = *jp;
  tri_lowest_dev(a_g, b, j + 1, E + j / ndiag, nullptr);
}
// one Lanczos iteration on the device index: scale V[j] (and copy it to xin), the caller's matvec
// xin -> w, alpha[j], the optional energy checkpoint, V[j+1] and its squared norm, j += 1
void launch_lz_pre(double* const* V, const int* jp, const double* norm2, double delta, double* beta, double* xin,
                   int64_t n, cudaStream_t s) {
  k_lz_scale<<<kRedBlocks, 256, 0, s>>>(V, jp, norm2, delta, beta, xin, n);
  LAUNCHED();
}
void launch_lz_post(double* const* V, int* jp, const double* w, const double* xin, double* alpha, double* beta,
                    double* norm2, double* E, int ndiag, bool checkpoint, int itmax, int64_t n, double* part,
                    cudaStream_t s) {
  k_dot_part<<<kRedBlocks, 256, 0, s>>>(w, xin, n, part);
  k_lz_sum<<<1, 256, 0, s>>>(part, kRedBlocks, alpha, jp, 0, 0);
  if (checkpoint) {
    const size_t sh = (size_t)(itmax + 1) * 8 * sizeof(double) + 16;
    k_lz_tri_lowest<<<1, 32, sh, s>>>(alpha, beta, jp, ndiag, E);
  }
  k_lz_axpy3<<<kRedBlocks, 256, 0, s>>>(V, jp, w, xin, alpha, beta, n, part);
  k_lz_sum<<<1, 256, 0, s>>>(part, kRedBlocks, norm2, jp, 1, 1);
  g_launches.fetch_add(checkpoint ? 5 : 4);
}
void lz_prepare_attributes(int itmax) {
  const size_t sh = (size_t)(itmax + 1) * 8 * sizeof(double) + 16;
  if (sh > 48 * 1024)
    MPSG_CUDA(cudaFuncSetAttribute(k_lz_tri_lowest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
}
void count_graph_launches(int64_t n) { g_launches.fetch_add(n); }

// One block per chain c: the lowest eigenpair of chain c's tridiagonal (alpha / beta at c * stride,
// n_of[c] rows; chains with n_of[c] <= 0 are skipped); E0 at c * estride, z at c * stride.
__global__ void k_tri_lowest_seg(const double* __restrict__ alpha, const double* __restrict__ beta,
                                 const int* __restrict__ n_of, int stride, double* E0, int estride, double* z) {
  const int c = blockIdx.x;
  const int n = n_of[c];
  if (n <= 0) return;
  tri_lowest_dev(alpha + (int64_t)c * stride, beta + (int64_t)c * stride, n, E0 + (int64_t)c * estride,
                 z ? z + (int64_t)c * stride : nullptr);
}
void launch_tri_lowest_seg(const double* alpha, const double* beta, const int* n_of, int nchains, int nmax, int stride,
                           double* E0, int estride, double* z, cudaStream_t s) {
  if (nchains <= 0 || nmax <= 0) return;
  const size_t sh = (size_t)nmax * 8 * sizeof(double) + 16;
  k_tri_lowest_seg<<<nchains, 32, sh, s>>>(alpha, beta, n_of, stride, E0, estride, z);
  LAUNCHED();
}

// ============================================================================ truncation
// rank[i] = position of value i when all values are ordered by (value desc, later insertion first),
// the iteration order of the reference's reversed std::multimap (src/BlockTensor.hpp:236-258).
// rank[i] = number of values ordered before value i: larger ones, and equal ones stored later (the
// reversed multimap).  Singular values are >= +0, so their IEEE bit patterns order like the values:
// the comparisons run on the integer pipe (an FP64 compare occupies this GPU's FP64 pipe for 16
// cycles per warp), over tiles of the values staged in shared memory.
constexpr int kRankTile = 2048;
__global__ void __launch_bounds__(256) k_trunc_rank(const double* __restrict__ S, int n, int32_t* rank) {
  __shared__ long long key[kRankTile];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr long long kAbs = 0x7fffffffffffffffll;  // -0 orders as +0
  const long long v = i < n ? (__double_as_longlong(S[i]) & kAbs) : 0;
  int r = 0;
  for (int t0 = 0; t0 < n; t0 += kRankTile) {
    const int tn = min(kRankTile, n - t0);
    __syncthreads();
    for (int j = threadIdx.x; j < tn; j += blockDim.x) key[j] = __double_as_longlong(S[t0 + j]) & kAbs;
    __syncthreads();
    if (i < n)
      for (int j = 0; j < tn; ++j) {
        const long long w = key[j];
        r += (w > v) | ((w == v) & (t0 + j > i));
      }
  }
  if (i < n) rank[i] = r;
}
// out3[0] = truncated weight, out3[1] = kept count, out3[2] = 1/norm of kept values (normalisation).
// One block.  The floating-point recurrences stay sequential in the reference's order (the norm over
// the values in storage order, the truncated weight over the values in rank order, the kept norm per
// sector then over the sectors), run by thread 0 on values the block stages in shared memory chunk by
// chunk; the scatter of the order, the per-sector counts and the per-sector partial sums run in
// parallel.  sec_of is non-decreasing (each sector's values contiguous, stored descending).
constexpr int kTruncThreads = 1024;
constexpr int kTruncChunk = 2048;
constexpr int kTruncSecSh = 2048;
__global__ void __launch_bounds__(kTruncThreads)
    k_trunc_select(const double* __restrict__ S, int n, const int32_t* __restrict__ sec_of, int nsec, int chimax,
                   int doTrunc, double tr_weight, const int32_t* __restrict__ rank, int32_t* order, int32_t* counts,
                   double* out3) {
  __shared__ double sv[kTruncChunk];
  __shared__ double part_sh[kTruncSecSh];
  __shared__ int start_sh[kTruncSecSh];
  __shared__ int s_stop, s_cnt;
  __shared__ double s_norm;
  const int tid = threadIdx.x;
  for (int i = tid; i < nsec; i += blockDim.x) counts[i] = 0;
  for (int i = tid; i < n; i += blockDim.x) order[rank[i]] = i;
  if (tid == 0) {
    s_stop = 0;
    s_cnt = 0;
    s_norm = 0.0;
  }
  __syncthreads();
  // norm of all values (truncated-weight mode), summed in storage order
  double nrm2 = 0.0;
  if (doTrunc) {
    for (int c0 = 0; c0 < n; c0 += kTruncChunk) {
      const int m = min(kTruncChunk, n - c0);
      for (int j = tid; j < m; j += blockDim.x) sv[j] = S[c0 + j];
      __syncthreads();
      if (tid == 0)
        for (int j = 0; j < m; ++j) nrm2 += sv[j] * sv[j];
      __syncthreads();
    }
    if (tid == 0) s_norm = sqrt(nrm2);
    __syncthreads();
  }
  const double norm = s_norm;
  // the kept prefix of the rank order
  double tw = doTrunc ? norm : 1.0;
  int cnt = 0;
  for (int c0 = 0; c0 < n; c0 += kTruncChunk) {
    const int m = min(kTruncChunk, n - c0);
    for (int j = tid; j < m; j += blockDim.x) sv[j] = S[order[c0 + j]];
    __syncthreads();
    if (tid == 0) {
      int r = 0;
      if (!doTrunc) {
        for (; r < m && cnt != chimax; ++r) {
          const double v = sv[r];
          if (!(fabs(v) > 1e-15)) {
            s_stop = 1;
            break;
          }
          tw -= v * v;
          ++cnt;
        }
        if (cnt == chimax) s_stop = 1;
      } else {
        for (; r < m && fabs(tw) > norm * tr_weight && cnt < chimax; ++r) {
          const double v = sv[r];
          tw -= (v * v) / norm;
          ++cnt;
        }
        if (r < m) s_stop = 1;
      }
      s_cnt = cnt;
    }
    __syncthreads();
    const int stop = s_stop;
    __syncthreads();
    if (stop) break;
  }
  if (doTrunc && tw < 0 && fabs(tw) < 1e-14) tw = 0.0;
  cnt = s_cnt;
  for (int r = tid; r < cnt; r += blockDim.x) atomicAdd(&counts[sec_of[order[r]]], 1);
  __syncthreads();
  // norm of the kept values: per sector (its first counts[sec] values, in storage order), then over
  // the sectors in order
  double k2 = 0.0;
  if (nsec <= kTruncSecSh) {
    for (int i = tid; i < nsec; i += blockDim.x) {
      part_sh[i] = 0.0;
      start_sh[i] = -1;
    }
    __syncthreads();
    for (int j = tid; j < n; j += blockDim.x)
      if (j == 0 || sec_of[j] != sec_of[j - 1]) start_sh[sec_of[j]] = j;
    __syncthreads();
    for (int sec = tid; sec < nsec; sec += blockDim.x) {
      const int st = start_sh[sec];
      if (st < 0) continue;
      const int c = counts[sec];
      double part = 0.0;
      for (int t = 0; t < c; ++t) part += S[st + t] * S[st + t];
      part_sh[sec] = part;
    }
    __syncthreads();
    if (tid != 0) return;
    for (int sec = 0; sec < nsec; ++sec)
      if (start_sh[sec] >= 0) k2 += part_sh[sec];
  } else {
    if (tid != 0) return;
    int i = 0;
    while (i < n) {
      const int sec = sec_of[i];
      int j = i;
      double part = 0.0;
      int taken = 0;
      while (j < n && sec_of[j] == sec) {
        if (taken < counts[sec]) {
          part += S[j] * S[j];
          ++taken;
        }
        ++j;
      }
      k2 += part;
      i = j;
    }
  }
  out3[0] = tw;
  out3[1] = (double)cnt;
  out3[2] = k2 > 0 ? 1.0 / sqrt(k2) : 0.0;
}
void launch_truncate(const double* S, int n, const int32_t* sec_of, int nsec, int chimax, int doTrunc,
                     double tr_weight, int32_t* rank_scratch, int32_t* counts, double* out3, cudaStream_t s) {
  if (n > 0) {
    k_trunc_rank<<<(n + 255) / 256, 256, 0, s>>>(S, n, rank_scratch);
    LAUNCHED();
  }
  k_trunc_select<<<1, kTruncThreads, 0, s>>>(S, n, sec_of, nsec, chimax, doTrunc, tr_weight, rank_scratch,
                                   rank_scratch + n, counts, out3);
  LAUNCHED();
}

}  // namespace mpsg
