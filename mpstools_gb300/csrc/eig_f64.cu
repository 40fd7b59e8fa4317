// Batched FP64 symmetric eigensolver for the density-matrix split (sector Gram matrices G = M^T M).
//
// Stages, each one launch over all sectors:
//   1. k_sytrd<CL>   Householder tridiagonalisation Q^T G Q = T.  One thread-block cluster of CL CTAs
//                    per sector; the CTAs own the matrix columns round-robin in shared memory; the
//                    Householder vector is copied from its owner, the product p = tau G v and the
//                    partial dot products are pushed through distributed shared memory; two
//                    cluster barriers per column.
//   2. k_tri_bisect  eigenvalues of T above the resolution floor by multisection on Sturm counts
//                    (a group of 4 lanes per eigenvalue, 4 points per round).
//   3. k_tri_invit   eigenvectors of T by inverse iteration with a partially pivoted tridiagonal LU,
//                    one thread per eigenvalue; the caller re-orthonormalises them (CholeskyQR).
//   4. k_ormtr       eigenvectors of G = Q z: the reflectors applied to blocks of 8 eigenvector
//                    columns held in shared memory, one warp per column.
// The tridiagonalisation follows the Householder method (Golub & Van Loan, Matrix Computations,
// sections 8.3.1 and 5.1.2); bisection and inverse iteration follow the Sturm-sequence and
// inverse-iteration methods of Wilkinson, The Algebraic Eigenvalue Problem, chapter 5.
// No wait in these kernels spins: cluster barriers are hardware barriers.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cfloat>

#include "mpsg_internal.h"
#include "eig_common.cuh"

namespace cg = cooperative_groups;

namespace mpsg {

static std::atomic<int64_t> g_eig_launches{0};
int64_t eig_launch_count() { return g_eig_launches.load(); }

// ----------------------------------------------------------------------------- 1. tridiagonalisation
// Shared memory of one CTA: own columns (ncol x n) | v (2 x n, double-buffered) | p (n) | w (n) |
// kpart (16) | scal (4: tau[2], beta[2]).
static __host__ __device__ size_t sytrd_smem_doubles(int n, int CL) {
  const int ncol = (n + CL - 1) / CL;
  return (size_t)ncol * n + 4 * (size_t)n + 16 + 4;
}
size_t sytrd_smem_bytes(int n, int CL) { return sizeof(double) * sytrd_smem_doubles(n, CL); }


// Householder vector of column j (held by the calling warp's CTA as local column `col`): alpha =
// x[j+1], the rest x[j+2..n-1].  Writes v (v[j+1] = 1) into this CTA's v buffer `slot`, tau and beta
// into its scal (the other CTAs copy them after the next cluster barrier), the reflector (without the
// unit entry) into column j of the global matrix, tau[j] and e[j].
__device__ void sytrd_householder(const SytrdOp& o, const double* col, int j, double* vbuf_local,
                                  double* scal_local, int slot, int lane) {
  const int n = o.n;
  double s2 = 0.0;
  for (int i = j + 2 + lane; i < n; i += 32) s2 = fma(col[i], col[i], s2);
  s2 = warp_sum(s2);
  const double alpha = col[j + 1];
  double tau = 0.0, beta = alpha, scale = 0.0;
  if (s2 > 0.0) {
    beta = -copysign(sqrt(alpha * alpha + s2), alpha);
    tau = (beta - alpha) / beta;
    scale = 1.0 / (alpha - beta);
  }
  double* vr = vbuf_local + (size_t)slot * n;
  for (int i = j + 1 + lane; i < n; i += 32) vr[i] = (i == j + 1) ? 1.0 : col[i] * scale;
  if (lane == 0) {
    scal_local[slot] = tau;
    scal_local[2 + slot] = beta;
  }
  for (int i = j + 2 + lane; i < n; i += 32) o.A[i + (int64_t)j * o.lda] = col[i] * scale;
  if (lane == 0) {
    o.tau[j] = tau;
    o.e[j] = beta;
  }
}

// Copy the Householder vector of step j (and its tau) from the CTA that computed it.
__device__ void sytrd_pull(cg::cluster_group& cluster, int CL, int r, int n, int j, double* vbuf, double* scal) {
  const int src = j % CL;  // owner of column j computed its reflector
  const int slot = j & 1;
  if (src == r) return;
  const double* rv = cluster.map_shared_rank(vbuf + (size_t)slot * n, src);
  double* lv = vbuf + (size_t)slot * n;
  for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) lv[i] = rv[i];
  if (threadIdx.x == 0) scal[slot] = *cluster.map_shared_rank(scal + slot, src);
}

template <int CL>
__global__ void __launch_bounds__(256) k_sytrd(const SytrdOp* __restrict__ ops) {
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const SytrdOp o = ops[blockIdx.x / CL];
  const int n = o.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  extern __shared__ double sm[];
  const int ncol = (n - r + CL - 1) / CL;  // local columns: global column r + lc*CL
  double* cols = sm;
  const int ncol_max = (n + CL - 1) / CL;
  double* vbuf = cols + (size_t)ncol_max * n;
  double* p = vbuf + 2 * (size_t)n;
  double* w = p + n;
  double* kpart = w + n;
  double* scal = kpart + 16;
  for (int lc = warp; lc < ncol; lc += nwarp) {
    const int c = r + lc * CL;
    for (int i = lane; i < n; i += 32) cols[(size_t)lc * n + i] = o.A[i + (int64_t)c * o.lda];
  }
  if (n >= 3 && r == 0 && warp == 0) sytrd_householder(o, cols, 0, vbuf, scal, 0, lane);
  if (n >= 1 && r == 0 && threadIdx.x == 0) o.d[0] = cols[0];
  cluster.sync();  // every CTA runs (distributed shared memory is addressable) and reflector 0 exists
  for (int j = 0; j + 2 < n; ++j) {
    const int slot = j & 1;
    sytrd_pull(cluster, CL, r, n, j, vbuf, scal);
    __syncthreads();
    const double* v = vbuf + (size_t)slot * n;
    const double tau = scal[slot];
    // (b) p_c = tau * G(:, c) . v for own columns c >= j+1, pushed to every CTA; partial v . p
    double kp = 0.0;
    const int lc0 = (j + 1 - r + CL - 1) / CL;  // first local column with global index >= j+1
    for (int lc = lc0 + warp; lc < ncol; lc += nwarp) {
      const int c = r + lc * CL;
      const double* a = cols + (size_t)lc * n;
      double s = 0.0;
      for (int i = j + 1 + lane; i < n; i += 32) s = fma(a[i], v[i], s);
      s = warp_sum(s) * tau;
      if (lane < CL) *cluster.map_shared_rank(p + c, lane) = s;
      kp = fma(s, v[c], kp);  // identical in every lane
    }
    __shared__ double red[8];
    if (lane == 0) red[warp] = kp;
    __syncthreads();
    if (threadIdx.x < CL) {
      double t = 0.0;
      for (int q = 0; q < nwarp; ++q) t += red[q];
      *cluster.map_shared_rank(kpart + r, threadIdx.x) = t;
    }
    cluster.sync();  // #1: p and the partial dots are everywhere
    double K = 0.0;
    for (int q = 0; q < CL; ++q) K += kpart[q];
    K *= 0.5 * tau;
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) w[i] = p[i] - K * v[i];
    __syncthreads();
    // (e) G(:, c) -= v w_c + w v_c on own columns; the owner of column j+1 updates it first and
    // computes the next Householder vector (lookahead) while its other warps continue.
    const int owner = (j + 1) % CL;
    const int lnext = (j + 1) / CL;
    if (r == owner && warp == 0) {
      double* a = cols + (size_t)lnext * n;
      const double wc = w[j + 1], vc = v[j + 1];
      for (int i = j + 1 + lane; i < n; i += 32) a[i] -= v[i] * wc + w[i] * vc;
      __syncwarp();
      if (lane == 0) o.d[j + 1] = a[j + 1];
      if (j + 3 < n) sytrd_householder(o, a, j + 1, vbuf, scal, slot ^ 1, lane);
    }
    for (int lc = lc0 + warp; lc < ncol; lc += nwarp) {
      if (r == owner && lc == lnext) continue;
      const int c = r + lc * CL;
      double* a = cols + (size_t)lc * n;
      const double wc = w[c], vc = v[c];
      for (int i = j + 1 + lane; i < n; i += 32) a[i] -= v[i] * wc + w[i] * vc;
    }
    cluster.sync();  // #2: columns updated, next Householder vector ready on its owner
  }
  // trailing 2 x 2 block: d[n-2] was recorded by the last step (or above for n == 2), e[n-2], d[n-1]
  if (n >= 2 && threadIdx.x == 0) {
    const int cA = n - 2, cB = n - 1;
    if (cA % CL == r) {
      const double* a = cols + (size_t)(cA / CL) * n;
      o.e[n - 2] = a[n - 1];
      o.tau[n - 2] = 0.0;
      if (n == 2) o.d[0] = a[0];
    }
    if (cB % CL == r) o.d[n - 1] = cols[(size_t)(cB / CL) * n + n - 1];
  }
  cluster.sync();  // no CTA leaves while another may still address its shared memory
}

template <int CL>
static void launch_sytrd_cl(const SytrdOp* ops, int nops, int nmax, cudaStream_t s) {
  const size_t smem = sytrd_smem_bytes(nmax, CL);
  MPSG_CUDA(cudaFuncSetAttribute(k_sytrd<CL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (CL > 8) MPSG_CUDA(cudaFuncSetAttribute(k_sytrd<CL>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nops * CL);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MPSG_CUDA(cudaLaunchKernelEx(&cfg, k_sytrd<CL>, ops));
  g_eig_launches.fetch_add(1);
}

int sytrd_cluster_size(int n) {
  if (n <= 48) return 1;
  if (n <= 96) return 2;
  if (n <= 192) return 4;
  if (n <= 320) return 8;
  return 16;
}
int sytrd_max_n() { return 640; }

void launch_sytrd(const SytrdOp* ops, int nops, int CL, int nmax, cudaStream_t s) {
  if (nops <= 0) return;
  MPSG_CHECK(nmax <= sytrd_max_n(), "sytrd: sector too large for the cluster kernel");
  switch (CL) {
    case 1: launch_sytrd_cl<1>(ops, nops, nmax, s); break;
    case 2: launch_sytrd_cl<2>(ops, nops, nmax, s); break;
    case 4: launch_sytrd_cl<4>(ops, nops, nmax, s); break;
    case 8: launch_sytrd_cl<8>(ops, nops, nmax, s); break;
    case 16: launch_sytrd_cl<16>(ops, nops, nmax, s); break;
    default: throw Err(1, "sytrd: unsupported cluster size");
  }
}

// ----------------------------------------------------------------------------- 0. scaling
// G <- 2^-p G with 2^p <= max |G| < 2^(p+1), per sector (exact): the eigenvalue stages below work on
// matrices of norm ~1 whatever the scale of the input (the division-free Sturm counts assume
// |T| <= 2^100; unnormalised tensors, e.g. a random MPS being orthonormalised, reach 2^400).  The
// eigenvalues only rank and select the vectors; the singular values are recomputed from |M v|.
__global__ void __launch_bounds__(256) k_gram_scale(const GramScaleOp* __restrict__ ops) {
  const GramScaleOp o = ops[blockIdx.x];
  double m = 0.0;
  for (int64_t e = threadIdx.x; e < (int64_t)o.n * o.n; e += blockDim.x)
    m = fmax(m, fabs(o.G[e % o.n + (e / o.n) * (int64_t)o.ld]));
  m = warp_max(m);
  __shared__ double red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  m = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
  if (!(m > 0.0) || !isfinite(m)) return;
  const double sc = ldexp(1.0, -ilogb(m));
  for (int64_t e = threadIdx.x; e < (int64_t)o.n * o.n; e += blockDim.x) o.G[e % o.n + (e / o.n) * (int64_t)o.ld] *= sc;
}
void launch_gram_scale(const GramScaleOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_gram_scale<<<nops, 256, 0, s>>>(ops);
  g_eig_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- 2. eigenvalues
// Number of eigenvalues of T below x from the sign changes of the characteristic-polynomial sequence
// p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2}, rescaled by exact powers of two (no division: an FP64
// division is a long instruction sequence on this GPU).  A zero p_i counts as a sign change.
__device__ int sturm_count(const double* d, const double* e2, int n, double x) {
  // signs compared through the bit patterns (integer pipe); magnitudes checked every 4 steps (the
  // recurrence cannot leave [2^-1000, 2^1000] from [2^-400, 2^400] in 4 steps for |T| <= 2^100)
  auto neg = [](double v) { return (int)((unsigned long long)__double_as_longlong(v) >> 63); };
  double p0 = 1.0, p1 = d[0] - x;
  if (p1 == 0.0) p1 = -DBL_MIN;
  int c = neg(p1);
  int i = 1;
  while (i < n) {
    const int iend = min(n, i + 4);
    for (; i < iend; ++i) {
      double p2 = fma(d[i] - x, p1, -e2[i - 1] * p0);
      if ((__double_as_longlong(p2) << 1) == 0) p2 = neg(p1) ? DBL_MIN : -DBL_MIN;  // zero: a sign change
      c += neg(p2) ^ neg(p1);
      p0 = p1;
      p1 = p2;
    }
    const int ex = (int)((__double_as_longlong(p1) >> 52) & 0x7ff) - 1023;  // binary exponent of p1
    if (ex > 400) { p0 *= 0x1p-400; p1 *= 0x1p-400; }
    else if (ex < -400) { p0 *= 0x1p+400; p1 *= 0x1p+400; }
  }
  return c;
}

// Per sector (one warp): e2 = e^2, Gershgorin interval, and the largest eigenvalue by multisection.
__global__ void k_tri_bounds(const TriOp* __restrict__ ops) {
  const TriOp o = ops[blockIdx.x];
  const int lane = threadIdx.x;
  const int n = o.n;
  double lo = DBL_MAX, hi = -DBL_MAX;
  for (int i = lane; i < n; i += 32) {
    const double r = (i > 0 ? fabs(o.e[i - 1]) : 0.0) + (i + 1 < n ? fabs(o.e[i]) : 0.0);
    lo = fmin(lo, o.d[i] - r);
    hi = fmax(hi, o.d[i] + r);
    if (i + 1 < n) o.e2[i] = o.e[i] * o.e[i];
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, off));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, off));
  }
  __syncwarp();
  const double tnorm = fmax(fabs(lo), fabs(hi));
  lo -= 2.0 * DBL_EPSILON * tnorm + DBL_MIN;
  hi += 2.0 * DBL_EPSILON * tnorm + DBL_MIN;
  // largest eigenvalue: count(x) <= n - 1 exactly when x <= lambda_max.  It only places the floor
  // (floor_rel * lambda_max, floor_rel = 32 n eps), so 1e-10 relative is enough: ~7 rounds of 32-point
  // multisection instead of ~11 to full precision.
  double a = lo, b = hi;
  for (int round = 0; round < 40 && b - a > 1e-10 * fmax(fabs(a), fabs(b)) + DBL_MIN; ++round) {
    const double x = a + (b - a) * (double)(lane + 1) / 33.0;
    const int c = sturm_count(o.d, o.e2, n, x);
    const unsigned below = __ballot_sync(0xffffffffu, c <= n - 1);
    const int k = below ? 31 - __clz(below) : -1;
    const double xa = k >= 0 ? __shfl_sync(0xffffffffu, x, k) : a;
    const double xb = k < 31 ? __shfl_sync(0xffffffffu, x, (k + 1) & 31) : b;
    a = xa;
    b = (k < 31) ? xb : b;
  }
  if (lane == 0) {
    o.meta[0] = 0.5 * (a + b);  // lambda_max
    o.meta[1] = DBL_MIN;
    o.meta[2] = lo;
    o.meta[3] = hi;
  }
}
void launch_tri_bounds(const TriOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_tri_bounds<<<nops, 32, 0, s>>>(ops);
  g_eig_launches.fetch_add(1);
}

// Multisection: LN lanes per (sector, eigenvalue index in descending order).  Each round the LN lanes
// count at the LN interior points of an equal division of [a, b] into LN + 1 parts, and the interval
// shrinks to the part that holds the eigenvalue (log2(LN + 1) bits per round, LN times the warps of
// one-thread bisection, whose single dependent chain per thread left the SMs with one warp each).
// Eigenvalues at or below the sector's floor (floor_rel * lambda_max) are not computed: W holds -1
// there.  W[k] = k-th largest eigenvalue.  LN divides 32, so a lane group never spans two warps.
constexpr int kBisectLanes = 4;
// Eigenvalues at or below 1e-30 (singular values at or below 1e-15) are never computed: the split's
// truncation drops every singular value <= 1e-15, and a zero or denormal-scale sector would otherwise
// give inverse iteration reciprocal pivots that overflow.
constexpr double kAbsFloor = 1e-30;

template <int LN>
__global__ void k_tri_bisect(const TriOp* __restrict__ ops, const int* __restrict__ op_of, const int* __restrict__ k_of,
                             int nthreads) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = gt / LN, g = gt % LN;
  if (t >= nthreads) return;  // whole lane groups leave together (blockDim.x is a multiple of LN)
  const int lane = threadIdx.x & 31;
  const unsigned gmask = ((1u << LN) - 1u) << (lane & ~(LN - 1));
  const TriOp o = ops[op_of[t]];
  const int k = k_of[t];  // 0 = largest
  const int n = o.n;
  const double lmax = o.meta[0];
  const double floor_v = fmax(o.floor_rel * fmax(lmax, 0.0), kAbsFloor);
  const int m = n - 1 - k;  // the eigenvalue with exactly m smaller ones
  if (sturm_count(o.d, o.e2, n, floor_v) > m) {  // same answer in every lane of the group
    if (g == 0) o.W[k] = -1.0;
    return;
  }
  const double frac = (double)(g + 1) / (double)(LN + 1);
  double a = floor_v, b = o.meta[3];
  for (int it = 0; it < 100 && b - a > 2.0 * DBL_EPSILON * fmax(fabs(a), fabs(b)) + DBL_MIN; ++it) {
    const double x = fma(b - a, frac, a);
    const unsigned above = (__ballot_sync(gmask, sturm_count(o.d, o.e2, n, x) > m) >> (lane & ~(LN - 1))) &
                           ((1u << LN) - 1u);
    // the counts grow with x: the first point above the eigenvalue bounds it from above, the one
    // before it from below
    const int first = above ? __ffs(above) - 1 : LN;
    const double xb = __shfl_sync(gmask, x, first < LN ? first : LN - 1, LN);
    const double xa = __shfl_sync(gmask, x, first > 0 ? first - 1 : 0, LN);
    if (first < LN) b = xb;
    if (first > 0) a = xa;
  }
  if (g == 0) o.W[k] = 0.5 * (a + b);
}
void launch_tri_bisect(const TriOp* ops, const int* op_of, const int* k_of, int nthreads, double,
                       cudaStream_t s) {
  if (nthreads <= 0) return;
  const int64_t lanes = (int64_t)kBisectLanes * nthreads;
  k_tri_bisect<kBisectLanes><<<(unsigned)((lanes + 127) / 128), 128, 0, s>>>(ops, op_of, k_of, nthreads);
  g_eig_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- 3. eigenvectors of T
// Eigenvectors of T by inverse iteration: three iterations from a deterministic pseudo-random start
// with one LU of T - lambda I.  Eigenvalues that bisection cannot tell apart (within kClusterGap *
// ||T|| of their predecessor in descending order, a few eps) form a cluster, handled in groups of at
// most kMaxGroup consecutive members: the thread of a group's first member computes the group's
// vectors one after another and orthogonalises each iterate against the group's earlier vectors
// (modified Gram-Schmidt, as LAPACK's dstein does), so that degenerate eigenvalues do not yield the
// same vector twice; the group's other threads return.  The caller still re-orthonormalises the
// eigenvector matrix (CholeskyQR).  Z column k receives the vector of W[k]; columns below the floor
// are zero.
constexpr double kClusterGap = 16.0 * DBL_EPSILON;
constexpr int kMaxGroup = 32;

__device__ __forceinline__ bool same_cluster(const TriOp& o, int j, double tnorm) {  // W[j - 1] ~ W[j]
  return j > 0 && o.W[j - 1] >= 0.0 && o.W[j] >= 0.0 && o.W[j - 1] - o.W[j] <= kClusterGap * tnorm;
}

__device__ void invit_one(const TriOp& o, int k, int k_first, double tnorm, double* z, double* base) {
  const int n = o.n;
  double *u0 = base, *u1 = base + n, *u2 = base + 2 * n, *mul = base + 3 * n;
  unsigned char* piv = (unsigned char*)(base + 4 * n);
  for (int i = 0; i < n; ++i) z[i] = hash_unit(k, i);
  tri_shift_factor(o.d, o.e, n, o.W[k], tnorm, u0, u1, u2, mul, piv);
  for (int it = 0; it < 3; ++it) {
    tri_shift_solve(n, z, u0, u1, u2, mul, piv);
    for (int j = k - 1; j >= k_first; --j) {  // the group's earlier vectors (already final)
      const double* y = o.Z + (int64_t)j * o.ldz;
      double dot = 0.0;
      for (int i = 0; i < n; ++i) dot = fma(y[i], z[i], dot);
      for (int i = 0; i < n; ++i) z[i] = fma(-dot, y[i], z[i]);
    }
    double amax = 0.0;
    for (int i = 0; i < n; ++i) amax = fmax(amax, fabs(z[i]));
    const double inv = amax > 0.0 ? 1.0 / amax : 0.0;  // keep the iterate in range
    for (int i = 0; i < n; ++i) z[i] *= inv;
  }
  double nrm = 0.0;
  for (int i = 0; i < n; ++i) nrm = fma(z[i], z[i], nrm);
  const double inv = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
  for (int i = 0; i < n; ++i) z[i] *= inv;
}

__global__ void k_tri_invit(const TriOp* __restrict__ ops, const int* __restrict__ op_of,
                            const int* __restrict__ k_of, int nthreads, double, double* scratch,
                            const int64_t* __restrict__ scratch_off) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nthreads) return;
  const TriOp o = ops[op_of[t]];
  const int n = o.n;
  const int k = k_of[t];
  const double tnorm = fmax(fabs(o.meta[2]), fabs(o.meta[3]));
  double* z = o.Z + (int64_t)k * o.ldz;
  if (o.W[k] < 0.0) {  // below the floor
    for (int i = 0; i < n; ++i) z[i] = 0.0;
    return;
  }
  int c0 = k;  // first member of the cluster
  while (same_cluster(o, c0, tnorm)) --c0;
  if ((k - c0) % kMaxGroup != 0) return;  // computed by the first thread of its group
  double* base = scratch + scratch_off[t];
  for (int m = k; m < n && m < k + kMaxGroup && (m == k || same_cluster(o, m, tnorm)); ++m)
    invit_one(o, m, k, tnorm, o.Z + (int64_t)m * o.ldz, base);
}
void launch_tri_invit(const TriOp* ops, const int* op_of, const int* k_of, int nthreads, double gap_rel,
                      double* scratch, const int64_t* scratch_off, cudaStream_t s) {
  if (nthreads <= 0) return;
  k_tri_invit<<<(nthreads + 31) / 32, 32, 0, s>>>(ops, op_of, k_of, nthreads, gap_rel, scratch, scratch_off);
  g_eig_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- 4. back-transformation
// Z <- H_0 H_1 ... H_{n-3} Z with H_j = I - tau_j v_j v_j^T (v_j: 1 at row j+1, reflector below it in
// column j of A).  One CTA per block of 8 columns of Z (first k columns only), one warp per column.
__global__ void __launch_bounds__(256) k_ormtr(const OrmtrOp* __restrict__ ops) {
  const OrmtrOp o = ops[blockIdx.x];
  const int n = o.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  extern __shared__ double zs[];  // 8 columns x n
  const int c = o.c0 + warp;
  const bool active = c < o.c1 && o.W[c] >= 0.0;  // eigenvectors below the floor are zero
  double* z = zs + (size_t)warp * n;
  if (active)
    for (int i = lane; i < n; i += 32) z[i] = o.Z[i + (int64_t)c * o.ldz];
  if (!active) return;  // no block-wide synchronisation below: each warp owns its column
  for (int j = n - 3; j >= 0; --j) {
    const double tau = o.tau[j];
    if (tau == 0.0) continue;
    const double* v = o.A + (int64_t)j * o.lda;  // v[j+1] = 1 implicitly, v[i] for i >= j+2
    double s = lane == 0 ? z[j + 1] : 0.0;
    for (int i = j + 2 + lane; i < n; i += 32) s = fma(v[i], z[i], s);
    s = warp_sum(s) * tau;
    if (lane == 0) z[j + 1] -= s;
    for (int i = j + 2 + lane; i < n; i += 32) z[i] -= s * v[i];
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) o.Z[i + (int64_t)c * o.ldz] = z[i];
}
void launch_ormtr(const OrmtrOp* ops, int nops, int nmax, cudaStream_t s) {
  if (nops <= 0) return;
  const size_t smem = sizeof(double) * 8 * (size_t)nmax;
  MPSG_CUDA(cudaFuncSetAttribute(k_ormtr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_ormtr<<<nops, 256, smem, s>>>(ops);
  g_eig_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- 5. CholeskyQR
// k_chol<CL>: C = L L^T for the k x k symmetric positive definite C (lower triangle read), one cluster
// of CL CTAs per sector.  Columns are distributed in panels of kPanel columns, panel b on CTA b % CL.
// Per panel: its owner factorises the panel in shared memory (columns in sequence, CTA barriers only),
// one cluster barrier, every CTA copies the panel from the owner's shared memory (distributed shared
// memory loads by all its threads) and applies the rank-kPanel update to its own later columns.
// Output: R = L^T in the upper triangle of C (column j of R = row j of L), rdiag[j] = 1 / R_jj,
// S[j] *= R_jj when S is given; info[0] = j + 1 for the first non-positive pivot (then treated as 1).
constexpr int kPanel = 16;
static __host__ __device__ size_t chol_smem_doubles(int k, int CL) {
  const int nb = (k + kPanel - 1) / kPanel;
  const int nbl = (nb + CL - 1) / CL;  // panels per CTA (at most)
  return (size_t)nbl * kPanel * k + (size_t)kPanel * k + 8;
}
size_t chol_smem_bytes(int k, int CL) { return sizeof(double) * chol_smem_doubles(k, CL); }

// GM = true (k beyond the cluster's shared memory): the own panels are factorised and updated in place
// in C in global memory (L2-resident); only the copied panel lives in shared memory.
template <int CL, bool GM>
__global__ void __launch_bounds__(256) k_chol(const CholQROp* __restrict__ ops) {
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const CholQROp o = ops[blockIdx.x / CL];
  const int k = o.k;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  extern __shared__ double sm[];
  const int nb = (k + kPanel - 1) / kPanel;
  const int nbl_max = (nb + CL - 1) / CL;
  double* cols = sm;                                        // local panel p (global panel r + p*CL): kPanel x k
  double* pbuf = GM ? sm : cols + (size_t)nbl_max * kPanel * k;  // current panel, copied from its owner
  // column jj of local panel lp (GM: the column of C itself; padding columns past k are never used
  // in GM mode, which works on the k real columns only)
  auto colptr = [&](double* base, int lp, int jj) -> double* {
    if (GM) return o.C + (int64_t)((r + lp * CL) * kPanel + jj) * o.ld;
    return base + ((size_t)lp * kPanel + jj) * k;
  };
  const int nbl = (nb - r + CL - 1) / CL;
  if (!GM)
    for (int lp = 0; lp < nbl; ++lp)
      for (int jj = warp; jj < kPanel; jj += nwarp) {
        const int c = (r + lp * CL) * kPanel + jj;
        double* dst = colptr(cols, lp, jj);
        for (int i = lane; i < k; i += 32) dst[i] = c < k ? o.C[i + (int64_t)c * o.ld] : 0.0;
      }
  cluster.sync();
  for (int b = 0; b < nb; ++b) {
    const int j0 = b * kPanel, jn = min(kPanel, k - j0);
    const int owner = b % CL;
    if (r == owner) {  // factorise panel b (its columns already hold all earlier panels' updates)
      const int lp = b / CL;
      for (int jj = 0; jj < jn; ++jj) {
        double* a = colptr(cols, lp, jj);
        const int j = j0 + jj;
        __shared__ double ljj_s;
        if (tid == 0) {
          double piv = a[j];
          if (!(piv > 0.0)) {
            atomicCAS(o.info, 0, j + 1);
            piv = 1.0;
          }
          const double l = sqrt(piv);
          ljj_s = l;
          o.rdiag[j] = 1.0 / l;
          if (o.S) o.S[j] *= l;
        }
        __syncthreads();
        const double l = ljj_s, inv = 1.0 / l;
        for (int i = j + tid; i < k; i += blockDim.x) a[i] = (i == j) ? l : a[i] * inv;
        __syncthreads();
        // update the rest of the panel: column j0+q -= L(:, j) L(j0+q, j), rows >= j0+q
        for (int q = jj + 1 + warp; q < jn; q += nwarp) {
          double* c = colptr(cols, lp, q);
          const double f = a[j0 + q];
          for (int i = j0 + q + lane; i < k; i += 32) c[i] -= a[i] * f;
        }
        __syncthreads();
      }
      // R = L^T rows of this panel
      for (int jj = warp; jj < jn; jj += nwarp) {
        const double* a = colptr(cols, lp, jj);
        const int j = j0 + jj;
        for (int i = j + lane; i < k; i += 32) o.C[j + (int64_t)i * o.ld] = a[i];
      }
    }
    cluster.sync();  // panel b factorised
    if (b + 1 == nb) break;
    // copy panel b (rows >= j0 + jn) from the owner's shared memory (GM: from C)
    if (GM) {
      for (int idx = tid; idx < jn * k; idx += blockDim.x) {
        const int i = idx % k, q = idx / k;
        if (i >= j0 + jn) pbuf[idx] = o.C[i + (int64_t)(j0 + q) * o.ld];
      }
    } else {
      const double* src = cluster.map_shared_rank(colptr(cols, b / CL, 0), owner);
      for (int idx = tid; idx < jn * k; idx += blockDim.x) {
        const int i = idx % k;
        if (i >= j0 + jn) pbuf[idx] = src[idx];
      }
    }
    __syncthreads();
    // rank-jn update of the own columns of later panels: C(i, c) -= sum_jj L(i, jj) L(c, jj), i >= c
    for (int lp = 0; lp < nbl; ++lp) {
      const int gb = r + lp * CL;
      if (gb <= b) continue;
      for (int jj = warp; jj < kPanel; jj += nwarp) {
        const int c = gb * kPanel + jj;
        if (c >= k) break;
        double* a = colptr(cols, lp, jj);
        double f[kPanel];
#pragma unroll
        for (int q = 0; q < kPanel; ++q) f[q] = q < jn ? pbuf[(size_t)q * k + c] : 0.0;
        for (int i = c + lane; i < k; i += 32) {
          double acc = a[i];
#pragma unroll
          for (int q = 0; q < kPanel; ++q) acc = fma(-pbuf[(size_t)q * k + i], f[q], acc);
          a[i] = acc;
        }
      }
    }
    __syncthreads();  // own columns updated before this CTA factorises or copies the next panel
  }
  cluster.sync();  // no CTA leaves while another may still read its panels
}

template <int CL, bool GM>
static void launch_chol_cl(const CholQROp* ops, int nops, int kmax, cudaStream_t s) {
  const size_t smem = GM ? sizeof(double) * ((size_t)kPanel * kmax + 8) : chol_smem_bytes(kmax, CL);
  MPSG_CUDA(cudaFuncSetAttribute(k_chol<CL, GM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (CL > 8) MPSG_CUDA(cudaFuncSetAttribute(k_chol<CL, GM>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nops * CL);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MPSG_CUDA(cudaLaunchKernelEx(&cfg, k_chol<CL, GM>, ops));
  g_eig_launches.fetch_add(1);
}
// the shared-memory cluster kernel up to k = 512; beyond, the global-memory variant (its copied panel,
// 16 x k doubles, has to fit in shared memory)
constexpr int kCholGlobal = 100;
int chol_max_k() { return 1600; }
int chol_cluster_size(int k) {
  // smallest cluster whose shared memory holds the panels (<= 200 KB per CTA)
  for (int CL : {1, 2, 4, 8, 16})
    if (chol_smem_bytes(k, CL) <= 200 * 1024 && (CL >= 16 || k <= 48 * CL)) return CL;
  if (chol_smem_bytes(k, 16) <= 227 * 1024) return 16;
  return kCholGlobal + 16;
}
void launch_chol(const CholQROp* ops, int nops, int code, int kmax, cudaStream_t s) {
  if (nops <= 0) return;
  MPSG_CHECK(kmax <= chol_max_k(), "Cholesky: sector wider than the cluster kernel's limit");
  switch (code) {
    case 1: launch_chol_cl<1, false>(ops, nops, kmax, s); break;
    case 2: launch_chol_cl<2, false>(ops, nops, kmax, s); break;
    case 4: launch_chol_cl<4, false>(ops, nops, kmax, s); break;
    case 8: launch_chol_cl<8, false>(ops, nops, kmax, s); break;
    case 16: launch_chol_cl<16, false>(ops, nops, kmax, s); break;
    case kCholGlobal + 16: launch_chol_cl<16, true>(ops, nops, kmax, s); break;
    default: throw Err(1, "Cholesky: unsupported cluster size");
  }
}

// X <- X R^-1 (R upper triangular from k_chol, rdiag its reciprocal diagonal) for rows [r0, r1) of
// one sector: one thread per row, forward substitution x_j = (x_j - sum_{i<j} x_i R_ij) / R_jj over a
// 32-row tile in shared memory (column-major tile: conflict-free).
__global__ void __launch_bounds__(32) k_trsm_rows(const TrsmRowsOp* __restrict__ ops) {
  const TrsmRowsOp o = ops[blockIdx.x];
  const int k = o.k, lane = threadIdx.x;
  extern __shared__ double xs[];  // k x 32
  const int row = o.r0 + lane;
  const bool act = row < o.r1;
  for (int j = 0; j < k; ++j) xs[(size_t)j * 32 + lane] = act ? o.X[row + (int64_t)j * o.ldx] : 0.0;
  __syncwarp();
  for (int j = 0; j < k; ++j) {
    const double* rc = o.R + (int64_t)j * o.ldr;  // column j of R: R(i, j), i <= j
    double a0 = xs[(size_t)j * 32 + lane], a1 = 0.0;
    int i = 0;
    for (; i + 1 < j; i += 2) {
      a0 = fma(-xs[(size_t)i * 32 + lane], rc[i], a0);
      a1 = fma(-xs[(size_t)(i + 1) * 32 + lane], rc[i + 1], a1);
    }
    if (i < j) a0 = fma(-xs[(size_t)i * 32 + lane], rc[i], a0);
    xs[(size_t)j * 32 + lane] = (a0 + a1) * o.rdiag[j];
  }
  __syncwarp();
  if (act)
    for (int j = 0; j < k; ++j) o.X[row + (int64_t)j * o.ldx] = xs[(size_t)j * 32 + lane];
}
void launch_trsm_rows(const TrsmRowsOp* ops, int nops, int kmax, cudaStream_t s) {
  if (nops <= 0) return;
  const size_t smem = sizeof(double) * 32 * (size_t)kmax;
  MPSG_CUDA(cudaFuncSetAttribute(k_trsm_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_trsm_rows<<<nops, 32, smem, s>>>(ops);
  g_eig_launches.fetch_add(1);
}

// cnt[t] = number of eigenvalues of sector t above the floor (W >= 0; W is descending).
__global__ void k_count_nonneg(const TriOp* __restrict__ ops, int* cnt) {
  const TriOp o = ops[blockIdx.x];
  __shared__ int c;
  if (threadIdx.x == 0) c = 0;
  __syncthreads();
  int mine = 0;
  for (int k = threadIdx.x; k < o.n; k += blockDim.x) mine += o.W[k] >= 0.0;
  atomicAdd(&c, mine);
  __syncthreads();
  if (threadIdx.x == 0) cnt[blockIdx.x] = c;
}
void launch_count_nonneg(const TriOp* ops, int nops, int* cnt, cudaStream_t s) {
  if (nops <= 0) return;
  k_count_nonneg<<<nops, 128, 0, s>>>(ops, cnt);
  g_eig_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- post-processing
// S[k] = sqrt(W[k]) (0 below the floor).
__global__ void k_eig_post(const EigPostOp* __restrict__ ops) {
  const EigPostOp o = ops[blockIdx.x];
  for (int k = threadIdx.x; k < o.n; k += blockDim.x) {
    const double w = o.W[k];
    o.S[k] = w > 0.0 ? sqrt(w) : 0.0;
  }
}
void launch_eig_post(const EigPostOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_eig_post<<<nops, 256, 0, s>>>(ops);
  g_eig_launches.fetch_add(1);
}

}  // namespace mpsg
