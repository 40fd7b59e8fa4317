// Batched FP64 symmetric eigensolver for the density-matrix split (sector Gram matrices G = M^T M).
//
// Stages, each one launch over all sectors:
//   1. k_sytrd<CL>   Householder tridiagonalisation Q^T G Q = T.  One thread-block cluster of CL CTAs
//                    per sector; the CTAs own the matrix columns round-robin in shared memory and
//                    exchange the Householder vector, the product p = tau G v and the partial dot
//                    products through distributed shared memory, two cluster barriers per column.
//   2. k_tri_bisect  eigenvalues of T above the resolution floor by bisection on Sturm counts
//                    (one thread per eigenvalue).
//   3. k_tri_invit   eigenvectors of T by inverse iteration with a partially pivoted tridiagonal LU;
//                    eigenvalues closer than gap_rel * lambda_max are solved by one thread in
//                    sequence and kept orthogonal to each other (modified Gram-Schmidt).
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

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// Householder vector of column j (held by the calling warp's CTA as local column `col`): alpha =
// x[j+1], the rest x[j+2..n-1].  Writes v (v[j+1] = 1) into every CTA's v buffer `slot`, tau and beta
// into every CTA's scal, the reflector (without the unit entry) into column j of the global matrix,
// tau[j] and e[j].
__device__ void sytrd_householder(cg::cluster_group& cluster, int CL, const SytrdOp& o, const double* col, int j,
                                  double* vbuf_local, double* scal_local, int slot, int lane) {
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
  for (int q = 0; q < CL; ++q) {
    double* vr = cluster.map_shared_rank(vbuf_local + (size_t)slot * n, q);
    for (int i = j + 1 + lane; i < n; i += 32) vr[i] = (i == j + 1) ? 1.0 : col[i] * scale;
    if (lane == 0) {
      double* sr = cluster.map_shared_rank(scal_local, q);
      sr[slot] = tau;
      sr[2 + slot] = beta;
    }
  }
  for (int i = j + 2 + lane; i < n; i += 32) o.A[i + (int64_t)j * o.lda] = col[i] * scale;
  if (lane == 0) {
    o.tau[j] = tau;
    o.e[j] = beta;
  }
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
  cluster.sync();  // every CTA of the cluster runs before distributed shared memory is written
  if (n >= 3 && r == 0 && warp == 0) sytrd_householder(cluster, CL, o, cols, 0, vbuf, scal, 0, lane);
  if (n >= 1 && r == 0 && threadIdx.x == 0) o.d[0] = cols[0];
  cluster.sync();
  for (int j = 0; j + 2 < n; ++j) {
    const int slot = j & 1;
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
      if (j + 3 < n) sytrd_householder(cluster, CL, o, a, j + 1, vbuf, scal, slot ^ 1, lane);
    }
    for (int lc = lc0 + warp; lc < ncol; lc += nwarp) {
      if (r == owner && lc == lnext) continue;
      const int c = r + lc * CL;
      double* a = cols + (size_t)lc * n;
      const double wc = w[c], vc = v[c];
      for (int i = j + 1 + lane; i < n; i += 32) a[i] -= v[i] * wc + w[i] * vc;
    }
    cluster.sync();  // #2: columns updated, next Householder vector everywhere
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

// ----------------------------------------------------------------------------- 2. eigenvalues
// Number of eigenvalues of T (diagonal d, off-diagonal e[0..n-2]) below x.
__device__ int sturm_count(const double* d, const double* e, int n, double x, double pivmin) {
  int c = 0;
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  c += q < 0.0;
  for (int i = 1; i < n; ++i) {
    q = d[i] - x - e[i - 1] * e[i - 1] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    c += q < 0.0;
  }
  return c;
}

// Per sector (one warp): Gershgorin interval, pivmin, and the largest eigenvalue by bisection.
__global__ void k_tri_bounds(const TriOp* __restrict__ ops) {
  const TriOp o = ops[blockIdx.x];
  const int lane = threadIdx.x;
  const int n = o.n;
  double lo = DBL_MAX, hi = -DBL_MAX, e2max = 0.0;
  for (int i = lane; i < n; i += 32) {
    const double r = (i > 0 ? fabs(o.e[i - 1]) : 0.0) + (i + 1 < n ? fabs(o.e[i]) : 0.0);
    lo = fmin(lo, o.d[i] - r);
    hi = fmax(hi, o.d[i] + r);
    if (i + 1 < n) e2max = fmax(e2max, o.e[i] * o.e[i]);
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, off));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, off));
    e2max = fmax(e2max, __shfl_xor_sync(0xffffffffu, e2max, off));
  }
  const double tnorm = fmax(fabs(lo), fabs(hi));
  const double pivmin = fmax(DBL_MIN, DBL_MIN * e2max);
  lo -= 2.0 * DBL_EPSILON * tnorm + pivmin;
  hi += 2.0 * DBL_EPSILON * tnorm + pivmin;
  // largest eigenvalue: multisection with 32 points per round (count(x) = n - 1 means x is inside the
  // last gap below lambda_max)
  double a = lo, b = hi;
  for (int round = 0; round < 40 && b - a > 2.0 * DBL_EPSILON * fmax(fabs(a), fabs(b)) + pivmin; ++round) {
    const double x = a + (b - a) * (double)(lane + 1) / 33.0;
    const int c = sturm_count(o.d, o.e, n, x, pivmin);
    const unsigned below = __ballot_sync(0xffffffffu, c <= n - 1);  // lambda_max >= x
    // highest lane whose x is still <= lambda_max
    const int k = below ? 31 - __clz(below) : -1;
    const double xa = k >= 0 ? __shfl_sync(0xffffffffu, x, k) : a;
    const double xb = k < 31 ? __shfl_sync(0xffffffffu, x, (k + 1) & 31) : b;
    a = xa;
    b = (k < 31) ? xb : b;
  }
  if (lane == 0) {
    o.meta[0] = 0.5 * (a + b);  // lambda_max
    o.meta[1] = pivmin;
    o.meta[2] = lo;
    o.meta[3] = hi;
  }
}
void launch_tri_bounds(const TriOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_tri_bounds<<<nops, 32, 0, s>>>(ops);
  g_eig_launches.fetch_add(1);
}

// One thread per (sector, eigenvalue index in descending order).  Eigenvalues at or below the sector's
// floor (floor_rel * lambda_max) are not computed: W holds -1 there.  W[k] = k-th largest eigenvalue.
__global__ void k_tri_bisect(const TriOp* __restrict__ ops, const int* __restrict__ op_of, const int* __restrict__ k_of,
                             int nthreads) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nthreads) return;
  const TriOp o = ops[op_of[t]];
  const int k = k_of[t];  // 0 = largest
  const int n = o.n;
  const double lmax = o.meta[0], pivmin = o.meta[1];
  const double floor_v = o.floor_rel * fmax(lmax, 0.0);
  // index from the bottom: the eigenvalue with exactly m = n-1-k smaller ones
  const int m = n - 1 - k;
  if (sturm_count(o.d, o.e, n, floor_v, pivmin) > m) {  // this eigenvalue is below the floor
    o.W[k] = -1.0;
    return;
  }
  double a = floor_v, b = o.meta[3];
  for (int it = 0; it < 100 && b - a > 2.0 * DBL_EPSILON * fmax(fabs(a), fabs(b)) + pivmin; ++it) {
    const double x = 0.5 * (a + b);
    if (sturm_count(o.d, o.e, n, x, pivmin) > m) b = x;
    else a = x;
  }
  o.W[k] = 0.5 * (a + b);
}
void launch_tri_bisect(const TriOp* ops, const int* op_of, const int* k_of, int nthreads, double,
                       cudaStream_t s) {
  if (nthreads <= 0) return;
  k_tri_bisect<<<(nthreads + 127) / 128, 128, 0, s>>>(ops, op_of, k_of, nthreads);
  g_eig_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- 3. eigenvectors of T
__device__ __forceinline__ double hash_unit(uint32_t a, uint32_t b) {  // deterministic value in [-1, 1)
  uint64_t z = ((uint64_t)a << 32) ^ b ^ 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// Solve (T - lam I) x = x in place with a partially pivoted LU of the tridiagonal (rows i, i+1 swapped
// when the subdiagonal entry is larger than the pivot); zero pivots are replaced by eps * tnorm.
// Scratch: u0 (pivots), u1, u2 (first and second superdiagonal of U), mul (multipliers), piv flags.
__device__ void tri_shift_solve(const double* d, const double* e, int n, double lam, double tnorm, double* x,
                                double* u0, double* u1, double* u2, double* mul, unsigned char* piv) {
  const double tiny = DBL_EPSILON * fmax(tnorm, DBL_MIN);
  // factor
  double dd = d[0] - lam, du = n > 1 ? e[0] : 0.0;
  for (int i = 0; i + 1 < n; ++i) {
    const double sub = e[i];
    const double dnext = d[i + 1] - lam;
    const double dunext = i + 2 < n ? e[i + 1] : 0.0;
    if (fabs(dd) >= fabs(sub)) {
      if (dd == 0.0) dd = tiny;
      const double l = sub / dd;
      u0[i] = dd; u1[i] = du; u2[i] = 0.0; mul[i] = l; piv[i] = 0;
      dd = dnext - l * du;
      du = dunext;
    } else {
      const double l = dd / sub;
      u0[i] = sub; u1[i] = dnext; u2[i] = dunext; mul[i] = l; piv[i] = 1;
      dd = du - l * dnext;
      du = -l * dunext;
    }
  }
  if (dd == 0.0) dd = tiny;
  u0[n - 1] = dd;
  // forward: apply the row interchanges and multipliers
  for (int i = 0; i + 1 < n; ++i) {
    if (piv[i]) {
      const double t = x[i];
      x[i] = x[i + 1];
      x[i + 1] = t - mul[i] * x[i];
    } else {
      x[i + 1] -= mul[i] * x[i];
    }
  }
  // back substitution with U (diagonal u0, superdiagonals u1, u2)
  x[n - 1] /= u0[n - 1];
  if (n >= 2) x[n - 2] = (x[n - 2] - u1[n - 2] * x[n - 1]) / u0[n - 2];
  for (int i = n - 3; i >= 0; --i) x[i] = (x[i] - u1[i] * x[i + 1] - u2[i] * x[i + 2]) / u0[i];
}

// One thread per group of consecutive eigenvalues (descending order) that lie closer than
// gap_rel * lambda_max to each other: each vector is found by three inverse iterations, and inside a
// group every iterate is orthogonalised against the group's earlier vectors.  Z column k receives the
// eigenvector of W[k] (unit norm); columns of eigenvalues below the floor are zero.
__global__ void k_tri_invit(const TriOp* __restrict__ ops, const int* __restrict__ op_of,
                            const int* __restrict__ k_of, int nthreads, double gap_rel, double* scratch,
                            const int64_t* __restrict__ scratch_off) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nthreads) return;
  const TriOp o = ops[op_of[t]];
  const int n = o.n;
  const int k0 = k_of[t];  // first eigenvalue of the candidate group
  const double lmax = o.meta[0];
  const double tnorm = fmax(fabs(o.meta[2]), fabs(o.meta[3]));
  const double gap = gap_rel * fmax(lmax, DBL_MIN);
  // a thread whose first eigenvalue continues the previous eigenvalue's group does nothing
  if (k0 > 0 && o.W[k0] >= 0.0 && o.W[k0 - 1] - o.W[k0] < gap) return;
  double* base = scratch + scratch_off[t];
  double *u0 = base, *u1 = base + n, *u2 = base + 2 * n, *mul = base + 3 * n;
  unsigned char* piv = (unsigned char*)(base + 4 * n);
  for (int k = k0; k < n; ++k) {
    if (k > k0 && !(o.W[k] >= 0.0 && o.W[k - 1] - o.W[k] < gap)) break;  // end of this group
    double* z = o.Z + (int64_t)k * o.ldz;
    const double lam = o.W[k];
    if (lam < 0.0) {  // below the floor
      for (int i = 0; i < n; ++i) z[i] = 0.0;
      continue;
    }
    for (int i = 0; i < n; ++i) z[i] = hash_unit(k, i);
    for (int it = 0; it < 3; ++it) {
      tri_shift_solve(o.d, o.e, n, lam, tnorm, z, u0, u1, u2, mul, piv);
      for (int q = k0; q < k; ++q) {  // orthogonalise against the group's earlier vectors
        const double* y = o.Z + (int64_t)q * o.ldz;
        double s = 0.0;
        for (int i = 0; i < n; ++i) s = fma(y[i], z[i], s);
        for (int i = 0; i < n; ++i) z[i] -= s * y[i];
      }
      double nrm = 0.0;
      for (int i = 0; i < n; ++i) nrm = fma(z[i], z[i], nrm);
      nrm = sqrt(nrm);
      const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
      for (int i = 0; i < n; ++i) z[i] *= inv;
    }
  }
}
void launch_tri_invit(const TriOp* ops, const int* op_of, const int* k_of, int nthreads, double gap_rel,
                      double* scratch, const int64_t* scratch_off, cudaStream_t s) {
  if (nthreads <= 0) return;
  k_tri_invit<<<(nthreads + 63) / 64, 64, 0, s>>>(ops, op_of, k_of, nthreads, gap_rel, scratch, scratch_off);
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
  const bool active = c < o.c1;
  double* z = zs + (size_t)warp * n;
  if (active)
    for (int i = lane; i < n; i += 32) z[i] = o.Z[i + (int64_t)c * o.ldz];
  for (int j = n - 3; j >= 0; --j) {
    const double tau = o.tau[j];
    if (tau == 0.0 || !active) continue;
    const double* v = o.A + (int64_t)j * o.lda;  // v[j+1] = 1 implicitly, v[i] for i >= j+2
    double s = lane == 0 ? z[j + 1] : 0.0;
    for (int i = j + 2 + lane; i < n; i += 32) s = fma(v[i], z[i], s);
    s = warp_sum(s) * tau;
    if (lane == 0) z[j + 1] -= s;
    for (int i = j + 2 + lane; i < n; i += 32) z[i] -= s * v[i];
    __syncwarp();
  }
  if (active)
    for (int i = lane; i < n; i += 32) o.Z[i + (int64_t)c * o.ldz] = z[i];
}
void launch_ormtr(const OrmtrOp* ops, int nops, int nmax, cudaStream_t s) {
  if (nops <= 0) return;
  const size_t smem = sizeof(double) * 8 * (size_t)nmax;
  MPSG_CUDA(cudaFuncSetAttribute(k_ormtr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_ormtr<<<nops, 256, smem, s>>>(ops);
  g_eig_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- post-processing
// S[k] = sqrt(W[k]) (0 below the floor); P = 1.5 I - 0.5 C for one Newton-Schulz orthonormalisation
// step of the eigenvector matrix (C = Z^T Z over the first k columns, k x k, leading dimension ld).
__global__ void k_eig_post(const EigPostOp* __restrict__ ops) {
  const EigPostOp o = ops[blockIdx.x];
  for (int k = threadIdx.x; k < o.n; k += blockDim.x) {
    const double w = o.W[k];
    o.S[k] = w > 0.0 ? sqrt(w) : 0.0;
  }
  for (int64_t idx = threadIdx.x; idx < (int64_t)o.n * o.n; idx += blockDim.x) {
    const int i = (int)(idx % o.n), j = (int)(idx / o.n);
    double* c = o.C + i + (int64_t)j * o.ldc;
    *c = (i == j ? 1.5 : 0.0) - 0.5 * *c;
  }
}
void launch_eig_post(const EigPostOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_eig_post<<<nops, 256, 0, s>>>(ops);
  g_eig_launches.fetch_add(1);
}

}  // namespace mpsg
