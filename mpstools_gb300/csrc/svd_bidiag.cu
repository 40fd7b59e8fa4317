// Batched FP64 singular value decomposition of the split's sector matrices through the bidiagonal
// form, with the global truncation decided before any singular vector is computed.  Every stage is
// one launch over all sectors of the split:
//   1. k_gebrd<CL>   Householder bidiagonalisation A = Q B P^T (Golub & Kahan; Golub & Van Loan,
//                    Matrix Computations, section 5.4.8).  One thread-block cluster of CL CTAs per
//                    sector, the columns round-robin in shared memory (in global memory for sectors
//                    too large for that); per column two or three cluster barriers: the left
//                    reflector is pulled from the CTA that owns the column, the right reflector of
//                    the row is formed from partial products every CTA pushes through distributed
//                    shared memory, each CTA summing the partials of a slice of the rows.
//   2. k_gk_setup    the Golub-Kahan tridiagonal T = [[0, B], [B^T, 0]] (rows interleaved, zero
//                    diagonal; eigenvalues +-sigma), scaled by a power of two.
//   3. k_gk_cut_*    per truncation segment: Sturm counts of all sectors at 32 points per round
//                    (log scale, one warp per sector) locate a cut x with at least chimax singular
//                    values >= x; only the values above the cut can be kept, and only they are computed.
//   4. k_gk_bisect   those singular values by multisection on Sturm counts of T.
//   5. k_gk_invit    eigenvectors of T for the values the truncation keeps (inverse iteration).
//   6. k_gk_vectors  (v, u) halves of each eigenvector: right and left singular vectors of B.
//   7. k_apply_refl  U = Q [U_B; 0] and V = P V_B with the stored reflectors.
// The singular values carry the absolute accuracy of a backward-stable SVD (~eps ||A||), like the
// LAPACK dgesvd of the reference, because T is formed from B without squaring A (the Gram-matrix
// route cannot resolve values below ~sqrt(eps) ||A||).  Sturm counts and inverse iteration follow
// Wilkinson, The Algebraic Eigenvalue Problem, chapter 5.  No wait in these kernels spins: cluster
// barriers are hardware barriers.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cstdlib>

#include "mpsg_internal.h"
#include "eig_common.cuh"

namespace cg = cooperative_groups;

namespace mpsg {

static std::atomic<int64_t> g_bd_launches{0};
int64_t bidiag_launch_count() { return g_bd_launches.load(); }

// ----------------------------------------------------------------------------- 1. bidiagonalisation
// Shared memory of one CTA: own columns (ncol x m) | v (m) | zp (m) | cb (m) | z (m) | ub (ncol) | scal (16)
static __host__ __device__ size_t gebrd_smem_doubles(int m, int n, int CL) {
  const int ncol = (n + CL - 1) / CL;
  return (size_t)ncol * m + 4 * (size_t)m + (size_t)ncol + 16;
}
static size_t gebrd_smem_bytes(int m, int n, int CL) { return sizeof(double) * gebrd_smem_doubles(m, n, CL); }
// the global-memory variant keeps only the reduction buffers in shared memory
static __host__ __device__ size_t gebrd_gm_smem_doubles(int m, int n, int CL) {
  return 4 * (size_t)m + (size_t)((n + CL - 1) / CL) + 16;
}
constexpr int kGebrdGlobal = 100;  // cluster-size code offset of the global-memory variant

// Left reflector of column j (`col`, rows j..m-1 current): v (v[j] = 1) into the CTA's v buffer, tau
// into scal[0]; with store (the owner of the column) the reflector's tail into column j of A,
// tauq[j] and d[j] = beta.  Every CTA computes the reflector from the same values with the same
// operations, so the copies agree bit for bit.
__device__ void gebrd_left(const GebrdOp& o, const double* col, int j, double* v, double* scal, int lane,
                           bool store = true) {
  const int m = o.m;
  double s2a = 0.0, s2b = 0.0;
  int i0 = j + 1 + lane;
  for (; i0 + 32 < m; i0 += 64) {
    s2a = fma(col[i0], col[i0], s2a);
    s2b = fma(col[i0 + 32], col[i0 + 32], s2b);
  }
  if (i0 < m) s2a = fma(col[i0], col[i0], s2a);
  const double s2 = warp_sum(s2a + s2b);
  const double alpha = col[j];
  double tau = 0.0, beta = alpha, scale = 0.0;
  if (s2 > 0.0) {
    beta = -copysign(sqrt(fma(alpha, alpha, s2)), alpha);
    tau = (beta - alpha) / beta;
    scale = 1.0 / (alpha - beta);
  }
  for (int i = j + lane; i < m; i += 32) {
    const double x = (i == j) ? 1.0 : col[i] * scale;
    v[i] = x;
    if (store && i > j) o.A[i + (int64_t)j * o.lda] = x;
  }
  if (lane == 0) {
    scal[0] = tau;
    if (store) {
      o.tauq[j] = tau;
      o.d[j] = beta;
    }
  }
}

// Column passes shared by the bidiagonalisation kernels.  The CTA's own columns are cols + lc * ldc,
// lc < ncol; lc1 / lc2 = first own column at or past global column j + 1 / j + 2.
// (a) A(j:m, c) -= v tau (v^T A(j:m, c)) on the own columns lc >= lc1, one warp per column; four
//     independent loads and partial sums in flight per lane (the global-memory variants wait on L2
//     latency otherwise).
__device__ __forceinline__ void gebrd_apply_left(double* cols, int64_t ldc, const double* v, double tau, int j, int m,
                                                 int lc1, int ncol, int warp, int nwarp, int lane) {
  for (int lc = lc1 + warp; lc < ncol; lc += nwarp) {
    double* a = cols + (size_t)lc * ldc;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int i = j + lane;
    for (; i + 96 < m; i += 128) {
      s0 = fma(v[i], a[i], s0);
      s1 = fma(v[i + 32], a[i + 32], s1);
      s2 = fma(v[i + 64], a[i + 64], s2);
      s3 = fma(v[i + 96], a[i + 96], s3);
    }
    for (; i < m; i += 32) s0 = fma(v[i], a[i], s0);
    const double w = warp_sum((s0 + s1) + (s2 + s3)) * tau;
    i = j + lane;
    for (; i + 96 < m; i += 128) {
      const double a0 = a[i], a1 = a[i + 32], a2 = a[i + 64], a3 = a[i + 96];
      a[i] = fma(-v[i], w, a0);
      a[i + 32] = fma(-v[i + 32], w, a1);
      a[i + 64] = fma(-v[i + 64], w, a2);
      a[i + 96] = fma(-v[i + 96], w, a3);
    }
    for (; i < m; i += 32) a[i] = fma(-v[i], w, a[i]);
  }
}
// (b) zp_i = sum over the own columns lc >= lc2 of A(i, c) A(j, c), rows j < i < m, thread t of nt
//     (four independent partial sums per row)
__device__ __forceinline__ void gebrd_row_partials(const double* cols, int64_t ldc, double* zp, int j, int m, int lc2,
                                                   int ncol, int t, int nt) {
  for (int i = j + 1 + t; i < m; i += nt) {
    double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0, acc3 = 0.0;
    int lc = lc2;
    for (; lc + 3 < ncol; lc += 4) {
      acc0 = fma(cols[(size_t)lc * ldc + i], cols[(size_t)lc * ldc + j], acc0);
      acc1 = fma(cols[(size_t)(lc + 1) * ldc + i], cols[(size_t)(lc + 1) * ldc + j], acc1);
      acc2 = fma(cols[(size_t)(lc + 2) * ldc + i], cols[(size_t)(lc + 2) * ldc + j], acc2);
      acc3 = fma(cols[(size_t)(lc + 3) * ldc + i], cols[(size_t)(lc + 3) * ldc + j], acc3);
    }
    for (; lc < ncol; ++lc) acc0 = fma(cols[(size_t)lc * ldc + i], cols[(size_t)lc * ldc + j], acc0);
    zp[i] = (acc0 + acc1) + (acc2 + acc3);
  }
}
// the own part of |A(j, c >= j+2)|^2 (one warp; the sum is in every lane)
__device__ __forceinline__ double gebrd_row_norm_partial(const double* cols, int64_t ldc, int j, int lc2, int ncol,
                                                         int lane) {
  double s = 0.0;
  for (int lc = lc2 + lane; lc < ncol; lc += 32) {
    const double x = cols[(size_t)lc * ldc + j];
    s = fma(x, x, s);
  }
  return warp_sum(s);
}
// (d) A(i, c) -= z_i u_c for rows j < i < m on the own columns lc >= lc2, thread t of nt (four loads
//     in flight before the stores)
__device__ __forceinline__ void gebrd_apply_right(double* cols, int64_t ldc, const double* z, const double* ub, int j,
                                                  int m, int lc2, int ncol, int t, int nt) {
  for (int i = j + 1 + t; i < m; i += nt) {
    const double zi = z[i];
    int lc = lc2;
    for (; lc + 3 < ncol; lc += 4) {
      double* a = cols + (size_t)lc * ldc + i;
      const double a0 = a[0], a1 = a[ldc], a2 = a[2 * ldc], a3 = a[3 * ldc];
      a[0] = fma(-zi, ub[lc], a0);
      a[ldc] = fma(-zi, ub[lc + 1], a1);
      a[2 * ldc] = fma(-zi, ub[lc + 2], a2);
      a[3 * ldc] = fma(-zi, ub[lc + 3], a3);
    }
    for (; lc < ncol; ++lc) cols[(size_t)lc * ldc + i] = fma(-zi, ub[lc], cols[(size_t)lc * ldc + i]);
  }
}

// GM = false: the CTA's columns live in shared memory; GM = true (sectors too large for that): they
// are worked on in place in the sector matrix in global memory (L2-resident), only the reduction
// buffers stay in shared memory.  The arithmetic is the same.
template <int CL, bool GM, int NT>
__global__ void __launch_bounds__(NT, 1) k_gebrd(const GebrdOp* __restrict__ ops) {
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const GebrdOp o = ops[blockIdx.x / CL];
  const int m = o.m, n = o.n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  extern __shared__ double sm[];
  const int ncol_max = (n + CL - 1) / CL;
  const int ncol = (n - r + CL - 1) / CL;  // own columns: global column r + lc * CL
  const int64_t ldc = GM ? (int64_t)CL * o.lda : m;  // stride between own columns
  double* cols = GM ? o.A + (int64_t)r * o.lda : sm;
  double* v = GM ? sm : cols + (size_t)ncol_max * m;  // current left reflector
  double* zp = v + m;                       // this CTA's partial products for the right reflector
  double* cb = zp + m;                      // column j+1 after the left update (staged by its owner,
                                            // copied by the others)
  double* z = cb + m;                       // right-update coefficients
  double* ub = z + m;                       // right reflector entries of the own columns
  double* scal = ub + ncol_max;             // [0] tau, [1] partial |row|^2, [2] alpha, [3] |row|^2, [4] alpha
  if (!GM)
    for (int lc = warp; lc < ncol; lc += nwarp) {
      const int c = r + lc * CL;
      for (int i = lane; i < m; i += 32) cols[(size_t)lc * m + i] = o.A[i + (int64_t)c * o.lda];
    }
  __syncthreads();
  if (r == 0 && warp == 0) gebrd_left(o, cols, 0, v, scal, lane);
  cluster.sync();  // every CTA runs (distributed shared memory is addressable), reflector 0 exists
  if (r != 0) {    // reflector 0 from its owner; every later one is computed in every CTA
    const double* rv = cluster.map_shared_rank(v, 0);
    for (int i = tid; i < m; i += blockDim.x) v[i] = rv[i];
    if (tid == 0) scal[0] = *cluster.map_shared_rank(scal, 0);
  }
  for (int j = 0; j + 1 < n; ++j) {
    __syncthreads();  // left reflector j in v, scal[0]
    // (a) left reflector j applied to the own columns c > j
    const double tau = scal[0];
    const int lc1 = (j + CL - r) / CL;      // first own column with c >= j + 1
    const int lc2 = (j + 1 + CL - r) / CL;  // first own column with c >= j + 2
    if (tau != 0.0) gebrd_apply_left(cols, ldc, v, tau, j, m, lc1, ncol, warp, nwarp, lane);
    __syncthreads();
    // (b) partial products of the right reflector of row j: zp_i = sum over own c >= j+2 of
    //     A(i, c) A(j, c), and the partial |A(j, c >= j+2)|^2; the owner of column j+1 stages it
    gebrd_row_partials(cols, ldc, zp, j, m, lc2, ncol, tid, blockDim.x);
    if (warp == 0) {
      const double s2 = gebrd_row_norm_partial(cols, ldc, j, lc2, ncol, lane);
      if (lane == 0) scal[1] = s2;
    }
    const int on = (j + 1) % CL, lnext = (j + 1) / CL;
    const bool own_next = (r == on);
    if (own_next) {
      const double* a = cols + (size_t)lnext * ldc;
      for (int i = j + 1 + tid; i < m; i += blockDim.x) cb[i] = a[i];
      if (tid == 0) scal[2] = a[j];
    }
    cluster.sync();  // #1: partials and column j+1 visible to the cluster
    // (c) the right reflector u (u_{j+1} = 1) zeroing A(j, j+2..): every CTA sums the partials
    if (warp == 0) {
      double s = lane < CL ? *cluster.map_shared_rank(scal + 1, lane) : 0.0;
      s = warp_sum(s);
      if (lane == 0) {
        scal[3] = s;
        scal[4] = *cluster.map_shared_rank(scal + 2, on);
      }
    }
    __syncthreads();
    const double nrm2 = scal[3], alpha = scal[4];
    double taup = 0.0, beta = alpha, sc = 0.0;
    if (nrm2 > 0.0) {
      beta = -copysign(sqrt(fma(alpha, alpha, nrm2)), alpha);
      taup = (beta - alpha) / beta;
      sc = 1.0 / (alpha - beta);
    }
    // z_i = taup (A(i, j+1) + sum_{c >= j+2} A(i, c) u_c), u_c = A(j, c) sc.  With 8 or more CTAs
    // each sums the partials of one slice of the rows (the sum of CL partials per row is FP64 work
    // of the order of the update itself) and the slices are exchanged after a cluster barrier;
    // smaller clusters sum all rows in every CTA.  Either way z_i is the same fixed-order sum.
    constexpr bool kSliced = CL >= 8;
    const int zlen = m - (j + 1);
    const int zcs = kSliced ? (zlen + CL - 1) / CL : zlen;
    const double* rcb = cluster.map_shared_rank(cb, on);
    if (taup != 0.0) {
      const int i0 = j + 1 + (kSliced ? r * zcs : 0);
      const int i1 = kSliced ? min(m, i0 + zcs) : m;
      for (int i = i0 + tid; i < i1; i += blockDim.x) {
        double part[CL];  // all CL remote loads in flight before the (fixed-order) sum
#pragma unroll
        for (int q = 0; q < CL; ++q) part[q] = cluster.map_shared_rank(zp, q)[i];
        double zs = 0.0;
#pragma unroll
        for (int q = 0; q < CL; ++q) zs += part[q];
        z[i] = taup * fma(sc, zs, rcb[i]);
      }
      for (int lc = lc2 + tid; lc < ncol; lc += blockDim.x) {
        const double u = cols[(size_t)lc * ldc + j] * sc;
        ub[lc] = u;
        o.Pr[(r + lc * CL) + (int64_t)j * o.n] = u;
      }
    }
    // column j+1 of the other CTAs: a copy of the owner's (read before the barrier below, so that the
    // owner may stage the next column without a further barrier)
    if (!own_next)
      for (int i = j + 1 + tid; i < m; i += blockDim.x) cb[i] = rcb[i];
    if (kSliced) cluster.sync();  // #1b: every CTA's slice of z, every copy of column j+1 taken
    if (kSliced && taup != 0.0)
      for (int i = j + 1 + tid; i < m; i += blockDim.x) {
        const int q = (i - (j + 1)) / zcs;
        if (q != r) z[i] = cluster.map_shared_rank(z, q)[i];
      }
    if (!kSliced) cluster.sync();  // every copy of column j+1 taken
    __syncthreads();
    // (d) A(i, c) -= z_i u_c for i > j on the own columns c >= j+2; warp 0 of every CTA forms column
    //     j+1 after the update (the owner in place) and left reflector j+1 from it (the owner stores it)
    if (warp == 0) {
      double* a = own_next ? cols + (size_t)lnext * ldc : cb;
      if (taup != 0.0)
        for (int i = j + 1 + lane; i < m; i += 32) a[i] -= z[i];
      __syncwarp();
      if (own_next && lane == 0) {
        o.e[j] = beta;
        o.taup[j] = taup;
      }
      gebrd_left(o, a, j + 1, v, scal, lane, own_next);
    }
    if (taup != 0.0 && tid >= 32) gebrd_apply_right(cols, ldc, z, ub, j, m, lc2, ncol, tid - 32, (int)blockDim.x - 32);
  }
  cluster.sync();  // no CTA leaves while the others may still read its shared memory
}


// ----------------------------------------------------------------------------- 1b. two-cluster sectors
// Sectors too large for one cluster's shared memory run in global memory; the largest of them are
// spread over G clusters of CL CTAs (CTA R = g CL + r owns the columns c = R mod G CL), so that
// G CL SMs share their FP64 work.  Per column: the left update, each CTA's partial products of the
// right reflector into global memory, one barrier over the G clusters, each cluster sums the
// partials of its rows (one slice per CTA, exchanged through distributed shared memory), the right
// update, and in every CTA the next left reflector from the copy of the next column.  The barriers count on a per-sector counter in global memory; every
// wait is bounded (~2 s of globaltimer), after which the CTA records *err and all CTAs of its
// cluster leave together (the other clusters' waits then expire as well); the host redoes those
// sectors on one cluster from the copy of their matrices.  All G clusters of a sector must be
// resident together: the host launches these sectors alone on their stream, at most as many as
// cudaOccupancyMaxActiveClusters allows, 2 x 16 CTAs each.
__device__ __forceinline__ uint64_t gebrd_globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned gebrd_ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// Barrier of the NC = G CL CTAs of a sector; false (in every CTA of the cluster) once a wait expired.
template <int CL>
__device__ bool gebrd_sector_sync(cg::cluster_group& cluster, unsigned* ctr, unsigned target, int* err, int* flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // this CTA's global writes (ordered before by the CTA barrier) are visible
    atomicAdd(ctr, 1u);
    const uint64_t t0 = gebrd_globaltimer();
    bool ok = true;
    while (gebrd_ld_acquire(ctr) < target) {
      if (gebrd_globaltimer() - t0 > 2000000000ull) {
        ok = false;
        break;
      }
      __nanosleep(32);
    }
    if (!ok) {
      atomicExch(err, 1);
      for (int q = 0; q < CL; ++q) *cluster.map_shared_rank(flag, q) = 1;
    }
    __threadfence();
  }
  cluster.sync();
  return flag[0] == 0;
}
size_t gebrd_mc_xg_doubles(int m, int clusters) {
  const size_t nc = (size_t)16 * clusters;
  return 2 * (nc * (size_t)m + nc + (size_t)m + 8);  // two sets: partials | row norms | column j+1 | alpha
}
// shared memory of a CTA: v (m) | z (m) | cb (m) | ub (ncol) | scal (8) | flag
size_t gebrd_mc_smem(int m, int n, int clusters) {
  const int NC = 16 * clusters;
  return sizeof(double) * (3 * (size_t)m + (size_t)((n + NC - 1) / NC) + 8) + 16;
}

template <int CL, int G, int NT>
__global__ void __launch_bounds__(NT, 1) k_gebrd_mc(const GebrdOp* __restrict__ ops) {
  constexpr int NC = CL * G;
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int g = (int)(blockIdx.x / CL) % G;
  const int R = g * CL + r;
  const GebrdOp o = ops[blockIdx.x / NC];
  const int m = o.m, n = o.n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = NT / 32;
  extern __shared__ double sm[];
  const int ncol_max = (n + NC - 1) / NC;
  const int ncol = (n - R + NC - 1) / NC;  // own columns: global column R + lc * NC
  const int64_t ldc = (int64_t)NC * o.lda;
  double* cols = o.A + (int64_t)R * o.lda;
  double* v = sm;                // current left reflector
  double* z = v + m;             // right-update coefficients
  double* cb = z + m;            // column j+1 (copy)
  double* ub = cb + m;           // right reflector entries of the own columns
  double* scal = ub + ncol_max;  // [0] tau, [3] |row|^2, [4] alpha
  int* flag = (int*)(scal + 8);
  // exchange buffers, two sets used in alternate columns (a CTA can be at most one column ahead of
  // another's reads): partial products (NC x m) | row-norm partials (NC) | column j+1 (m) | alpha
  const size_t xset = (size_t)NC * m + NC + m + 8;
  unsigned nb = 0;
  if (tid == 0) flag[0] = 0;
  // every CTA of the cluster runs and has cleared its flag before a peer may set it (a wait that
  // expires writes the flags of the whole cluster through distributed shared memory)
  cluster.sync();
  if (R == 0 && warp == 0) gebrd_left(o, cols, 0, v, scal, lane);
  if (!gebrd_sector_sync<CL>(cluster, o.ctr, NC * ++nb, o.err, flag)) return;
  if (R != 0) {  // reflector 0 from the sector matrix; every later one is computed in every CTA
    for (int i = tid; i < m; i += NT) v[i] = i == 0 ? 1.0 : __ldcg(o.A + i);
    if (tid == 0) scal[0] = __ldcg(o.tauq);
  }
  for (int j = 0; j + 1 < n; ++j) {
    double* zpg = o.xg + (size_t)(j & 1) * xset;
    double* nrg = zpg + (size_t)NC * m;
    double* cbuf = nrg + NC;
    double* galpha = cbuf + m;
    __syncthreads();  // left reflector j in v, scal[0]
    // (a) left reflector j applied to the own columns c > j
    const double tau = scal[0];
    const int lc1 = (j + NC - R) / NC;      // first own column with c >= j + 1
    const int lc2 = (j + 1 + NC - R) / NC;  // first own column with c >= j + 2
    if (tau != 0.0) gebrd_apply_left(cols, ldc, v, tau, j, m, lc1, ncol, warp, nwarp, lane);
    __syncthreads();
    // (b) partial products and row-norm partial of this CTA into global memory; the owner of column
    //     j+1 copies it there
    gebrd_row_partials(cols, ldc, zpg + (size_t)R * m, j, m, lc2, ncol, tid, NT);
    if (warp == 0) {
      const double s2 = gebrd_row_norm_partial(cols, ldc, j, lc2, ncol, lane);
      if (lane == 0) nrg[R] = s2;
    }
    const int on = (j + 1) % NC, lnext = (j + 1) / NC;
    const bool own_next = (R == on);
    if (own_next) {
      const double* a = cols + (size_t)lnext * ldc;
      for (int i = j + 1 + tid; i < m; i += NT) cbuf[i] = a[i];
      if (tid == 0) galpha[0] = a[j];
    }
    if (!gebrd_sector_sync<CL>(cluster, o.ctr, NC * ++nb, o.err, flag)) return;
    // (c) the right reflector from the NC partials (fixed order); z for this CTA's slice of the rows
    if (warp == 0) {
      double s2 = 0.0;
      for (int q = lane; q < NC; q += 32) s2 += __ldcg(nrg + q);
      s2 = warp_sum(s2);
      if (lane == 0) {
        scal[3] = s2;
        scal[4] = __ldcg(galpha);
      }
    }
    __syncthreads();
    const double nrm2 = scal[3], alpha = scal[4];
    double taup = 0.0, beta = alpha, sc = 0.0;
    if (nrm2 > 0.0) {
      beta = -copysign(sqrt(fma(alpha, alpha, nrm2)), alpha);
      taup = (beta - alpha) / beta;
      sc = 1.0 / (alpha - beta);
    }
    const int zlen = m - (j + 1);
    const int zcs = (zlen + CL - 1) / CL;
    if (taup != 0.0) {
      // 8 lanes per row, each summing NC / 8 partials (all loads in flight at once), then a fixed
      // butterfly over the 8 lanes: one L2 round trip per row
      constexpr int TPR = 8, PPT = NC / TPR;
      static_assert(NC % TPR == 0, "partials per lane");
      const int i0 = j + 1 + r * zcs, i1 = min(m, i0 + zcs);
      for (int k0 = warp * 32; k0 < zcs * TPR; k0 += NT) {  // whole warps per iteration
        const int k = k0 + lane;
        const int i = i0 + k / TPR, t = k % TPR;
        double zs = 0.0;
        if (i < i1) {
          double part[PPT];
#pragma unroll
          for (int u = 0; u < PPT; ++u) part[u] = __ldcg(zpg + (size_t)(t * PPT + u) * m + i);
#pragma unroll
          for (int u = 0; u < PPT; ++u) zs += part[u];
        }
        zs += __shfl_xor_sync(0xffffffffu, zs, 1);
        zs += __shfl_xor_sync(0xffffffffu, zs, 2);
        zs += __shfl_xor_sync(0xffffffffu, zs, 4);
        if (t == 0 && i < i1) z[i] = taup * fma(sc, zs, __ldcg(cbuf + i));
      }
      for (int lc = lc2 + tid; lc < ncol; lc += NT) {
        const double u = cols[(size_t)lc * ldc + j] * sc;
        ub[lc] = u;
        o.Pr[(R + lc * NC) + (int64_t)j * o.n] = u;
      }
    }
    if (!own_next)
      for (int i = j + 1 + tid; i < m; i += NT) cb[i] = __ldcg(cbuf + i);
    cluster.sync();  // the cluster's slices of z
    if (taup != 0.0)
      for (int i = j + 1 + tid; i < m; i += NT) {
        const int q = (i - (j + 1)) / zcs;
        if (q != r) z[i] = cluster.map_shared_rank(z, q)[i];
      }
    __syncthreads();
    // (d) the right update; warp 0 of every CTA forms column j+1 after it (the owner in place) and
    //     left reflector j+1 from it (the owner stores it)
    if (warp == 0) {
      double* a = own_next ? cols + (size_t)lnext * ldc : cb;
      if (taup != 0.0)
        for (int i = j + 1 + lane; i < m; i += 32) a[i] -= z[i];
      __syncwarp();
      if (own_next && lane == 0) {
        o.e[j] = beta;
        o.taup[j] = taup;
      }
      gebrd_left(o, a, j + 1, v, scal, lane, own_next);
    }
    if (taup != 0.0 && tid >= 32) gebrd_apply_right(cols, ldc, z, ub, j, m, lc2, ncol, tid - 32, NT - 32);
  }
  cluster.sync();  // no CTA leaves while the others may still read its shared memory
}

template <int CL, bool GM, int NT = 256>
static void launch_gebrd_cl(const GebrdOp* ops, int nops, size_t smem, cudaStream_t s) {
  MPSG_CUDA(cudaFuncSetAttribute(k_gebrd<CL, GM, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (CL > 8) MPSG_CUDA(cudaFuncSetAttribute(k_gebrd<CL, GM, NT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nops * CL);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MPSG_CUDA(cudaLaunchKernelEx(&cfg, k_gebrd<CL, GM, NT>, ops));
  g_bd_launches.fetch_add(1);
}

static int gebrd_cl_cap() {
  static int cap = [] {
    const char* e = std::getenv("MPSG_GEBRD_MAX_CLUSTER");
    const int v = e ? std::atoi(e) : 16;
    return (v == 1 || v == 2 || v == 4 || v == 8) ? v : 16;
  }();
  return cap;
}

static int gebrd_gm_threads() {
  static int nt = [] {
    const char* e = std::getenv("MPSG_GEBRD_GM_THREADS");
    const int v = e ? std::atoi(e) : 512;
    return (v == 256 || v == 1024) ? v : 512;
  }();
  return nt;
}
static int gebrd_sm_threads() {
  static int nt = [] {
    const char* e = std::getenv("MPSG_GEBRD_THREADS");
    const int v = e ? std::atoi(e) : 256;
    return v == 512 ? 512 : 256;
  }();
  return nt;
}

// Cluster size of a sector: CL in 1..16 for the shared-memory kernel, kGebrdGlobal + CL for the
// global-memory one (sectors whose columns do not fit the cluster's shared memory), 0 if neither fits.
int gebrd_cluster_size(int m, int n) {
  int CL = n <= 48 ? 1 : n <= 96 ? 2 : n <= 192 ? 4 : n <= 320 ? 8 : 16;
  CL = std::min(CL, gebrd_cl_cap());
  int c = CL;
  while (c <= 16 && gebrd_smem_bytes(m, n, c) > 220 * 1024) c *= 2;
  if (c <= 16) return c;
  c = std::min(16, gebrd_cl_cap());
  return sizeof(double) * gebrd_gm_smem_doubles(m, n, c) <= 220 * 1024 ? kGebrdGlobal + c : 0;
}


// Sectors whose FP64 work is worth two clusters: global-memory sectors with m n^2 above 3e8
// (about 670 x 670); MPSG_GEBRD_CLUSTERS=1 keeps every sector on one cluster.
int gebrd_mc_clusters(int m, int n) {
  static const int cap = [] {
    const char* e = std::getenv("MPSG_GEBRD_CLUSTERS");
    return e && std::atoi(e) == 1 ? 1 : 2;
  }();
  if (cap < 2 || gebrd_cl_cap() < 16) return 1;
  const int code = gebrd_cluster_size(m, n);
  if (code <= kGebrdGlobal) return 1;
  return (double)m * n * n > 3e8 ? 2 : 1;
}

template <int G>
static void launch_gebrd_mc_g(const GebrdOp* ops, int nops, size_t smem, cudaStream_t s) {
  constexpr int CL = 16, NT = 512;
  auto kern = k_gebrd_mc<CL, G, NT>;
  MPSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MPSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nops * CL * G);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // every cluster of the launch must be able to be resident at once (the clusters of a sector wait
  // on each other)
  int active = 0;
  MPSG_CUDA(cudaOccupancyMaxActiveClusters(&active, (void*)kern, &cfg));
  MPSG_CHECK(active >= nops * G, "bidiagonalisation: the two-cluster sectors cannot all be resident");
  MPSG_CUDA(cudaLaunchKernelEx(&cfg, kern, ops));
  g_bd_launches.fetch_add(1);
}

// two-cluster sectors resident at once: the active 16-CTA clusters of the kernel (one per GPC of at
// least 16 SMs) over two, at the kernel's largest shared memory
int gebrd_mc_capacity() {
  static const int cap = [] {
    auto kern = k_gebrd_mc<16, 2, 512>;
    const size_t smem = 227 * 1024;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(32);
    cfg.blockDim = dim3(512);
    cfg.dynamicSmemBytes = 16 * 1024;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int active = 0;
    if (cudaOccupancyMaxActiveClusters(&active, (void*)kern, &cfg) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return active / 2;
  }();
  return cap;
}

void launch_gebrd_mc(const GebrdOp* ops, int nops, int clusters, size_t smem, cudaStream_t s) {
  if (nops <= 0) return;
  MPSG_CHECK(clusters == 2, "bidiagonalisation: unsupported cluster count");
  launch_gebrd_mc_g<2>(ops, nops, smem, s);
}

// dynamic shared memory of one sector's CTAs (a launch takes the largest over its sectors)
size_t gebrd_smem(int m, int n, int code) {
  const bool gm = code > kGebrdGlobal;
  const int CL = gm ? code - kGebrdGlobal : code;
  return sizeof(double) * (gm ? gebrd_gm_smem_doubles(m, n, CL) : gebrd_smem_doubles(m, n, CL));
}

void launch_gebrd(const GebrdOp* ops, int nops, int code, size_t smem, cudaStream_t s) {
  if (nops <= 0) return;
  MPSG_CHECK(smem <= 227 * 1024, "bidiagonalisation: sector too large for the cluster");
  switch (code) {
    case 1: launch_gebrd_cl<1, false>(ops, nops, smem, s); break;
    case 2: launch_gebrd_cl<2, false>(ops, nops, smem, s); break;
    case 4: launch_gebrd_cl<4, false>(ops, nops, smem, s); break;
    case 8:
      if (gebrd_sm_threads() == 512) launch_gebrd_cl<8, false, 512>(ops, nops, smem, s);
      else launch_gebrd_cl<8, false>(ops, nops, smem, s);
      break;
    case 16:
      if (gebrd_sm_threads() == 512) launch_gebrd_cl<16, false, 512>(ops, nops, smem, s);
      else launch_gebrd_cl<16, false>(ops, nops, smem, s);
      break;
    case kGebrdGlobal + 1: launch_gebrd_cl<1, true>(ops, nops, smem, s); break;
    case kGebrdGlobal + 2: launch_gebrd_cl<2, true>(ops, nops, smem, s); break;
    case kGebrdGlobal + 4: launch_gebrd_cl<4, true>(ops, nops, smem, s); break;
    case kGebrdGlobal + 8: launch_gebrd_cl<8, true>(ops, nops, smem, s); break;
    case kGebrdGlobal + 16:
      // threads of the global-memory variant: more warps hide the L2 latency of its column accesses
      switch (gebrd_gm_threads()) {
        case 256: launch_gebrd_cl<16, true, 256>(ops, nops, smem, s); break;
        case 512: launch_gebrd_cl<16, true, 512>(ops, nops, smem, s); break;
        default: launch_gebrd_cl<16, true, 1024>(ops, nops, smem, s); break;
      }
      break;
    default: throw Err(1, "bidiagonalisation: unsupported cluster size");
  }
}

// ----------------------------------------------------------------------------- 2. Golub-Kahan matrix
// b = (d0, e0, d1, e1, ..., d_{n-1}) * 2^-p with 2^p <= max |b| < 2^(p+1) (exact scaling: the
// division-free Sturm counts below assume entries of order one); meta = (2^p, 2^-p, Gershgorin bound).
__global__ void __launch_bounds__(128) k_gk_setup(const GkOp* __restrict__ ops) {
  const GkOp o = ops[blockIdx.x];
  const int n = o.n, N = 2 * n;
  double mx = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    mx = fmax(mx, fabs(o.d[i]));
    if (i + 1 < n) mx = fmax(mx, fabs(o.e[i]));
  }
  mx = warp_max(mx);
  __shared__ double red[4];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  mx = fmax(fmax(red[0], red[1]), fmax(red[2], red[3]));
  if (!(mx > 0.0) || !isfinite(mx)) {  // a zero sector: no singular value above any floor
    for (int k = threadIdx.x; k + 1 < N; k += blockDim.x) o.b[k] = o.b2[k] = 0.0;
    if (threadIdx.x == 0) o.meta[0] = o.meta[1] = o.meta[2] = 0.0;
    return;
  }
  const int p = ilogb(mx);
  const double sc = ldexp(1.0, -p);
  double rs = 0.0;
  for (int k = threadIdx.x; k + 1 < N; k += blockDim.x) {
    const double x = ((k & 1) ? o.e[k >> 1] : o.d[k >> 1]) * sc;
    o.b[k] = x;
    o.b2[k] = x * x;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < N; k += blockDim.x)
    rs = fmax(rs, (k > 0 ? fabs(o.b[k - 1]) : 0.0) + (k + 1 < N ? fabs(o.b[k]) : 0.0));
  rs = warp_max(rs);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = rs;
  __syncthreads();
  if (threadIdx.x == 0) {
    rs = fmax(fmax(red[0], red[1]), fmax(red[2], red[3]));
    o.meta[0] = ldexp(1.0, p);
    o.meta[1] = sc;
    o.meta[2] = rs * (1.0 + 8.0 * DBL_EPSILON) + DBL_MIN;
  }
}
void launch_gk_setup(const GkOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_gk_setup<<<nops, 128, 0, s>>>(ops);
  g_bd_launches.fetch_add(1);
}

// Number of eigenvalues of the zero-diagonal tridiagonal matrix (squared off-diagonals b2, order N)
// below x, from the sign changes of p_i = -x p_{i-1} - b2_{i-1} p_{i-2}, rescaled by exact powers of
// two (no division).  A zero p_i counts as a sign change.
// The off-diagonals are loaded kGkBlk steps ahead of the dependent chain (one load latency per block
// instead of per step); with |b| < 2 and x <= 4 a block of 8 steps grows |p| by at most 2^24, so the
// magnitude check once per block keeps p inside [2^-1000, 2^1000].
constexpr int kGkBlk = 8;
__device__ int gk_count(const double* __restrict__ b2, int N, double x) {
  // signs from the high words (32-bit integer operations; 64-bit integer operations on the bit
  // patterns measured twice as slow); an exact zero counts as a sign change (it is replaced by the
  // smallest normal number of the sign opposite to its predecessor)
  double p0 = 1.0, p1 = -x;
  if (p1 == 0.0) p1 = -DBL_MIN;
  int s1 = (int)((unsigned)__double2hiint(p1) >> 31);
  int c = s1;
  int i = 1;
  auto step = [&](double b2v) {
    double p2 = fma(-x, p1, -b2v * p0);
    const int hi = __double2hiint(p2);
    int s2 = (int)((unsigned)hi >> 31);
    if (((hi & 0x7fffffff) | __double2loint(p2)) == 0) {
      p2 = s1 ? DBL_MIN : -DBL_MIN;
      s2 = s1 ^ 1;
    }
    c += s1 ^ s2;
    s1 = s2;
    p0 = p1;
    p1 = p2;
  };
  for (; i + kGkBlk <= N; i += kGkBlk) {
    double bb[kGkBlk];
#pragma unroll
    for (int u = 0; u < kGkBlk; ++u) bb[u] = __ldg(b2 + i - 1 + u);
#pragma unroll
    for (int u = 0; u < kGkBlk; ++u) step(bb[u]);
    const int ex = ((__double2hiint(p1) >> 20) & 0x7ff) - 1023;
    if (ex > 400 || ex < -400) {
      const double f = ex > 0 ? 0x1p-400 : 0x1p+400;
      p0 *= f;
      p1 *= f;
    }
  }
  for (; i < N; ++i) step(__ldg(b2 + i - 1));
  return c;
}
// singular values of the sector >= x (unscaled x)
__device__ __forceinline__ int gk_ge(const GkOp& o, double x) {
  if (!(o.meta[0] > 0.0)) return 0;
  const double xs = x * o.meta[1];
  if (xs >= o.meta[2]) return 0;
  return 2 * o.n - gk_count(o.b2, 2 * o.n, xs);
}

// ----------------------------------------------------------------------------- 3. the cut
// Per truncation segment a cut x such that at least chimax of the segment's singular values are >= x
// (or the floor when fewer than chimax exceed it): multisection on log2(x), 32 points per round; each
// round counts every sector at the 32 points with one warp per sector over the whole GPU (a Sturm
// count is a dependent FP64 chain; a single CTA would run all of them through one SM's FP64 pipe),
// then one thread per segment keeps the part of the interval where the count still reaches chimax.
// Four rounds narrow log2(x) by 33^4: the values computed beyond the kept chimax are those within a
// relative 1e-4 or so of the cut.
struct CutState {
  double lo, hi, xlo;
  int32_t tot[32];
  int32_t floor_tot, done, pad;
};
constexpr int kCutRounds = 4;

__global__ void k_gk_cut_init(const GkOp* __restrict__ ops, const int32_t* __restrict__ seg, double floor_abs,
                              CutState* st) {
  const int c = blockIdx.x, s0 = seg[c], s1 = seg[c + 1];
  double hb = 0.0;
  for (int q = s0 + threadIdx.x; q < s1; q += blockDim.x) hb = fmax(hb, ops[q].meta[2] * ops[q].meta[0]);
  hb = warp_max(hb);
  __shared__ double red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = hb;
  __syncthreads();
  if (threadIdx.x == 0) {
    double h = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) h = fmax(h, red[w]);
    CutState& x = st[c];
    x.lo = log2(floor_abs);
    x.hi = h > 0.0 ? log2(h) + 1.0 : x.lo;
    x.xlo = floor_abs;
    x.floor_tot = 0;
    x.done = h > floor_abs ? 0 : 1;
    for (int i = 0; i < 32; ++i) x.tot[i] = 0;
  }
}
// singular values >= the floor, per segment (one thread per sector)
__global__ void k_gk_cut_floor(const GkOp* __restrict__ ops, const int32_t* __restrict__ op_seg, int nops,
                               double floor_abs, CutState* st) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nops) return;
  const int c = gk_ge(ops[q], floor_abs);
  if (c) atomicAdd(&st[op_seg[q]].floor_tot, c);
}
// one warp per sector: lane i counts at the i-th of 32 interior points of the segment's interval
__global__ void k_gk_cut_round(const GkOp* __restrict__ ops, const int32_t* __restrict__ op_seg, CutState* st) {
  const int q = blockIdx.x, lane = threadIdx.x;
  CutState& x = st[op_seg[q]];
  if (x.done) return;
  const double lo = x.lo, hi = x.hi;
  const int c = gk_ge(ops[q], exp2(lo + (hi - lo) * (double)(lane + 1) / 33.0));
  if (c) atomicAdd(&x.tot[lane], c);
}
// one thread per segment: after the floor count (round < 0) or a multisection round
__global__ void k_gk_cut_pick(CutState* st, int nseg, int chimax, int round) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nseg) return;
  CutState& x = st[c];
  if (x.done) return;
  if (round < 0) {
    if (x.floor_tot <= chimax) x.done = 1;  // every value above the floor can be kept
    return;
  }
  int best = -1;  // the counts fall with x
  for (int i = 0; i < 32; ++i)
    if (x.tot[i] >= chimax) best = i;
  const double lo = x.lo, hi = x.hi;
  double nlo = lo, nhi = lo + (hi - lo) * 1.0 / 33.0;
  if (best >= 0) {
    nlo = lo + (hi - lo) * (double)(best + 1) / 33.0;
    nhi = best < 31 ? lo + (hi - lo) * (double)(best + 2) / 33.0 : hi;
  }
  x.lo = nlo;
  x.hi = nhi;
  for (int i = 0; i < 32; ++i) x.tot[i] = 0;
  if (round == kCutRounds - 1) x.xlo = exp2(nlo);  // total(>= 2^nlo) >= chimax by construction
}
__global__ void k_gk_cut_final(const GkOp* __restrict__ ops, int nops) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nops) return;
  *ops[q].kcomp = gk_ge(ops[q], *ops[q].xlo);
}
void launch_gk_cut(const GkOp* ops, const int32_t* seg, const int32_t* op_seg, int nops, int nseg, int chimax,
                   double floor_abs, void* state, cudaStream_t s) {
  if (nseg <= 0 || nops <= 0) return;
  CutState* st = (CutState*)state;
  k_gk_cut_init<<<nseg, 256, 0, s>>>(ops, seg, floor_abs, st);
  k_gk_cut_floor<<<(nops + 63) / 64, 64, 0, s>>>(ops, op_seg, nops, floor_abs, st);
  k_gk_cut_pick<<<(nseg + 63) / 64, 64, 0, s>>>(st, nseg, chimax, -1);
  for (int r = 0; r < kCutRounds; ++r) {
    k_gk_cut_round<<<nops, 32, 0, s>>>(ops, op_seg, st);
    k_gk_cut_pick<<<(nseg + 63) / 64, 64, 0, s>>>(st, nseg, chimax, r);
  }
  k_gk_cut_final<<<(nops + 63) / 64, 64, 0, s>>>(ops, nops);
  g_bd_launches.fetch_add(4 + 2 * kCutRounds);
}
size_t gk_cut_state_bytes() { return sizeof(CutState); }
double* gk_cut_xlo(void* state, int c) { return &((CutState*)state)[c].xlo; }

// ----------------------------------------------------------------------------- 4. singular values
// LN lanes per (sector, k): the k-th largest singular value (the eigenvalue of T with exactly
// 2n - 1 - k smaller ones) for k < kcomp by multisection on [cut, Gershgorin bound]; S[k] = 0 past
// kcomp.  The LN interior points of each round are spaced evenly in the bit patterns of the bounds
// (positive doubles order like their bits): geometric spacing while the interval spans binades,
// linear within one, so every value needs about the same number of rounds however small it is.
// One warp per block: the groups spread over all SMs (the counts are dependent FP64 chains).
// S is unscaled and descending.
constexpr int kGkLanes = 8;
template <int LN>
__global__ void __launch_bounds__(32) k_gk_bisect(const GkOp* __restrict__ ops, const int32_t* __restrict__ op_of,
                                                  const int32_t* __restrict__ k_of, int nthreads) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = gt / LN, g = gt % LN;
  if (t >= nthreads) return;  // whole lane groups leave together (blockDim.x is a multiple of LN)
  const int lane = threadIdx.x & 31;
  const unsigned gmask = ((1u << LN) - 1u) << (lane & ~(LN - 1));
  const GkOp o = ops[op_of[t]];
  const int k = k_of[t];
  if (k >= *o.kcomp) {
    if (g == 0) o.S[k] = 0.0;
    return;
  }
  const int N = 2 * o.n;
  const int m = N - 1 - k;
  long long ia = __double_as_longlong(*o.xlo * o.meta[1]), ib = __double_as_longlong(o.meta[2]);
  for (int it = 0; it < 200 && ib - ia > 2; ++it) {
    // LN points strictly inside (ia, ib); once the interval holds fewer than LN + 1 patterns some of
    // them coincide (the counts stay monotone in the point, so the bracketing below still holds)
    const long long step = (ib - ia) / (LN + 1) > 0 ? (ib - ia) / (LN + 1) : 1;
    const long long ix = min(ia + step * (g + 1), ib - 1);
    const unsigned above =
        (__ballot_sync(gmask, gk_count(o.b2, N, __longlong_as_double(ix)) > m) >> (lane & ~(LN - 1))) &
        ((1u << LN) - 1u);
    // the counts grow with x: the first point above the eigenvalue bounds it from above, the one
    // before it from below
    const int first = above ? __ffs(above) - 1 : LN;
    const long long xb = __shfl_sync(gmask, ix, first < LN ? first : LN - 1, LN);
    const long long xa = __shfl_sync(gmask, ix, first > 0 ? first - 1 : 0, LN);
    if (first < LN) ib = xb;
    if (first > 0) ia = xa;
  }
  if (g == 0) o.S[k] = 0.5 * (__longlong_as_double(ia) + __longlong_as_double(ib)) * o.meta[0];
}
static int gk_lanes() {
  static const int v = [] {
    const char* e = std::getenv("MPSG_GK_LANES");
    const int x = e ? std::atoi(e) : kGkLanes;
    return (x == 2 || x == 4 || x == 8) ? x : kGkLanes;
  }();
  return v;
}
void launch_gk_bisect(const GkOp* ops, const int32_t* op_of, const int32_t* k_of, int nthreads, cudaStream_t s) {
  if (nthreads <= 0) return;
  const int ln = gk_lanes();
  const int64_t lanes = (int64_t)ln * nthreads;
  const unsigned grid = (unsigned)((lanes + 31) / 32);
  if (ln == 2) k_gk_bisect<2><<<grid, 32, 0, s>>>(ops, op_of, k_of, nthreads);
  else if (ln == 4) k_gk_bisect<4><<<grid, 32, 0, s>>>(ops, op_of, k_of, nthreads);
  else k_gk_bisect<8><<<grid, 32, 0, s>>>(ops, op_of, k_of, nthreads);
  g_bd_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- 5. eigenvectors of T
// One thread per kept singular value: three inverse iterations with one partially pivoted LU of
// T - sigma I (zero diagonal) from a deterministic pseudo-random start.  The LU factors and the iterate
// live in a scratch interleaved across the threads of the launch (element i of thread t at
// i * stride + t), so that a warp's loads of step i are contiguous; the solves carry their running
// values in registers.  Values above the noise level (4 N eps ||T||) that bisection cannot tell apart
// (within kGkClusterGap * ||T|| of their predecessor) are handled in groups of at most kGkGroup: the
// group's first thread computes its members one after another, each orthogonalised against the
// group's earlier ones (modified Gram-Schmidt).  Values at the noise level have no well-defined
// vectors: any orthonormal completion is an exact SVD to rounding, so they are computed independently
// (each iterate lies in the near-null space of T).  The vectors are re-orthonormalised afterwards
// (CholeskyQR of the singular-vector matrices).
constexpr double kGkClusterGap = 16.0 * DBL_EPSILON;
constexpr int kGkGroup = 32;

__device__ __forceinline__ bool gk_same_cluster(const GkOp& o, int j) {
  if (j <= 0) return false;
  const double tn = o.meta[2], noise = 4.0 * (2 * o.n) * DBL_EPSILON * tn;
  const double a = o.S[j - 1] * o.meta[1], b = o.S[j] * o.meta[1];
  return b > noise && a - b <= kGkClusterGap * tn;
}

// partially pivoted LU of T - lam I (zero diagonal, off-diagonals b) into strided factors: reciprocal
// pivots u0, superdiagonals u1, u2, multipliers, interchange flags (rows i, i+1 swapped when the
// subdiagonal entry is larger than the pivot; zero pivots replaced by eps * tnorm)
__device__ void gk_factor(const double* __restrict__ b, int N, double lam, double tnorm, double* __restrict__ f,
                          int64_t st) {
  double *u0 = f, *u1 = f + N * st, *u2 = f + 2 * N * st, *mul = f + 3 * N * st, *piv = f + 4 * N * st;
  const double tiny = DBL_EPSILON * fmax(tnorm, DBL_MIN);
  double dd = -lam, du = N > 1 ? b[0] : 0.0;
  for (int i = 0; i + 1 < N; ++i) {
    const double sub = b[i];
    const double dnext = -lam;
    const double dunext = i + 2 < N ? b[i + 1] : 0.0;
    const int64_t o = i * st;
    if (fabs(dd) >= fabs(sub)) {
      if (dd == 0.0) dd = tiny;
      const double inv = 1.0 / dd;
      const double l = sub * inv;
      u0[o] = inv; u1[o] = du; u2[o] = 0.0; mul[o] = l; piv[o] = 0.0;
      dd = dnext - l * du;
      du = dunext;
    } else {
      const double l = dd / sub;
      u0[o] = 1.0 / sub; u1[o] = dnext; u2[o] = dunext; mul[o] = l; piv[o] = 1.0;
      dd = du - l * dnext;
      du = -l * dunext;
    }
  }
  if (dd == 0.0) dd = tiny;
  u0[(N - 1) * st] = 1.0 / dd;
}
// Whole-vector rescaling by a power of two (exact) when an entry passed 2^166: brings the largest
// entry back to ~2^100 (the caller normalises the result).
__device__ __forceinline__ double gk_rescale_factor(double amax) { return ldexp(1.0, 100 - ilogb(amax)); }
__device__ void gk_scale_all(int N, double* x, int64_t st, double f) {
  for (int k = 0; k < N; ++k) x[k * st] *= f;
}

// x <- c (T - lam I)^-1 x with the factors of gk_factor, c > 0.  The loads of each block of kGkRows
// rows are issued before its dependent chain (the chain is what bounds this kernel: a dependent FP64
// operation takes ~64 cycles on this GPU), and the magnitude is checked once per block: partial
// pivoting keeps |mul| <= 1 (growth <= 2 per forward step) and the pivots >= eps ||T|| (growth
// <= 2^53 per backward step), so no entry leaves the range within a block.
constexpr int kGkRows = 8;
__device__ void gk_solve(int N, double* __restrict__ x, const double* __restrict__ f, int64_t st) {
  const double *u0 = f, *u1 = f + N * st, *u2 = f + 2 * N * st, *mul = f + 3 * N * st, *piv = f + 4 * N * st;
  // forward: L^-1 with the interchanges; cur = x_i as updated so far
  double cur = x[0];
  int i = 0;
  for (; i + kGkRows < N; i += kGkRows) {
    double nx[kGkRows], mm[kGkRows], pv[kGkRows];
#pragma unroll
    for (int u = 0; u < kGkRows; ++u) {
      const int64_t o = (int64_t)(i + u) * st;
      nx[u] = x[o + st];
      mm[u] = mul[o];
      pv[u] = piv[o];
    }
    double amax = 0.0;
#pragma unroll
    for (int u = 0; u < kGkRows; ++u) {
      double xi, xn;
      if (pv[u] != 0.0) {
        xi = nx[u];
        xn = cur - mm[u] * nx[u];
      } else {
        xi = cur;
        xn = nx[u] - mm[u] * cur;
      }
      x[(int64_t)(i + u) * st] = xi;
      cur = xn;
      amax = fmax(amax, fabs(xn));
    }
    if (amax > 0x1p+166) {
      const double sc = gk_rescale_factor(amax);
      gk_scale_all(N, x, st, sc);
      cur *= sc;
    }
  }
  for (; i + 1 < N; ++i) {
    const int64_t o = (int64_t)i * st;
    const double nxt = x[o + st], m = mul[o];
    double xi, xn;
    if (piv[o] != 0.0) {
      xi = nxt;
      xn = cur - m * nxt;
    } else {
      xi = cur;
      xn = nxt - m * cur;
    }
    x[o] = xi;
    cur = xn;
  }
  if (fabs(cur) > 0x1p+166) {
    const double sc = gk_rescale_factor(fabs(cur));
    gk_scale_all(N, x, st, sc);
    cur *= sc;
  }
  // backward: U^-1, x_{i+1} and x_{i+2} carried in registers
  double x1 = cur * u0[(int64_t)(N - 1) * st], x2 = 0.0;
  if (fabs(x1) > 0x1p+166) {
    const double sc = gk_rescale_factor(fabs(x1));
    gk_scale_all(N, x, st, sc);
    x1 *= sc;
  }
  x[(int64_t)(N - 1) * st] = x1;
  i = N - 2;
  for (; i - kGkRows + 1 >= 0; i -= kGkRows) {
    double xv[kGkRows], a0[kGkRows], a1[kGkRows], a2[kGkRows];
#pragma unroll
    for (int u = 0; u < kGkRows; ++u) {
      const int64_t o = (int64_t)(i - u) * st;
      xv[u] = x[o];
      a0[u] = u0[o];
      a1[u] = u1[o];
      a2[u] = u2[o];
    }
    double amax = 0.0;
#pragma unroll
    for (int u = 0; u < kGkRows; ++u) {
      const double xi = (xv[u] - a1[u] * x1 - a2[u] * x2) * a0[u];
      x[(int64_t)(i - u) * st] = xi;
      x2 = x1;
      x1 = xi;
      amax = fmax(amax, fabs(xi));
    }
    if (amax > 0x1p+166) {  // the whole vector, its register copies included
      const double sc = gk_rescale_factor(amax);
      gk_scale_all(N, x, st, sc);
      x1 *= sc;
      x2 *= sc;
    }
  }
  for (; i >= 0; --i) {
    const int64_t o = (int64_t)i * st;
    double xi = (x[o] - u1[o] * x1 - u2[o] * x2) * u0[o];
    if (fabs(xi) > 0x1p+166) {
      const double sc = gk_rescale_factor(fabs(xi));
      gk_scale_all(N, x, st, sc);
      xi *= sc;
      x1 *= sc;
    }
    x[o] = xi;
    x2 = x1;
    x1 = xi;
  }
}

// member k of a group whose first member is k_first; x: strided iterate; the result goes to Z column k
__device__ void gk_invit_one(const GkOp& o, int k, int k_first, double* x, double* f, int64_t st) {
  const int N = 2 * o.n;
  for (int i = 0; i < N; ++i) x[i * st] = hash_unit(k, i);
  gk_factor(o.b, N, o.S[k] * o.meta[1], o.meta[2], f, st);
  for (int it = 0; it < 3; ++it) {
    gk_solve(N, x, f, st);
    for (int j = k - 1; j >= k_first; --j) {
      const double* y = o.Z + (int64_t)j * o.ldz;
      double dot = 0.0;
      for (int i = 0; i < N; ++i) dot = fma(y[i], x[i * st], dot);
      for (int i = 0; i < N; ++i) x[i * st] = fma(-dot, y[i], x[i * st]);
    }
    double amax = 0.0;
    for (int i = 0; i < N; ++i) amax = fmax(amax, fabs(x[i * st]));
    const double inv = amax > 0.0 ? 1.0 / amax : 0.0;
    for (int i = 0; i < N; ++i) x[i * st] *= inv;
  }
  double nrm = 0.0;
  for (int i = 0; i < N; ++i) nrm = fma(x[i * st], x[i * st], nrm);
  const double inv = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
  double* z = o.Z + (int64_t)k * o.ldz;
  for (int i = 0; i < N; ++i) z[i] = x[i * st] * inv;
}

// threads list (op, k) for k < kept(op), kept counts from the truncation; scratch: 6 * nmax2 doubles
// per listed thread, interleaved with stride nthreads
// cpw chains per warp (lanes cpw..31 idle): a warp's FP64 instruction occupies its SMSP's FP64 pipe for
// the same time however few lanes are active, so fewer chains per warp spread them over more SMSPs
__global__ void k_gk_invit(const GkOp* __restrict__ ops, const int32_t* __restrict__ op_of,
                           const int32_t* __restrict__ k_of, const int32_t* __restrict__ kept, int nthreads, int nmax2,
                           double* scratch, int cpw) {
  const int lane = threadIdx.x & 31;
  if (lane >= cpw) return;
  const int t = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * cpw + lane;
  if (t >= nthreads) return;
  const int op = op_of[t];
  const GkOp o = ops[op];
  const int k = k_of[t], kk = kept[op];
  int c0 = k;
  while (gk_same_cluster(o, c0)) --c0;
  if ((k - c0) % kGkGroup != 0) return;  // computed by the first thread of its group
  const int64_t st = nthreads;
  double* x = scratch + t;
  double* f = scratch + (int64_t)nmax2 * st + t;
  for (int mm = k; mm < kk && mm < k + kGkGroup && (mm == k || gk_same_cluster(o, mm)); ++mm)
    gk_invit_one(o, mm, k, x, f, st);
}
void launch_gk_invit(const GkOp* ops, const int32_t* op_of, const int32_t* k_of, const int32_t* kept, int nthreads,
                     int nmax2, double* scratch, cudaStream_t s) {
  if (nthreads <= 0) return;
  static const int cpw = [] {
    const char* e = std::getenv("MPSG_INVIT_CPW");
    const int v = e ? std::atoi(e) : 8;
    return (v == 1 || v == 2 || v == 4 || v == 16 || v == 32) ? v : 8;
  }();
  const int nwarps = (nthreads + cpw - 1) / cpw;
  k_gk_invit<<<nwarps, 32, 0, s>>>(ops, op_of, k_of, kept, nthreads, nmax2, scratch, cpw);
  g_bd_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- 6. (v, u) halves
// One warp per kept vector: x = (v0, u0, v1, u1, ...) -> V(:, k) = v / |v|, U(:, k) = (u / |u|; 0).
__global__ void __launch_bounds__(256) k_gk_vectors(const GkVecOp* __restrict__ ops, int nops) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= nops) return;
  const GkVecOp o = ops[w];
  const double* x = o.Z + (int64_t)o.k * o.ldz;
  double sv = 0.0, su = 0.0;
  for (int i = lane; i < o.n; i += 32) {
    sv = fma(x[2 * i], x[2 * i], sv);
    su = fma(x[2 * i + 1], x[2 * i + 1], su);
  }
  sv = warp_sum(sv);
  su = warp_sum(su);
  const double iv = sv > 0.0 ? 1.0 / sqrt(sv) : 0.0, iu = su > 0.0 ? 1.0 / sqrt(su) : 0.0;
  double* V = o.V + (int64_t)o.k * o.ldv;
  double* U = o.U + (int64_t)o.k * o.ldu;
  for (int i = lane; i < o.n; i += 32) V[i] = x[2 * i] * iv;
  for (int i = lane; i < o.m; i += 32) U[i] = i < o.n ? x[2 * i + 1] * iu : 0.0;
}
void launch_gk_vectors(const GkVecOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_gk_vectors<<<(nops + 7) / 8, 256, 0, s>>>(ops, nops);
  g_bd_launches.fetch_add(1);
}

// ----------------------------------------------------------------------------- 7. back-transformation
// X <- H_0 H_1 ... H_{nref-1} X for columns [c0, c1): the reflectors applied last to first, one warp
// per column of X held in shared memory (8 columns per CTA).
__global__ void __launch_bounds__(256) k_apply_refl(const ReflOp* __restrict__ ops) {
  const ReflOp o = ops[blockIdx.x];
  const int len = o.len;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  extern __shared__ double xs[];  // 8 columns x len
  const int c = o.c0 + warp;
  if (c >= o.c1) return;  // no block-wide synchronisation below: each warp owns its column
  double* x = xs + (size_t)warp * len;
  double* X = o.X + (int64_t)c * o.ldx;
  for (int i = lane; i < len; i += 32) x[i] = X[i];
  __syncwarp();
  for (int j = o.nref - 1; j >= 0; --j) {
    const double tau = o.tau[j];
    if (tau == 0.0) continue;
    const int r0 = j + o.off;
    const double* rj = o.R + (int64_t)j * o.ldr;
    double s = lane == 0 ? x[r0] : 0.0;
    for (int i = r0 + 1 + lane; i < len; i += 32) s = fma(rj[i], x[i], s);
    s = warp_sum(s) * tau;
    if (lane == 0) x[r0] -= s;
    for (int i = r0 + 1 + lane; i < len; i += 32) x[i] = fma(-s, rj[i], x[i]);
    __syncwarp();
  }
  for (int i = lane; i < len; i += 32) X[i] = x[i];
}
// warps (columns) per CTA for columns of lenmax rows (at most 8, within 220 KB of shared memory)
static int apply_refl_warps(int lenmax) {
  const int w = (int)((220 * 1024) / (sizeof(double) * (size_t)std::max(lenmax, 1)));
  return std::max(1, std::min(8, w));
}
void launch_apply_refl(const ReflOp* ops, int nops, int lenmax, cudaStream_t s) {
  if (nops <= 0) return;
  const int nw = apply_refl_warps(lenmax);
  const size_t smem = sizeof(double) * nw * (size_t)std::max(lenmax, 1);
  MPSG_CHECK(smem <= 227 * 1024, "back-transformation: sector too tall for the shared-memory column block");
  MPSG_CUDA(cudaFuncSetAttribute(k_apply_refl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_apply_refl<<<nops, 32 * nw, smem, s>>>(ops);
  g_bd_launches.fetch_add(1);
}
int apply_refl_cols_per_block(int lenmax) { return apply_refl_warps(lenmax); }

// ----------------------------------------------------------------------------- complex sectors
// The complex split (TEBD) reduces each complex sector to a REAL bidiagonal: LAPACK's zgebrd
// conventions (zlarfg: beta real, H = I - tau v v^H with H^H x = beta e1; the left reflector applied
// as A <- A - conj(tau) v (v^H A), the right one built from the conjugated row and applied as
// A <- A - taup (A u) u^H).  Stages 2-6 above then run unchanged on the real bidiagonal; U = Q [U_B; 0]
// and V = P V_B are formed with the complex reflectors (k_zapply_refl).  Shared-memory cluster
// variant only (sectors that do not fit stay on the library solver).
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
// conj(a) b + c
__device__ __forceinline__ double2 zfma_c(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}
// a b + c
__device__ __forceinline__ double2 zfma(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
__device__ __forceinline__ double2 zrecip(double2 a) {
  const double d = 1.0 / fma(a.x, a.x, a.y * a.y);
  return make_double2(a.x * d, -a.y * d);
}
__device__ __forceinline__ double2 zwarp_sum(double2 a) { return make_double2(warp_sum(a.x), warp_sum(a.y)); }
// zlarfg on alpha and |x_tail|^2: beta (real), tau, scale = 1 / (alpha - beta)
__device__ __forceinline__ void zlarfg_coef(double2 alpha, double s2, double& beta, double2& tau, double2& scale) {
  beta = alpha.x;
  tau = make_double2(0.0, 0.0);
  scale = make_double2(0.0, 0.0);
  if (s2 > 0.0 || alpha.y != 0.0) {
    beta = -copysign(sqrt(fma(alpha.x, alpha.x, fma(alpha.y, alpha.y, s2))), alpha.x);
    tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
    scale = zrecip(make_double2(alpha.x - beta, alpha.y));
  }
}
// left reflector of column j (col, rows j..m-1): v, tau (scal[0]); with store the tail into A, tauq, d
__device__ void zgebrd_left(const ZGebrdOp& o, const double2* col, int j, double2* v, double2* scal, int lane,
                            bool store) {
  const int m = o.m;
  double s2 = 0.0;
  for (int i = j + 1 + lane; i < m; i += 32) s2 = fma(col[i].x, col[i].x, fma(col[i].y, col[i].y, s2));
  s2 = warp_sum(s2);
  double beta;
  double2 tau, scale;
  zlarfg_coef(col[j], s2, beta, tau, scale);
  for (int i = j + lane; i < m; i += 32) {
    const double2 x = (i == j) ? make_double2(1.0, 0.0) : zmul(col[i], scale);
    v[i] = x;
    if (store && i > j) o.A[i + (int64_t)j * o.lda] = x;
  }
  if (lane == 0) {
    scal[0] = tau;
    if (store) {
      o.tauq[j] = tau;
      o.d[j] = beta;
    }
  }
}
static __host__ __device__ size_t zgebrd_smem_elems(int m, int n, int CL) {
  const int ncol = (n + CL - 1) / CL;
  return (size_t)ncol * m + 4 * (size_t)m + (size_t)ncol + 8;
}
size_t zgebrd_smem(int m, int n, int CL) { return sizeof(double2) * zgebrd_smem_elems(m, n, CL); }
int zgebrd_cluster_size(int m, int n) {
  int CL = n <= 48 ? 1 : n <= 96 ? 2 : n <= 192 ? 4 : n <= 320 ? 8 : 16;
  while (CL <= 16 && zgebrd_smem(m, n, CL) > 220 * 1024) CL *= 2;
  return CL <= 16 ? CL : 0;
}

template <int CL>
__global__ void __launch_bounds__(256, 1) k_zgebrd(const ZGebrdOp* __restrict__ ops) {
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const ZGebrdOp o = ops[blockIdx.x / CL];
  const int m = o.m, n = o.n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  extern __shared__ double2 zsm[];
  const int ncol_max = (n + CL - 1) / CL;
  const int ncol = (n - r + CL - 1) / CL;  // own columns: global column r + lc * CL
  double2* cols = zsm;
  double2* v = cols + (size_t)ncol_max * m;
  double2* zp = v + m;
  double2* cb = zp + m;
  double2* z = cb + m;
  double2* ub = z + m;
  double2* scal = ub + ncol_max;  // [0] tau, [1] partial |row|^2 (x), [2] alpha, [3] |row|^2 (x), [4] alpha
  for (int lc = warp; lc < ncol; lc += nwarp) {
    const int c = r + lc * CL;
    for (int i = lane; i < m; i += 32) cols[(size_t)lc * m + i] = o.A[i + (int64_t)c * o.lda];
  }
  __syncthreads();
  if (r == 0 && warp == 0) zgebrd_left(o, cols, 0, v, scal, lane, true);
  cluster.sync();
  if (r != 0) {
    const double2* rv = cluster.map_shared_rank(v, 0);
    for (int i = tid; i < m; i += blockDim.x) v[i] = rv[i];
    if (tid == 0) scal[0] = *cluster.map_shared_rank(scal, 0);
  }
  for (int j = 0; j + 1 < n; ++j) {
    __syncthreads();
    // (a) A(j:m, c) -= v conj(tau) (v^H A(j:m, c)) on the own columns c > j
    const double2 tau = scal[0];
    const int lc1 = (j + CL - r) / CL, lc2 = (j + 1 + CL - r) / CL;
    if (tau.x != 0.0 || tau.y != 0.0)
      for (int lc = lc1 + warp; lc < ncol; lc += nwarp) {
        double2* a = cols + (size_t)lc * m;
        double2 s = make_double2(0.0, 0.0);
        for (int i = j + lane; i < m; i += 32) s = zfma_c(v[i], a[i], s);
        const double2 w = zmul(zconj(tau), zwarp_sum(s));
        for (int i = j + lane; i < m; i += 32) {
          const double2 t = zmul(v[i], w);
          a[i] = make_double2(a[i].x - t.x, a[i].y - t.y);
        }
      }
    __syncthreads();
    // (b) zp_i = sum over own c >= j+2 of A(i, c) conj(A(j, c)); partial |A(j, c >= j+2)|^2
    for (int i = j + 1 + tid; i < m; i += blockDim.x) {
      double2 acc = make_double2(0.0, 0.0);
      for (int lc = lc2; lc < ncol; ++lc) acc = zfma_c(cols[(size_t)lc * m + j], cols[(size_t)lc * m + i], acc);
      zp[i] = acc;
    }
    if (warp == 0) {
      double s2 = 0.0;
      for (int lc = lc2 + lane; lc < ncol; lc += 32) {
        const double2 x = cols[(size_t)lc * m + j];
        s2 = fma(x.x, x.x, fma(x.y, x.y, s2));
      }
      s2 = warp_sum(s2);
      if (lane == 0) scal[1] = make_double2(s2, 0.0);
    }
    const int on = (j + 1) % CL, lnext = (j + 1) / CL;
    const bool own_next = (r == on);
    if (own_next) {
      const double2* a = cols + (size_t)lnext * m;
      for (int i = j + 1 + tid; i < m; i += blockDim.x) cb[i] = a[i];
      if (tid == 0) scal[2] = a[j];
    }
    cluster.sync();  // #1
    // (c) right reflector from y = conj(row j): alpha' = conj(A(j, j+1)); u_c = y_c sc, z = taup A u
    if (warp == 0) {
      double s2 = lane < CL ? cluster.map_shared_rank(scal + 1, lane)->x : 0.0;
      s2 = warp_sum(s2);
      if (lane == 0) {
        scal[3] = make_double2(s2, 0.0);
        scal[4] = *cluster.map_shared_rank(scal + 2, on);
      }
    }
    __syncthreads();
    const double nrm2 = scal[3].x;
    double betap;
    double2 taup, sc;
    zlarfg_coef(zconj(scal[4]), nrm2, betap, taup, sc);
    const bool has_refl = taup.x != 0.0 || taup.y != 0.0;
    constexpr bool kSliced = CL >= 8;
    const int zlen = m - (j + 1);
    const int zcs = kSliced ? (zlen + CL - 1) / CL : zlen;
    const double2* rcb = cluster.map_shared_rank(cb, on);
    if (has_refl) {
      const int i0 = j + 1 + (kSliced ? r * zcs : 0);
      const int i1 = kSliced ? min(m, i0 + zcs) : m;
      for (int i = i0 + tid; i < i1; i += blockDim.x) {
        double2 zs = make_double2(0.0, 0.0);
        for (int q = 0; q < CL; ++q) {
          const double2 p = cluster.map_shared_rank(zp, q)[i];
          zs = make_double2(zs.x + p.x, zs.y + p.y);
        }
        z[i] = zmul(taup, zfma(sc, zs, rcb[i]));
      }
      for (int lc = lc2 + tid; lc < ncol; lc += blockDim.x) {
        const double2 u = zmul(zconj(cols[(size_t)lc * m + j]), sc);
        ub[lc] = u;
        o.Pr[(r + lc * CL) + (int64_t)j * o.n] = u;
      }
    }
    if (!own_next)
      for (int i = j + 1 + tid; i < m; i += blockDim.x) cb[i] = rcb[i];
    if (kSliced) cluster.sync();  // #1b
    if (kSliced && has_refl)
      for (int i = j + 1 + tid; i < m; i += blockDim.x) {
        const int q = (i - (j + 1)) / zcs;
        if (q != r) z[i] = cluster.map_shared_rank(z, q)[i];
      }
    if (!kSliced) cluster.sync();
    __syncthreads();
    // (d) A(i, c) -= z_i conj(u_c), i > j, own c >= j+2; column j+1 (u = 1) in every CTA's warp 0, then
    //     left reflector j+1 from it
    if (warp == 0) {
      double2* a = own_next ? cols + (size_t)lnext * m : cb;
      if (has_refl)
        for (int i = j + 1 + lane; i < m; i += 32) a[i] = make_double2(a[i].x - z[i].x, a[i].y - z[i].y);
      __syncwarp();
      if (own_next && lane == 0) {
        o.e[j] = betap;
        o.taup[j] = taup;
      }
      zgebrd_left(o, a, j + 1, v, scal, lane, own_next);
    }
    if (has_refl && tid >= 32)
      for (int i = j + 1 + tid - 32; i < m; i += (int)blockDim.x - 32) {
        const double2 zi = z[i];
        for (int lc = lc2; lc < ncol; ++lc) {
          double2* a = cols + (size_t)lc * m + i;
          const double2 t = zmul(zi, zconj(ub[lc]));
          *a = make_double2(a->x - t.x, a->y - t.y);
        }
      }
  }
  cluster.sync();
}
template <int CL>
static void launch_zgebrd_cl(const ZGebrdOp* ops, int nops, size_t smem, cudaStream_t s) {
  MPSG_CUDA(cudaFuncSetAttribute(k_zgebrd<CL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (CL > 8) MPSG_CUDA(cudaFuncSetAttribute(k_zgebrd<CL>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
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
  MPSG_CUDA(cudaLaunchKernelEx(&cfg, k_zgebrd<CL>, ops));
  g_bd_launches.fetch_add(1);
}
void launch_zgebrd(const ZGebrdOp* ops, int nops, int CL, size_t smem, cudaStream_t s) {
  if (nops <= 0) return;
  MPSG_CHECK(smem <= 227 * 1024, "complex bidiagonalisation: sector too large for the cluster");
  switch (CL) {
    case 1: launch_zgebrd_cl<1>(ops, nops, smem, s); break;
    case 2: launch_zgebrd_cl<2>(ops, nops, smem, s); break;
    case 4: launch_zgebrd_cl<4>(ops, nops, smem, s); break;
    case 8: launch_zgebrd_cl<8>(ops, nops, smem, s); break;
    case 16: launch_zgebrd_cl<16>(ops, nops, smem, s); break;
    default: throw Err(1, "complex bidiagonalisation: unsupported cluster size");
  }
}

// X_out = H_0 ... H_{nref-1} X_in for the columns [c0, c1) of one op, one warp per column (column in
// shared memory as complex values): the reflectors applied last to first, x -= tau v (v^H x).
__global__ void __launch_bounds__(256) k_zapply_refl(const ZReflOp* __restrict__ ops) {
  const ZReflOp o = ops[blockIdx.x];
  const int len = o.len;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  extern __shared__ double2 zx[];
  const int c = o.c0 + warp;
  if (c >= o.c1) return;  // no block-wide synchronisation below
  double2* x = zx + (size_t)warp * len;
  for (int i = lane; i < len; i += 32)
    x[i] = make_double2(i < o.rows_in ? o.Xin[i + (int64_t)c * o.ldi] : 0.0, 0.0);
  __syncwarp();
  for (int j = o.nref - 1; j >= 0; --j) {
    const double2 tau = o.tau[j];
    if (tau.x == 0.0 && tau.y == 0.0) continue;
    const int r0 = j + o.off;
    const double2* rj = o.R + (int64_t)j * o.ldr;
    double2 s = lane == 0 ? x[r0] : make_double2(0.0, 0.0);
    for (int i = r0 + 1 + lane; i < len; i += 32) s = zfma_c(rj[i], x[i], s);
    const double2 st = zmul(tau, zwarp_sum(s));
    __syncwarp();
    if (lane == 0) x[r0] = make_double2(x[r0].x - st.x, x[r0].y - st.y);
    for (int i = r0 + 1 + lane; i < len; i += 32) {
      const double2 t = zmul(rj[i], st);
      x[i] = make_double2(x[i].x - t.x, x[i].y - t.y);
    }
    __syncwarp();
  }
  for (int i = lane; i < len; i += 32) o.Xout[i + (int64_t)c * o.ldo] = x[i];
}
void launch_zapply_refl(const ZReflOp* ops, int nops, int lenmax, cudaStream_t s) {
  if (nops <= 0) return;
  const int nw = std::max(1, std::min(8, (int)((220 * 1024) / (sizeof(double2) * (size_t)std::max(lenmax, 1)))));
  const size_t smem = sizeof(double2) * nw * (size_t)std::max(lenmax, 1);
  MPSG_CHECK(smem <= 227 * 1024, "complex back-transformation: sector too tall");
  MPSG_CUDA(cudaFuncSetAttribute(k_zapply_refl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_zapply_refl<<<nops, 32 * nw, smem, s>>>(ops);
  g_bd_launches.fetch_add(1);
}
int zapply_refl_cols_per_block(int lenmax) {
  return std::max(1, std::min(8, (int)((220 * 1024) / (sizeof(double2) * (size_t)std::max(lenmax, 1)))));
}

}  // namespace mpsg
