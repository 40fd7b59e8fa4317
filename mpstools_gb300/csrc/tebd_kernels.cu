// Kernels of the complex (TEBD) path.  Complex block tensors are planar: the real parts of all
// blocks, then the imaginary parts at a fixed offset (the layout's element count); the SVD works on
// interleaved complex sector matrices (cuSOLVER's layout).
#include <cuda_runtime.h>

#include <atomic>
#include <cfloat>

#include "mpsg_internal.h"

namespace mpsg {

static std::atomic<int64_t> g_tebd_launches{0};
int64_t tebd_launch_count() { return g_tebd_launches.load(); }

// dst(i, j) = re(i, j) + i im(i, j) (conj_trans: dst(j, i) = re(i, j) - i im(i, j)), leading dimension ldd
__global__ void k_cgather(const CGatherOp* __restrict__ ops) {
  const CGatherOp o = ops[blockIdx.x];
  const int64_t tot = (int64_t)o.rows * o.cols;
  for (int64_t e = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.y * blockDim.x) {
    const int i = (int)(e % o.rows), j = (int)(e / o.rows);
    const int64_t s = i + (int64_t)j * o.lds;
    if (o.conj_trans) o.dst[j + (int64_t)i * o.ldd] = make_double2(o.re[s], -o.im[s]);
    else o.dst[i + (int64_t)j * o.ldd] = make_double2(o.re[s], o.im[s]);
  }
}
void launch_cgather(const CGatherOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_cgather<<<dim3(nops, 16), 256, 0, s>>>(ops);
  g_tebd_launches.fetch_add(1);
}

// planar dst(i, j) = rs[i] cs[j] (conj_trans ? conj(src(j, i)) : src(i, j))
__global__ void k_cscatter(const CScatterOp* __restrict__ ops) {
  const CScatterOp o = ops[blockIdx.x];
  const int64_t tot = (int64_t)o.rows * o.cols;
  for (int64_t e = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.y * blockDim.x) {
    const int i = (int)(e % o.rows), j = (int)(e / o.rows);
    double2 v = o.conj_trans ? o.src[j + (int64_t)i * o.lds] : o.src[i + (int64_t)j * o.lds];
    if (o.conj_trans) v.y = -v.y;
    double f = 1.0;
    if (o.rs) f *= o.rs[i];
    if (o.cs) f *= o.cs[j];
    const int64_t d = i + (int64_t)j * o.ldd;
    o.re[d] = v.x * f;
    o.im[d] = v.y * f;
  }
}
void launch_cscatter(const CScatterOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_cscatter<<<dim3(nops, 16), 256, 0, s>>>(ops);
  g_tebd_launches.fetch_add(1);
}

// Complex FixPhase (helperfunctions.hpp FixPhase for Complex): for singular index i let ind be the
// first index of the largest |V(j, i)| (the row i of Vt = V^H); U(:, i) and V(:, i) are multiplied by
// w = conj(V(ind, i)) / |V(ind, i)|, which removes the phase of Vt(i, ind) from the row of Vt and
// gives it to the column of U.  One block per sector, one warp per singular index.
__global__ void k_cfixphase(const CPhaseOp* __restrict__ ops) {
  const CPhaseOp o = ops[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int i = warp; i < o.k; i += nwarp) {
    double2* v = o.V + (int64_t)i * o.ldv;
    double best = -1.0;
    int ind = 0x7fffffff;
    for (int j = lane; j < o.n; j += 32) {
      const double a = v[j].x * v[j].x + v[j].y * v[j].y;
      if (a > best) { best = a; ind = j; }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const double b2 = __shfl_xor_sync(0xffffffffu, best, off);
      const int i2 = __shfl_xor_sync(0xffffffffu, ind, off);
      if (b2 > best || (b2 == best && i2 < ind)) { best = b2; ind = i2; }
    }
    if (!(best > 0.0)) continue;
    const double2 p = v[ind];
    const double inv = 1.0 / sqrt(best);
    const double wr = p.x * inv, wi = -p.y * inv;
    __syncwarp();
    for (int j = lane; j < o.n; j += 32) {
      const double2 x = v[j];
      v[j] = make_double2(x.x * wr - x.y * wi, x.x * wi + x.y * wr);
    }
    double2* u = o.U + (int64_t)i * o.ldu;
    for (int j = lane; j < o.m; j += 32) {
      const double2 x = u[j];
      u[j] = make_double2(x.x * wr - x.y * wi, x.x * wi + x.y * wr);
    }
  }
}
void launch_cfixphase(const CPhaseOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_cfixphase<<<nops, 256, 0, s>>>(ops);
  g_tebd_launches.fetch_add(1);
}

// out[b] = max over the block of re^2 + im^2 (BlockMatrix::squeeze decides on |x| > thresh)
__global__ void k_cblock_max2(const CBlockOp* __restrict__ ops, double* out) {
  const CBlockOp o = ops[blockIdx.x];
  double m = 0.0;
  for (int64_t e = threadIdx.x; e < o.n; e += blockDim.x) m = fmax(m, o.re[e] * o.re[e] + o.im[e] * o.im[e]);
  __shared__ double red[256];
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}
void launch_cblock_max2(const CBlockOp* ops, int nops, double* out, cudaStream_t s) {
  if (nops <= 0) return;
  k_cblock_max2<<<nops, 256, 0, s>>>(ops, out);
  g_tebd_launches.fetch_add(1);
}

// out[b] = w * sum_ij |x_ij|^2 ll_i^2 lr_j^2 (local diagonal operator on lambda Gamma lambda)
__global__ void k_cmeasure(const CMeasureOp* __restrict__ ops, double* out) {
  const CMeasureOp o = ops[blockIdx.x];
  const int64_t tot = (int64_t)o.rows * o.cols;
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) {
    const int i = (int)(e % o.rows), j = (int)(e / o.rows);
    const double f = o.ll[i] * o.lr[j];
    acc += (o.re[e] * o.re[e] + o.im[e] * o.im[e]) * f * f;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = o.w * red[0];
}
void launch_cmeasure(const CMeasureOp* ops, int nops, double* out, cudaStream_t s) {
  if (nops <= 0) return;
  k_cmeasure<<<nops, 256, 0, s>>>(ops, out);
  g_tebd_launches.fetch_add(1);
}

// out[b] = Re <a, b> = sum a_re b_re + a_im b_im over one block pair (mixed two-site expectation values
// of the adjoint)
__global__ void k_cdot_re(const CDotOp* __restrict__ ops, double* out) {
  const CDotOp o = ops[blockIdx.x];
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < o.n; e += blockDim.x) acc = fma(o.ar[e], o.br[e], fma(o.ai[e], o.bi[e], acc));
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}
void launch_cdot_re(const CDotOp* ops, int nops, double* out, cudaStream_t s) {
  if (nops <= 0) return;
  k_cdot_re<<<nops, 256, 0, s>>>(ops, out);
  g_tebd_launches.fetch_add(1);
}

// ---- complex density-matrix split (G = M^H M, batched Hermitian eigensolver, U = M V / s)
__global__ void k_cgram_pad(const CGramPad* __restrict__ ops) {
  const CGramPad o = ops[blockIdx.x];
  for (int i = o.n + threadIdx.x; i < o.nc; i += blockDim.x) o.A[i + (int64_t)i * o.nc] = make_double2(-1.0, 0.0);
}
void launch_cgram_pad(const CGramPad* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_cgram_pad<<<nops, 128, 0, s>>>(ops);
  g_tebd_launches.fetch_add(1);
}
// The n non-padding eigenvalues of the slot (any order) ranked descending (ties by index); V column
// rank = the eigenvector, S[rank] = sqrt(lambda) or 0 below the resolution floor 32 n eps lambda_max.
__global__ void k_cgram_post(const CGramPost* __restrict__ ops) {
  const CGramPost o = ops[blockIdx.x];
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
    if (rank >= n) continue;
    o.S[rank] = lj > floor_l ? sqrt(lj) : 0.0;
    const double2* w = o.W + (int64_t)j * nc;
    double2* v = o.V + (int64_t)rank * n;
    for (int r = 0; r < n; ++r) v[r] = w[r];
  }
}
void launch_cgram_post(const CGramPost* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_cgram_post<<<nops, 128, 0, s>>>(ops);
  g_tebd_launches.fetch_add(1);
}
// S_j = |M v_j| (the value the pair carries), u_j = M v_j / S_j; unresolved columns (S_j == 0) cleared.
__global__ void k_ccolnorm(const CColNorm* __restrict__ ops) {
  const CColNorm o = ops[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int j = warp; j < o.k; j += nwarp) {
    double2* u = o.U + (int64_t)j * o.ldu;
    if (o.S[j] == 0.0) {
      for (int r = lane; r < o.m; r += 32) u[r] = make_double2(0.0, 0.0);
      continue;
    }
    double acc = 0.0;
    for (int r = lane; r < o.m; r += 32) acc = fma(u[r].x, u[r].x, fma(u[r].y, u[r].y, acc));
    for (int off = 16; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    const double nrm = sqrt(acc);
    const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
    for (int r = lane; r < o.m; r += 32) u[r] = make_double2(u[r].x * inv, u[r].y * inv);
    __syncwarp();
    if (lane == 0) o.S[j] = nrm;
  }
}
void launch_ccolnorm(const CColNorm* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return;
  k_ccolnorm<<<nops, 256, 0, s>>>(ops);
  g_tebd_launches.fetch_add(1);
}

// dst = 1 / src (0 where src is 0: padding)
__global__ void k_recip(double* dst, const double* src, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i] != 0.0 ? 1.0 / src[i] : 0.0;
}
void launch_recip(double* dst, const double* src, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  k_recip<<<(int)std::min<int64_t>((n + 255) / 256, 1024), 256, 0, s>>>(dst, src, n);
  g_tebd_launches.fetch_add(1);
}

}  // namespace mpsg
