// Segmented Lanczos vector kernels of the batched-chain engine: the Krylov vectors of all chains are
// one concatenated vector, chain c owning the elements [segoff[c], segoff[c + 1]); every reduction
// and every scalar (alpha, beta, norms) is per chain, scalars of chain c at c * stride.  Grid: x =
// chunks of one chain's range, y = chain.
#include <cuda_runtime.h>

#include <atomic>

#include "mpsg_internal.h"

namespace mpsg {

static std::atomic<int64_t> g_batch_launches{0};
int64_t batch_launch_count() { return g_batch_launches.load(); }

constexpr int kSegChunks = 32;

__device__ __forceinline__ double seg_block_sum(double v) {  // blockDim.x == 256
  __shared__ double red[8];
#pragma unroll
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 8) t = red[threadIdx.x];
  if (warp == 0) {
#pragma unroll
    for (int off = 4; off; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  }
  return t;  // valid in thread 0
}

__global__ void k_sdot_part(const double* __restrict__ x, const double* __restrict__ y,
                            const int64_t* __restrict__ segoff, double* part) {
  const int c = blockIdx.y;
  const int64_t i0 = segoff[c], i1 = segoff[c + 1];
  double s = 0.0;
  for (int64_t i = i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < i1; i += (int64_t)gridDim.x * blockDim.x)
    s = fma(x[i], y[i], s);
  s = seg_block_sum(s);
  if (threadIdx.x == 0) part[(int64_t)c * gridDim.x + blockIdx.x] = s;
}
__global__ void k_ssum_parts(const double* __restrict__ part, int np, double* out, int ostride) {
  const int c = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[(int64_t)c * np + i];
  s = seg_block_sum(s);
  if (threadIdx.x == 0) out[(int64_t)c * ostride] = s;
}
void launch_sdot(const double* x, const double* y, const int64_t* segoff, int nseg, double* part, double* out,
                 int ostride, cudaStream_t s) {
  if (nseg <= 0) return;
  k_sdot_part<<<dim3(kSegChunks, nseg), 256, 0, s>>>(x, y, segoff, part);
  k_ssum_parts<<<nseg, 256, 0, s>>>(part, kSegChunks, out, ostride);
  g_batch_launches.fetch_add(2);
}

// x_c *= 1 / sqrt(norm2_c) (0 when below delta); beta_c = sqrt(norm2_c)
__global__ void k_sscale_by_norm(double* x, const int64_t* __restrict__ segoff, const double* norm2, int stride,
                                 double delta, double* beta_out) {
  const int c = blockIdx.y;
  const double k = sqrt(norm2[(int64_t)c * stride]);
  const double sc = (k < delta) ? 0.0 : 1.0 / k;
  if (beta_out && blockIdx.x == 0 && threadIdx.x == 0) beta_out[(int64_t)c * stride] = k;
  const int64_t i0 = segoff[c], i1 = segoff[c + 1];
  for (int64_t i = i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < i1; i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= sc;
}
void launch_sscale_by_norm(double* x, const int64_t* segoff, int nseg, const double* norm2, int stride, double delta,
                           double* beta_out, cudaStream_t s) {
  if (nseg <= 0) return;
  k_sscale_by_norm<<<dim3(kSegChunks, nseg), 256, 0, s>>>(x, segoff, norm2, stride, delta, beta_out);
  g_batch_launches.fetch_add(1);
}

// out_c = w_c - alpha_c v_c - beta_c vprev_c, and |out_c|^2
__global__ void k_saxpy3(double* __restrict__ out, const double* __restrict__ w, const double* __restrict__ v,
                         const double* __restrict__ vp, const double* alpha, const double* beta, int stride,
                         const int64_t* __restrict__ segoff, double* part) {
  const int c = blockIdx.y;
  const double a = -alpha[(int64_t)c * stride];
  const double b = vp ? -beta[(int64_t)c * stride] : 0.0;
  const int64_t i0 = segoff[c], i1 = segoff[c + 1];
  double s = 0.0;
  for (int64_t i = i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < i1; i += (int64_t)gridDim.x * blockDim.x) {
    double o = v[i] * a + w[i];
    if (vp) o = o + vp[i] * b;
    out[i] = o;
    s = fma(o, o, s);
  }
  s = seg_block_sum(s);
  if (threadIdx.x == 0) part[(int64_t)c * gridDim.x + blockIdx.x] = s;
}
void launch_saxpy3(double* out, const double* w, const double* v, const double* vprev, const double* alpha,
                   const double* beta, int stride, const int64_t* segoff, int nseg, double* part, double* norm2_out,
                   cudaStream_t s) {
  if (nseg <= 0) return;
  k_saxpy3<<<dim3(kSegChunks, nseg), 256, 0, s>>>(out, w, v, vprev, alpha, beta, stride, segoff, part);
  k_ssum_parts<<<nseg, 256, 0, s>>>(part, kSegChunks, norm2_out, stride);
  g_batch_launches.fetch_add(2);
}

// y_c = sum_{j < nv_c} z_c[j] V_j (chain c's range)
__global__ void k_scombine(double* y, const double* const* __restrict__ V, const int* __restrict__ nv_of,
                           const double* __restrict__ z, int zstride, const int64_t* __restrict__ segoff) {
  const int c = blockIdx.y;
  const int nv = nv_of[c];
  const double* zc = z + (int64_t)c * zstride;
  const int64_t i0 = segoff[c], i1 = segoff[c + 1];
  for (int64_t i = i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < i1; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < nv; ++j) s = fma(V[j][i], zc[j], s);
    y[i] = s;
  }
}
void launch_scombine(double* y, const double* const* V, const int* nv_of, const double* z, int zstride,
                     const int64_t* segoff, int nseg, cudaStream_t s) {
  if (nseg <= 0) return;
  k_scombine<<<dim3(kSegChunks, nseg), 256, 0, s>>>(y, V, nv_of, z, zstride, segoff);
  g_batch_launches.fetch_add(1);
}

int seg_chunks() { return kSegChunks; }

}  // namespace mpsg
