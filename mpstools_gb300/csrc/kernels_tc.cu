// Tensor-core (tcgen05) grouped block GEMM for the mixed-precision matvec (sm_103a).
//
// Operands live in "tile images": for a block with R rows (M or N index) and K columns, row tiles
// of 128 rows and K chunks of 128 bytes (32 tf32 / 64 bf16 values) are stored as 16 KiB images
// in the exact shared-memory layout that tcgen05.mma reads (K-major, 128-byte swizzle: the 16-byte
// piece p of row r sits at r*128 + ((p ^ (r & 7)) * 16)).  Image (row_tile, k_chunk) is at
// offset (row_tile * nkc + k_chunk) * 16 KiB; padding rows / columns are zero.  Each value is
// split into hi = round(x) and lo = round(x - hi) in the operand type; NPROD = 3 accumulates
// hi*hi + hi*lo + lo*hi, NPROD = 1 only hi*hi.  Accumulation is FP32 in tensor memory.
//
// One persistent CTA per SM: warp 0 streams images with cp.async.bulk (TMA bulk copies), warp 1
// issues tcgen05.mma from one thread, warps 2-5 drain the double-buffered TMEM accumulator
// (tcgen05.ld) and write either FP64 column-major blocks or hi/lo tile images for the next stage.
// Every mbarrier wait is bounded (about 2 s of globaltimer); on expiry the CTA records an error
// code in *err, stops issuing work, frees its tensor memory and returns.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <atomic>
#include <cstdint>

#include "mpsg_internal.h"
#include "tc_types.h"

namespace mpsg {

extern std::atomic<int64_t> g_tc_launches;

namespace tc {

constexpr int kImg = 16384;
constexpr int kThreads = 192;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when the ~2 s limit expired (error code recorded) or another CTA failed.
__device__ __noinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  while (true) {
    for (int i = 0; i < 32; ++i)
      if (mbar_try_wait(bar, parity)) return true;
    if (*reinterpret_cast<volatile int*>(err) != 0) return false;
    if (globaltimer() - t0 > 2000000000ull) {
      atomicCAS(err, 0, code);
      return false;
    }
  }
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major, 128-byte swizzle shared-memory matrix descriptor (start address, SBO = 1024 bytes)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major), encoded 1
  d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset: 8 rows x 128 bytes
  d |= (uint64_t)1 << 46;              // descriptor version
  d |= (uint64_t)2 << 61;              // 128-byte swizzle
  return d;
}
// instruction descriptor: D = F32, A/B format, K-major A and B, N = 128, M = 128
template <int KIND>
__host__ __device__ constexpr uint32_t instr_desc() {
  return (1u << 4) | ((KIND == 0 ? 2u : 1u) << 7) | ((KIND == 0 ? 2u : 1u) << 10) | ((128u >> 3) << 17) |
         ((128u >> 4) << 24);
}
template <int KIND>
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  constexpr uint32_t id = instr_desc<KIND>();
  if (KIND == 0)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::
            "r"(d_tmem),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
  else
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::
            "r"(d_tmem),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
// hi/lo split of one value in the operand type; returns bit patterns
template <int KIND>
__device__ __forceinline__ void split_hilo(float x, uint32_t& hi, uint32_t& lo) {
  if (KIND == 0) {
    hi = to_tf32(x);
    lo = to_tf32(x - __uint_as_float(hi));
  } else {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    hi = (uint32_t)__bfloat16_as_ushort(h);
    lo = (uint32_t)__bfloat16_as_ushort(l);
  }
}

// ============================================================================ FP64 -> tile images
// One CTA converts one image; ops[] are prefix-indexed by img0.
template <int KIND, int NCOMP>
__global__ void __launch_bounds__(256) k_to_images(const TcConv* __restrict__ ops, int nops, const TcBases B) {
  constexpr int KC = (KIND == 0) ? 32 : 64;  // values per 128-byte row chunk
  constexpr int VP = (KIND == 0) ? 4 : 8;    // values per 16-byte piece
  const int img = blockIdx.x;
  int lo = 0, hi = nops - 1;
  while (lo < hi) {  // last op with img0 <= img
    const int mid = (lo + hi + 1) >> 1;
    if (ops[mid].img0 <= img) lo = mid; else hi = mid - 1;
  }
  const TcConv o = ops[lo];
  const int li = img - o.img0;
  const int rt = li / o.nkc, kc = li % o.nkc;
  const double* __restrict__ src = B.f64[o.src_slot] + o.src_off;
  uint8_t* dhi = const_cast<uint8_t*>(B.img[o.dst_slot]) + o.dst_off + (int64_t)li * kImg;
  uint8_t* dlo = dhi + B.lo_off[o.dst_slot];
  for (int pid = threadIdx.x; pid < 1024; pid += 256) {
    const int r = pid & 127, p = pid >> 7;
    const int row = rt * 128 + r;
    uint32_t h[VP], l[VP];
#pragma unroll
    for (int e = 0; e < VP; ++e) {
      const int k = kc * KC + p * VP + e;
      float x = 0.f;
      if (row < o.R && k < o.K) x = (float)(src[(int64_t)row * o.rs + (int64_t)k * o.ks] * o.scale);
      split_hilo<KIND>(x, h[e], l[e]);
    }
    const int off = r * 128 + ((p ^ (r & 7)) << 4);
    uint4 vh, vl;
    if (KIND == 0) {
      vh = make_uint4(h[0], h[1], h[2], h[3]);
      vl = make_uint4(l[0], l[1], l[2], l[3]);
    } else {
      vh = make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16), h[4] | (h[5] << 16), h[6] | (h[7] << 16));
      vl = make_uint4(l[0] | (l[1] << 16), l[2] | (l[3] << 16), l[4] | (l[5] << 16), l[6] | (l[7] << 16));
    }
    *reinterpret_cast<uint4*>(dhi + off) = vh;
    if (NCOMP == 2) *reinterpret_cast<uint4*>(dlo + off) = vl;
  }
}

// ============================================================================ persistent grouped GEMM
template <int KIND, int NPROD>
__global__ void __launch_bounds__(kThreads, 1) k_tc_gemm(const TcProb* __restrict__ prob, const TcSeg* __restrict__ seg,
                                                        const TcTile* __restrict__ tiles, int ntiles, const TcBases B) {
  constexpr int NCOMP = (NPROD == 3) ? 2 : 1;
  constexpr int STAGE_BYTES = 2 * NCOMP * kImg;
  constexpr int STAGES = (NCOMP == 2) ? 3 : 6;
  constexpr int KC = (KIND == 0) ? 32 : 64;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accf = empty + STAGES;
  uint64_t* acce = accf + 2;
  uint64_t* mdone = acce + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mdone + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* err = B.err;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&accf[a], 1);
      mbar_init(&acce[a], 4);
    }
    mbar_init(mdone, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {  // ---------------------------------------------------------------- producer
      int stage = 0;
      uint32_t phase = 0;
      int issued = 0;
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const TcTile tl = tiles[t];
        if (tl.prob < 0) continue;  // padding of a host-chosen block schedule
        const TcProb P = prob[tl.prob];
        for (int s = P.seg0; s < P.seg1; ++s) {
          const TcSeg S = seg[s];
          const uint8_t* a0 = B.img[S.a_slot] + S.a_off + (int64_t)tl.mt * S.nkc * kImg;
          const uint8_t* b0 = B.img[S.b_slot] + S.b_off + (int64_t)tl.nt * S.nkc * kImg;
          for (int kc = 0; kc < S.nkc; ++kc) {
            if (!mbar_wait(&empty[stage], phase ^ 1, err, 1)) goto producer_done;
            uint8_t* st = smem + stage * STAGE_BYTES;
            mbar_expect_tx(&full[stage], STAGE_BYTES);
            bulk_g2s(st, a0 + (int64_t)kc * kImg, kImg, &full[stage]);
            bulk_g2s(st + NCOMP * kImg, b0 + (int64_t)kc * kImg, kImg, &full[stage]);
            if (NCOMP == 2) {
              bulk_g2s(st + kImg, a0 + B.lo_off[S.a_slot] + (int64_t)kc * kImg, kImg, &full[stage]);
              bulk_g2s(st + 3 * kImg, b0 + B.lo_off[S.b_slot] + (int64_t)kc * kImg, kImg, &full[stage]);
            }
            ++issued;
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
    producer_done:
      // drain: every issued stage must have landed before the CTA may exit
      for (int i = 0; i < STAGES && i < issued; ++i) {
        int s = stage - 1 - i;
        uint32_t ph = phase;
        if (s < 0) {
          s += STAGES;
          ph ^= 1;
        }
        mbar_wait(&full[s], ph, err, 5);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // ---------------------------------------------------------------- MMA issuer
      int stage = 0;
      uint32_t phase = 0;
      int local = 0;
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const TcTile tl = tiles[t];
        if (tl.prob < 0) continue;
        const TcProb P = prob[tl.prob];
        const int acc = local & 1;
        const uint32_t accph = (local >> 1) & 1;
        ++local;
        if (!mbar_wait(&acce[acc], accph ^ 1, err, 2)) goto mma_done;
        tc_fence_after();
        const uint32_t d = tmem + acc * 128;
        uint32_t accum = 0;
        for (int s = P.seg0; s < P.seg1; ++s) {
          const int nkc = seg[s].nkc;
          for (int kc = 0; kc < nkc; ++kc) {
            if (!mbar_wait(&full[stage], phase, err, 3)) goto mma_done;
            tc_fence_after();
            const uint32_t base = smem_u32(smem + stage * STAGE_BYTES);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint64_t ah = sw128_desc(base + kk * 32);
              const uint64_t bh = sw128_desc(base + NCOMP * kImg + kk * 32);
              mma<KIND>(d, ah, bh, accum);
              accum = 1;
              if (NPROD == 3) {
                const uint64_t al = sw128_desc(base + kImg + kk * 32);
                const uint64_t bl = sw128_desc(base + 3 * kImg + kk * 32);
                mma<KIND>(d, ah, bl, 1);
                mma<KIND>(d, al, bh, 1);
              }
            }
            mma_commit(&empty[stage]);
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
        mma_commit(&accf[acc]);
      }
    mma_done:
      // all issued MMAs must be complete before tensor memory is released
      mma_commit(mdone);
      mbar_wait(mdone, 0, err, 6);
    }
  } else {  // ------------------------------------------------------------------------ epilogue
    const int q = warp & 3;  // TMEM lane quarter owned by this warp
    const int r = q * 32 + lane;
    int local = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const TcTile tl = tiles[t];
      if (tl.prob < 0) continue;
      const TcProb P = prob[tl.prob];
      const int acc = local & 1;
      const uint32_t accph = (local >> 1) & 1;
      ++local;
      if (!mbar_wait(&accf[acc], accph, err, 4)) break;
      tc_fence_after();
      const bool zero = (P.seg0 == P.seg1);
      const int m = tl.mt * 128 + r;
#pragma unroll 1
      for (int cc = 0; cc < 4; ++cc) {
        uint32_t v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + acc * 128 + cc * 32, v);
        const int n0 = tl.nt * 128 + cc * 32;
        if (P.mode == 0) {
          if (m < P.M) {
            double* c = B.f64[P.c_slot] + P.c_off + m;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int n = n0 + j;
              if (n < P.N) {
                const double val = zero ? 0.0 : (double)__uint_as_float(v[j]);
                double* cp = c + (int64_t)n * P.ldc;
                *cp = P.beta ? (*cp + val) : val;
              }
            }
          }
        } else {
          const int kc = n0 / KC;
          if (kc < P.c_nkc) {
            uint8_t* dhi = const_cast<uint8_t*>(B.img[P.c_slot]) + P.c_off + ((int64_t)tl.mt * P.c_nkc + kc) * kImg;
            uint8_t* dlo = dhi + B.lo_off[P.c_slot];
            const int e0 = n0 - kc * KC;  // element offset of this 32-column piece inside the chunk
            const bool rowok = (m < P.M) && !zero;
            if (KIND == 0) {
#pragma unroll
              for (int pp = 0; pp < 8; ++pp) {
                uint32_t h[4], l[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                  const int j = pp * 4 + e;
                  const float x = (rowok && n0 + j < P.N) ? __uint_as_float(v[j]) : 0.f;
                  split_hilo<0>(x, h[e], l[e]);
                }
                const int p = (e0 >> 2) + pp;
                const int off = r * 128 + ((p ^ (r & 7)) << 4);
                *reinterpret_cast<uint4*>(dhi + off) = make_uint4(h[0], h[1], h[2], h[3]);
                if (NCOMP == 2) *reinterpret_cast<uint4*>(dlo + off) = make_uint4(l[0], l[1], l[2], l[3]);
              }
            } else {
#pragma unroll
              for (int pp = 0; pp < 4; ++pp) {
                uint32_t h[8], l[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                  const int j = pp * 8 + e;
                  const float x = (rowok && n0 + j < P.N) ? __uint_as_float(v[j]) : 0.f;
                  split_hilo<1>(x, h[e], l[e]);
                }
                const int p = (e0 >> 3) + pp;
                const int off = r * 128 + ((p ^ (r & 7)) << 4);
                *reinterpret_cast<uint4*>(dhi + off) =
                    make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16), h[4] | (h[5] << 16), h[6] | (h[7] << 16));
                if (NCOMP == 2)
                  *reinterpret_cast<uint4*>(dlo + off) =
                      make_uint4(l[0] | (l[1] << 16), l[2] | (l[3] << 16), l[4] | (l[5] << 16), l[6] | (l[7] << 16));
              }
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[acc]);
    }
  }
  // ---------------------------------------------------------------------------- teardown
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
  }
}

}  // namespace tc

std::atomic<int64_t> g_tc_launches{0};

static size_t tc_smem_bytes(int nprod) {
  const int ncomp = nprod == 3 ? 2 : 1;
  const int stages = ncomp == 2 ? 3 : 6;
  return (size_t)stages * 2 * ncomp * tc::kImg + 1024 + 256;
}

void launch_tc_gemm(int kind, int nprod, const TcProb* prob, const TcSeg* seg, const TcTile* tiles, int ntiles,
                    const TcBases& B, int nsm, cudaStream_t s, int grid_override) {
  if (ntiles <= 0) return;
  const int grid = grid_override > 0 ? grid_override : (ntiles < nsm ? ntiles : nsm);
  const size_t sh = tc_smem_bytes(nprod);
#define MPSG_TC_CASE(K, P)                                                                         \
  if (kind == K && nprod == P) {                                                                   \
    cudaFuncSetAttribute(tc::k_tc_gemm<K, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh); \
    tc::k_tc_gemm<K, P><<<grid, tc::kThreads, sh, s>>>(prob, seg, tiles, ntiles, B);                \
  }
  MPSG_TC_CASE(0, 1)
  MPSG_TC_CASE(0, 3)
  MPSG_TC_CASE(1, 1)
  MPSG_TC_CASE(1, 3)
#undef MPSG_TC_CASE
  g_tc_launches.fetch_add(1);
}

void launch_tc_convert(int kind, int ncomp, const TcConv* ops, int nops, int nimg, const TcBases& B, cudaStream_t s) {
  if (nimg <= 0 || nops <= 0) return;
  if (kind == 0 && ncomp == 1) tc::k_to_images<0, 1><<<nimg, 256, 0, s>>>(ops, nops, B);
  if (kind == 0 && ncomp == 2) tc::k_to_images<0, 2><<<nimg, 256, 0, s>>>(ops, nops, B);
  if (kind == 1 && ncomp == 1) tc::k_to_images<1, 1><<<nimg, 256, 0, s>>>(ops, nops, B);
  if (kind == 1 && ncomp == 2) tc::k_to_images<1, 2><<<nimg, 256, 0, s>>>(ops, nops, B);
  g_tc_launches.fetch_add(1);
}

int64_t tc_launch_count() { return g_tc_launches.load(); }

}  // namespace mpsg
