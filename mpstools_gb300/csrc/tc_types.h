// Descriptors of the tensor-core (tcgen05) grouped GEMM and the FP64 -> tile-image conversion.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace mpsg {

// One product term: A images (row tile = output row tile) and B images (row tile = output
// column tile), nkc chunks of K.  Offsets are bytes of the hi component inside the slot's arena.
struct TcSeg {
  int64_t a_off, b_off;
  int32_t nkc;
  int8_t a_slot, b_slot;
};
// Output block: mode 0 = FP64 column-major (c_off in elements, ldc), mode 1 = hi/lo tile images
// (c_off in bytes, c_nkc K chunks) for the next contraction stage.
struct TcProb {
  int64_t c_off;
  int32_t ldc, M, N, seg0, seg1, c_nkc;
  int8_t mode, c_slot, beta;
};
struct TcTile {
  int32_t prob, mt, nt;  // prob < 0: padding (no work)
};
// FP64 block (element (row, k) at src[row*rs + k*ks], R rows, K columns) -> images from img0 on
struct TcConv {
  int64_t src_off, dst_off;
  int32_t R, K, rs, ks, nkc, img0;
  double scale;
  int8_t src_slot, dst_slot;
};
struct TcBases {
  const uint8_t* img[6];
  int64_t lo_off[6];
  double* f64[6];
  int* err;
};

// kind: 0 = kind::tf32, 1 = kind::f16 with bf16 operands; nprod: 1 or 3 (hi/lo split)
// grid_override > 0: that many persistent CTAs (a block schedule laid out for it); tiles with
// prob < 0 are padding and skipped
void launch_tc_gemm(int kind, int nprod, const TcProb* prob, const TcSeg* seg, const TcTile* tiles, int ntiles,
                    const TcBases& B, int nsm, cudaStream_t s, int grid_override = 0);
void launch_tc_convert(int kind, int ncomp, const TcConv* ops, int nops, int nimg, const TcBases& B, cudaStream_t s);
int64_t tc_launch_count();

}  // namespace mpsg
