// Host-side core types of libmpsg (context, MPO terms, GEMM / lincomb plans).
#pragma once
#include <cublas_v2.h>
#include <cusolverDn.h>

#include "../../include/mpsg.h"
#include "mpsg_internal.h"

namespace mpsg {

extern thread_local std::string g_last_error;

struct Ctx : std::enable_shared_from_this<Ctx> {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own = nullptr;
  cusolverDnHandle_t solver = nullptr;
  gesvdjInfo_t svdp = nullptr;
  double* part = nullptr;     // reduction partials (kRedBlocks) + 64 scalars
  double* hscal = nullptr;    // pinned host scalars
  int svd_method = 4;         // 4: own bidiagonal SVD; 0: Jacobi SVD (gesvdj); 1-3: density matrix
  explicit Ctx(int dev);
  ~Ctx();
  void* dmalloc(size_t bytes);
  void dfree(void* p);
  cusolverDnHandle_t svd_handle();
  cusolverDnParams_t params = nullptr;
  cusolverDnParams_t solver_params();
  cublasHandle_t blas = nullptr;
  cublasHandle_t blas_handle();  // bound to `stream`
  // worker streams / solver handles for concurrent per-sector eigen-solves (created on first use)
  std::vector<cudaStream_t> wstreams;
  std::vector<cusolverDnHandle_t> whandles;
  std::vector<cublasHandle_t> wblas;
  int nworkers();
  // fork(n): worker streams 0..n-1 wait for the work queued on `stream` so far; join(n): `stream`
  // waits for the work queued on them.  Independent launches between the two run concurrently.
  std::vector<cudaEvent_t> wevents;
  cudaEvent_t fork_event = nullptr;
  void fork(int n);
  void join(int n);
  void sync();
  // side stream at the lowest priority (the library's own streams run at the highest): work queued
  // there fills the SMs that the main stream's kernels leave idle
  cudaStream_t side = nullptr;
  cudaStream_t side_stream();
};

// ---------------------------------------------------------------- tensors
TensorP make_tensor(Ctx* ctx, int nphys, const Layout& lay, bool zero);
Layout layout_of(const Tensor& t);
TensorP tensor_from_host(Ctx* ctx, int nphys, int n, const uint64_t* q, const uint32_t* p, const int32_t* rows,
                         const int32_t* cols, const double* data);
void tensor_to_host(const Tensor& t, std::vector<double>& packed);  // blocks in key order, concatenated
// the same packed layout written straight into dst (device gather, one device-to-host copy)
void tensor_pack_to_host(const Tensor& t, double* dst);
TensorP tensor_copy(const Tensor& t);

// ---------------------------------------------------------------- MPO (MPOMat<1,T>)
struct OpEl {  // element (out, in) of a SparseOperator<1,T>
  uint32_t out, in;
  double v;
};
struct MPOEntry {  // W[wl, wr], elements in (in, out) order
  uint32_t wl, wr;
  std::vector<OpEl> ops;
};
struct MPO {
  std::vector<MPOEntry> e;  // (wl, wr) ascending
  int Dl = 0, Dr = 0;
};
typedef std::vector<Q> ItoKey;
MPO mpo_from_c(const mpsg_mpo* w);
ItoKey itokey_from_c(const mpsg_itokey* ik);

// ---------------------------------------------------------------- grouped GEMM plan
// Operands are (base slot, element offset) pairs so a plan can be re-bound to new buffers.
struct GSegH {
  int baseA, baseB;
  int64_t offA, offB;
  int lda, ldb, K, tA, tB;
  double alpha;
};
struct GProbH {
  int baseC;
  int64_t offC;
  int ldc, M, N, seg0, seg1, beta;
};
struct GemmPlan {
  Ctx* ctx = nullptr;
  std::shared_ptr<Ctx> keep;
  std::vector<GProbH> hprob;
  std::vector<GSegH> hseg;
  GProb* dprob = nullptr;
  GSeg* dseg = nullptr;
  GTile* dtile = nullptr;
  int ntiles = 0;
  std::vector<int> prob_tile0;  // first tile of each problem (set by upload), then the tile count
  double flops = 0;
  void add_problem(int baseC, int64_t offC, int ldc, int M, int N, bool accumulate, const std::vector<GSegH>& segs);
  int nprob() const { return (int)hprob.size(); }
  void upload(Ctx* ctx);
  void run(const double* const* bases);
  void run_range(const double* const* bases, int p0, int p1);  // problems [p0, p1) only
  GemmPlan() {}
  GemmPlan(const GemmPlan&) = delete;
  ~GemmPlan();
};

struct LincombPlan {
  std::vector<LCOut> hout;
  std::vector<LCTerm> hterm;
  int64_t maxn = 0;
  void add(double* dst, int64_t n, const std::vector<std::pair<const double*, double>>& terms);
  void run(Ctx* ctx);
};
void run_copyops(Ctx* ctx, const std::vector<CopyOp>& ops);

}  // namespace mpsg
