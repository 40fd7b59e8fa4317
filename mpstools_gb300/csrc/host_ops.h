// Contraction plans and algorithms of the DMRG hot path (host orchestration of the kernels).
#pragma once
#include <functional>
#include <memory>

#include "host_core.h"
#include "tc_types.h"

namespace mpsg {

// Arena of blocks addressed by an arbitrary ordered key (internal intermediates).
template <class K>
struct KeyedArena {
  struct B {
    int32_t r, c;
    int64_t off;
  };
  std::map<K, B> m;
  int64_t nelem = 0;
  void add(const K& k, int r, int c) {
    if (m.count(k)) return;
    B b{r, c, nelem};
    m[k] = b;
    nelem += ((int64_t)r * c + kAlign - 1) / kAlign * kAlign;
  }
  const B& at(const K& k) const { return m.at(k); }
};

// 5-index key of a combined environment block (L~ / R~) or intermediate
struct K5 {
  Q x, y;
  uint32_t w, s, t;
  bool operator<(const K5& o) const {
    if (x != o.x) return x < o.x;
    if (y != o.y) return y < o.y;
    if (w != o.w) return w < o.w;
    if (s != o.s) return s < o.s;
    return t < o.t;
  }
};

// Matvec  theta' = L W1 W2 R theta  (contractTwosite), factored as
//   L~(a',a;wm,s1',s1) = sum_wl W1[wl,wm](s1->s1') L(a',a;wl)
//   R~(b',b;wm,s2',s2) = sum_wr W2[wm,wr](s2->s2') R(b',b;wr)
//   X(a',b;wm,s1',s2)  = sum_s1 L~(a',a;wm,s1',s1) theta(a,b;s1,s2)          (stage A)
//   theta'(a',b';s1',s2') = sum_{wm,s2,b} X(a',b;wm,s1',s2) R~(b',b;wm,s2',s2)^T   (stage C)
struct MatvecPlan {
  Ctx* ctx = nullptr;
  std::shared_ptr<Ctx> keep;
  KeyedArena<K5> lt, rt, xa;
  double* dLt = nullptr;
  double* dRt = nullptr;
  double* dX = nullptr;
  Layout out;                // output layout (reference structure unless given)
  GemmPlan stageA, stageC;
  LincombPlan build_lt, build_rt;
  double flops = 0;          // algorithmic FLOPs of one matvec (stage A + stage C)
  double flops_ref = 0;      // FLOPs of the reference's per-term schedule (2 GEMMs per term)
  double flops_factored = 0;   // F_A + F_B + F_C of the factored (L.theta first) schedule
  int64_t bytes_alg = 0;     // 8*(|L|+|R|+2|theta|)
  // tensor-core path (prec != FP64): operands as hi/lo tile images
  int prec = MPSG_PREC_FP64;
  int kind = 0, nprod = 3, nsm = 148;
  uint8_t* dimg[4] = {nullptr, nullptr, nullptr, nullptr};  // L~, theta, X, R~ images
  int64_t img_hi[4] = {0, 0, 0, 0};                         // bytes of the hi component per arena
  TcProb* dprob[2] = {nullptr, nullptr};
  TcSeg* dseg[2] = {nullptr, nullptr};
  TcTile* dtile[2] = {nullptr, nullptr};
  int ntile[2] = {0, 0};
  int tgrid[2] = {0, 0};   // persistent CTAs of each stage (0: min(tiles, SMs))
  int tsched[2] = {0, 0};  // block schedule chosen for each stage (tc_schedule_name)
  TcConv* dconv_theta = nullptr;
  int nconv_theta = 0, nimg_theta = 0;
  int* derr = nullptr;
  // a tensor-core plan also carries the FP64 stage tables (same combined environments and blocks):
  // use_fp64() switches run() to them, e.g. for an FP64 energy or an FP64 Lanczos finish
  bool fp64 = false;
  void use_fp64();
  void run(const double* theta_in, double* theta_out);
  void check_error();  // throws MPSG_ERR_TIMEOUT when a bounded device wait expired
  int launches_per_run() const {
    if (prec != MPSG_PREC_FP64 && !fp64) return 3;
    return (stageA.hprob.empty() ? 0 : 1) + (stageC.hprob.empty() ? 0 : 1);
  }
  ~MatvecPlan();
};
// Block schedules of the tcgen05 stages, chosen per plan by timing (autotuner): 0 = tiles in
// longest-K-first order dealt round-robin to the persistent CTAs, 1 = the same order dealt in a
// snake (alternate rounds reversed), 2 = greedy longest-processing-time assignment (each tile, longest
// first, to the CTA with the least estimated work; lists padded).  The choice is cached per
// block-size signature.  tuned / cache_hits count the signatures timed and the plans served from
// the cache.
const char* tc_schedule_name(int s);
void tc_autotune_counts(int64_t* tuned, int64_t* cache_hits);
// schedules of the most recent tensor-core plan; timing6 (optional): best ms of each schedule in the
// most recent timing, stage A then stage C (-1 where not timed)
void tc_last_schedules(int32_t* sched2, float* timing6 = nullptr);
// FP64 plan applied with the stage-A intermediate in the library's fixed device array (noalloc.cu)
void matvec_noalloc(MatvecPlan& P, const double* theta_in, double* theta_out);
// device address of that array on `device` (the current device); resolved once per device
double* noalloc_scratch_address(int device);
std::unique_ptr<MatvecPlan> build_matvec(Ctx* ctx, const Tensor& L, const Tensor& R, const Layout& th_in,
                                         const MPO& W1, const MPO& W2, const ItoKey& ik0, const ItoKey& ik1,
                                         const Layout* out_layout, int prec = MPSG_PREC_FP64);
// Block keys reachable from `th` by repeated application of the matvec (reference semantics).
Layout theta_closure(const Tensor& L, const Tensor& R, const Layout& th, const MPO& W1, const MPO& W2,
                     const ItoKey& ik0, const ItoKey& ik1);

// Environment update (addContractionLayer) factored as two grouped GEMM stages.
// A grouped FP64 GEMM stage (GemmPlan) run on the tensor cores: every operand block of the plan is
// converted to hi/lo tile images (transposes folded into the conversion's strides, the segment's
// alpha into its A operand) and the products run through the tcgen05 grouped GEMM with FP64 output
// blocks, from and to the same base slots as the FP64 plan.
struct TcStage {
  Ctx* ctx = nullptr;
  int kind = 0, nprod = 3, nsm = 148;
  uint8_t* dimg = nullptr;
  int64_t img_hi = 0;
  TcConv* dconv = nullptr;
  int nconv = 0, nimg = 0;
  TcProb* dprob = nullptr;
  TcSeg* dseg = nullptr;
  TcTile* dtile = nullptr;
  int ntile = 0, grid = 0;
  int* derr = nullptr;
  void build(Ctx* c, const GemmPlan& g, int prec);
  void run(const double* const* bases);  // conversions + GEMM on ctx->stream
  ~TcStage();
};
struct EnvPlan {
  Ctx* ctx = nullptr;
  std::shared_ptr<Ctx> keep;
  int prec = MPSG_PREC_FP64;             // tensor-core precisions: both stages as TcStage
  std::unique_ptr<TcStage> tc1, tc2;
  KeyedArena<K5> ct;      // combined environment (L~ or R~)
  KeyedArena<K5> tt;      // intermediate T
  double* dCt = nullptr;
  double* dT = nullptr;
  Layout out;
  GemmPlan st1, st2;
  LincombPlan build_ct;
  double flops = 0;
  // A: lower tensor data; Aup: upper tensor data (nullptr: the lower tensor is also the upper one)
  void run(const double* A, double* out_d, const double* Aup = nullptr);
  ~EnvPlan();
};
// Aup (optional): separate upper tensor, the two-tensor addContractionLayer(BL, A, mpo, Ap, ...)
std::unique_ptr<EnvPlan> build_env(Ctx* ctx, const Tensor& BL, const Tensor& A, const MPO& W, const ItoKey& ik,
                                   int direction, const Tensor* Aup = nullptr, int prec = MPSG_PREC_FP64);
TensorP env_update(Ctx* ctx, const Tensor& BL, const Tensor& A, const MPO& W, const ItoKey& ik, int direction,
                   double* flops_out, const Tensor* Aup = nullptr, int prec = MPSG_PREC_FP64);

// theta(a,b;s1,s2) = A1(a,c;s1) A2(c,b;s2)
TensorP theta_form(Ctx* ctx, const Tensor& A1, const Tensor& A2, const Layout* layout);

// Complex SVD of the sectors of the TEBD split on the bidiagonal route: sector i is the complex
// ms x ns matrix (ms >= ns, leading dimension ms) at zM + offM (overwritten); its ns values go to
// dS (the sectors' values consecutive, descending; values below 1e-16 are 0) and M = U diag(S) V^H
// with U (ms x ns, ldu) and V (ns x ns, ldv), columns of values below 1e-16 zero.  Returns false
// when a sector does not fit the shared-memory cluster kernel or its vectors would need the Jacobi
// route (the caller then uses the library solver; counted in split_fallback_count()).
struct ZSvdSec {
  int ms, ns;
  int64_t offM;
  double2 *U, *V;
  int ldu, ldv;
};
bool zsvd_bidiag(Ctx* ctx, const std::vector<ZSvdSec>& secs, double2* zM, double* dS);

// split (two-site, direction 0) with global truncation
struct SplitResult {
  TensorP U, Vt, lam;
  double tw = 0;
  int chi = 0;
  std::vector<double> tw_seg;  // per segment (one entry without segments)
  std::vector<int> chi_seg;
};
// absorb: 0 none, +1 lambda into Vt (rows), -1 lambda into U (columns).  seg_q0 (optional, ascending):
// th is a direct sum of independent chains, chain c holding the centre charges from seg_q0[c] up to
// the next entry; truncation, truncated weight, kept count and normalisation are then per chain.
// number of charge sectors of density-matrix splits (own eigensolver) redone on the exact Jacobi
// route because the CholeskyQR of their singular vectors failed
int64_t split_fallback_count();
// on_bidiag (optional): called once the bidiagonalisation launches are queued (bidiagonal route), with
// the event those launches wait for; work queued on other streams after that event becomes ready
// together with them, so that the higher-priority cluster launches are placed first.
SplitResult split2(Ctx* ctx, const Tensor& th, const ItoKey& ik0, const ItoKey& ik1, int chimax, bool doTrunc,
                   double tr_weight, bool normalize, int absorb, const std::vector<Q>* seg_q0 = nullptr,
                   const std::vector<int>* seg_absorb = nullptr,  // per-segment absorb
                   const std::function<void(cudaEvent_t)>& on_bidiag = {});

// prepareMatrix(BL1, lambda, BL2, "r", multiply=true, truncate=true, delta): right-orthonormalise BL2,
// multiply U*D into BL1 (BL1 may be null at the left edge).
void prepare_matrix_r(Ctx* ctx, TensorP* BL1, TensorP& BL2, TensorP* lam_out, double delta);
// prepareMatrix(BL1, lambda, BL2, "l", multiply=true): left-orthonormalise BL1, multiply D*Vd into BL2
// from the left (BL2 may be null at the right edge); singular values <= delta dropped.
void prepare_matrix_l(Ctx* ctx, TensorP& BL1, TensorP* BL2, TensorP* lam_out, double delta);

struct LanczosStats {
  int64_t matvecs = 0;
  double matvec_flops = 0;
  double matvec_seconds = 0;
  double seconds = 0;
};
struct LanczosResult {
  double E0 = 0;
  int iterations = 0;
  int n = 0;
};
// TSLanzcosEngine::simulate + getState(0): psi receives the ground state (layout of th_init).
// The energy test runs every ndiag iterations (reference: 5) and passes when
// |E - E_prev| < max(delta, tol_rel*|E|); stall_rel > 0 also stops once |E - E_prev| is below
// stall_rel*|E| and stopped shrinking (the noise floor of a low-precision matvec).
// energy-test tolerance and stall level of the Lanczos for a matvec precision (0 for FP64)
double prec_tol(int prec);
double prec_stall(int prec);
// <psi|H|psi> / <psi|psi> with one matvec of the plan (FP64 for MPSG_PREC_MIXED energies).
double rayleigh_quotient(Ctx* ctx, MatvecPlan& mv, const Tensor& psi, LanczosStats* st);
// The same Rayleigh quotient queued on the context's low-priority side stream, so that it runs on
// the SMs the work queued after it (the split of psi) leaves idle.  psi must stay alive and
// unchanged until finish(), which waits for the result.
struct EnergyJob {
  Ctx* ctx = nullptr;
  std::unique_ptr<MatvecPlan> mv;
  LanczosStats* st = nullptr;
  const Tensor* psi = nullptr;
  bool launched = false;
  double* buf = nullptr;  // H psi (nw) | reduction partials | the two dot products
  int64_t nw = 0;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // matvec start / end, dots done
  bool pending() const { return ctx != nullptr; }
  // prepare: take the plan and the state (nothing queued); launch: queue the matvec and the dot
  // products on the side stream after `after` (an event of the main stream's work; nullptr: all of it)
  void prepare(Ctx* c, std::unique_ptr<MatvecPlan> plan, const Tensor& psi, LanczosStats* s);
  void launch(cudaEvent_t after);
  double finish();
  void release();
  ~EnergyJob() { release(); }
};
LanczosResult lanczos(Ctx* ctx, MatvecPlan& mv, const Tensor& th_init, Tensor& psi, int itmax, double delta,
                      bool testenergy, bool reorth, LanczosStats* st, double tol_rel = 0.0, int ndiag = 5,
                      double stall_rel = 0.0, const double* proj = nullptr);
// Lanczos in precision `prec` (mpsg_prec): FP64 is the reference loop; TF32/TF32X3/BF16/BF16X3 run
// the loop with the tensor-core matvec and a precision-adapted energy test; AUTO runs TF32X3 first
// and finishes with FP64 iterations restarted from the mixed-precision ground state; MIXED runs
// TF32X3 and measures the energy as the FP64 Rayleigh quotient of its ground state.
LanczosResult lanczos_prec(Ctx* ctx, const Tensor& L, const Tensor& R, const Layout& sx, const MPO& W1, const MPO& W2,
                           const ItoKey& ik0, const ItoKey& ik1, const Tensor& th_init, Tensor& psi, int itmax,
                           double delta, bool testenergy, bool reorth, int prec, LanczosStats* st,
                           const double* proj = nullptr,  // proj: state the Krylov space stays orthogonal to
                           EnergyJob* energy = nullptr);  // MIXED: E0 left to energy->finish()

}  // namespace mpsg
