// Internal declarations of libmpsg: block-sparse tensors, device launch descriptors.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace mpsg {

typedef uint64_t Q;  // packed U(1) charge word (AbKeyType::_qn); + and - wrap like the reference

struct Err : std::runtime_error {
  int code;
  Err(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define MPSG_CUDA(x)                                                                          \
  do {                                                                                        \
    cudaError_t e_ = (x);                                                                     \
    if (e_ != cudaSuccess)                                                                    \
      throw ::mpsg::Err(2, std::string(#x) + ": " + cudaGetErrorString(e_) + " @" +           \
                               std::to_string(__LINE__));                                     \
  } while (0)
#define MPSG_CHECK(c, msg)                    \
  do {                                        \
    if (!(c)) throw ::mpsg::Err(1, (msg));    \
  } while (0)

// TensorKeyType<2,Ns,AbKeyType> order: charges [0],[1] then indices (0),(1)
struct BKey {
  Q q0 = 0, q1 = 0;
  uint32_t p0 = 0, p1 = 0;
  bool operator<(const BKey& o) const {
    if (q0 != o.q0) return q0 < o.q0;
    if (q1 != o.q1) return q1 < o.q1;
    if (p0 != o.p0) return p0 < o.p0;
    return p1 < o.p1;
  }
  bool operator==(const BKey& o) const { return q0 == o.q0 && q1 == o.q1 && p0 == o.p0 && p1 == o.p1; }
};
inline BKey K1(Q a, Q b, uint32_t p) { BKey k; k.q0 = a; k.q1 = b; k.p0 = p; return k; }
inline BKey K2(Q a, Q b, uint32_t p, uint32_t pp) { BKey k; k.q0 = a; k.q1 = b; k.p0 = p; k.p1 = pp; return k; }

struct Block {
  BKey k;
  int32_t r = 0, c = 0;
  int64_t off = 0;  // element offset into the arena (multiple of kAlign)
};
constexpr int64_t kAlign = 16;  // 128-byte aligned blocks

struct Ctx;

// Block-sparse tensor with a device arena.  Padding between blocks is kept zero.
struct Tensor {
  Ctx* ctx = nullptr;
  std::shared_ptr<Ctx> keep;  // keeps the context (memory pool, stream) alive
  int nphys = 1;
  std::vector<Block> b;         // sorted by key
  std::map<BKey, int> idx;      // key -> position in b
  int64_t nelem = 0;            // arena length (elements)
  double* d = nullptr;          // device arena
  Tensor() {}
  Tensor(const Tensor&) = delete;
  Tensor& operator=(const Tensor&) = delete;
  ~Tensor();
  int find(const BKey& k) const {
    auto it = idx.find(k);
    return it == idx.end() ? -1 : it->second;
  }
  const double* ptr(int i) const { return d + b[i].off; }
  double* ptr(int i) { return d + b[i].off; }
};
typedef std::shared_ptr<Tensor> TensorP;

// Structure-only description used by planners before allocation.
struct Layout {
  std::vector<Block> b;
  std::map<BKey, int> idx;
  int64_t nelem = 0;
  void add(const BKey& k, int r, int c) {
    Block x;
    x.k = k; x.r = r; x.c = c;
    b.push_back(x);
  }
  void finalize();  // sort, assign offsets, build index; duplicate keys are an error
};

// ----------------------------------------------------------------------------- device descriptors
// Operands are addressed as (base slot, element offset); the base pointers are passed to the
// kernel by value, so one uploaded descriptor set serves every call with new buffers.
struct Bases {
  const double* p[8];
};
struct GSeg {  // one product term alpha*op(A)*op(B) accumulated into a problem
  int64_t offA, offB;
  int32_t lda, ldb, K;
  int8_t baseA, baseB, tA, tB;
  double alpha;
};
struct GProb {  // C (M x N, col-major, ldc) = [C +] sum_segments alpha*op(A)*op(B)
  int64_t offC;
  int32_t ldc, M, N, seg0, seg1;
  int8_t baseC, beta;
};
struct GTile {  // rows m0 .. m0 + 16 mi, columns n0 .. n0 + 16 nj of problem `prob` (mi, nj in 1..4)
  int32_t prob, m0, n0;
  int8_t mi, nj;
};
struct LCOut {  // dst[0..n) = sum_t coef_t * src_t[0..n)
  double* dst;
  int64_t n;
  int32_t t0, t1;
};
struct LCTerm {
  const double* src;
  double coef;
};
struct CopyOp {  // dst(i,j) = scale * rs[i] * cs[j] * (trans ? src(j,i) : src(i,j)); dst is rows x cols
  const double* src;
  double* dst;
  const double* rs;
  const double* cs;
  int32_t rows, cols, lds, ldd, trans;
  double scale;
};
struct GramPost {  // eigenpairs of an nc x nc slot (padding eigenvalues -1) -> s descending (0 if unresolved), V
  const double* W;   // eigenvectors, column j at W + j*ldw (rows 0..n-1 belong to the sector)
  const double* lam; // nc eigenvalues, any order
  double* V;
  double* S;
  int32_t n, ldw, nc;
};
struct ColNorm {  // U (m x k, column j at U + j*ldu): s_j = |U(:, j)|, U(:, j) /= s_j; columns with S[j] == 0 zeroed
  double* U;
  double* S;
  int32_t m, k, ldu;
};
struct CholOp {  // square n x n matrix C (leading dimension ld) of one sector, and its singular values S
  double* C;
  double* S;
  int32_t n, ld;
};
// ---- batched FP64 symmetric eigensolver (eig_f64.cu)
struct SytrdOp {  // n x n symmetric matrix A (full storage); out: diagonal d, off-diagonal e, reflectors in A
  double* A;
  double* d;
  double* e;
  double* tau;
  int32_t n, lda;
};
struct TriOp {  // tridiagonal (d, e) of one sector -> W (eigenvalues, descending; -1 below the floor), Z
  const double* d;
  const double* e;
  double* e2;    // e^2 (written by launch_tri_bounds)
  double* W;
  double* Z;
  double* meta;  // 4 doubles: lambda_max, pivmin, Gershgorin lo, hi
  double floor_rel;
  int32_t n, ldz;
};
struct OrmtrOp {  // columns [c0, c1) of Z <- Q Z with the reflectors of SytrdOp (columns with W < 0 skipped)
  const double* A;
  const double* tau;
  const double* W;
  double* Z;
  int32_t n, lda, ldz, c0, c1;
};
struct EigPostOp {  // S = sqrt(W) (0 below the floor)
  const double* W;
  double* S;
  int32_t n;
};
struct CholQROp {  // Cholesky of the k x k Gram matrix C (ld) of one sector: R = L^T in C's upper triangle
  double* C;
  double* rdiag;  // 1 / R_jj
  double* S;      // optional: S_j *= R_jj
  int* info;      // first non-positive pivot + 1 (0: none)
  int32_t k, ld;
};
struct TrsmRowsOp {  // rows [r0, r1) of X (ldx) <- X R^-1, R upper (ldr), k columns
  double* X;
  const double* R;
  const double* rdiag;
  int32_t k, ldx, ldr, r0, r1;
};
// ---- bidiagonal SVD of the split (svd_bidiag.cu)
struct GebrdOp {  // m x n (m >= n) sector matrix A (lda) -> B = Q^T A P upper bidiagonal (d, e)
  double* A;      // overwritten: column j below the diagonal = tail of left reflector j (unit at row j)
  double* d;      // n
  double* e;      // n (e[n-1] unused)
  double* tauq;   // n
  double* taup;   // n (taup[n-1] unused)
  double* Pr;     // n x n (ld n): column j = tail of right reflector j at rows j+2.. (unit at row j+1)
  int32_t m, n, lda;
  // sectors spread over several clusters (k_gebrd_mc): exchange buffers (gebrd_mc_xg_doubles), the
  // sector's barrier counter (zero at launch) and the launch's error flag (set when a wait expired)
  double* xg = nullptr;
  unsigned int* ctr = nullptr;
  int* err = nullptr;
};
// complex sector matrix (m >= n, interleaved re/im) -> B = Q^H A P real upper bidiagonal (d, e); the
// reflectors as in GebrdOp, complex (zgebrd conventions: real beta, H = I - tau v v^H applied as H^H)
struct ZGebrdOp {
  double2* A;
  double* d;
  double* e;
  double2* tauq;
  double2* taup;
  double2* Pr;
  int32_t m, n, lda;
};
// X_out (len x [c0, c1), ldo) = H_0 ... H_{nref-1} X_in with X_in real (ldi, rows >= rows_in are zero)
struct ZReflOp {
  const double2* R;    // reflector j: unit at row j + off, tail below it in column j (ldr)
  const double2* tau;  // nref
  const double* Xin;
  double2* Xout;
  int32_t len, nref, off, ldr, ldi, ldo, rows_in, c0, c1;
};
int zgebrd_cluster_size(int m, int n);  // 0: does not fit the shared-memory cluster kernel
size_t zgebrd_smem(int m, int n, int CL);
void launch_zgebrd(const ZGebrdOp* ops, int nops, int CL, size_t smem, cudaStream_t s);
void launch_zapply_refl(const ZReflOp* ops, int nops, int lenmax, cudaStream_t s);
int zapply_refl_cols_per_block(int lenmax);  // columns per op of launch_zapply_refl
struct GkOp {  // Golub-Kahan tridiagonal [[0, B], [B^T, 0]] (interleaved, zero diagonal) of one sector
  const double* d;    // n (bidiagonal)
  const double* e;    // n - 1
  double* b;          // 2n - 1 off-diagonals, scaled by 2^-p (max |b| in [1, 2))
  double* b2;         // their squares
  double* S;          // n: singular values (unscaled), descending; 0 past the computed ones
  double* Z;          // 2n x kept: eigenvectors (v0, u0, v1, u1, ...) of the kept values
  double* meta;       // [0] 2^p, [1] 2^-p, [2] Gershgorin bound of the scaled matrix
  const double* xlo;  // the segment's cut: singular values >= *xlo are computed
  int32_t* kcomp;     // number of singular values >= *xlo
  int32_t n, ldz;
};
struct GkVecOp {  // split the GK eigenvector of kept value k into V (n x k) and U (m x k, zero rows >= n)
  const double* Z;
  double* U;
  double* V;
  int32_t n, m, ldz, ldu, ldv, k;
};
struct ReflOp {  // columns [c0, c1) of X (len rows, ldx) <- H_0 H_1 ... H_{nref-1} X,
                 // H_j = I - tau_j r_j r_j^T, r_j = unit at row j + off, R(i, j) below it
  const double* R;
  const double* tau;
  double* X;
  int32_t len, nref, off, ldr, ldx, c0, c1;
};
// ---- complex (TEBD) path (tebd_kernels.cu); planar blocks: re at p, im at p + plane offset
struct CGatherOp {  // interleaved dst(i, j) = re(i, j) + i im(i, j); conj_trans: dst(j, i) = conj(...)
  const double* re;
  const double* im;
  double2* dst;
  int32_t rows, cols, lds, ldd, conj_trans;
};
struct CScatterOp {  // planar dst(i, j) = rs[i] cs[j] (conj_trans ? conj(src(j, i)) : src(i, j))
  const double2* src;
  double* re;
  double* im;
  const double* rs;
  const double* cs;
  int32_t rows, cols, lds, ldd, conj_trans;
};
struct CPhaseOp {  // complex FixPhase of one sector: U (m x k), V (n x k) with Vt = V^H
  double2* U;
  double2* V;
  int32_t m, n, k, ldu, ldv;
};
struct CBlockOp {  // one planar block of n elements
  const double* re;
  const double* im;
  int64_t n;
};
struct CMeasureOp {  // w * sum |x_ij|^2 ll_i^2 lr_j^2
  const double* re;
  const double* im;
  const double* ll;
  const double* lr;
  int32_t rows, cols;
  double w;
};
struct CGramPad {  // complex nc x nc slot: diagonal entries [n, nc) set to -1 (ranked below the spectrum)
  double2* A;
  int32_t nc, n;
};
struct CGramPost {  // eigenpairs of a padded complex Gram slot -> V (n x n, descending), S (sqrt, floored)
  const double2* W;
  const double* lam;
  double2* V;
  double* S;
  int32_t n, nc;
};
struct CColNorm {  // complex U (m x k, ldu): S_j = |U_j|, U_j /= S_j; columns with S_j == 0 cleared
  double2* U;
  double* S;
  int32_t m, k, ldu;
};
struct GramScaleOp {  // n x n matrix G (leading dimension ld), scaled in place by a power of two
  double* G;
  int32_t n, ld;
};
struct CDotOp {  // Re sum conj(a) b = sum a_re b_re + a_im b_im over n elements
  const double* ar;
  const double* ai;
  const double* br;
  const double* bi;
  int64_t n;
};
struct GramPad {  // diagonal entries [n, nc) of an nc x nc slot set to -1
  double* A;
  int32_t nc, n;
};
struct PhaseOp {  // FixPhase on one sector: Q (m x k, ldq) and P (n x k, ldp); sign from P columns
  double* Qm;
  double* Pm;
  int32_t m, n, k, ldq, ldp;
};

// ----------------------------------------------------------------------------- launchers (kernels.cu)
void launch_gemm_f64(const GProb* prob, const GSeg* seg, const GTile* tile, int ntiles, const Bases& bases,
                     cudaStream_t s);
void launch_lincomb(const LCOut* outs, const LCTerm* terms, int nout, int64_t maxn, cudaStream_t s);
void launch_copyops(const CopyOp* ops, int nops, cudaStream_t s);
void launch_fixphase(const PhaseOp* ops, int nops, int maxk, cudaStream_t s);
void launch_gram_post(const GramPost* ops, int nops, cudaStream_t s);
void launch_gram_pad(const GramPad* ops, int nops, cudaStream_t s);
void launch_colnorm(const ColNorm* ops, int nops, cudaStream_t s);
// C_jj = 1 where C_jj == 0 (zero columns of U stay zero through C = R^T R, U R^-1)
void launch_chol_unit_zero_diag(const CholOp* ops, int nops, cudaStream_t s);
// S_j *= |R_jj| for the Cholesky factor R stored in C's upper triangle
void launch_chol_scale_s(const CholOp* ops, int nops, cudaStream_t s);
// Lanczos vector kernels; `part` is a scratch array of kRedBlocks doubles
constexpr int kRedBlocks = 608;
void launch_dot(const double* x, const double* y, int64_t n, double* part, double* out, cudaStream_t s);
void launch_scale_by_norm(double* x, int64_t n, const double* norm2, double delta, double* beta_out,
                          cudaStream_t s);
void launch_axpy3(double* out, const double* w, const double* v, const double* vprev, const double* alpha,
                  const double* beta, int64_t n, double* part, double* norm2_out, cudaStream_t s);
// y[i] = sum_j V[j][i] * c[j]  (j < nv), optionally y -= instead of =; V is a device array of pointers
void launch_combine(double* y, const double* const* V, int nv, const double* c, int64_t n, int subtract,
                    cudaStream_t s);
// c[j] = <V_j, x> for j < nv (block partials reduced deterministically); part_nv holds 64*nv doubles
void launch_project(const double* const* V, int nv, const double* x, int64_t n, double* part_nv, double* c,
                    cudaStream_t s);
// graph-replayed Lanczos iteration (kernels_f64.cu): the iteration index *jp on the device
void launch_lz_pre(double* const* V, const int* jp, const double* norm2, double delta, double* beta, double* xin,
                   int64_t n, cudaStream_t s);
void launch_lz_post(double* const* V, int* jp, const double* w, const double* xin, double* alpha, double* beta,
                    double* norm2, double* E, int ndiag, bool checkpoint, int itmax, int64_t n, double* part,
                    cudaStream_t s);
void lz_prepare_attributes(int itmax);
void count_graph_launches(int64_t n);  // kernels a graph replay ran (for the launch statistics)
// lowest eigenpair of the symmetric tridiagonal (alpha[0..n), offdiag beta[1..n)); z may be null
void launch_tri_lowest(const double* alpha, const double* beta, int n, double* E0, double* z, cudaStream_t s);
void launch_tri_lowest_seg(const double* alpha, const double* beta, const int* n_of, int nchains, int nmax, int stride,
                           double* E0, int estride, double* z, cudaStream_t s);
// segmented Lanczos vector operations (batch_kernels.cu): chain c owns [segoff[c], segoff[c + 1]),
// its scalars sit at c * stride; `part` holds seg_chunks() doubles per chain
int seg_chunks();
int64_t batch_launch_count();
void launch_sdot(const double* x, const double* y, const int64_t* segoff, int nseg, double* part, double* out,
                 int ostride, cudaStream_t s);
void launch_sscale_by_norm(double* x, const int64_t* segoff, int nseg, const double* norm2, int stride, double delta,
                           double* beta_out, cudaStream_t s);
void launch_saxpy3(double* out, const double* w, const double* v, const double* vprev, const double* alpha,
                   const double* beta, int stride, const int64_t* segoff, int nseg, double* part, double* norm2_out,
                   cudaStream_t s);
void launch_scombine(double* y, const double* const* V, const int* nv_of, const double* z, int zstride,
                     const int64_t* segoff, int nseg, cudaStream_t s);
// bidiagonal SVD (svd_bidiag.cu)
int gebrd_cluster_size(int m, int n);  // 0: the sector does not fit the cluster kernel
// clusters of 16 CTAs for a global-memory sector (1 or 2) and the doubles of its exchange buffers
int gebrd_mc_clusters(int m, int n);
size_t gebrd_mc_xg_doubles(int m, int clusters);
size_t gebrd_mc_smem(int m, int n, int clusters);  // dynamic shared memory of one sector's CTAs
int gebrd_mc_capacity();  // two-cluster sectors that can be resident at once
// the sectors of ops (all with gebrd_mc_clusters == clusters) on clusters x 16 CTAs each
void launch_gebrd_mc(const GebrdOp* ops, int nops, int clusters, size_t smem, cudaStream_t s);
size_t gebrd_smem(int m, int n, int code);  // dynamic shared memory of one sector's CTAs
void launch_gebrd(const GebrdOp* ops, int nops, int code, size_t smem, cudaStream_t s);
void launch_gk_setup(const GkOp* ops, int nops, cudaStream_t s);
// per segment [seg[c], seg[c + 1]) of ops (op_seg: segment of each op): the cut x of the segment such
// that at least chimax of its values are >= x (or floor_abs when fewer than chimax exceed it), kept in
// the segment's state (gk_cut_state_bytes() per segment; the ops' xlo point at gk_cut_xlo(state, c));
// kcomp per op
void launch_gk_cut(const GkOp* ops, const int32_t* seg, const int32_t* op_seg, int nops, int nseg, int chimax,
                   double floor_abs, void* state, cudaStream_t s);
size_t gk_cut_state_bytes();
double* gk_cut_xlo(void* state, int c);
// S[k] of every (op_of[t], k_of[t]) with k < kcomp; 0 past kcomp
void launch_gk_bisect(const GkOp* ops, const int32_t* op_of, const int32_t* k_of, int nthreads, cudaStream_t s);
// Z column k for every listed (op, k), k < kept[op]; nmax2 = the largest 2n; scratch: 6 * nmax2 doubles
// per listed thread
void launch_gk_invit(const GkOp* ops, const int32_t* op_of, const int32_t* k_of, const int32_t* kept, int nthreads,
                     int nmax2, double* scratch, cudaStream_t s);
void launch_gk_vectors(const GkVecOp* ops, int nops, cudaStream_t s);
void launch_apply_refl(const ReflOp* ops, int nops, int lenmax, cudaStream_t s);
int apply_refl_cols_per_block(int lenmax);  // columns of X per ReflOp (c1 - c0 at most)
int64_t bidiag_launch_count();
// global truncation over concatenated singular values (see kernels.cu)
void launch_truncate(const double* S, int n, const int32_t* sec_of, int nsec, int chimax, int doTrunc,
                     double tr_weight, int32_t* rank_scratch, int32_t* counts, double* out3, cudaStream_t s);
void launch_fill(double* x, int64_t n, double v, cudaStream_t s);
int64_t kernel_launch_count();
int64_t tebd_launch_count();
void launch_cgather(const CGatherOp* ops, int nops, cudaStream_t s);
void launch_cscatter(const CScatterOp* ops, int nops, cudaStream_t s);
void launch_cfixphase(const CPhaseOp* ops, int nops, cudaStream_t s);
void launch_cblock_max2(const CBlockOp* ops, int nops, double* out, cudaStream_t s);
void launch_cmeasure(const CMeasureOp* ops, int nops, double* out, cudaStream_t s);
void launch_cdot_re(const CDotOp* ops, int nops, double* out, cudaStream_t s);
void launch_gram_scale(const GramScaleOp* ops, int nops, cudaStream_t s);
void launch_cgram_pad(const CGramPad* ops, int nops, cudaStream_t s);
void launch_cgram_post(const CGramPost* ops, int nops, cudaStream_t s);
void launch_ccolnorm(const CColNorm* ops, int nops, cudaStream_t s);
void launch_recip(double* dst, const double* src, int64_t n, cudaStream_t s);
int64_t eig_launch_count();
int sytrd_cluster_size(int n);
int sytrd_max_n();
size_t sytrd_smem_bytes(int n, int CL);
void launch_sytrd(const SytrdOp* ops, int nops, int CL, int nmax, cudaStream_t s);
void launch_tri_bounds(const TriOp* ops, int nops, cudaStream_t s);
void launch_tri_bisect(const TriOp* ops, const int* op_of, const int* k_of, int nthreads, double floor_rel_unused,
                       cudaStream_t s);
void launch_tri_invit(const TriOp* ops, const int* op_of, const int* k_of, int nthreads, double gap_rel,
                      double* scratch, const int64_t* scratch_off, cudaStream_t s);
void launch_ormtr(const OrmtrOp* ops, int nops, int nmax, cudaStream_t s);
void launch_eig_post(const EigPostOp* ops, int nops, cudaStream_t s);
void launch_count_nonneg(const TriOp* ops, int nops, int* cnt, cudaStream_t s);
size_t chol_smem_bytes(int k, int CL);
int chol_cluster_size(int k);
int chol_max_k();
void launch_chol(const CholQROp* ops, int nops, int CL, int kmax, cudaStream_t s);
void launch_trsm_rows(const TrsmRowsOp* ops, int nops, int kmax, cudaStream_t s);

}  // namespace mpsg
