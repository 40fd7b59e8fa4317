/*
 * mpsg.h -- C ABI of libmpsg, the GB300 (sm_103a) DMRG hot path of MPSTools.
 *
 * Plain C types only: pointers, sizes, enums and opaque handles.  Block-sparse
 * tensors are U(1) BlockMatrix objects: a sorted list of dense column-major
 * blocks, each keyed by two packed charge words (AbKeyType::_qn) and 0..2
 * physical / MPO-auxiliary indices (TensorKeyType<2,Ns,AbKeyType>), with the
 * payload in one device arena per tensor.
 *
 * Every entry point returns an mpsg_status; on failure mpsg_last_error()
 * holds a one-line message.  Nothing aborts the process.
 */
#ifndef MPSG_H_
#define MPSG_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  MPSG_OK = 0,
  MPSG_ERR_ARG = 1,           /* invalid argument or inconsistent block structure */
  MPSG_ERR_CUDA = 2,          /* CUDA runtime error */
  MPSG_ERR_SOLVER = 3,        /* cuSOLVER / dense eigen- or SVD-solver failure */
  MPSG_ERR_NOMEM = 4,         /* device allocation failed */
  MPSG_ERR_TIMEOUT = 5,       /* a bounded device-side wait ran out */
  MPSG_ERR_NOT_CONVERGED = 6  /* reported by solvers that do not treat this as success */
} mpsg_status;

/* Arithmetic of the matvec / environment contractions.  The Lanczos recurrence,
 * reorthogonalisation, SVD, truncation bookkeeping and energy measurement are
 * always FP64. */
typedef enum {
  MPSG_PREC_FP64 = 0,    /* FP64 FMA on CUDA cores (drop-in path) */
  MPSG_PREC_TF32 = 1,    /* tcgen05 kind::tf32, FP32 accumulate */
  MPSG_PREC_TF32X3 = 2,  /* tcgen05 kind::tf32 with hi/lo split (3 products), FP32 accumulate */
  MPSG_PREC_BF16 = 3,    /* tcgen05 kind::f16 (bf16), FP32 accumulate */
  MPSG_PREC_BF16X3 = 4,  /* tcgen05 kind::f16 (bf16) hi/lo split (3 products), FP32 accumulate */
  MPSG_PREC_AUTO = 5,    /* Lanczos only: TF32X3 Lanczos to its precision floor, then the reference's
                            FP64 Lanczos restarted from that state (energy test every iteration) */
  MPSG_PREC_MIXED = 6    /* Lanczos only: TF32X3 Lanczos to its precision floor; the energy is the FP64
                            Rayleigh quotient <psi|H|psi> / <psi|psi> of its ground state (one FP64
                            matvec) */
} mpsg_prec;

typedef struct mpsg_ctx_s* mpsg_ctx;
typedef struct mpsg_tensor_s* mpsg_tensor;
typedef struct mpsg_dmrg_s* mpsg_dmrg;

/* One MPO matrix MPOMat<1,T> (src/MPOTypes.hpp:839-889): term i is the element
 * (out[i], in[i]) = value[i] of the sparse operator W[wl[i], wr[i]]. */
typedef struct {
  int32_t nterms;
  const uint32_t* wl;
  const uint32_t* wr;
  const uint32_t* out;
  const uint32_t* in;
  const double* value;
  int32_t Dl, Dr;
} mpsg_mpo;

/* i_to_key<AbKeyType> (src/tensormap.hpp:280-298): local state -> charge word. */
typedef struct {
  int32_t d;
  const uint64_t* charge;
} mpsg_itokey;

/* ------------------------------------------------------------------ context */
mpsg_status mpsg_ctx_create(int32_t device, mpsg_ctx* out);
void mpsg_ctx_destroy(mpsg_ctx ctx);
const char* mpsg_last_error(void);
/* stream: a cudaStream_t (NULL = the library's own non-blocking stream). */
mpsg_status mpsg_ctx_set_stream(mpsg_ctx ctx, void* stream);
mpsg_status mpsg_ctx_sync(mpsg_ctx ctx);
/* Waits for the context's work and returns the device memory the library's stream-ordered
 * allocations keep cached (the default memory pool of the device) to the driver. */
mpsg_status mpsg_ctx_trim(mpsg_ctx ctx);
/* Number of kernels this library launched on ctx since creation. */
int64_t mpsg_ctx_kernel_launches(mpsg_ctx ctx);
/* The tensor-core matvec's block-schedule autotuner (process-wide): signatures timed, plans served
 * from its cache, the schedule of each stage of the most recent tensor-core plan (0 round robin,
 * 1 snake, 2 greedy longest-processing-time) and, of the most recent timing, the best time in ms of
 * each schedule for stage A (entries 0-2) and stage C (3-5; -1 where not timed).  Any pointer may be
 * null. */
void mpsg_tc_autotune_info(int64_t* tuned, int64_t* cache_hits, int32_t* last_schedule2, float* last_timing6);
/* How often the library's own SVD routes (svd methods 3 and 4) left their fast path: charge sectors
 * redone on the Jacobi route (singular vectors too dependent for CholeskyQR, or more kept vectors
 * than the cluster Cholesky takes), sectors of a two-cluster bidiagonalisation whose barrier wait
 * expired (redone on one cluster), and TEBD splits handed to the complex Jacobi SVD (one per split). */
int64_t mpsg_split_fallbacks(void);
/* Two-site SVD used by split and canonicalisation (BoostSVD, blas/lapack_routines.cpp:614-634):
 * 4 = the library's own exact SVD (default): Householder bidiagonalisation of each charge sector,
 *     singular values by bisection on the Golub-Kahan tridiagonal (absolute accuracy ~eps ||M||, as
 *     dgesvd), computed only down to the global top-chimax cut of the split (all of them down to
 *     1e-15 with doTrunc, whose weight bound needs the norm of all values); singular vectors only
 *     for the kept values (inverse iteration, CholeskyQR, reflector back-transformation).  A split
 *     with a sector of more than about 6900 rows (taken tall) runs on route 0 as a whole; a sector
 *     with more than 1600 kept values has its vectors redone on route 0 (mpsg_split_fallbacks);
 * 0 = one-sided Jacobi SVD of each charge sector (cuSOLVER gesvdj, FP64, exact),
 * 1, 2, 3 = eigen-decomposition of each sector's reduced density matrix G = M^T M (FP64) with the
 *     eigensolver of cuSOLVER batched by size class (1), cuSOLVER per sector on concurrent streams (2)
 *     or the library's own batched eigensolver (3).  The left vectors are re-orthonormalised
 *     (CholeskyQR); singular values below sqrt(32 n eps) of their sector's largest are not resolved
 *     by G and are dropped, and a kept value s carries an absolute error up to ~n eps s_max^2 / s. */
mpsg_status mpsg_ctx_set_svd_method(mpsg_ctx ctx, int32_t method);

/* ------------------------------------------------------------------ tensors
 * nphys: 0 = lambda (DiagBlockMatrix: keys (q,q), blocks are n x 1 vectors),
 *        1 = single-site MPS tensor or environment (q0,q1; p0),
 *        2 = two-site theta (q0,q1; p0,p1).
 * q holds 2*nblocks charge words, p holds nphys*nblocks indices.  host_data
 * holds the blocks in the given order, column-major, concatenated (NULL: zeros).
 * Blocks are stored sorted by key; duplicate keys are an error. */
mpsg_status mpsg_tensor_create(mpsg_ctx ctx, int32_t nphys, int32_t nblocks, const uint64_t* q,
                               const uint32_t* p, const int32_t* rows, const int32_t* cols,
                               const double* host_data, mpsg_tensor* out);
mpsg_status mpsg_tensor_shape(mpsg_tensor t, int32_t* nphys, int32_t* nblocks, int64_t* nelem);
/* Copies structure (sorted key order) and, if host_data != NULL, the payload. */
mpsg_status mpsg_tensor_export(mpsg_tensor t, uint64_t* q, uint32_t* p, int32_t* rows, int32_t* cols,
                               double* host_data);
/* Zero-copy view: device base pointer and the element offset of every block. */
mpsg_status mpsg_tensor_device_view(mpsg_tensor t, double** dptr, int64_t* offsets);
void mpsg_tensor_destroy(mpsg_tensor t);

/* ------------------------------------------------------------------ hot-path drop-ins */

/* contractTwosite(Aout, BL, BR, A, mpol, mpor, itokey)  -- src/MPSfunctions.hpp:949-981.
 * out receives a new tensor holding exactly the blocks the reference creates. */
mpsg_status mpsg_contract_twosite(mpsg_ctx ctx, mpsg_tensor L, mpsg_tensor R, mpsg_tensor theta,
                                  const mpsg_mpo* Wl, const mpsg_mpo* Wr, const mpsg_itokey* ikl,
                                  const mpsg_itokey* ikr, mpsg_prec prec, mpsg_tensor* out);

/* addContractionLayer(BL, A, mpo, itokey, direction)  -- src/MPSfunctions.hpp:442-493.
 * prec: MPSG_PREC_FP64 (the reference's arithmetic), or TF32 / TF32X3 / BF16 / BF16X3: both grouped
 * products on the tensor cores with FP32 accumulation (relative deviation from FP64 of ~1e-7 for
 * TF32X3, ~1e-5 BF16X3, ~1e-3 TF32, ~1e-2 BF16, relative to the largest output entry). */
mpsg_status mpsg_add_contraction_layer(mpsg_ctx ctx, mpsg_tensor BL, mpsg_tensor A, const mpsg_mpo* W,
                                       const mpsg_itokey* ik, int32_t direction, mpsg_prec prec,
                                       mpsg_tensor* out);

/* Persistent matvec plan for repeated application (the Lanczos use of contractTwosite,
 * src/lanzcos.hpp:197): theta_layout fixes the block structure of both the input and the
 * output vector (every block the matvec can reach must be present; see mpsg_theta_closure).
 * The combined environments are built once; execute() is asynchronous on the context stream
 * and reads/writes device arenas laid out like theta_layout (mpsg_tensor_device_view). */
typedef struct mpsg_matvec_plan_s* mpsg_matvec_plan;
mpsg_status mpsg_matvec2_plan_create(mpsg_ctx ctx, mpsg_tensor L, mpsg_tensor R, mpsg_tensor theta_layout,
                                     const mpsg_mpo* Wl, const mpsg_mpo* Wr, const mpsg_itokey* ikl,
                                     const mpsg_itokey* ikr, mpsg_prec prec, mpsg_matvec_plan* out);
mpsg_status mpsg_matvec2_plan_execute(mpsg_matvec_plan plan, const double* theta_in, double* theta_out);
/* mpsg_matvec2_plan_execute for callers that may not allocate device memory: hosts whose own
 * allocator owns the whole GPU memory budget and forbids libraries from allocating, and
 * latency-bound loops that may not block on an allocation.  No counterpart in MPSTools (the reference runs on the CPU).
 * It calls no cudaMalloc / cudaFree or other allocating routine: the stage-A intermediate is
 * kept in a fixed 8 MiB device array inside the library (held by every GPU that loads it until
 * the process exits).  FP64 plans only; plans whose intermediate exceeds 1 Mi FP64 elements are
 * rejected with MPSG_ERR_ARG.  mpsg_ctx_create resolves the array's device address
 * (cudaGetSymbolAddress) for its device, which loads the array when the library is set up; a
 * device reset (cudaDeviceReset) while the library is loaded is not supported.  All calls share
 * the array, so calls that overlap on the GPU (other streams, other threads) race; nothing in
 * it needs clearing, every intermediate block is overwritten before it is read.  Runs on the
 * context's stream, the current device must be the plan's device. */
mpsg_status mpsg_matvec2_plan_execute_noalloc(mpsg_matvec_plan plan, const double* theta_in, double* theta_out);
/* info[0] algorithmic FLOPs of one application, info[1] FLOPs of the reference's per-term
 * schedule, info[2] algorithmic bytes 8*(|L|+|R|+2|theta|), info[3] kernel launches per application. */
mpsg_status mpsg_matvec2_plan_info(mpsg_matvec_plan plan, double* info4);
void mpsg_matvec2_plan_destroy(mpsg_matvec_plan plan);
/* Smallest superset of theta's blocks closed under the matvec (the structure the reference's
 * Lanczos vectors reach); out holds zeros in the added blocks and theta's values elsewhere. */
mpsg_status mpsg_theta_closure(mpsg_ctx ctx, mpsg_tensor L, mpsg_tensor R, mpsg_tensor theta, const mpsg_mpo* Wl,
                               const mpsg_mpo* Wr, const mpsg_itokey* ikl, const mpsg_itokey* ikr,
                               mpsg_tensor* out);

/* Two-tensor addContractionLayer(BL, A, mpo, Ap, itokey, direction): A is the lower (ket) tensor,
 * Ap the upper (bra) one -- src/MPSfunctions.hpp:500-556 (add_out_sub :360-434). */
mpsg_status mpsg_add_contraction_layer2(mpsg_ctx ctx, mpsg_tensor BL, mpsg_tensor A, mpsg_tensor Ap,
                                        const mpsg_mpo* W, const mpsg_itokey* ik, int32_t direction, mpsg_prec prec,
                                        mpsg_tensor* out);
/* computeOverlap(a, b): identity-MPO layers over N sites, a lower and b upper; entry (0,0) of the first
 * block of the final environment -- src/MPSfunctions.hpp:2066-2085. */
mpsg_status mpsg_overlap(mpsg_ctx ctx, int32_t N, const mpsg_tensor* a, const mpsg_tensor* b, const mpsg_itokey* ik,
                         double* out);
/* MPO::measure(mps) for N site tensors and N MPO tensors (energies, local operators as D = 1 MPOs)
 * -- src/MPOTypes.hpp:990-1020. */
mpsg_status mpsg_mpo_measure(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* W,
                             const mpsg_itokey* ik, double* out);

/* BlockMatrix<2>(A1, A2): theta formation  -- src/BlockTensor.hpp:285-301. */
mpsg_status mpsg_theta(mpsg_ctx ctx, mpsg_tensor A1, mpsg_tensor A2, mpsg_tensor* out);

/* split(A, mps, lambda, itokey, 0, chimax, doTrunc, tr_weight, normalize)
 * -- src/MPSfunctions.hpp:1142-1278 (two-site, direction 0): U (left, A-form),
 * lambda (normalised when normalize != 0), Vt (right, B-form). */
mpsg_status mpsg_split2(mpsg_ctx ctx, mpsg_tensor theta, const mpsg_itokey* ikl, const mpsg_itokey* ikr,
                        uint32_t chimax, int32_t doTrunc, double tr_weight, int32_t normalize,
                        mpsg_tensor* U, mpsg_tensor* Vt, mpsg_tensor* lambda, double* tw, uint32_t* chi);

/* TSLanzcosEngine(L,R,mpsl,mpsr,mpol,mpor,itokeyl,itokeyr).simulate(itmax,delta,testenergy)
 * followed by getState(0)  -- src/lanzcos.hpp:100-114,165-278,81-92.
 * reorth != 0 adds full FP64 reorthogonalisation (the reference has none).  testenergy = 0: the
 * reference stops when the residual |H psi - E psi| of the current Ritz vector (one extra matvec
 * every 5 iterations) falls below delta; that test is not implemented here yet, the loop then stops
 * only at breakdown (norm of the new vector < delta) or after itmax iterations.  The same holds for
 * the testenergy argument of the DMRG entry points. */
mpsg_status mpsg_lanczos2(mpsg_ctx ctx, mpsg_tensor L, mpsg_tensor R, mpsg_tensor mpsl, mpsg_tensor mpsr,
                          const mpsg_mpo* Wl, const mpsg_mpo* Wr, const mpsg_itokey* ikl,
                          const mpsg_itokey* ikr, int32_t itmax, double delta, int32_t testenergy,
                          mpsg_prec prec, int32_t reorth, mpsg_tensor* state, double* E0,
                          int32_t* iterations);

/* ------------------------------------------------------------------ DMRG engine
 * DMRGengine<AbKeyType,Real>(mps, mpo)  -- src/container.hpp:236-438.  The engine
 * copies the site tensors; MPO and itokey arrays are copied too. */
mpsg_status mpsg_dmrg_create(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* mpos,
                             const mpsg_itokey* itokeys, mpsg_dmrg* out);
/* prec: Lanczos / matvec arithmetic (the environment updates stay FP64 unless
 * mpsg_dmrg_set_env_prec says otherwise); reorth: full reorthogonalisation in Lanczos;
 * lanmax: Lanczos iteration cap (reference: 500). */
mpsg_status mpsg_dmrg_set_options(mpsg_dmrg e, mpsg_prec prec, int32_t reorth, int32_t lanmax);
/* The options in effect (set by mpsg_dmrg_set_options or restored by mpsg_dmrg_load); any output
 * pointer may be NULL.  No reference counterpart (the reference keeps them as engine members). */
/* Arithmetic of doStep's environment updates (default MPSG_PREC_FP64; TF32 / TF32X3 / BF16 / BF16X3
 * run them on the tensor cores, about five times faster at chi = 2048, but H then carries their
 * ~1e-7 (TF32X3) relative error into every energy: meant for the early sweeps of a chi ramp). */
mpsg_status mpsg_dmrg_set_env_prec(mpsg_dmrg e, mpsg_prec prec);
mpsg_status mpsg_dmrg_get_options(mpsg_dmrg e, int32_t* prec, int32_t* reorth, int32_t* lanmax);
/* DMRGengine::simulate(maxsteps, EnConv, chimax, doTrunc, tr_weight, delta, testenergy):
 * orthonormalize("rl"), computeR, sweeps, final doStep(0,-1).  E = last Lanczos energy.  The
 * reference's two further arguments keep their defaults here: leaveoutlast = false (with true the
 * left sweeps skip doStep(N-2, -1): schedule the sweeps with mpsg_dmrg_prepare / mpsg_dmrg_do_step)
 * and targetstate = 0 (the Lanczos ground state; for excited states see mpsg_dmrg_excited_simulate). */
mpsg_status mpsg_dmrg_simulate(mpsg_dmrg e, uint32_t maxsteps, double EnConv, uint32_t chimax,
                               int32_t doTrunc, double tr_weight, double delta, int32_t testenergy,
                               double* E);
/* The pieces of simulate, for callers that schedule sweeps themselves. */
mpsg_status mpsg_dmrg_prepare(mpsg_dmrg e);
mpsg_status mpsg_dmrg_do_step(mpsg_dmrg e, int32_t site, int32_t dir, uint32_t chimax, int32_t doTrunc,
                              double tr_weight, double delta, int32_t testenergy, double* E);
/* Environments of the current MPS without canonicalising it: L[-1..center-1] from the left
 * edge and R[N..center+2] from the right edge (getLMin / getRMax / addContractionLayer), so a
 * mixed-canonical state (e.g. a checkpoint) can be resumed at bond (center, center+1). */
mpsg_status mpsg_dmrg_build_environments(mpsg_dmrg e, int32_t center);
/* Copy of an environment: which = 0 for L[site], 1 for R[site]. */
mpsg_status mpsg_dmrg_env(mpsg_dmrg e, int32_t which, int32_t site, mpsg_tensor* out);
/* Step records appended by every doStep. */
int32_t mpsg_dmrg_nsteps(mpsg_dmrg e);
mpsg_status mpsg_dmrg_steps(mpsg_dmrg e, int32_t* site, int32_t* dir, int32_t* iters, int32_t* chi,
                            double* E, double* tw);
/* Accumulated counters: [0] matvecs, [1] matvec FLOPs (algorithmic), [2] Lanczos iteration
 * seconds (device events around the batched iterations), [3] env-update seconds, [4] split
 * seconds, [5] Lanczos seconds (wall), [6] env-update FLOPs, [7] wall seconds of simulate,
 * [8] device seconds of all doStep calls (events), [9] number of doStep calls. */
mpsg_status mpsg_dmrg_stats(mpsg_dmrg e, double* stats10);
/* The counters of mpsg_dmrg_stats followed by [10] wall seconds of doStep before the eigensolver
 * (theta layout, closure and formation) and [11] wall seconds of the eigensolver calls (matvec plan,
 * Lanczos, MIXED's FP64 energy, AUTO's FP64 finish); the first min(n, 12) entries are written. */
mpsg_status mpsg_dmrg_stats_ext(mpsg_dmrg e, double* stats, int32_t n);
mpsg_status mpsg_dmrg_site(mpsg_dmrg e, int32_t site, mpsg_tensor* out);
mpsg_status mpsg_dmrg_lambda(mpsg_dmrg e, int32_t bond, mpsg_tensor* out);
/* MPO::measure(mps) in FP64 on the GPU  -- src/MPOTypes.hpp:990-1020. */
mpsg_status mpsg_dmrg_measure_energy(mpsg_dmrg e, double* E);
/* MPO::measure of the engine's state with another MPO (N tensors), e.g. a local operator
 * -- src/MPOTypes.hpp:990-1020. */
mpsg_status mpsg_dmrg_measure_mpo(mpsg_dmrg e, const mpsg_mpo* W, double* out);

/* ---------------------------------------------------------------- TEBD (complex FP64, Vidal form)
 * TEBDengine (src/container.hpp:1195-1406) from a product state: Gamma tensors complex (planar on
 * the device), lambdas real.  The two-site gate of bond b is exp(-i dt h_b) built from the MPO like
 * MPO::getNNGate (src/MPOTypes.hpp:1090-1209); each bond update is applyGate
 * (src/MPSfunctions.hpp:1492-1548) with the complex split (per charge sector the context's SVD
 * method: by default the library's complex bidiagonal SVD, cuSOLVER's zgesvdj for method 0 and where
 * a split does not fit the bidiagonal route; complex FixPhase, the reference's truncation,
 * dropDangling, squeeze(1e-15)). */
typedef struct mpsg_tebd_s* mpsg_tebd;
/* local_state[s]: index into ik[s] of site s (e.g. the Neel state s % 2). */
mpsg_status mpsg_tebd_create(mpsg_ctx ctx, int32_t N, const int32_t* local_state, const mpsg_mpo* W,
                             const mpsg_itokey* ik, mpsg_tebd* out);
/* Second-order Trotter evolution (TEBDengine::simulate "second" without intermediate measurements):
 * odd bonds dt/2, then steps x (even dt, odd dt) with the last odd step dt/2. */
mpsg_status mpsg_tebd_second_order(mpsg_tebd e, int32_t steps, double dt, uint32_t chimax, int32_t doTrunc,
                                   double tr_weight, int32_t normalize);
/* SparseLocalOperator::measure (src/MPOTypes.hpp:532-563) of a diagonal operator on
 * lambda(site-1) Gamma(site) lambda(site). */
mpsg_status mpsg_tebd_measure_diag(mpsg_tebd e, int32_t site, const double* op_diag, int32_t d, double* out);
/* lambda of bond b (b = -1 .. N-1) as an nphys = 0 tensor (n x 1 blocks keyed (q, q)). */
mpsg_status mpsg_tebd_lambda(mpsg_tebd e, int32_t bond, mpsg_tensor* out);
/* Gamma(site): block table and interleaved (re, im) column-major data in key order. */
mpsg_status mpsg_tebd_gamma_shape(mpsg_tebd e, int32_t site, int32_t* nblocks, int64_t* nelem);
mpsg_status mpsg_tebd_gamma_export(mpsg_tebd e, int32_t site, uint64_t* q, uint32_t* p, int32_t* rows,
                                   int32_t* cols, double* data_interleaved);
/* wall seconds of the evolution, of the split part, and bond updates applied. */
mpsg_status mpsg_tebd_stats(mpsg_tebd e, double* seconds, double* split_seconds, int64_t* gates);
/* 1 (default): the disjoint bonds of a time slice are updated together (one theta formation, split
 * and scatter for the slice, gates / truncation / normalisation per bond); 0: one bond at a time
 * (doTimeSlice order).  The results are the same. */
mpsg_status mpsg_tebd_set_batch_layers(mpsg_tebd e, int32_t batch_layers);
void mpsg_tebd_destroy(mpsg_tebd e);
/* MPO::getNNGate: dense (d1 d2) x (d1 d2) gate exp(-(dt_im + i dt_re) h_b), index o1 + d1*o2,
 * column-major, interleaved complex -- src/MPOTypes.hpp:1090-1209. */
mpsg_status mpsg_nn_gate(const mpsg_mpo* W1, const mpsg_mpo* W2, int32_t site1, int32_t N, double dt_re, double dt_im,
                         int32_t d1, int32_t d2, double* out_interleaved);
/* The bond Hamiltonian h_b that MPO::getNNGate exponentiates (boundary-aware one-half weights of
 * the on-site terms), real (d1 d2) x (d1 d2), index o1 + d1*o2, column-major
 * -- src/MPOTypes.hpp:1090-1209. */
mpsg_status mpsg_bond_hamiltonian(const mpsg_mpo* W1, const mpsg_mpo* W2, int32_t site1, int32_t N, int32_t d1,
                                  int32_t d2, double* out);
/* Tangent of the gate G = exp(-i dt h_b) along a real symmetric direction dh (d1 d2 square, same
 * index): (dG/dtheta) G^H for h_b(theta) with dh_b/dtheta = dh, interleaved complex.  Used by the
 * TEBD adjoint; no counterpart in the reference (MPO::getNNGate, src/MPOTypes.hpp:1090-1209, is the
 * gate it differentiates). */
mpsg_status mpsg_nn_gate_tangent(const mpsg_mpo* W1, const mpsg_mpo* W2, int32_t site1, int32_t N, double dt,
                                 const double* dh, int32_t d1, int32_t d2, double* out_interleaved);
/* TEBD adjoint (no counterpart in the reference, which has no gradients; the forward map is
 * TEBDengine::simulate "second", src/container.hpp:1272-1406): runs the schedule of
 * mpsg_tebd_second_order (normalised, same truncation) from the engine's current state, returns
 * value = <O> of the diagonal operator obs_diag (d entries) on site obs_site at the end, and
 * grad[b] = d value / d theta_b for one parameter per bond entering h_b with derivative dh_b:
 * dh holds N-1 real matrices, bond b's of size (d_b d_{b+1})^2 (index o1 + d_b o2, column-major),
 * one after another.  Truncation and renormalisation are not differentiated (exact when nothing is
 * truncated).  The forward states are kept every checkpoint_every layers (<= 0: about the square
 * root of the layer count) and recomputed segment by segment in the backward pass.  The engine ends
 * at the evolved state, as after mpsg_tebd_second_order. */
mpsg_status mpsg_tebd_adjoint_second_order(mpsg_tebd e, int32_t steps, double dt, uint32_t chimax, int32_t doTrunc,
                                           double tr_weight, int32_t obs_site, const double* obs_diag, int32_t d,
                                           const double* dh, int32_t checkpoint_every, double* value, double* grad);
/* wall seconds spent in mpsg_tebd_adjoint_second_order (forward, recomputation and backward). */
mpsg_status mpsg_tebd_adjoint_seconds(mpsg_tebd e, double* seconds);
void mpsg_dmrg_destroy(mpsg_dmrg e);
/* DMRGengine::simulate(mps, delta_ortho, ...) (src/container.hpp:441-570): two-site DMRG whose Lanczos
 * keeps every Krylov vector orthogonal to the target state (N site tensors, e.g. a converged ground
 * state), in the current basis through overlap environments; E = the last step's energy (the lowest
 * state orthogonal to the target in the engine's sector).  delta_ortho is accepted and unused, as in
 * the reference.  Deviation: the reference's last update forms the target's two-site state from its
 * site 0 twice; here from sites 0 and 1. */
mpsg_status mpsg_dmrg_excited_simulate(mpsg_dmrg e, const mpsg_tensor* target, double delta_ortho, uint32_t maxsteps,
                                       double EnConv, uint32_t chimax, int32_t doTrunc, double tr_weight, double delta,
                                       int32_t testenergy, int32_t leaveoutlast, double* E);
/* applyMPO (src/MPSfunctions.hpp:2088-2346): the exact product W|psi> of an MPO (N tensors) and an MPS
 * (N site tensors); out receives N new site tensors.  New bond charges are propagated from the left
 * ((b, w) takes charge(a, w') + q(s_out) when first seen); a new charge sector is the direct sum over
 * the MPO channels of the old sectors that reach it (largest size per channel, zero padding). */
mpsg_status mpsg_apply_mpo(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* W, const mpsg_itokey* ik,
                           mpsg_tensor* out);
/* compressTwoSite (src/MPSfunctions.hpp:2797-2940): variational two-site fit of W|psi> at bond
 * dimension <= chimax (initial guess: W applied to psi truncated to chimax / D, D the MPO dimension
 * at site 1; sweeps until the convergence measure grows, maxstep sweeps or |conv| < delta).  out
 * receives the fitted site tensors, conv the reference's measure (n1^2 + n2^2 - 2 |<fit|psi>|) / n1^2
 * (its overlap term is with psi, as the reference computes it). */
mpsg_status mpsg_compress_two_site(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* W,
                                   const mpsg_itokey* ik, uint32_t chimax, uint32_t maxstep, double delta,
                                   int32_t doTrunc, double tr_weight, mpsg_tensor* out, double* conv);
/* compress (src/MPSfunctions.hpp:2349-2510): variational single-site compression of psi to bond
 * dimension <= chimax.  psi is first swept with prepareSite (left over sites 0 .. N-2, right over
 * N-2 .. 1; with normalize over all sites, which normalises it); the initial guess is psi truncated to
 * chimax with those lambdas; single-site sweeps (contractSingle with the identity MPO) until the
 * measure grows, maxstep sweeps or |conv| < delta; site 0 fitted once more; the fit left and right
 * canonicalised.  out receives the fit, conv = |fit - psi|^2 / |psi|^2.  maxstep must be >= 1 (with 0 the
 * reference reads an environment it never built). */
mpsg_status mpsg_compress(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_itokey* ik, uint32_t chimax,
                          uint32_t maxstep, double delta, int32_t normalize, mpsg_tensor* out, double* conv);
/* compressSingleSite (src/MPSfunctions.hpp:2667-2792): variational single-site fit of W|psi> (the
 * initial guess and the measure as mpsg_compress_two_site; the bond dimensions stay those of the
 * initial guess). */
mpsg_status mpsg_compress_single_site(mpsg_ctx ctx, int32_t N, const mpsg_tensor* sites, const mpsg_mpo* W,
                                      const mpsg_itokey* ik, uint32_t chimax, uint32_t maxstep, double delta,
                                      mpsg_tensor* out, double* conv);
/* SSDMRGengine::simulate (src/container.hpp:827-925): single-site DMRG (no bond growth) from the
 * engine's state: orthonormalize("rl"), sweeps until |dE| < EnConv or more than maxsteps sweeps, then
 * doStep(0, -1); E = the last step's energy.  Each update is SSLanzcosEngine on one site
 * (contractSingle, src/MPSfunctions.hpp:857-885) and prepareSite without truncation; the matvec
 * precision of mpsg_dmrg_set_options applies. */
mpsg_status mpsg_dmrg_ss_simulate(mpsg_dmrg e, uint32_t maxsteps, double EnConv, double delta, int32_t testenergy,
                                  double* E);
/* Portable checkpoint of the engine's state (what MPSBase::save keeps, src/MPSTypes.hpp:377-426, in a
 * documented little-endian format instead of a Boost binary archive): per site the charge map, the
 * MPO tensor and the site tensor, then the lambdas.  Format "MPSGCKP1": see checkpoint.cpp; the
 * Python module mpstools_gb300.checkpoint reads and writes the same files (e.g. for states made by
 * the CPU oracle).  mpsg_dmrg_load creates an engine on ctx; simulate() or build_environments()
 * continues from the loaded state.  Version-2 files also keep the engine's options (matvec
 * precision, reorthogonalisation, Lanczos limit), which load restores; version-1 files load with the
 * FP64 defaults.  The environment-update precision (mpsg_dmrg_set_env_prec) is not kept: a loaded
 * engine updates its environments in FP64 until it is set again.  The loader rejects (MPSG_ERR_ARG) files whose indices fall outside the declared
 * MPO / local dimensions or whose declared sizes exceed the file, before allocating for them. */
mpsg_status mpsg_dmrg_save(mpsg_dmrg e, const char* path);
mpsg_status mpsg_dmrg_load(mpsg_ctx ctx, const char* path, mpsg_dmrg* out);

/* ---------------------------------------------------------------- batched chains
 * Many independent DMRGengine runs (src/container.hpp:292-438) in lockstep: every global step each
 * chain performs its own next doStep, and the work of all chains goes through one launch per matvec
 * stage, one batched split and one environment update per sweep direction (the chains form a
 * block-diagonal direct sum: charges of chain i shifted by i << 32, MPO channels concatenated).
 * Lanczos reductions, convergence, truncation and normalisation stay per chain.  No counterpart in
 * the reference, which runs one chain per process; the per-chain results follow DMRGengine. */
typedef struct mpsg_batch_s* mpsg_batch;
/* chains: engines created with mpsg_dmrg_create on ctx (charges below 2^32, the same i_to_key at the
 * sites that update together); they must outlive the batch and are updated in place. */
mpsg_status mpsg_batch_create(mpsg_ctx ctx, int32_t nchains, const mpsg_dmrg* chains, mpsg_batch* out);
/* matvec precision (FP64, a mixed mode, AUTO or MIXED: per chain the FP64 Rayleigh quotient of its
 * TF32X3 ground state, one FP64 matvec of the direct sum for all chains) and the Lanczos iteration
 * cap of every chain. */
mpsg_status mpsg_batch_set_options(mpsg_batch b, mpsg_prec prec, int32_t lanmax);
/* DMRGengine::simulate of every chain with exactly `sweeps` sweeps (orthonormalize("rl"), then the
 * sweeps, then the final doStep(0, -1)); energies[c] = the last step's energy of chain c.  Each
 * chain's step records are available through mpsg_dmrg_steps. */
mpsg_status mpsg_batch_simulate(mpsg_batch b, uint32_t sweeps, uint32_t chimax, int32_t doTrunc, double tr_weight,
                                double delta, int32_t testenergy, double* energies);
/* st[11]: global steps, chain steps, matvecs (one per lockstep iteration), matvec FLOPs (all chains),
 * matvec kernel launches, Lanczos seconds, split seconds, environment seconds, wall seconds, device
 * seconds of the sweeps, seconds of the preparation (orthonormalisation and right environments). */
mpsg_status mpsg_batch_stats(mpsg_batch b, double* st);
void mpsg_batch_destroy(mpsg_batch b);

#ifdef __cplusplus
}
#endif
#endif /* MPSG_H_ */
