// ============================================================================
// oracle.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// A CPU restatement, in plain C++17 with OpenMP, of the MPSTools DMRG hot path.
// It exists only to check the GPU library (tests/), to be run once inside
// __graft_entry__.smoke() as the checker, and to be timed as the CPU baseline
// in bench.py.  Nothing in mpstools_gb300/ links, loads or calls it.
//
// What it restates (reference paths are relative to the MPSTools tree):
//   AbKeyType / TensorKeyType ordering ............ src/keyTypes.hpp:20-124,166-343
//   BlockMatrix<2>(A1,A2) theta formation ......... src/BlockTensor.hpp:285-301
//   BlockMatrix scalar product / +=, *= .......... src/BlockTensor.hpp:443-544
//   DiagBlockMatrix::truncate(chimax) ............. src/BlockTensor.hpp:234-276
//   DiagBlockMatrix::truncate(tr_weight,chimax) ... src/BlockTensor.hpp:85-136
//   lambda*B, B*lambda ............................ src/BlockTensor.hpp:653-690
//   add_out_sub_2 / addContractionLayer ........... src/MPSfunctions.hpp:276-352,442-493
//   doContraction / contractTwosite ............... src/MPSfunctions.hpp:726-804,949-981
//   split (two-site) .............................. src/MPSfunctions.hpp:1142-1278
//   dropDangling(L,lambda,R) ...................... src/MPSfunctions.hpp:1444-1484
//   prepareBlock / prepareMatrix .................. src/MPSfunctions.hpp:21-269
//   prepareSite / orthonormalize .................. src/MPSTypes.hpp:585-621, src/MPSfunctions.hpp:1756-1792
//   getLMin / getRMax / computeR .................. src/MPSfunctions.hpp:1917-2037
//   TSLanzcosEngine::simulate / getState .......... src/lanzcos.hpp:81-92,165-278
//   DMRGengine::doStep / simulate ................. src/container.hpp:292-337,381-438
//   MPO::measure .................................. src/MPOTypes.hpp:990-1020
//   MPO::getNNGate (two-site gate exp(-i dt h_b)) . src/MPOTypes.hpp:1090-1209
//   applyGate ..................................... src/MPSfunctions.hpp:1492-1548
//   TEBDengine doTimeSlice / second-order simulate  src/container.hpp:1195-1233,1325-1395
//   SparseLocalOperator::measure (on lambda Gamma lambda) src/MPOTypes.hpp:532-563
//   complex FixPhase .............................. blas/helperfunctions.hpp:52-67
//   HeisenbergMPO / SpinlessFermionsMPO ........... src/Hamiltonians.hpp:84-131,527-566
//   SparseOperator product ........................ src/MPOTypes.hpp:200-230
//   BoostSVD -> rsvd (dgesvd 'S','S') + FixPhase .. blas/lapack_routines.cpp:334-366,614-634,
//                                                   blas/helperfunctions.hpp:36-51
//   tridiag -> dstev .............................. blas/lapack_routines.cpp:429-445
//   cut ........................................... blas/helperfunctions.hpp:69-89
//
// Dense BLAS/LAPACK come from the OpenBLAS that numpy/scipy bundle, opened with
// dlopen at run time (the same Fortran routines the reference calls through MKL:
// dgemm, ddot, dgesvd, dstev).
//
// Parity unpinned: MPSTools ships no tests, fixtures or golden vectors, and it
// cannot be built here (Boost and MKL are absent), so no output of the
// reference itself checks this restatement.  It is checked instead against
// independent answers: exact diagonalisation energies, dense contractions of
// the same operands, and numpy restatements of the reference's split,
// truncation and Lanczos (tests/).
// ============================================================================
#include <dlfcn.h>
#include <omp.h>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <map>
#include <set>
#include <string>
#include <vector>
#include <algorithm>
#include <complex>

namespace orc {

typedef uint64_t Q;  // packed U(1) charge word (AbKeyType::_qn)

// ---------------------------------------------------------------- BLAS binding
typedef void (*dgemm_t)(const char*, const char*, const int*, const int*, const int*,
                        const double*, const double*, const int*, const double*, const int*,
                        const double*, double*, const int*, size_t, size_t);
typedef double (*ddot_t)(const int*, const double*, const int*, const double*, const int*);
typedef void (*dgesvd_t)(const char*, const char*, const int*, const int*, double*, const int*,
                         double*, double*, const int*, double*, const int*, double*, const int*,
                         int*, size_t, size_t);
typedef void (*dstev_t)(const char*, const int*, double*, double*, double*, const int*, double*,
                        int*, size_t);
typedef void (*setthreads_t)(int);

static dgemm_t p_dgemm = nullptr;
static ddot_t p_ddot = nullptr;
static dgesvd_t p_dgesvd = nullptr;
static dstev_t p_dstev = nullptr;

static void* sym(void* h, const char* a, const char* b) {
  void* p = dlsym(h, a);
  if (!p) p = dlsym(h, b);
  return p;
}

// ---------------------------------------------------------------- dense matrix
struct Mat {
  int r = 0, c = 0;
  std::vector<double> d;  // column-major
  Mat() {}
  Mat(int r_, int c_) : r(r_), c(c_), d((size_t)r_ * c_, 0.0) {}
  double& operator()(int i, int j) { return d[(size_t)i + (size_t)j * r]; }
  double operator()(int i, int j) const { return d[(size_t)i + (size_t)j * r]; }
};

// out = alpha * op(A) * op(B)   (MatMatProd, blas/blasroutines.cpp:837-849)
static Mat gemm(double alpha, const Mat& A, char ta, const Mat& B, char tb) {
  int m = (ta == 'n') ? A.r : A.c;
  int k = (ta == 'n') ? A.c : A.r;
  int n = (tb == 'n') ? B.c : B.r;
  Mat C(m, n);
  if (m == 0 || n == 0) return C;
  if (k == 0) return C;
  int lda = std::max(1, A.r), ldb = std::max(1, B.r), ldc = std::max(1, m);
  double beta = 0.0;
  char TA = ta == 'n' ? 'N' : 'T', TB = tb == 'n' ? 'N' : 'T';
  p_dgemm(&TA, &TB, &m, &n, &k, &alpha, A.d.data(), &lda, B.d.data(), &ldb, &beta, C.d.data(),
          &ldc, 1, 1);
  return C;
}
static void addto(Mat& y, const Mat& x) {
  for (size_t i = 0; i < y.d.size(); ++i) y.d[i] += x.d[i];
}
static void scale(Mat& y, double s) {
  for (auto& v : y.d) v *= s;
}
static double dot(size_t n, const double* a, const double* b) {
  // ddot_ with int sizes; blocks never exceed 2^31 elements here
  int nn = (int)n, one = 1;
  if (nn == 0) return 0.0;
  return p_ddot(&nn, a, &one, b, &one);
}

// BoostSVD: U (m x k), D (k), Vt (k x n), k=min(m,n); dgesvd 'S','S' then FixPhase.
static int svd(const Mat& M, Mat& U, std::vector<double>& D, Mat& Vt) {
  int m = M.r, n = M.c, k = std::min(m, n);
  U = Mat(m, k);
  Vt = Mat(k, n);
  D.assign(k, 0.0);
  if (k == 0) return 0;
  Mat A = M;
  char J = 'S';
  int lda = m, ldu = m, ldvt = k, info = 0;
  int lwork = -1;
  double wq = 0;
  p_dgesvd(&J, &J, &m, &n, A.d.data(), &lda, D.data(), U.d.data(), &ldu, Vt.d.data(), &ldvt, &wq,
           &lwork, &info, 1, 1);
  lwork = std::max((int)wq, std::max(3 * k + std::max(m, n), 5 * k));
  std::vector<double> work(lwork);
  p_dgesvd(&J, &J, &m, &n, A.d.data(), &lda, D.data(), U.d.data(), &ldu, Vt.d.data(), &ldvt,
           work.data(), &lwork, &info, 1, 1);
  // FixPhase: sign of the (first) abs-max entry of each row of Vt made positive
  for (int i = 0; i < k; ++i) {
    int ind = 0;
    double val = 0;
    for (int j = 0; j < n; ++j)
      if (std::fabs(Vt(i, j)) > val) { val = std::fabs(Vt(i, j)); ind = j; }
    double phi = Vt(i, ind) > 0 ? 1.0 : -1.0;
    for (int j = 0; j < n; ++j) Vt(i, j) *= phi;
    for (int j = 0; j < m; ++j) U(j, i) *= phi;
  }
  return info;
}

// tridiag: dstev on diag (n) / sub (n-1); eigenvalues ascending overwrite diag
static int tridiag(std::vector<double>& diag, std::vector<double> sub, std::vector<double>* z) {
  int n = (int)diag.size();
  if (n == 0) return 0;
  sub.resize(std::max(1, n - 1));
  char J = z ? 'V' : 'N';
  int ldz = std::max(1, n), info = 0;
  std::vector<double> work(std::max(1, 2 * n - 2));
  std::vector<double> dummy(1);
  double* zp = dummy.data();
  if (z) { z->assign((size_t)n * n, 0.0); zp = z->data(); }
  p_dstev(&J, &n, diag.data(), sub.data(), zp, &ldz, work.data(), &info, 1);
  return info;
}

// ---------------------------------------------------------------- keys
// TensorKeyType<2,Ns,AbKeyType>: ordered by charge [0], charge [1], then the
// physical/MPO indices (0),(1) -- src/keyTypes.hpp:276-303
struct Key {
  Q q0 = 0, q1 = 0;
  uint32_t p0 = 0, p1 = 0;  // p1 unused for single-site keys (always 0)
  bool operator<(const Key& o) const {
    if (q0 != o.q0) return q0 < o.q0;
    if (q1 != o.q1) return q1 < o.q1;
    if (p0 != o.p0) return p0 < o.p0;
    return p1 < o.p1;
  }
  bool operator==(const Key& o) const {
    return q0 == o.q0 && q1 == o.q1 && p0 == o.p0 && p1 == o.p1;
  }
};
static Key K1(Q a, Q b, uint32_t p) { Key k; k.q0 = a; k.q1 = b; k.p0 = p; return k; }
static Key K2(Q a, Q b, uint32_t p, uint32_t pp) { Key k; k.q0 = a; k.q1 = b; k.p0 = p; k.p1 = pp; return k; }

typedef std::map<Key, Mat> BM;                   // BlockMatrix<Ns,AbKeyType,Real>
typedef std::map<Q, std::vector<double>> Diag;   // DiagBlockMatrix<AbKeyType,Real>

// OpKeyType<1>: [0]=in, (0)=out; map order is (in, out)
struct OpKey {
  uint32_t in, out;
  bool operator<(const OpKey& o) const { return in != o.in ? in < o.in : out < o.out; }
};
typedef std::map<OpKey, double> SparseOp;
struct WKey {
  uint32_t wl, wr;
  bool operator<(const WKey& o) const { return wl != o.wl ? wl < o.wl : wr < o.wr; }
};
struct MPOMat {
  std::map<WKey, SparseOp> m;
  int Dl = 0, Dr = 0;
};
typedef std::vector<Q> ItoKey;

// ---------------------------------------------------------------- BlockMatrix ops
static double bm_dot(const BM& a, const BM& b) {  // BlockMatrix::operator* (BlockTensor.hpp:521-544)
  double v = 0;
  for (auto& x : a) {
    auto it = b.find(x.first);
    if (it == b.end()) continue;
    v += dot(x.second.d.size(), it->second.d.data(), x.second.d.data());
  }
  return v;
}
static void bm_scale(BM& a, double s) { for (auto& x : a) scale(x.second, s); }
static void bm_add(BM& a, const BM& b) {  // operator+= (BlockTensor.hpp:443-462)
  for (auto& x : b) {
    auto it = a.find(x.first);
    if (it == a.end()) a[x.first] = x.second; else addto(it->second, x.second);
  }
}
static BM bm_scaled(const BM& a, double s) { BM c = a; bm_scale(c, s); return c; }
static void merge(BM& a, const BM& b) { for (auto& x : b) a[x.first] = x.second; }

// BlockMatrix<2>(B1,B2): theta formation (BlockTensor.hpp:285-301)
static BM theta_form(const BM& B1, const BM& B2) {
  BM out;
  for (auto& a : B1)
    for (auto& b : B2)
      if (a.first.q1 == b.first.q0)
        out[K2(a.first.q0, b.first.q1, a.first.p0, b.first.p0)] = gemm(1.0, a.second, 'n', b.second, 'n');
  return out;
}

// lambda*B : rows scaled by lambda[B.q0] ; B*lambda : columns scaled by lambda[B.q1]
static BM lam_times(const Diag& lam, const BM& B) {
  BM out;
  for (auto& b : B) {
    auto l = lam.find(b.first.q0);
    if (l == lam.end()) continue;
    Mat t = b.second;
    for (int j = 0; j < t.c; ++j)
      for (int i = 0; i < t.r; ++i) t(i, j) *= l->second[i];
    out[b.first] = t;
  }
  return out;
}
static BM times_lam(const BM& B, const Diag& lam) {
  BM out;
  for (auto& b : B) {
    auto l = lam.find(b.first.q1);
    if (l == lam.end()) continue;
    Mat t = b.second;
    for (int j = 0; j < t.c; ++j)
      for (int i = 0; i < t.r; ++i) t(i, j) *= l->second[j];
    out[b.first] = t;
  }
  return out;
}

static double diag_norm(const Diag& l) {
  double n = 0;
  for (auto& x : l) n += dot(x.second.size(), x.second.data(), x.second.data());
  return std::sqrt(n);
}
static void diag_normalize(Diag& l) {
  double n = diag_norm(l);
  for (auto& x : l)
    for (auto& v : x.second) v *= 1.0 / n;
}

// DiagBlockMatrix::truncate(chimax): keep top-chi values (> 1e-15) of a multimap
// sorted by value; among equal values the later-inserted one comes first.
static std::pair<double, int> truncate_chi(Diag& lam, int chi, bool normalize) {
  std::multimap<double, Q> m;
  for (auto& x : lam)
    for (double v : x.second) m.insert(std::make_pair(v, x.first));
  std::multimap<Q, double> im;
  int cnt = 0;
  double tw = 1.0;
  for (auto r = m.rbegin(); r != m.rend() && cnt != chi && std::fabs(r->first) > 1e-15; ++r) {
    tw -= r->first * r->first;
    im.insert(std::make_pair(r->second, r->first));
    ++cnt;
  }
  lam.clear();
  for (auto& x : im) lam[x.first].push_back(x.second);
  if (normalize) diag_normalize(lam);
  return std::make_pair(tw, cnt);
}
// DiagBlockMatrix::truncate(tr_weight, chimax)
static std::pair<double, int> truncate_tw(Diag& lam, double tr_weight, int chimax, bool normalize) {
  std::multimap<double, Q> m;
  double tw = diag_norm(lam), norm = diag_norm(lam);
  for (auto& x : lam)
    for (double v : x.second) m.insert(std::make_pair(v, x.first));
  std::multimap<Q, double> im;
  int chi = 0;
  for (auto r = m.rbegin(); r != m.rend() && std::fabs(tw) > norm * tr_weight && chi < chimax; ++r) {
    tw -= (r->first * r->first) / norm;
    im.insert(std::make_pair(r->second, r->first));
    ++chi;
  }
  if (tw < 0 && std::fabs(tw) < 1e-14) tw = 0.0;
  lam.clear();
  for (auto& x : im) lam[x.first].push_back(x.second);
  if (normalize) diag_normalize(lam);
  return std::make_pair(tw, chi);
}

// dropDangling(L, lambda, R) (MPSfunctions.hpp:1444-1484)
static void drop_dangling(BM& L, const Diag& lam, BM& R) {
  for (auto it = L.begin(); it != L.end();) {
    auto l = lam.find(it->first.q1);
    if (l == lam.end()) { it = L.erase(it); continue; }
    int k = (int)l->second.size();
    if (it->second.c > k) {
      Mat t(it->second.r, k);
      for (int j = 0; j < k; ++j)
        for (int i = 0; i < t.r; ++i) t(i, j) = it->second(i, j);
      it->second = t;
    }
    ++it;
  }
  for (auto it = R.begin(); it != R.end();) {
    auto l = lam.find(it->first.q0);
    if (l == lam.end()) { it = R.erase(it); continue; }
    int k = (int)l->second.size();
    if (it->second.r > k) {
      Mat t(k, it->second.c);
      for (int j = 0; j < t.c; ++j)
        for (int i = 0; i < k; ++i) t(i, j) = it->second(i, j);
      it->second = t;
    }
    ++it;
  }
}

// ---------------------------------------------------------------- env update
// add_out_sub_2 (MPSfunctions.hpp:276-352); with a separate upper tensor Ap it is add_out_sub
// (MPSfunctions.hpp:360-434): lower blocks from A, upper blocks from Ap.
static BM add_out_sub_2(const std::map<uint32_t, std::vector<BM::const_iterator>>& BLits, const BM& A,
                        const MPOMat& mpo, Q p, const ItoKey& ik, int direction, const BM* Ap = nullptr) {
  const BM& Aup = Ap ? *Ap : A;
  const int idir = direction > 0 ? 1 : 0;
  BM B;
  for (auto& a : A)
    if ((idir ? a.first.q1 : a.first.q0) == p) B[a.first] = a.second;
  BM Bout;
  static const std::vector<BM::const_iterator> empty;
  for (auto& o : mpo.m) {
    const uint32_t kwo[2] = {o.first.wl, o.first.wr};
    const uint32_t o_in = kwo[1 - idir];
    for (auto& oi : o.second) {
      Q kyout = ik[oi.first.out];
      Key key_b = direction > 0 ? K1(p - kyout, p, oi.first.out) : K1(p, p + kyout, oi.first.out);
      auto posb = B.find(key_b);
      if (posb == B.end()) continue;
      auto bl = BLits.find(o_in);
      const std::vector<BM::const_iterator>& its = bl == BLits.end() ? empty : bl->second;
      for (auto itBL : its) {
        const Key& kb = itBL->first;
        if (direction > 0 && kb.p0 != kwo[0]) continue;
        if (direction <= 0 && kb.p0 != kwo[1]) continue;
        if (direction > 0 && kb.q1 != key_b.q0) continue;
        if (direction <= 0 && kb.q1 != key_b.q1) continue;
        Q kyin = ik[oi.first.in];
        Key key_a = direction > 0 ? K1(kb.q0, kb.q0 + kyin, oi.first.in) : K1(kb.q0 - kyin, kb.q0, oi.first.in);
        auto posa = Aup.find(key_a);
        if (posa == Aup.end()) continue;
        Mat T2;
        if (direction > 0) {
          Mat T1 = gemm(1.0, itBL->second, 't', posa->second, 'n');
          T2 = gemm(1.0, T1, 't', posb->second, 'n');
        } else {
          Mat T1 = gemm(1.0, posa->second, 'n', itBL->second, 'n');
          T2 = gemm(1.0, T1, 'n', posb->second, 't');
        }
        scale(T2, oi.second);
        Key ky = idir ? K1(key_a.q1, key_b.q1, kwo[1]) : K1(key_a.q0, key_b.q0, kwo[0]);
        auto y = Bout.find(ky);
        if (y != Bout.end()) addto(T2, y->second);
        Bout[ky] = T2;
      }
    }
  }
  return Bout;
}

// addContractionLayer (MPSfunctions.hpp:442-493); the two-tensor overload (MPSfunctions.hpp:500-556)
// when Ap is given (A lower, Ap upper)
static BM add_contraction_layer(const BM& BL, const BM& A, const MPOMat& mpo, const ItoKey& ik,
                                int direction, int maxthreads, const BM* Ap = nullptr) {
  const int idir = direction > 0 ? 1 : 0;
  std::set<Q> outs;
  for (auto& a : A) outs.insert(idir ? a.first.q1 : a.first.q0);
  std::vector<Q> outgoing(outs.begin(), outs.end());
  std::map<uint32_t, std::vector<BM::const_iterator>> BLits;
  for (auto it = BL.begin(); it != BL.end(); ++it) BLits[it->first.p0].push_back(it);
  std::vector<BM> bouts(maxthreads);
  const int n = (int)outgoing.size();
#pragma omp parallel for num_threads(maxthreads) schedule(dynamic)
  for (int i = 0; i < n; ++i) {
    BM Bi = add_out_sub_2(BLits, A, mpo, outgoing[i], ik, direction, Ap);
    merge(bouts[omp_get_thread_num()], Bi);
  }
  BM out;
  for (auto& b : bouts) merge(out, b);
  return out;
}

// ---------------------------------------------------------------- matvec
// doContraction (two-site) (MPSfunctions.hpp:726-804)
static void do_contraction(BM& Aout, const std::vector<BM::const_iterator>& BLits, const BM& BR,
                           const BM& Ain, const MPOMat& mpol, const MPOMat& mpor, const ItoKey& ik0,
                           const ItoKey& ik1) {
  for (auto itBL : BLits) {
    const Key& kl = itBL->first;
    for (auto& o1 : mpol.m) {
      for (auto& o2 : mpor.m) {
        if (o1.first.wl != kl.p0) continue;
        if (o2.first.wl != o1.first.wr) continue;
        const uint32_t o_out = o2.first.wr;
        for (auto& oil : o1.second) {
          for (auto& oir : o2.second) {
            Q kylo = ik0[oil.first.out] + ik1[oir.first.out];
            auto pos = Ain.find(K2(kl.q1, kl.q1 + kylo, oil.first.out, oir.first.out));
            if (pos == Ain.end()) continue;
            Q kyup = ik0[oil.first.in] + ik1[oir.first.in];
            auto posR = BR.find(K1(kl.q0 + kyup, kl.q1 + kylo, o_out));
            if (posR == BR.end()) continue;
            double num = oil.second * oir.second;
            Key key_out = K2(kl.q0, posR->first.q0, oil.first.in, oir.first.in);
            Mat T1 = gemm(num, itBL->second, 'n', pos->second, 'n');
            Mat T2 = gemm(1.0, T1, 'n', posR->second, 't');
            auto y = Aout.find(key_out);
            if (y != Aout.end()) addto(T2, y->second);
            Aout[key_out] = T2;
          }
        }
      }
    }
  }
}

// contractTwosite (MPSfunctions.hpp:949-981)
static BM contract_twosite(const BM& BL, const BM& BR, const BM& A, const MPOMat& mpol,
                           const MPOMat& mpor, const ItoKey& ik0, const ItoKey& ik1, int maxthreads) {
  std::map<Q, std::vector<BM::const_iterator>> BLits;
  for (auto it = BL.begin(); it != BL.end(); ++it) BLits[it->first.q0].push_back(it);
  std::vector<Q> lefts;
  for (auto& x : BLits) lefts.push_back(x.first);
  std::vector<BM> aout(maxthreads);
  const int n = (int)lefts.size();
#pragma omp parallel for num_threads(maxthreads) schedule(dynamic)
  for (int i = 0; i < n; ++i)
    do_contraction(aout[omp_get_thread_num()], BLits.at(lefts[i]), BR, A, mpol, mpor, ik0, ik1);
  BM out;
  for (auto& a : aout) merge(out, a);
  return out;
}

// ---------------------------------------------------------------- split
struct SplitOut {
  BM U, Vt;
  Diag lam;
  double tw = 0;
  int chi = 0;
};
// split (two-site) (MPSfunctions.hpp:1142-1278); consumes A
static SplitOut split2(const BM& A, const ItoKey& ik0, const ItoKey& ik1, int chimax, bool doTrunc,
                       double tr_weight, bool normalize, int maxthreads) {
  std::map<Q, std::vector<BM::const_iterator>> blocks;
  std::map<Q, std::map<uint32_t, std::pair<int, int>>> RX, RY;  // (start,size)
  std::set<Q> QC;
  for (auto a = A.begin(); a != A.end(); ++a) {
    Q qc = a->first.q0 + ik0[a->first.p0];
    blocks[qc].push_back(a);
    RX[qc][a->first.p0] = std::make_pair(0, a->second.r);
    RY[qc][a->first.p1] = std::make_pair(0, a->second.c);
    QC.insert(qc);
  }
  std::map<Q, int> sizex, sizey;
  for (auto& r : RX) {
    int s = 0;
    for (auto& x : r.second) { x.second.first = s; s += x.second.second; }
    sizex[r.first] = s;
  }
  for (auto& r : RY) {
    int s = 0;
    for (auto& x : r.second) { x.second.first = s; s += x.second.second; }
    sizey[r.first] = s;
  }
  std::vector<Q> qcv(QC.begin(), QC.end());
  const int N = (int)qcv.size();
  std::vector<BM> PM(maxthreads), RM(maxthreads);
  std::vector<Diag> LM(maxthreads);
#pragma omp parallel for num_threads(maxthreads) schedule(dynamic)
  for (int i = 0; i < N; ++i) {
    const int th = omp_get_thread_num();
    Q qc = qcv[i];
    Mat tmp(sizex.at(qc), sizey.at(qc)), U, Vt;
    std::vector<double> D;
    for (auto b : blocks.at(qc)) {
      auto rx = RX.at(qc).at(b->first.p0);
      auto ry = RY.at(qc).at(b->first.p1);
      for (int j = 0; j < b->second.c; ++j)
        for (int ii = 0; ii < b->second.r; ++ii) tmp(rx.first + ii, ry.first + j) = b->second(ii, j);
    }
    svd(tmp, U, D, Vt);
    int chi = (int)D.size();
    for (auto& x : RX.at(qc)) {
      Mat u(x.second.second, chi);
      for (int j = 0; j < chi; ++j)
        for (int ii = 0; ii < u.r; ++ii) u(ii, j) = U(x.second.first + ii, j);
      PM[th][K1(qc - ik0[x.first], qc, x.first)] = u;
    }
    LM[th][qc] = D;
    for (auto& y : RY.at(qc)) {
      Mat v(chi, y.second.second);
      for (int j = 0; j < v.c; ++j)
        for (int ii = 0; ii < chi; ++ii) v(ii, j) = Vt(ii, y.second.first + j);
      RM[th][K1(qc, qc + ik1[y.first], y.first)] = v;
    }
  }
  SplitOut o;
  for (int t = 0; t < maxthreads; ++t) {
    merge(o.Vt, RM[t]);
    merge(o.U, PM[t]);
    for (auto& x : LM[t]) o.lam[x.first] = x.second;
  }
  if (!chimax && doTrunc) chimax = 100;
  if (!chimax && !doTrunc) chimax = 200;
  std::pair<double, int> t;
  if (!doTrunc) t = truncate_chi(o.lam, chimax, normalize);
  else t = truncate_tw(o.lam, tr_weight, chimax, normalize);
  o.tw = t.first;
  o.chi = t.second;
  drop_dangling(o.U, o.lam, o.Vt);
  return o;
}

// ---------------------------------------------------------------- Lanczos
struct LanczosOut {
  double E0 = 0;
  int iterations = 0;
  std::vector<double> es;  // eigenvalues (ascending) after the final tridiag
  BM state;
};
// TSLanzcosEngine::simulate(itmax, delta, testenergy) + getState(0) (lanzcos.hpp:165-278, 81-92)
static LanczosOut lanczos(const BM& L, const BM& R, const BM& Ainit, const MPOMat& mpol,
                          const MPOMat& mpor, const ItoKey& ik0, const ItoKey& ik1, int itmax,
                          double delta, bool testenergy, int maxthreads, double* t_matvec) {
  int it = 0;
  const int Ndiag = 5;
  std::vector<BM> As;
  double k = 0, e = 0, eold = 1e100;
  bool first = true;
  std::vector<double> es, ks, estmp;
  BM A0, A1 = Ainit, A2, A3;
  while (true) {
    k = std::sqrt(bm_dot(A1, A1));
    if (std::fabs(k) < delta) break;
    if (!first) ks.push_back(k);
    bm_scale(A1, 1.0 / k);
    auto t0 = std::chrono::steady_clock::now();
    A2 = contract_twosite(L, R, A1, mpol, mpor, ik0, ik1, maxthreads);
    if (t_matvec) *t_matvec += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    As.push_back(A1);
    e = bm_dot(A2, A1);
    es.push_back(e);
    if (it % Ndiag == 0 && it != 0) {
      if (testenergy) {
        estmp = es;
        tridiag(estmp, ks, nullptr);
        if (std::fabs(estmp[0] - eold) < delta) break;
        eold = estmp[0];
      } else {
        // residual test (lanzcos.hpp:215-235): the Ritz vector A4 = sum_i As[i] z(i,0) of the current
        // tridiagonal matrix, A6 = H A4 - E0 A4, stop when |A6| < delta (one extra matvec)
        estmp = es;
        std::vector<double> z;
        tridiag(estmp, ks, &z);
        BM A4 = bm_scaled(As[0], z[0]);
        for (size_t i = 1; i < es.size(); ++i) bm_add(A4, bm_scaled(As[i], z[i]));
        auto t1 = std::chrono::steady_clock::now();
        BM A5 = contract_twosite(L, R, A4, mpol, mpor, ik0, ik1, maxthreads);
        if (t_matvec) *t_matvec += std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
        BM A6 = bm_scaled(A4, -estmp[0]);
        bm_add(A6, A5);
        if (std::fabs(std::sqrt(bm_dot(A6, A6))) < delta) break;
      }
    }
    if (!first) {
      A3 = bm_scaled(A1, -e);
      bm_add(A3, A2);
      bm_scale(A0, -k);
      bm_add(A3, A0);
      A0 = A1;
      A1 = A3;
    } else {
      A0 = A1;
      A3 = bm_scaled(A1, -e);
      bm_add(A3, A2);
      A1 = A3;
      first = false;
    }
    it++;
    if (it >= itmax) break;
  }
  LanczosOut o;
  o.iterations = (int)es.size();  // number of Krylov vectors (matvecs) entering the ground state
  if (!es.empty()) {
    std::vector<double> z;
    tridiag(es, ks, &z);
    o.es = es;
    o.E0 = es[0];
    // getState(0) = sum_i As[i] * z(i,0)
    BM A = bm_scaled(As[0], z[0]);
    for (size_t i = 1; i < es.size(); ++i) bm_add(A, bm_scaled(As[i], z[i]));
    o.state = A;
  }
  return o;
}

// ---------------------------------------------------------------- MPS and canonical forms
struct MPS {
  std::vector<BM> s;
  std::map<int, Diag> lam;
  BM leftDummy, rightDummy;
  std::vector<ItoKey> ik;
};

// prepareBlock (MPSfunctions.hpp:21-142), dir "r": right-orthonormalise the blocks of BL2 with
// left charge keyout; U*D is multiplied into the BL1 blocks whose right charge is keyout.
static bool prepare_block_r(const std::vector<Key>& out, BM& BL1, const BM& BL2, BM& BLp, Diag& lam,
                            bool truncate, double delta) {
  Q keyout = out[0].q0;
  int SIZE1 = BL2.at(out[0]).r, SIZE2 = 0;
  std::vector<std::pair<int, int>> rng;
  for (auto& k : out) { rng.push_back(std::make_pair(SIZE2, BL2.at(k).c)); SIZE2 += BL2.at(k).c; }
  Mat tmp(SIZE1, SIZE2);
  for (size_t b = 0; b < out.size(); ++b) {
    const Mat& m = BL2.at(out[b]);
    for (int j = 0; j < m.c; ++j)
      for (int i = 0; i < m.r; ++i) tmp(i, rng[b].first + j) = m(i, j);
  }
  Mat U, Vd;
  std::vector<double> D;
  svd(tmp, U, D, Vd);
  if (truncate) {
    size_t l = 0;
    while (l < D.size() && std::fabs(D[l]) > delta) ++l;
    D.resize(l);
    Mat Ut(U.r, (int)l), Vt((int)l, Vd.c);
    for (int j = 0; j < (int)l; ++j)
      for (int i = 0; i < U.r; ++i) Ut(i, j) = U(i, j);
    for (int j = 0; j < Vd.c; ++j)
      for (int i = 0; i < (int)l; ++i) Vt(i, j) = Vd(i, j);
    U = Ut;
    Vd = Vt;
  }
  int n = (int)D.size();
  if (!n) return true;
  lam[keyout] = D;
  for (size_t b = 0; b < out.size(); ++b) {
    Mat t(n, rng[b].second);
    for (int j = 0; j < t.c; ++j)
      for (int i = 0; i < n; ++i) t(i, j) = Vd(i, rng[b].first + j);
    BLp[out[b]] = t;
  }
  for (auto& x : BL1) {
    if (x.first.q1 != keyout) continue;
    Mat t = gemm(1.0, x.second, 'n', U, 'n');
    for (int j = 0; j < t.c; ++j)
      for (int i = 0; i < t.r; ++i) t(i, j) *= D[j];
    x.second = t;
  }
  return false;
}
// prepareMatrix dir "r" (MPSfunctions.hpp:210-268)
static void prepare_matrix_r(BM& BL1, Diag& lam, BM& BL2, bool truncate, double delta) {
  std::map<Q, std::vector<Key>> Tkeys;
  for (auto& b : BL2) Tkeys[b.first.q0].push_back(b.first);
  Diag lamn;
  BM BLp;
  std::set<Q> er;
  for (auto& t : Tkeys) {
    bool e = prepare_block_r(t.second, BL1, BL2, BLp, lamn, truncate, delta);
    if (e) er.insert(t.first);
  }
  for (auto it = BL1.begin(); it != BL1.end();) {
    if (er.count(it->first.q1)) it = BL1.erase(it); else ++it;
  }
  BL2 = BLp;
  lam = lamn;
}
// orthonormalize(mps,"rl") (MPSfunctions.hpp:1776-1784)
static void orthonormalize_rl(MPS& mps) {
  const int N = (int)mps.s.size();
  for (int site = N - 1; site >= 0; --site) {
    if (site != 0) prepare_matrix_r(mps.s[site - 1], mps.lam[site - 1], mps.s[site], true, 1e-16);
    else prepare_matrix_r(mps.leftDummy, mps.lam[-1], mps.s[0], true, 1e-16);
  }
}

static BM get_lmin() {  // getLMin (MPSfunctions.hpp:1917-1926)
  BM L;
  Mat m(1, 1);
  m(0, 0) = 1.0;
  L[K1(0, 0, 0)] = m;
  return L;
}
static BM get_rmax(const BM& last) {  // getRMax (MPSfunctions.hpp:1996-2022)
  BM R;
  std::set<Q> ps;
  for (auto& a : last) ps.insert(a.first.q1);
  for (Q p : ps) {
    int m = 0;
    for (auto& a : last)
      if (a.first.q1 == p) { m = a.second.c; break; }
    Mat id(m, m);
    for (int i = 0; i < m; ++i) id(i, i) = 1.0;
    R[K1(p, p, 0)] = id;
  }
  return R;
}

// MPO::measure(MPS) (MPOTypes.hpp:990-1020)
static double mpo_measure(const std::vector<BM>& s, const std::vector<MPOMat>& mpo,
                          const std::vector<ItoKey>& ik, int maxthreads) {
  BM L = get_lmin();
  for (size_t x = 0; x < s.size(); ++x) L = add_contraction_layer(L, s[x], mpo[x], ik[x], 1, maxthreads);
  double out = 0;
  for (auto& l : L)
    if (l.first.q0 == l.first.q1) {
      int n = std::min(l.second.r, l.second.c);
      for (int i = 0; i < n; ++i) out += l.second(i, i);
    }
  return out;
}

// ---------------------------------------------------------------- DMRG engine
struct StepRec {
  int site, dir, iters, chi;
  double E, tw;
};
struct DMRG {
  MPS mps;
  std::vector<MPOMat> mpo;
  std::map<int, BM> L, R;
  int lanmax = 500;
  std::vector<StepRec> steps;
  double t_matvec = 0, t_env = 0, t_split = 0, t_total = 0;
  int maxthreads = 1;
  int matvec_threads = 8;
};

// DMRGengine::doStep (container.hpp:292-337)
static StepRec dmrg_step(DMRG& g, int site, int dir, int chimax, bool doTrunc, double tr_weight,
                         double delta, bool testenergy) {
  MPS& mps = g.mps;
  BM theta = theta_form(mps.s[site], mps.s[site + 1]);
  LanczosOut lo = lanczos(g.L[site - 1], g.R[site + 2], theta, g.mpo[site], g.mpo[site + 1],
                          mps.ik[site], mps.ik[site + 1], g.lanmax, delta, testenergy,
                          std::min(g.maxthreads, g.matvec_threads), &g.t_matvec);
  auto t0 = std::chrono::steady_clock::now();
  SplitOut so = split2(lo.state, mps.ik[site], mps.ik[site + 1], chimax, doTrunc, tr_weight, true, g.maxthreads);
  auto t1 = std::chrono::steady_clock::now();
  g.t_split += std::chrono::duration<double>(t1 - t0).count();
  if (dir > 0) {
    mps.s[site] = so.U;
    mps.s[site + 1] = lam_times(so.lam, so.Vt);
  } else {
    mps.s[site] = times_lam(so.U, so.lam);
    mps.s[site + 1] = so.Vt;
  }
  mps.lam[site] = so.lam;
  if (dir > 0)
    g.L[site] = add_contraction_layer(g.L[site - 1], mps.s[site], g.mpo[site], mps.ik[site], 1, g.maxthreads);
  else
    g.R[site + 1] = add_contraction_layer(g.R[site + 2], mps.s[site + 1], g.mpo[site + 1], mps.ik[site + 1], -1, g.maxthreads);
  g.t_env += std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
  StepRec r;
  r.site = site; r.dir = dir; r.iters = lo.iterations; r.chi = so.chi; r.E = lo.E0; r.tw = so.tw;
  g.steps.push_back(r);
  return r;
}

// DMRGengine::simulate (container.hpp:381-438)
static double dmrg_simulate(DMRG& g, int maxsteps, double EnConv, int chimax, bool doTrunc,
                            double tr_weight, double delta, bool testenergy) {
  auto t0 = std::chrono::steady_clock::now();
  MPS& mps = g.mps;
  const int N = (int)mps.s.size();
  orthonormalize_rl(mps);
  g.R.clear();
  g.R[N] = get_rmax(mps.s[N - 1]);
  auto te = std::chrono::steady_clock::now();
  for (int s = N - 1; s >= 2; --s)
    g.R[s] = add_contraction_layer(g.R[s + 1], mps.s[s], g.mpo[s], mps.ik[s], 0, g.maxthreads);
  g.t_env += std::chrono::duration<double>(std::chrono::steady_clock::now() - te).count();
  g.L.clear();
  g.L[-1] = get_lmin();
  double globalE = 1e100;
  StepRec out;
  int step = 0;
  while (true) {
    for (int site = 0; site < N - 2; ++site) out = dmrg_step(g, site, 1, chimax, doTrunc, tr_weight, delta, testenergy);
    for (int site = N - 2; site > 0; --site) out = dmrg_step(g, site, -1, chimax, doTrunc, tr_weight, delta, testenergy);
    ++step;
    bool conv = std::fabs(globalE - out.E) < EnConv;
    if (step >= maxsteps) conv = true;
    globalE = out.E;
    if (conv) break;
  }
  out = dmrg_step(g, 0, -1, chimax, doTrunc, tr_weight, delta, testenergy);
  g.t_total += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return out.E;
}

// ---------------------------------------------------------------- model MPOs
static SparseOp opmul(const SparseOp& a, const SparseOp& b) {  // SparseOperator::operator*=
  SparseOp t;
  for (auto& i : a)
    for (auto& j : b)
      if (i.first.in == j.first.out) {
        OpKey k{j.first.in, i.first.out};
        t[k] += i.second * j.second;
      }
  return t;
}
static SparseOp opscale(SparseOp a, double s) { for (auto& x : a) x.second *= s; return a; }
static SparseOp op(std::initializer_list<std::pair<std::pair<uint32_t, uint32_t>, double>> l) {
  SparseOp o;  // entries given as ((out,in), value)
  for (auto& x : l) o[OpKey{x.first.second, x.first.first}] = x.second;
  return o;
}
static void squeeze(MPOMat& M, double th) {
  for (auto& x : M.m)
    for (auto it = x.second.begin(); it != x.second.end();) {
      if (std::fabs(it->second) < th) it = x.second.erase(it); else ++it;
    }
}
// HeisenbergMPO(Jz,Jxy,B) (Hamiltonians.hpp:84-131)
static std::vector<MPOMat> heisenberg(int N, const double* Jz, const double* Jxy, const double* B) {
  SparseOp Sz = op({{{0, 0}, -0.5}, {{1, 1}, 0.5}}), Sp = op({{{1, 0}, 1.0}}), Sm = op({{{0, 1}, 1.0}}),
           id = op({{{0, 0}, 1.0}, {{1, 1}, 1.0}});
  std::vector<MPOMat> W(N);
  MPOMat M;
  M.m[{0, 0}] = opscale(Sz, -B[0]);
  M.m[{0, 1}] = opscale(Sm, Jxy[0] / 2.);
  M.m[{0, 2}] = opscale(Sp, Jxy[0] / 2.);
  M.m[{0, 3}] = opscale(Sz, Jz[0]);
  M.m[{0, 4}] = id;
  M.Dl = 1; M.Dr = 5;
  squeeze(M, 1e-16);
  W[0] = M;
  M = MPOMat();
  M.m[{0, 0}] = id;
  M.m[{1, 0}] = Sp;
  M.m[{2, 0}] = Sm;
  M.m[{3, 0}] = Sz;
  M.m[{4, 0}] = opscale(Sz, -B[N - 1]);
  M.Dl = 5; M.Dr = 1;
  squeeze(M, 1e-16);
  W[N - 1] = M;
  for (int s = 1; s < N - 1; ++s) {
    MPOMat Mb;
    Mb.m[{0, 0}] = id;
    Mb.m[{1, 0}] = Sp;
    Mb.m[{2, 0}] = Sm;
    Mb.m[{3, 0}] = Sz;
    Mb.m[{4, 0}] = opscale(Sz, -B[s]);
    Mb.m[{4, 1}] = opscale(Sm, Jxy[s] / 2.);
    Mb.m[{4, 2}] = opscale(Sp, Jxy[s] / 2.);
    Mb.m[{4, 3}] = opscale(Sz, Jz[s]);
    Mb.m[{4, 4}] = id;
    Mb.Dl = 5; Mb.Dr = 5;
    squeeze(Mb, 1e-16);
    W[s] = Mb;
  }
  return W;
}
// SpinlessFermionsMPO(V,t,mu) (Hamiltonians.hpp:527-566)
static std::vector<MPOMat> spinless(int N, const double* V, const double* t, const double* mu) {
  SparseOp n = op({{{0, 0}, 0.0}, {{1, 1}, 1.0}}), cd = op({{{1, 0}, 1.0}}), c = op({{{0, 1}, 1.0}}),
           id = op({{{0, 0}, 1.0}, {{1, 1}, 1.0}}), p = op({{{0, 0}, 1.0}, {{1, 1}, -1.0}});
  std::vector<MPOMat> W(N);
  MPOMat M;
  M.m[{0, 0}] = opscale(n, -mu[0]);
  M.m[{0, 1}] = opscale(opmul(c, p), t[0]);
  M.m[{0, 2}] = opscale(opmul(cd, p), -t[0]);
  M.m[{0, 3}] = opscale(n, V[0]);
  M.m[{0, 4}] = id;
  M.Dl = 1; M.Dr = 5;
  squeeze(M, 1e-16);
  W[0] = M;
  M = MPOMat();
  M.m[{0, 0}] = id;
  M.m[{1, 0}] = cd;
  M.m[{2, 0}] = c;
  M.m[{3, 0}] = n;
  M.m[{4, 0}] = opscale(n, -mu[N - 1]);
  M.Dl = 5; M.Dr = 1;
  squeeze(M, 1e-16);
  W[N - 1] = M;
  for (int s = 1; s < N - 1; ++s) {
    MPOMat Mb;
    Mb.m[{0, 0}] = id;
    Mb.m[{1, 0}] = cd;
    Mb.m[{2, 0}] = c;
    Mb.m[{3, 0}] = n;
    Mb.m[{4, 0}] = opscale(n, -mu[s]);
    Mb.m[{4, 1}] = opscale(opmul(c, p), t[s]);
    Mb.m[{4, 2}] = opscale(opmul(cd, p), -t[s]);
    Mb.m[{4, 3}] = opscale(n, V[s]);
    Mb.m[{4, 4}] = id;
    Mb.Dl = 5; Mb.Dr = 5;
    squeeze(Mb, 1e-16);
    W[s] = Mb;
  }
  return W;
}

}  // namespace orc

// ============================================================================ C ABI for ctypes
using namespace orc;


// ================================================================ complex FP64 (TEBD)
typedef std::complex<double> cplx;
typedef void (*zgemm_t)(const char*, const char*, const int*, const int*, const int*, const cplx*, const cplx*,
                        const int*, const cplx*, const int*, const cplx*, cplx*, const int*, size_t, size_t);
typedef void (*zgesvd_t)(const char*, const char*, const int*, const int*, cplx*, const int*, double*, cplx*,
                         const int*, cplx*, const int*, cplx*, const int*, double*, int*, size_t, size_t);
static zgemm_t p_zgemm = nullptr;
static zgesvd_t p_zgesvd = nullptr;

struct CMat {
  int r = 0, c = 0;
  std::vector<cplx> d;  // column-major
  CMat() {}
  CMat(int r_, int c_) : r(r_), c(c_), d((size_t)r_ * c_, cplx(0.0, 0.0)) {}
  cplx& operator()(int i, int j) { return d[(size_t)i + (size_t)j * r]; }
  cplx operator()(int i, int j) const { return d[(size_t)i + (size_t)j * r]; }
};
typedef std::map<Key, CMat> CBM;

// out = op(A) op(B), op in 'n', 't', 'c' (MatMatProd for Complex)
static CMat cgemm(const CMat& A, char ta, const CMat& B, char tb) {
  int m = (ta == 'n') ? A.r : A.c;
  int k = (ta == 'n') ? A.c : A.r;
  int n = (tb == 'n') ? B.c : B.r;
  CMat C(m, n);
  if (m == 0 || n == 0 || k == 0) return C;
  int lda = std::max(1, A.r), ldb = std::max(1, B.r), ldc = std::max(1, m);
  cplx one(1.0, 0.0), zero(0.0, 0.0);
  char TA = ta == 'n' ? 'N' : (ta == 't' ? 'T' : 'C'), TB = tb == 'n' ? 'N' : (tb == 't' ? 'T' : 'C');
  p_zgemm(&TA, &TB, &m, &n, &k, &one, A.d.data(), &lda, B.d.data(), &ldb, &zero, C.d.data(), &ldc, 1, 1);
  return C;
}

// BoostSVD for Complex: zgesvd 'S','S', then the complex FixPhase (the phase of the first abs-max
// entry of each row of Vt removed from that row and given to the column of U).
static int csvd(const CMat& M, CMat& U, std::vector<double>& D, CMat& Vt) {
  int m = M.r, n = M.c, k = std::min(m, n);
  U = CMat(m, k);
  Vt = CMat(k, n);
  D.assign(k, 0.0);
  if (k == 0) return 0;
  CMat A = M;
  char J = 'S';
  int lda = m, ldu = m, ldvt = k, info = 0, lwork = -1;
  cplx wq;
  std::vector<double> rwork(5 * (size_t)k + 8);
  p_zgesvd(&J, &J, &m, &n, A.d.data(), &lda, D.data(), U.d.data(), &ldu, Vt.d.data(), &ldvt, &wq, &lwork,
           rwork.data(), &info, 1, 1);
  lwork = std::max((int)wq.real(), 2 * k + std::max(m, n));
  std::vector<cplx> work(lwork);
  p_zgesvd(&J, &J, &m, &n, A.d.data(), &lda, D.data(), U.d.data(), &ldu, Vt.d.data(), &ldvt, work.data(), &lwork,
           rwork.data(), &info, 1, 1);
  for (int i = 0; i < k; ++i) {
    int ind = 0;
    double val = 0;
    for (int j = 0; j < n; ++j)
      if (std::abs(Vt(i, j)) > val) { val = std::abs(Vt(i, j)); ind = j; }
    const double phi = std::arg(Vt(i, ind));
    const cplx e = std::exp(cplx(0.0, -phi)), ec = std::exp(cplx(0.0, phi));
    for (int j = 0; j < n; ++j) Vt(i, j) *= e;
    for (int j = 0; j < m; ++j) U(j, i) *= ec;
  }
  return info;
}

// BlockMatrix::squeeze(thresh): erase blocks whose entries are all <= thresh in magnitude
static void csqueeze(CBM& B, double thresh) {
  for (auto it = B.begin(); it != B.end();) {
    bool keep = false;
    for (auto& v : it->second.d)
      if (std::abs(v) > thresh) { keep = true; break; }
    if (!keep) it = B.erase(it);
    else ++it;
  }
}

// lambda * B (rows by the left charge), B * lambda (columns by the right charge), and the divisions;
// blocks whose charge has no lambda are dropped (src/BlockTensor.hpp:653-733)
static CBM lam_scale(const Diag& lam, const CBM& B, bool left, bool divide) {
  CBM out;
  for (auto& b : B) {
    auto l = lam.find(left ? b.first.q0 : b.first.q1);
    if (l == lam.end()) continue;
    CMat t = b.second;
    for (int j = 0; j < t.c; ++j)
      for (int i = 0; i < t.r; ++i) {
        const double f = left ? l->second[i] : l->second[j];
        t(i, j) = divide ? t(i, j) * (1.0 / f) : t(i, j) * f;
      }
    out[b.first] = t;
  }
  return out;
}

// BlockMatrix<2>(A1, A2)
static CBM ctheta(const CBM& B1, const CBM& B2) {
  CBM out;
  for (auto& a : B1)
    for (auto& b : B2)
      if (a.first.q1 == b.first.q0) {
        Key k = K2(a.first.q0, b.first.q1, a.first.p0, b.first.p0);
        CMat t = cgemm(a.second, 'n', b.second, 'n');
        auto y = out.find(k);
        if (y != out.end())
          for (size_t i = 0; i < t.d.size(); ++i) t.d[i] += y->second.d[i];
        out[k] = t;
      }
  return out;
}

template <class M>
static void drop_dangling_t(std::map<Key, M>& L, const Diag& lam, std::map<Key, M>& R) {
  for (auto it = L.begin(); it != L.end();) {
    auto l = lam.find(it->first.q1);
    if (l == lam.end()) { it = L.erase(it); continue; }
    const int k = (int)l->second.size();
    if (it->second.c > k) {
      M t(it->second.r, k);
      for (int j = 0; j < k; ++j)
        for (int i = 0; i < t.r; ++i) t(i, j) = it->second(i, j);
      it->second = t;
    }
    ++it;
  }
  for (auto it = R.begin(); it != R.end();) {
    auto l = lam.find(it->first.q0);
    if (l == lam.end()) { it = R.erase(it); continue; }
    const int k = (int)l->second.size();
    if (it->second.r > k) {
      M t(k, it->second.c);
      for (int j = 0; j < t.c; ++j)
        for (int i = 0; i < k; ++i) t(i, j) = it->second(i, j);
      it->second = t;
    }
    ++it;
  }
}

struct CSplitOut {
  CBM U, Vt;
  Diag lam;
  double tw = 0;
  int chi = 0;
};
// split (two-site) for Complex (MPSfunctions.hpp:1142-1278): sectors by centre charge, zgesvd,
// global truncation, dropDangling
static CSplitOut csplit2(const CBM& A, const ItoKey& ik0, const ItoKey& ik1, int chimax, bool doTrunc,
                         double tr_weight, bool normalize) {
  std::map<Q, std::vector<CBM::const_iterator>> blocks;
  std::map<Q, std::map<uint32_t, std::pair<int, int>>> RX, RY;
  for (auto a = A.begin(); a != A.end(); ++a) {
    Q qc = a->first.q0 + ik0[a->first.p0];
    blocks[qc].push_back(a);
    RX[qc][a->first.p0] = std::make_pair(0, a->second.r);
    RY[qc][a->first.p1] = std::make_pair(0, a->second.c);
  }
  std::map<Q, int> sx, sy;
  for (auto& r : RX) { int s = 0; for (auto& x : r.second) { x.second.first = s; s += x.second.second; } sx[r.first] = s; }
  for (auto& r : RY) { int s = 0; for (auto& x : r.second) { x.second.first = s; s += x.second.second; } sy[r.first] = s; }
  CSplitOut o;
  for (auto& bq : blocks) {
    const Q qc = bq.first;
    CMat tmp(sx.at(qc), sy.at(qc)), U, Vt;
    std::vector<double> D;
    for (auto b : bq.second) {
      auto rx = RX.at(qc).at(b->first.p0);
      auto ry = RY.at(qc).at(b->first.p1);
      for (int j = 0; j < b->second.c; ++j)
        for (int i = 0; i < b->second.r; ++i) tmp(rx.first + i, ry.first + j) = b->second(i, j);
    }
    csvd(tmp, U, D, Vt);
    const int chi = (int)D.size();
    for (auto& x : RX.at(qc)) {
      CMat u(x.second.second, chi);
      for (int j = 0; j < chi; ++j)
        for (int i = 0; i < u.r; ++i) u(i, j) = U(x.second.first + i, j);
      o.U[K1(qc - ik0[x.first], qc, x.first)] = u;
    }
    o.lam[qc] = D;
    for (auto& y : RY.at(qc)) {
      CMat v(chi, y.second.second);
      for (int j = 0; j < v.c; ++j)
        for (int i = 0; i < chi; ++i) v(i, j) = Vt(i, y.second.first + j);
      o.Vt[K1(qc, qc + ik1[y.first], y.first)] = v;
    }
  }
  if (!chimax && doTrunc) chimax = 100;
  if (!chimax && !doTrunc) chimax = 200;
  std::pair<double, int> t = doTrunc ? truncate_tw(o.lam, tr_weight, chimax, normalize)
                                     : truncate_chi(o.lam, chimax, normalize);
  o.tw = t.first;
  o.chi = t.second;
  drop_dangling_t(o.U, o.lam, o.Vt);
  return o;
}

// Two-site gate G[(o1,o2),(i1,i2)] = exp(-(dt_im + i dt_re) h_b), h_b = sum_i W1[row, i] (x) W2[i, 0]
// with the boundary-aware halves of the on-site channels (MPO::getNNGate).  Dense d1*d2 square,
// index o1 + d1*o2.
struct Gate {
  int d1 = 0, d2 = 0;
  std::vector<cplx> g;  // (d1 d2) x (d1 d2), column-major
  cplx at(int o1, int o2, int i1, int i2) const { return g[(size_t)(o1 + d1 * o2) + (size_t)(i1 + d1 * i2) * d1 * d2]; }
};
static void jacobi_eig_sym(int n, std::vector<double>& A, std::vector<double>& V, std::vector<double>& E) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i + (size_t)i * n] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[p + (size_t)q * n] * A[p + (size_t)q * n];
    if (off < 1e-32) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p + (size_t)q * n];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = A[p + (size_t)p * n], aqq = A[q + (size_t)q * n];
        const double th = 0.5 * (aqq - app) / apq;
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- J^T A J
          const double akp = A[k + (size_t)p * n], akq = A[k + (size_t)q * n];
          A[k + (size_t)p * n] = c * akp - s * akq;
          A[k + (size_t)q * n] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[p + (size_t)k * n], aqk = A[q + (size_t)k * n];
          A[p + (size_t)k * n] = c * apk - s * aqk;
          A[q + (size_t)k * n] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k + (size_t)p * n], vkq = V[k + (size_t)q * n];
          V[k + (size_t)p * n] = c * vkp - s * vkq;
          V[k + (size_t)q * n] = s * vkp + c * vkq;
        }
      }
  }
  E.resize(n);
  for (int i = 0; i < n; ++i) E[i] = A[i + (size_t)i * n];
}
static Gate nn_gate(const MPOMat& m1, const MPOMat& m2, int site1, int N, double dt_re, double dt_im, int d1, int d2) {
  const int site2 = site1 + 1;
  const int D = d1 * d2;
  std::vector<double> H((size_t)D * D, 0.0);
  auto add = [&](uint32_t r1, uint32_t c1, uint32_t r2, uint32_t c2, double w1, double w2) {
    auto a = m1.m.find(WKey{r1, c1});
    auto b = m2.m.find(WKey{r2, c2});
    if (a == m1.m.end() || b == m2.m.end()) return;
    for (auto& x : a->second)
      for (auto& y : b->second) {
        const int o = (int)x.first.out + d1 * (int)y.first.out, in = (int)x.first.in + d1 * (int)y.first.in;
        H[o + (size_t)in * D] += x.second * w1 * y.second * w2;
      }
  };
  const uint32_t lend = (uint32_t)m1.Dl - 1, last = (uint32_t)m1.Dr - 1;
  for (uint32_t i = 0; i <= last; ++i) {
    if (site1 == 0 && site2 != N - 1) {
      if (i == 0) add(0, i, i, 0, 1.0, 1.0);
      else if (i == last) add(0, i, i, 0, 1.0, 0.5);
      else add(0, i, i, 0, 1.0, 1.0);
    }
    if (site2 == N - 1 && site1 != 0) {
      if (i == 0) add(lend, i, i, 0, 0.5, 1.0);
      else if (i == last) add(lend, i, i, 0, 1.0, 1.0);
      else add(lend, i, i, 0, 1.0, 1.0);
    }
    if (site2 != N - 1 && site1 != 0) {
      if (i == 0) add(lend, i, i, 0, 0.5, 1.0);
      else if (i == last) add(lend, i, i, 0, 1.0, 0.5);
      else add(lend, i, i, 0, 1.0, 1.0);
    }
  }
  for (auto& h : H)
    if (std::fabs(h) < 1e-14) h = 0.0;  // gate.squeeze(1e-14) before the exponential
  std::vector<double> V, E;
  std::vector<double> A = H;
  jacobi_eig_sym(D, A, V, E);
  Gate G;
  G.d1 = d1;
  G.d2 = d2;
  G.g.assign((size_t)D * D, cplx(0, 0));
  for (int x = 0; x < D; ++x)
    for (int y = 0; y < D; ++y) {
      cplx s(0, 0);
      for (int k = 0; k < D; ++k) s += V[x + (size_t)k * D] * std::exp(-cplx(dt_im, dt_re) * E[k]) * V[y + (size_t)k * D];
      G.g[x + (size_t)y * D] = std::abs(s) < 1e-15 ? cplx(0, 0) : s;  // gateC.squeeze(1e-15)
    }
  return G;
}

// Vidal-form state: Gamma[s] (s = 0..N-1), lambda[b] for b = -1..N-1 (stored at b+1)
struct TEBDState {
  int N = 0;
  std::vector<CBM> G;
  std::vector<Diag> lam;
  std::vector<ItoKey> ik;
};
// product state: Gamma[s] = (q_s, q_s + q(sigma_s); sigma_s) = [[1]], all lambdas [1]
static TEBDState tebd_product(const std::vector<int>& local, const std::vector<ItoKey>& ik) {
  TEBDState st;
  st.N = (int)local.size();
  st.ik = ik;
  st.G.resize(st.N);
  st.lam.resize(st.N + 1);
  Q q = 0;
  st.lam[0][q] = {1.0};
  for (int s = 0; s < st.N; ++s) {
    const Q q1 = q + ik[s][local[s]];
    CMat one(1, 1);
    one(0, 0) = cplx(1.0, 0.0);
    st.G[s][K1(q, q1, (uint32_t)local[s])] = one;
    st.lam[s + 1][q1] = {1.0};
    q = q1;
  }
  return st;
}
// applyGate (MPSfunctions.hpp:1492-1548) on bond (site, site+1)
static std::pair<double, int> apply_gate(TEBDState& st, int site, const Gate& gate, int chimax, bool doTrunc,
                                         double tr_weight, bool normalize) {
  const Diag &ll = st.lam[site], &lc = st.lam[site + 1], &lr = st.lam[site + 2];
  CBM Ml = lam_scale(lc, lam_scale(ll, st.G[site], true, false), false, false);
  CBM Mr = lam_scale(lr, st.G[site + 1], false, false);
  CBM Ain = ctheta(Ml, Mr), th;
  for (auto& a : Ain) {
    const uint32_t i1 = a.first.p0, i2 = a.first.p1;
    for (int o2 = 0; o2 < gate.d2; ++o2)
      for (int o1 = 0; o1 < gate.d1; ++o1) {
        const cplx g = gate.at(o1, o2, (int)i1, (int)i2);
        if (g == cplx(0, 0)) continue;
        Key k = K2(a.first.q0, a.first.q1, (uint32_t)o1, (uint32_t)o2);
        CMat t = a.second;
        for (auto& v : t.d) v *= g;
        auto y = th.find(k);
        if (y != th.end())
          for (size_t i = 0; i < t.d.size(); ++i) t.d[i] += y->second.d[i];
        th[k] = t;
      }
  }
  csqueeze(th, 1e-15);
  CSplitOut o = csplit2(th, st.ik[site], st.ik[site + 1], chimax, doTrunc, tr_weight, normalize);
  csqueeze(o.U, 1e-15);
  csqueeze(o.Vt, 1e-15);
  st.G[site] = lam_scale(ll, o.U, true, true);
  st.G[site + 1] = lam_scale(lr, o.Vt, false, true);
  st.lam[site + 1] = o.lam;
  return std::make_pair(o.tw, o.chi);
}
// doTimeSlice: bonds start, start+2, ... (container.hpp:1195-1233)
static void tebd_slice(TEBDState& st, const std::vector<Gate>& gates, int start, int chimax, bool doTrunc,
                       double tr_weight, bool normalize, std::vector<double>* tw) {
  for (int site = start; site < st.N - 1; site += 2) {
    auto r = apply_gate(st, site, gates[site], chimax, doTrunc, tr_weight, normalize);
    if (tw) (*tw)[site] = r.first;
  }
}
// second-order Trotter (TEBDengine::simulate "second", without intermediate measurements):
// odd/2, then steps x (even, odd) with the last odd step halved
static void tebd_second_order(TEBDState& st, const std::vector<MPOMat>& mpo, int steps, double dt, int chimax,
                              bool doTrunc, double tr_weight, bool normalize) {
  std::vector<Gate> full, half;
  for (int s = 0; s + 1 < st.N; ++s) {
    const int d1 = (int)st.ik[s].size(), d2 = (int)st.ik[s + 1].size();
    full.push_back(nn_gate(mpo[s], mpo[s + 1], s, st.N, dt, 0.0, d1, d2));
    half.push_back(nn_gate(mpo[s], mpo[s + 1], s, st.N, dt / 2, 0.0, d1, d2));
  }
  tebd_slice(st, half, 1, chimax, doTrunc, tr_weight, normalize, nullptr);
  for (int step = 1; step <= steps; ++step) {
    tebd_slice(st, full, 0, chimax, doTrunc, tr_weight, normalize, nullptr);
    tebd_slice(st, step < steps ? full : half, 1, chimax, doTrunc, tr_weight, normalize, nullptr);
  }
}
// SparseLocalOperator::measure for a diagonal operator diag(op) on lambda Gamma lambda
static double tebd_measure_diag(const TEBDState& st, int site, const std::vector<double>& op) {
  CBM M = lam_scale(st.lam[site + 1], lam_scale(st.lam[site], st.G[site], true, false), false, false);
  double mean = 0;
  for (auto& b : M) {
    double nrm = 0;
    for (auto& v : b.second.d) nrm += std::norm(v);
    mean += op[b.first.p0] * nrm;
  }
  return mean;
}

struct orc_bm_t { BM m; int nphys; };
struct orc_mpo_t { MPOMat w; };
struct orc_dmrg_t { DMRG g; };

extern "C" {

int orc_init(const char* path) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) { fprintf(stderr, "oracle: dlopen(%s) failed: %s\n", path, dlerror()); return 1; }
  p_dgemm = (dgemm_t)sym(h, "scipy_dgemm_", "dgemm_");
  p_ddot = (ddot_t)sym(h, "scipy_ddot_", "ddot_");
  p_dgesvd = (dgesvd_t)sym(h, "scipy_dgesvd_", "dgesvd_");
  p_dstev = (dstev_t)sym(h, "scipy_dstev_", "dstev_");
  p_zgemm = (zgemm_t)sym(h, "scipy_zgemm_", "zgemm_");
  p_zgesvd = (zgesvd_t)sym(h, "scipy_zgesvd_", "zgesvd_");
  setthreads_t st = (setthreads_t)sym(h, "scipy_openblas_set_num_threads", "openblas_set_num_threads");
  if (st) st(1);  // OpenMP parallelism is over charge sectors, as in the reference
  if (!p_dgemm || !p_ddot || !p_dgesvd || !p_dstev || !p_zgemm || !p_zgesvd) return 2;
  return 0;
}

// nphys: 0 (lambda: key (q,q), cols=1), 1 (q0,q1;p0), 2 (q0,q1;p0,p1). data concatenated col-major.
void* orc_bm_new(int nphys, int nblocks, const uint64_t* q, const uint32_t* p, const int32_t* rows,
                 const int32_t* cols, const double* data) {
  orc_bm_t* b = new orc_bm_t;
  b->nphys = nphys;
  size_t off = 0;
  for (int i = 0; i < nblocks; ++i) {
    Key k;
    k.q0 = q[2 * i];
    k.q1 = q[2 * i + 1];
    if (nphys >= 1) k.p0 = p[nphys * i];
    if (nphys >= 2) k.p1 = p[nphys * i + 1];
    Mat m(rows[i], cols[i]);
    if (data) std::memcpy(m.d.data(), data + off, sizeof(double) * m.d.size());
    off += m.d.size();
    b->m[k] = m;
  }
  return b;
}
int orc_bm_nblocks(void* b) { return (int)((orc_bm_t*)b)->m.size(); }
int orc_bm_nphys(void* b) { return ((orc_bm_t*)b)->nphys; }
long orc_bm_size(void* b) {
  long s = 0;
  for (auto& x : ((orc_bm_t*)b)->m) s += (long)x.second.d.size();
  return s;
}
void orc_bm_export(void* bb, uint64_t* q, uint32_t* p, int32_t* rows, int32_t* cols, double* data) {
  orc_bm_t* b = (orc_bm_t*)bb;
  size_t i = 0, off = 0;
  for (auto& x : b->m) {
    q[2 * i] = x.first.q0;
    q[2 * i + 1] = x.first.q1;
    if (b->nphys >= 1) p[b->nphys * i] = x.first.p0;
    if (b->nphys >= 2) p[b->nphys * i + 1] = x.first.p1;
    rows[i] = x.second.r;
    cols[i] = x.second.c;
    if (data) std::memcpy(data + off, x.second.d.data(), sizeof(double) * x.second.d.size());
    off += x.second.d.size();
    ++i;
  }
}
void orc_bm_free(void* b) { delete (orc_bm_t*)b; }

static void* wrap_bm(const BM& m, int nphys) {
  orc_bm_t* b = new orc_bm_t;
  b->m = m;
  b->nphys = nphys;
  return b;
}
static void* wrap_diag(const Diag& d) {
  orc_bm_t* b = new orc_bm_t;
  b->nphys = 0;
  for (auto& x : d) {
    Mat m((int)x.second.size(), 1);
    m.d = x.second;
    b->m[K1(x.first, x.first, 0)] = m;
  }
  return b;
}

void* orc_mpo_new(int nterms, const uint32_t* wl, const uint32_t* wr, const uint32_t* out,
                  const uint32_t* in, const double* val, int Dl, int Dr) {
  orc_mpo_t* o = new orc_mpo_t;
  for (int i = 0; i < nterms; ++i) o->w.m[{wl[i], wr[i]}][OpKey{in[i], out[i]}] = val[i];
  o->w.Dl = Dl;
  o->w.Dr = Dr;
  return o;
}
int orc_mpo_nterms(void* m) {
  int n = 0;
  for (auto& x : ((orc_mpo_t*)m)->w.m) n += (int)x.second.size();
  return n;
}
void orc_mpo_export(void* mm, uint32_t* wl, uint32_t* wr, uint32_t* out, uint32_t* in, double* val,
                    int32_t* DlDr) {
  orc_mpo_t* m = (orc_mpo_t*)mm;
  int i = 0;
  for (auto& x : m->w.m)
    for (auto& y : x.second) {
      wl[i] = x.first.wl; wr[i] = x.first.wr; out[i] = y.first.out; in[i] = y.first.in; val[i] = y.second;
      ++i;
    }
  DlDr[0] = m->w.Dl;
  DlDr[1] = m->w.Dr;
}
void orc_mpo_free(void* m) { delete (orc_mpo_t*)m; }

// model builders: out_sites receives N handles
int orc_mpo_heisenberg(int N, const double* Jz, const double* Jxy, const double* B, void** out_sites) {
  auto W = heisenberg(N, Jz, Jxy, B);
  for (int i = 0; i < N; ++i) { orc_mpo_t* o = new orc_mpo_t; o->w = W[i]; out_sites[i] = o; }
  return 0;
}
int orc_mpo_spinless(int N, const double* V, const double* t, const double* mu, void** out_sites) {
  auto W = spinless(N, V, t, mu);
  for (int i = 0; i < N; ++i) { orc_mpo_t* o = new orc_mpo_t; o->w = W[i]; out_sites[i] = o; }
  return 0;
}

void* orc_theta(void* A1, void* A2) {
  return wrap_bm(theta_form(((orc_bm_t*)A1)->m, ((orc_bm_t*)A2)->m), 2);
}
void* orc_contract_twosite(void* L, void* R, void* th, void* W1, void* W2, const uint64_t* ik0,
                           int d0, const uint64_t* ik1, int d1, int nthreads) {
  ItoKey a(ik0, ik0 + d0), b(ik1, ik1 + d1);
  return wrap_bm(contract_twosite(((orc_bm_t*)L)->m, ((orc_bm_t*)R)->m, ((orc_bm_t*)th)->m,
                                  ((orc_mpo_t*)W1)->w, ((orc_mpo_t*)W2)->w, a, b, nthreads), 2);
}
void* orc_add_contraction_layer(void* BL, void* A, void* W, const uint64_t* ik, int d, int dir, int nthreads) {
  ItoKey a(ik, ik + d);
  return wrap_bm(add_contraction_layer(((orc_bm_t*)BL)->m, ((orc_bm_t*)A)->m, ((orc_mpo_t*)W)->w, a, dir, nthreads), 1);
}
// two-tensor addContractionLayer(BL, A, mpo, Ap, itokey, dir) (MPSfunctions.hpp:500-556): A lower, Ap upper
void* orc_add_contraction_layer2(void* BL, void* A, void* Ap, void* W, const uint64_t* ik, int d, int dir,
                                 int nthreads) {
  ItoKey a(ik, ik + d);
  return wrap_bm(add_contraction_layer(((orc_bm_t*)BL)->m, ((orc_bm_t*)A)->m, ((orc_mpo_t*)W)->w, a, dir, nthreads,
                                       &((orc_bm_t*)Ap)->m),
                 1);
}
// computeOverlap(a, b) (MPSfunctions.hpp:2066-2085): identity MPO (D = 1) layers, a lower, b upper.
// ik holds the sites' i_to_key tables back to back, d[s] entries for site s.
double orc_overlap(int N, void* const* a, void* const* b, const uint64_t* ik, const int* d, int nthreads) {
  BM L = get_lmin();
  size_t off = 0;
  for (int s = 0; s < N; ++s) {
    ItoKey k(ik + off, ik + off + d[s]);
    off += d[s];
    MPOMat id;
    for (int i = 0; i < d[s]; ++i) id.m[{0u, 0u}][OpKey{(uint32_t)i, (uint32_t)i}] = 1.0;
    id.Dl = id.Dr = 1;
    L = add_contraction_layer(L, ((orc_bm_t*)a[s])->m, id, k, 1, nthreads, &((orc_bm_t*)b[s])->m);
  }
  return L.empty() ? 0.0 : L.begin()->second(0, 0);
}
// MPO::measure(mps) (MPOTypes.hpp:990-1020) on given site tensors and MPO tensors
double orc_mpo_measure(int N, void* const* sites, void* const* W, const uint64_t* ik, const int* d, int nthreads) {
  std::vector<BM> s;
  std::vector<MPOMat> w;
  std::vector<ItoKey> k;
  size_t off = 0;
  for (int i = 0; i < N; ++i) {
    s.push_back(((orc_bm_t*)sites[i])->m);
    w.push_back(((orc_mpo_t*)W[i])->w);
    k.push_back(ItoKey(ik + off, ik + off + d[i]));
    off += d[i];
  }
  return mpo_measure(s, w, k, nthreads);
}
int orc_split(void* th, const uint64_t* ik0, int d0, const uint64_t* ik1, int d1, int chimax,
              int doTrunc, double tr_weight, int normalize, int nthreads, void** U, void** Vt,
              void** lam, double* tw, int* chi) {
  ItoKey a(ik0, ik0 + d0), b(ik1, ik1 + d1);
  SplitOut o = split2(((orc_bm_t*)th)->m, a, b, chimax, doTrunc != 0, tr_weight, normalize != 0, nthreads);
  *U = wrap_bm(o.U, 1);
  *Vt = wrap_bm(o.Vt, 1);
  *lam = wrap_diag(o.lam);
  *tw = o.tw;
  *chi = o.chi;
  return 0;
}
int orc_lanczos(void* L, void* R, void* theta, void* W1, void* W2, const uint64_t* ik0, int d0,
                const uint64_t* ik1, int d1, int itmax, double delta, int testenergy, int nthreads,
                double* E0, int* iters, void** state) {
  ItoKey a(ik0, ik0 + d0), b(ik1, ik1 + d1);
  LanczosOut o = lanczos(((orc_bm_t*)L)->m, ((orc_bm_t*)R)->m, ((orc_bm_t*)theta)->m,
                         ((orc_mpo_t*)W1)->w, ((orc_mpo_t*)W2)->w, a, b, itmax, delta,
                         testenergy != 0, nthreads, nullptr);
  *E0 = o.E0;
  *iters = o.iterations;
  *state = wrap_bm(o.state, 2);
  return 0;
}

// DMRG engine: sites[N] single-site block matrices, mpos[N], itokeys N*d charges
void* orc_dmrg_new(int N, void** sites, void** mpos, const uint64_t* itokeys, int d) {
  orc_dmrg_t* e = new orc_dmrg_t;
  e->g.mps.s.resize(N);
  e->g.mpo.resize(N);
  e->g.mps.ik.resize(N);
  for (int i = 0; i < N; ++i) {
    e->g.mps.s[i] = ((orc_bm_t*)sites[i])->m;
    e->g.mpo[i] = ((orc_mpo_t*)mpos[i])->w;
    e->g.mps.ik[i] = ItoKey(itokeys + (size_t)i * d, itokeys + (size_t)(i + 1) * d);
  }
  Mat m(1, 1);
  m(0, 0) = 1.0;
  e->g.mps.leftDummy[K1(0, 0, 0)] = m;
  return e;
}
void orc_dmrg_set_threads(void* e, int maxthreads, int matvec_threads) {
  ((orc_dmrg_t*)e)->g.maxthreads = maxthreads;
  ((orc_dmrg_t*)e)->g.matvec_threads = matvec_threads;
}
double orc_dmrg_simulate(void* e, int maxsteps, double EnConv, int chimax, int doTrunc,
                         double tr_weight, double delta, int testenergy) {
  return dmrg_simulate(((orc_dmrg_t*)e)->g, maxsteps, EnConv, chimax, doTrunc != 0, tr_weight, delta, testenergy != 0);
}
// single doStep, for bounded CPU-baseline samples (requires a prior dmrg_prepare)
int orc_dmrg_prepare(void* ee) {
  DMRG& g = ((orc_dmrg_t*)ee)->g;
  MPS& mps = g.mps;
  const int N = (int)mps.s.size();
  orthonormalize_rl(mps);
  g.R.clear();
  g.R[N] = get_rmax(mps.s[N - 1]);
  for (int s = N - 1; s >= 2; --s)
    g.R[s] = add_contraction_layer(g.R[s + 1], mps.s[s], g.mpo[s], mps.ik[s], 0, g.maxthreads);
  g.L.clear();
  g.L[-1] = get_lmin();
  return 0;
}
// replace one environment (which = 0: L[site], 1: R[site]) with a given block matrix
int orc_dmrg_set_env(void* ee, int which, int site, void* bm) {
  DMRG& g = ((orc_dmrg_t*)ee)->g;
  (which ? g.R : g.L)[site] = ((orc_bm_t*)bm)->m;
  return 0;
}
// environments of the current (mixed-canonical) MPS around bond (center, center+1)
int orc_dmrg_build_envs(void* ee, int center) {
  DMRG& g = ((orc_dmrg_t*)ee)->g;
  MPS& mps = g.mps;
  const int N = (int)mps.s.size();
  g.L.clear();
  g.L[-1] = get_lmin();
  for (int s = 0; s < center; ++s)
    g.L[s] = add_contraction_layer(g.L[s - 1], mps.s[s], g.mpo[s], mps.ik[s], 1, g.maxthreads);
  g.R.clear();
  g.R[N] = get_rmax(mps.s[N - 1]);
  for (int s = N - 1; s >= center + 2; --s)
    g.R[s] = add_contraction_layer(g.R[s + 1], mps.s[s], g.mpo[s], mps.ik[s], 0, g.maxthreads);
  return 0;
}
double orc_dmrg_do_step(void* ee, int site, int dir, int chimax, int doTrunc, double tr_weight,
                        double delta, int testenergy) {
  return dmrg_step(((orc_dmrg_t*)ee)->g, site, dir, chimax, doTrunc != 0, tr_weight, delta, testenergy != 0).E;
}
int orc_dmrg_nsteps(void* e) { return (int)((orc_dmrg_t*)e)->g.steps.size(); }
void orc_dmrg_steps(void* ee, int32_t* site, int32_t* dir, int32_t* iters, int32_t* chi, double* E, double* tw) {
  auto& s = ((orc_dmrg_t*)ee)->g.steps;
  for (size_t i = 0; i < s.size(); ++i) {
    site[i] = s[i].site; dir[i] = s[i].dir; iters[i] = s[i].iters; chi[i] = s[i].chi; E[i] = s[i].E; tw[i] = s[i].tw;
  }
}
void orc_dmrg_times(void* ee, double* t4) {
  auto& g = ((orc_dmrg_t*)ee)->g;
  t4[0] = g.t_total; t4[1] = g.t_matvec; t4[2] = g.t_env; t4[3] = g.t_split;
}
void* orc_dmrg_site(void* e, int s) { return wrap_bm(((orc_dmrg_t*)e)->g.mps.s[s], 1); }
void* orc_dmrg_lambda(void* e, int bond) { return wrap_diag(((orc_dmrg_t*)e)->g.mps.lam[bond]); }
void* orc_dmrg_env(void* e, int which, int s) {
  auto& g = ((orc_dmrg_t*)e)->g;
  return wrap_bm(which ? g.R[s] : g.L[s], 1);
}
double orc_dmrg_measure(void* ee, int nthreads) {
  auto& g = ((orc_dmrg_t*)ee)->g;
  return mpo_measure(g.mps.s, g.mpo, g.mps.ik, nthreads);
}
void orc_dmrg_free(void* e) { delete (orc_dmrg_t*)e; }


// ---- TEBD: product state, second-order evolution, diagonal local measurement, export
struct orc_tebd_t { TEBDState st; std::vector<MPOMat> mpo; };
void* orc_tebd_new(int N, const int* local, void* const* W, const uint64_t* ik, const int* d) {
  orc_tebd_t* t = new orc_tebd_t;
  std::vector<ItoKey> iks;
  size_t off = 0;
  for (int s = 0; s < N; ++s) {
    iks.push_back(ItoKey(ik + off, ik + off + d[s]));
    off += d[s];
    t->mpo.push_back(((orc_mpo_t*)W[s])->w);
  }
  t->st = tebd_product(std::vector<int>(local, local + N), iks);
  return t;
}
void orc_tebd_second_order(void* tt, int steps, double dt, int chimax, int doTrunc, double tr_weight, int normalize) {
  orc_tebd_t* t = (orc_tebd_t*)tt;
  tebd_second_order(t->st, t->mpo, steps, dt, chimax, doTrunc != 0, tr_weight, normalize != 0);
}
double orc_tebd_measure_diag(void* tt, int site, const double* op, int d) {
  return tebd_measure_diag(((orc_tebd_t*)tt)->st, site, std::vector<double>(op, op + d));
}
// complex block export of Gamma[site]: sizes via orc_tebd_gamma_info, data interleaved (re, im)
int orc_tebd_gamma_info(void* tt, int site, long* nelem) {
  const CBM& g = ((orc_tebd_t*)tt)->st.G[site];
  long n = 0;
  for (auto& b : g) n += (long)b.second.d.size();
  *nelem = n;
  return (int)g.size();
}
void orc_tebd_gamma_export(void* tt, int site, uint64_t* q, uint32_t* p, int32_t* rows, int32_t* cols, double* data) {
  const CBM& g = ((orc_tebd_t*)tt)->st.G[site];
  size_t i = 0, off = 0;
  for (auto& b : g) {
    q[2 * i] = b.first.q0; q[2 * i + 1] = b.first.q1; p[i] = b.first.p0;
    rows[i] = b.second.r; cols[i] = b.second.c;
    for (auto& v : b.second.d) { data[off++] = v.real(); data[off++] = v.imag(); }
    ++i;
  }
}
void* orc_tebd_lambda(void* tt, int bond) { return wrap_diag(((orc_tebd_t*)tt)->st.lam[bond + 1]); }
// the dense two-site gate (d1 d2 x d1 d2, column-major, index o1 + d1 o2), interleaved complex
void orc_nn_gate(void* W1, void* W2, int site1, int N, double dt_re, double dt_im, int d1, int d2, double* out) {
  Gate G = nn_gate(((orc_mpo_t*)W1)->w, ((orc_mpo_t*)W2)->w, site1, N, dt_re, dt_im, d1, d2);
  for (size_t i = 0; i < G.g.size(); ++i) { out[2 * i] = G.g[i].real(); out[2 * i + 1] = G.g[i].imag(); }
}
void orc_tebd_free(void* t) { delete (orc_tebd_t*)t; }

}  // extern "C"
