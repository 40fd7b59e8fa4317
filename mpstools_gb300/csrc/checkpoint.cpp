// Portable checkpoint of a DMRG state (what MPSBase::save / DMRGengine keep across runs,
// src/MPSTypes.hpp:377-426, src/container.hpp:87-146, in a documented format instead of a Boost
// binary archive): the site tensors, the lambdas, the charge maps and the MPO, so that a long run can
// resume and states can move between the CPU oracle and the GPU engine.
//
// File format "MPSGCKP1" (little-endian; tensors FP64, blocks in key order, each block column-major):
//   char[8] "MPSGCKP1"; u32 version (2; version 1 files lack the settings record and still load);
//   u32 N
//   version >= 2: u32 prec (mpsg_prec); u32 reorth; u32 lanmax; u64 updates (doStep calls made)
//   per site s = 0 .. N-1:
//     u32 d; u64 charge[d]                                   (i_to_key)
//     u32 Dl; u32 Dr; u32 nterms; nterms x {u32 wl, wr, out, in; f64 value}   (MPOMat)
//     u32 nblocks; nblocks x {u64 q0, q1; u32 p; i32 rows, cols}; f64 data[sum rows * cols]
//   u32 nlambda; nlambda x {i32 bond; u32 nblocks; nblocks x {u64 q; i32 n}; f64 data[sum n]}
//   char[8] "MPSGEND!"
#include <cstdio>
#include <cstring>

#include "engine.h"

namespace mpsg {
namespace {

constexpr char kMagic[8] = {'M', 'P', 'S', 'G', 'C', 'K', 'P', '1'};
constexpr char kEnd[8] = {'M', 'P', 'S', 'G', 'E', 'N', 'D', '!'};
constexpr uint32_t kVersion = 2;

struct File {
  FILE* f = nullptr;
  File(const char* path, const char* mode) : f(std::fopen(path, mode)) {
    if (!f) throw Err(1, std::string("cannot open checkpoint file ") + path);
  }
  ~File() {
    if (f) std::fclose(f);
  }
  void put(const void* p, size_t n) {
    if (n && std::fwrite(p, 1, n, f) != n) throw Err(1, "checkpoint write failed");
  }
  void get(void* p, size_t n) {
    if (n && std::fread(p, 1, n, f) != n) throw Err(1, "checkpoint file truncated");
  }
  // bytes left after the read position (checked before any allocation sized by the file)
  int64_t remaining() {
    const long cur = std::ftell(f);
    if (cur < 0 || std::fseek(f, 0, SEEK_END) != 0) throw Err(1, "checkpoint file is not seekable");
    const long end = std::ftell(f);
    if (end < 0 || std::fseek(f, cur, SEEK_SET) != 0) throw Err(1, "checkpoint file is not seekable");
    return (int64_t)end - (int64_t)cur;
  }
  template <class T>
  void put(T v) {
    put(&v, sizeof(T));
  }
  template <class T>
  T get() {
    T v;
    get(&v, sizeof(T));
    return v;
  }
};

// sanity bounds of a header field read from a file (a corrupt file must not drive huge allocations)
uint32_t bounded(uint32_t v, uint32_t hi, const char* what) {
  if (v > hi) throw Err(1, std::string("checkpoint: implausible ") + what);
  return v;
}

void write_tensor(File& f, const Tensor& t) {
  std::vector<double> data;
  tensor_to_host(t, data);
  f.put<uint32_t>((uint32_t)t.b.size());
  for (const Block& b : t.b) {
    f.put<uint64_t>(b.k.q0);
    f.put<uint64_t>(b.k.q1);
    f.put<uint32_t>(b.k.p0);
    f.put<int32_t>(b.r);
    f.put<int32_t>(b.c);
  }
  f.put(data.data(), sizeof(double) * data.size());
}

// Site tensor of local dimension d: block physical indices must be < d, and the data the block
// table declares must be present in the file before anything is allocated for it.
TensorP read_tensor(File& f, Ctx* ctx, uint32_t d) {
  const uint32_t n = bounded(f.get<uint32_t>(), 1u << 24, "block count");
  if ((int64_t)n * 28 > f.remaining()) throw Err(1, "checkpoint file truncated (block table)");
  std::vector<uint64_t> q(2 * (size_t)n);
  std::vector<uint32_t> p(n);
  std::vector<int32_t> r(n), c(n);
  int64_t total = 0;
  for (uint32_t i = 0; i < n; ++i) {
    q[2 * i] = f.get<uint64_t>();
    q[2 * i + 1] = f.get<uint64_t>();
    p[i] = f.get<uint32_t>();
    r[i] = f.get<int32_t>();
    c[i] = f.get<int32_t>();
    if (r[i] < 0 || c[i] < 0 || r[i] > (1 << 20) || c[i] > (1 << 20)) throw Err(1, "checkpoint: implausible block size");
    if (p[i] >= d) throw Err(1, "checkpoint: block physical index out of range of the site's itokey");
    total += (int64_t)r[i] * c[i];
  }
  if (total > ((int64_t)1 << 34)) throw Err(1, "checkpoint: implausible tensor size");
  if (total * (int64_t)sizeof(double) > f.remaining()) throw Err(1, "checkpoint file truncated (block data)");
  std::vector<double> data((size_t)std::max<int64_t>(total, 1));
  f.get(data.data(), sizeof(double) * (size_t)total);
  return tensor_from_host(ctx, 1, (int)n, q.data(), p.data(), r.data(), c.data(), data.data());
}

}  // namespace
}  // namespace mpsg

using namespace mpsg;

extern "C" {

mpsg_status mpsg_dmrg_save(mpsg_dmrg e, const char* path) {
  API_BEGIN
  MPSG_CHECK(e && e->e && path, "null argument");
  Engine& x = *e->e;
  File f(path, "wb");
  f.put(kMagic, 8);
  f.put<uint32_t>(kVersion);
  f.put<uint32_t>((uint32_t)x.N);
  f.put<uint32_t>((uint32_t)x.prec);
  f.put<uint32_t>(x.reorth ? 1u : 0u);
  f.put<uint32_t>((uint32_t)x.lanmax);
  f.put<uint64_t>((uint64_t)x.updates_done());
  for (int s = 0; s < x.N; ++s) {
    f.put<uint32_t>((uint32_t)x.ik[s].size());
    for (Q q : x.ik[s]) f.put<uint64_t>(q);
    const MPO& m = x.mpo[s];
    uint32_t nt = 0;
    for (auto& en : m.e) nt += (uint32_t)en.ops.size();
    f.put<uint32_t>((uint32_t)m.Dl);
    f.put<uint32_t>((uint32_t)m.Dr);
    f.put<uint32_t>(nt);
    for (auto& en : m.e)
      for (auto& op : en.ops) {
        f.put<uint32_t>(en.wl);
        f.put<uint32_t>(en.wr);
        f.put<uint32_t>(op.out);
        f.put<uint32_t>(op.in);
        f.put<double>(op.v);
      }
    write_tensor(f, *x.mps[s]);
  }
  f.put<uint32_t>((uint32_t)x.lam.size());
  for (auto& kv : x.lam) {
    const Tensor& l = *kv.second;
    std::vector<double> data;
    tensor_to_host(l, data);
    f.put<int32_t>(kv.first);
    f.put<uint32_t>((uint32_t)l.b.size());
    for (const Block& b : l.b) {
      f.put<uint64_t>(b.k.q0);
      f.put<int32_t>(b.r);
    }
    f.put(data.data(), sizeof(double) * data.size());
  }
  f.put(kEnd, 8);
  API_END
}

mpsg_status mpsg_dmrg_load(mpsg_ctx ctx, const char* path, mpsg_dmrg* out) {
  API_BEGIN
  MPSG_CHECK(ctx && path && out, "null argument");
  File f(path, "rb");
  char magic[8];
  f.get(magic, 8);
  MPSG_CHECK(std::memcmp(magic, kMagic, 8) == 0, "not an MPSG checkpoint file");
  const uint32_t version = f.get<uint32_t>();
  MPSG_CHECK(version == 1 || version == 2, "unsupported checkpoint version");
  const int N = (int)bounded(f.get<uint32_t>(), 1u << 20, "site count");
  MPSG_CHECK(N >= 3, "DMRG needs at least 3 sites");
  std::unique_ptr<Engine> e(new Engine());
  e->ctx = C(ctx);
  e->keep = e->ctx->shared_from_this();
  e->N = N;
  if (version >= 2) {  // run settings; a version-1 file resumes with the FP64 defaults
    const uint32_t prec = f.get<uint32_t>();
    MPSG_CHECK(prec <= (uint32_t)MPSG_PREC_MIXED, "checkpoint: unknown matvec precision");
    e->prec = (mpsg_prec)prec;
    e->reorth = f.get<uint32_t>() != 0;
    e->lanmax = (int)bounded(f.get<uint32_t>(), 1000, "Lanczos iteration limit");
    MPSG_CHECK(e->lanmax >= 1, "checkpoint: Lanczos iteration limit must be in [1, 1000]");
    e->updates_base = (int64_t)f.get<uint64_t>();
  }
  for (int s = 0; s < N; ++s) {
    const uint32_t d = bounded(f.get<uint32_t>(), 1u << 16, "local dimension");
    ItoKey ik(d);
    for (uint32_t i = 0; i < d; ++i) ik[i] = f.get<uint64_t>();
    e->ik.push_back(ik);
    std::vector<uint32_t> wl, wr, o, in;
    std::vector<double> v;
    mpsg_mpo m{};
    m.Dl = (int32_t)bounded(f.get<uint32_t>(), 1u << 16, "MPO dimension");
    m.Dr = (int32_t)bounded(f.get<uint32_t>(), 1u << 16, "MPO dimension");
    const uint32_t nt = bounded(f.get<uint32_t>(), 1u << 24, "MPO term count");
    if ((int64_t)nt * 24 > f.remaining()) throw Err(1, "checkpoint file truncated (MPO terms)");
    for (uint32_t t = 0; t < nt; ++t) {
      wl.push_back(f.get<uint32_t>());
      wr.push_back(f.get<uint32_t>());
      o.push_back(f.get<uint32_t>());
      in.push_back(f.get<uint32_t>());
      v.push_back(f.get<double>());
      if (wl.back() >= (uint32_t)m.Dl || wr.back() >= (uint32_t)m.Dr || o.back() >= d || in.back() >= d)
        throw Err(1, "checkpoint: MPO term index out of range");
    }
    m.nterms = (int32_t)nt;
    m.wl = wl.data();
    m.wr = wr.data();
    m.out = o.data();
    m.in = in.data();
    m.value = v.data();
    e->mpo.push_back(mpo_from_c(&m));
    e->mps.push_back(read_tensor(f, e->ctx, d));
  }
  const uint32_t nl = bounded(f.get<uint32_t>(), 1u << 20, "lambda count");
  for (uint32_t i = 0; i < nl; ++i) {
    const int32_t bond = f.get<int32_t>();
    const uint32_t n = bounded(f.get<uint32_t>(), 1u << 24, "lambda block count");
    if ((int64_t)n * 12 > f.remaining()) throw Err(1, "checkpoint file truncated (lambda table)");
    std::vector<uint64_t> q(2 * (size_t)n);
    std::vector<uint32_t> p(n, 0);
    std::vector<int32_t> r(n), c(n, 1);
    int64_t total = 0;
    for (uint32_t j = 0; j < n; ++j) {
      q[2 * j] = q[2 * j + 1] = f.get<uint64_t>();
      r[j] = f.get<int32_t>();
      if (r[j] < 0 || r[j] > (1 << 20)) throw Err(1, "checkpoint: implausible lambda size");
      total += r[j];
    }
    if (total * (int64_t)sizeof(double) > f.remaining()) throw Err(1, "checkpoint file truncated (lambda data)");
    std::vector<double> data((size_t)std::max<int64_t>(total, 1));
    f.get(data.data(), sizeof(double) * (size_t)total);
    e->lam[bond] = tensor_from_host(e->ctx, 0, (int)n, q.data(), p.data(), r.data(), c.data(), data.data());
  }
  char end[8];
  f.get(end, 8);
  MPSG_CHECK(std::memcmp(end, kEnd, 8) == 0, "checkpoint end marker missing");
  mpsg_dmrg d = new mpsg_dmrg_s;
  d->e = e.release();
  *out = d;
  API_END
}

}  // extern "C"
