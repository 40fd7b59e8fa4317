"""CPU test: the C++ adapter printed in INTEGRATION.md compiles against include/mpsg.h.

The adapter is what a maintainer adds next to MPSTools' headers.  MPSTools itself cannot be built
here (it needs Boost), so the test compiles the snippet (syntax and types only, no link) against a
minimal stand-in for the reference types it touches, written from their interfaces:
AbKeyType(q, 1) / getQ() (src/keyTypes.hpp:20-31), TensorKeyType<2,Ns,K> with operator[] for the
charge keys, operator() for the physical indices and a (key0, key1, std::vector<uint>) constructor
(:166-200), BlockMatrix as a map from keys to column-major matrices (src/BlockTensor.hpp:279-379),
MPOMat<1,T> as a map from ukey<2> to SparseOperator with public Dl / Dr (src/MPOTypes.hpp:839-885),
SparseOperator entries keyed by OpKeyType<1> (operator[] the in index, operator() the out index,
src/keyTypes.hpp:383-421), i_to_key as a map from local state to AbKeyType (src/tensormap.hpp:280-298)
and mps_exception (src/MPSTypes.hpp:25).
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STANDIN = r"""
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>
typedef double Real;
typedef unsigned int uint;
struct AbKeyType {
  unsigned long q = 0;
  AbKeyType() {}
  AbKeyType(const unsigned long& in, const int&) : q(in) {}
  unsigned long getQ() const { return q; }
  bool operator<(const AbKeyType& o) const { return q < o.q; }
};
template <size_t Nb, size_t Ns, class K>
struct TensorKeyType {
  K k[Nb];
  uint p[Ns > 0 ? Ns : 1];
  TensorKeyType() {}
  TensorKeyType(const K& a, const K& b, const std::vector<uint>& ps) {
    k[0] = a;
    k[1] = b;
    for (size_t i = 0; i < Ns; ++i) p[i] = ps[i];
  }
  K operator[](int i) const { return k[i]; }
  uint operator()(int i) const { return p[i]; }
  bool operator<(const TensorKeyType& o) const { return k[0] < o.k[0]; }
};
struct column_major {};
template <class T, class L>
struct matrix {
  std::vector<T> v;
  size_t r = 0, c = 0;
  matrix() {}
  matrix(size_t r_, size_t c_) : v(r_ * c_), r(r_), c(c_) {}
  size_t size1() const { return r; }
  size_t size2() const { return c; }
  std::vector<T>& data() { return v; }
  const std::vector<T>& data() const { return v; }
};
template <int Ns, class K, class T>
struct BlockMatrix : std::map<TensorKeyType<2, Ns, K>, matrix<T, column_major>> {};
struct ukey2 {
  uint k[2];
  uint operator[](int i) const { return k[i]; }
  bool operator<(const ukey2& o) const { return k[0] < o.k[0] || (k[0] == o.k[0] && k[1] < o.k[1]); }
};
struct OpKeyType1 {
  uint in, out;
  uint operator[](int) const { return in; }
  uint operator()(int) const { return out; }
  bool operator<(const OpKeyType1& o) const { return in < o.in || (in == o.in && out < o.out); }
};
template <int Ns, class T>
struct SparseOperator : std::map<OpKeyType1, T> {};
template <int Ns, class T>
struct MPOMat : std::map<ukey2, SparseOperator<Ns, T>> {
  uint Dl = 0, Dr = 0;
};
template <class K>
struct i_to_key : std::map<uint, K> {};
struct mps_exception : std::runtime_error {
  explicit mps_exception(const std::string& s) : std::runtime_error(s) {}
};
"""


def _snippet():
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        text = f.read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    assert blocks, "INTEGRATION.md holds no C++ block"
    return blocks[0]


def test_integration_adapter_compiles(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "adapter.cpp"
    src.write_text(STANDIN + "\n#include <algorithm>\n" + _snippet() + "\n")
    out = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"), str(src)],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
