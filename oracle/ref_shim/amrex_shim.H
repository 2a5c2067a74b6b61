// amrex_shim.H — ORACLE test infrastructure: the few AMReX types and
// functions that PeleC's hot-path headers use (Source/MOL.H, MOL.cpp,
// Riemann.H, Diffterm.H, Utilities.H, EBStencilTypes.H, Constants.H,
// Timestep.H), restated for one CPU and AMREX_SPACEDIM = 3 so that those reference
// sources compile unchanged where they lie.  AMReX itself is absent (the
// reference's Submodules tree is empty); each piece below states the AMReX
// semantics it follows.  Built only by oracle/ref_build.py.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#define AMREX_SPACEDIM 3
#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST_DEVICE
#define AMREX_GPU_CONSTANT
#define AMREX_FORCE_INLINE inline
#define AMREX_D_DECL(a, b, c) a, b, c
#define AMREX_D_TERM(a, b, c) a b c
#define AMREX_D_PICK(a, b, c) c
#define BL_PROFILE(x)
#define AMREX_ALWAYS_ASSERT_WITH_MESSAGE(c, m) \
  do {                                          \
    if (!(c)) amrex::Abort(m);                  \
  } while (0)

#ifdef PC_COUNT_FLOPS
#include "flop_count.hpp"
#endif

namespace amrex {

#ifdef PC_COUNT_FLOPS
using Real = pcc::CReal;  // the flop-counting build (flop_count.hpp)
#else
using Real = double;
#endif

// amrex::min / amrex::max (AMReX_Algorithm.H): std::min / std::max.
template <class T>
constexpr const T& min(const T& a, const T& b) noexcept { return std::min(a, b); }
template <class T>
constexpr const T& max(const T& a, const T& b) noexcept { return std::max(a, b); }

namespace Math {
template <class T>
constexpr T pi() { return T(3.1415926535897932384626433832795029); }
}  // namespace Math

template <class T>
using Vector = std::vector<T>;

[[noreturn]] inline void Abort(const char* msg = "") { throw std::runtime_error(std::string("amrex::Abort: ") + msg); }
[[noreturn]] inline void Error(const char* msg = "") { Abort(msg); }

struct Dim3 {
  int x, y, z;
};

// IntVect: three integers with componentwise arithmetic.
struct IntVect {
  int v[3] = {0, 0, 0};
  constexpr IntVect() = default;
  constexpr explicit IntVect(int a) : v{a, a, a} {}
  constexpr IntVect(int a, int b, int c) : v{a, b, c} {}
  int& operator[](int d) { return v[d]; }
  int operator[](int d) const { return v[d]; }
  IntVect operator+(const IntVect& o) const { return {v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]}; }
  IntVect operator-(const IntVect& o) const { return {v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]}; }
  IntVect operator-() const { return {-v[0], -v[1], -v[2]}; }
  bool operator<(const IntVect& o) const {  // lexicographic, k slowest
    for (int d = 2; d >= 0; --d)
      if (v[d] != o.v[d]) return v[d] < o.v[d];
    return false;
  }
  static IntVect TheDimensionVector(int d) { return {d == 0, d == 1, d == 2}; }
};

struct RealVect {
  Real v[3] = {0.0, 0.0, 0.0};
  RealVect() = default;
  RealVect(Real a, Real b, Real c) : v{a, b, c} {}
  Real& operator[](int d) { return v[d]; }
  Real operator[](int d) const { return v[d]; }
  RealVect operator-(const RealVect& o) const { return {v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]}; }
  Real radSquared() const { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
};

// Cell-centred box [lo, hi] (node-centred boxes are represented by their
// index range, which is all the reference's loops use).
struct Box {
  IntVect lo, hi;
  Box() = default;
  Box(const IntVect& l, const IntVect& h) : lo(l), hi(h) {}
  const IntVect& smallEnd() const { return lo; }
  const IntVect& bigEnd() const { return hi; }
  int smallEnd(int d) const { return lo[d]; }
  int bigEnd(int d) const { return hi[d]; }
  void setSmall(int d, int x) { lo[d] = x; }
  void setBig(int d, int x) { hi[d] = x; }
  bool ok() const { return lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2]; }
  long long numPts() const {
    return ok() ? (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) : 0;
  }
  bool contains(const IntVect& p) const {
    for (int d = 0; d < 3; ++d)
      if (p[d] < lo[d] || p[d] > hi[d]) return false;
    return true;
  }
};
inline Box grow(Box b, int n) {
  for (int d = 0; d < 3; ++d) {
    b.lo[d] -= n;
    b.hi[d] += n;
  }
  return b;
}
inline Box grow(Box b, int dir, int n) {
  b.lo[dir] -= n;
  b.hi[dir] += n;
  return b;
}
inline Box surroundingNodes(Box b, int dir) {
  b.hi[dir] += 1;
  return b;
}

// Array4 (AMReX_Array4.H): a non-owning view, i fastest, component slowest.
template <class T>
struct Array4 {
  T* p = nullptr;
  long long jstride = 0, kstride = 0, nstride = 0;
  Dim3 begin{0, 0, 0}, end{0, 0, 0};
  int ncomp = 0;
  Array4() = default;
  Array4(T* ptr, Dim3 b, Dim3 e, int nc) : p(ptr), begin(b), end(e), ncomp(nc) {
    jstride = e.x - b.x;
    kstride = jstride * (e.y - b.y);
    nstride = kstride * (e.z - b.z);
  }
  template <class U, class = std::enable_if_t<std::is_same<const U, T>::value && !std::is_same<U, T>::value>>
  Array4(const Array4<U>& o)
      : p(o.p), jstride(o.jstride), kstride(o.kstride), nstride(o.nstride), begin(o.begin), end(o.end),
        ncomp(o.ncomp) {}
  T& operator()(int i, int j, int k) const {
    return p[(i - begin.x) + (j - begin.y) * jstride + (k - begin.z) * kstride];
  }
  T& operator()(int i, int j, int k, int n) const {
    return p[(i - begin.x) + (j - begin.y) * jstride + (k - begin.z) * kstride + n * nstride];
  }
  T& operator()(const IntVect& iv) const { return (*this)(iv[0], iv[1], iv[2]); }
  T& operator()(const IntVect& iv, int n) const { return (*this)(iv[0], iv[1], iv[2], n); }
};

// EBCellFlag (AMReX_EBCellFlag.H) of a regular cell: every neighbour
// connected, not covered, regular.
struct EBCellFlag {
  bool isConnected(const IntVect&) const { return true; }
  bool isConnected(int, int, int) const { return true; }
  bool isCovered() const { return false; }
  bool isRegular() const { return true; }
  bool isSingleValued() const { return false; }
};
// The flag array of an all-regular box: every index reads a regular flag.
template <>
struct Array4<EBCellFlag const> {
  EBCellFlag f{};
  EBCellFlag operator()(int, int, int) const { return f; }
  EBCellFlag operator()(const IntVect&) const { return f; }
};

template <class T, std::size_t N>
struct GpuArray {
  T arr[N];
  T& operator[](int i) { return arr[i]; }
  const T& operator[](int i) const { return arr[i]; }
  T* data() { return arr; }
  const T* data() const { return arr; }
  static constexpr std::size_t size() { return N; }
};

struct Arena {};
inline Arena* The_Async_Arena() {
  static Arena a;
  return &a;
}

// FArrayBox: an owning box of ncomp doubles, zero-initialised.
struct FArrayBox {
  Box bx;
  int nc = 0;
  std::vector<Real> data;
  FArrayBox() = default;
  FArrayBox(const Box& b, int ncomp, Arena* = nullptr) { resize(b, ncomp); }
  void resize(const Box& b, int ncomp, Arena* = nullptr) {
    bx = b;
    nc = ncomp;
    data.assign((std::size_t)b.numPts() * ncomp, 0.0);
  }
  const Box& box() const { return bx; }
  int nComp() const { return nc; }
  Array4<Real> array() {
    return Array4<Real>(data.data(), Dim3{bx.lo[0], bx.lo[1], bx.lo[2]},
                        Dim3{bx.hi[0] + 1, bx.hi[1] + 1, bx.hi[2] + 1}, nc);
  }
  Array4<Real> array(int start) {
    Array4<Real> a = array();
    a.p += start * a.nstride;
    a.ncomp = nc - start;
    return a;
  }
};

struct GeometryData {
  Real prob_lo[3] = {0.0, 0.0, 0.0};
  Real dx[3] = {1.0, 1.0, 1.0};
  Real ProbLo(int d) const { return prob_lo[d]; }
  Real CellSize(int d) const { return dx[d]; }
};
struct Geometry {
  GeometryData gd;
  GeometryData data() const { return gd; }
  GpuArray<Real, 3> InvCellSizeArray() const { return {{1.0 / gd.dx[0], 1.0 / gd.dx[1], 1.0 / gd.dx[2]}}; }
  GpuArray<Real, 3> CellSizeArray() const { return {{gd.dx[0], gd.dx[1], gd.dx[2]}}; }
};

// ParallelFor over a box (k slowest, i fastest).  Iterations write disjoint
// elements in the reference's loops, so the k planes run in parallel.
template <class F>
inline void ParallelFor(const Box& b, F&& f) {
#pragma omp parallel for schedule(static)
  for (int k = b.lo[2]; k <= b.hi[2]; ++k)
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
      for (int i = b.lo[0]; i <= b.hi[0]; ++i) f(i, j, k);
}
template <class F>
inline void ParallelFor(const Box& b, int ncomp, F&& f) {
  for (int n = 0; n < ncomp; ++n) {
#pragma omp parallel for schedule(static)
    for (int k = b.lo[2]; k <= b.hi[2]; ++k)
      for (int j = b.lo[1]; j <= b.hi[1]; ++j)
        for (int i = b.lo[0]; i <= b.hi[0]; ++i) f(i, j, k, n);
  }
}
// Loop: the serial form of ParallelFor, used where the body reduces into a
// captured variable (Timestep.H).
template <class F>
inline void Loop(const Box& b, F&& f) {
  for (int k = b.lo[2]; k <= b.hi[2]; ++k)
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
      for (int i = b.lo[0]; i <= b.hi[0]; ++i) f(i, j, k);
}
template <class F>
inline void ParallelFor(int n, F&& f) {
  for (int i = 0; i < n; ++i) f(i);
}

}  // namespace amrex
