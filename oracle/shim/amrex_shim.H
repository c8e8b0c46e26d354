// Minimal host-only stand-ins for the AMReX types that OpenCFD-AMR's point
// kernels use, written for this project so that the reference's kernel headers
// (Source/kernel/*.H, Source/EB/*.H, Source/CHEM/*.H) compile unmodified on the
// CPU.  This is test infrastructure (the oracle), never part of the product.
//
// Semantics follow AMReX's public documentation:
//   * Array4<T>: non-owning view, element (i,j,k,n) at
//       p[(i-begin.x) + (j-begin.y)*jstride + (k-begin.z)*kstride + n*nstride]
//   * GpuArray<T,N>: aggregate fixed array
//   * EBCellFlag: 32-bit word, bits 0-1 cell type (0 regular, 1 single-valued,
//     3 covered), bits 4..30 connectivity to the 27 neighbours at bit
//     4 + (i+1) + 3*(j+1) + 9*(k+1)
#ifndef OCFD_AMREX_SHIM_H
#define OCFD_AMREX_SHIM_H

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cstdlib>

#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST
#define AMREX_GPU_HOST_DEVICE
#define AMREX_FORCE_INLINE inline
#define AMREX_SPACEDIM 3
#define AMREX_DEVICE_PRINTF(...) std::printf(__VA_ARGS__)

#ifdef OCFD_COUNT_FLOPS
#include "flop_real.H"
#endif

namespace amrex {

#ifdef OCFD_COUNT_FLOPS
using Real = CountedReal;
#else
using Real = double;
#endif

namespace literals {
inline constexpr Real operator""_rt(long double x) { return Real(x); }
}

struct Dim3 { int x, y, z; };

template <class T>
struct Array4 {
    T* p = nullptr;
    long long jstride = 0, kstride = 0, nstride = 0;
    Dim3 begin{0, 0, 0};
    Dim3 end{0, 0, 0};  // exclusive
    int ncomp = 0;

    Array4() = default;
    Array4(T* p_, long long js, long long ks, long long ns, Dim3 b, Dim3 e, int nc)
        : p(p_), jstride(js), kstride(ks), nstride(ns), begin(b), end(e), ncomp(nc) {}
    // Array4<T> -> Array4<T const>
    template <class U>
    Array4(Array4<U> const& o)
        : p(o.p), jstride(o.jstride), kstride(o.kstride), nstride(o.nstride),
          begin(o.begin), end(o.end), ncomp(o.ncomp) {}

    long long idx(int i, int j, int k, int n) const {
        return (long long)(i - begin.x) + (long long)(j - begin.y) * jstride +
               (long long)(k - begin.z) * kstride + (long long)n * nstride;
    }
    T& operator()(int i, int j, int k) const { return p[idx(i, j, k, 0)]; }
    T& operator()(int i, int j, int k, int n) const { return p[idx(i, j, k, n)]; }
};

template <class T, int N>
struct GpuArray {
    T arr[N];
    T& operator[](int i) { return arr[i]; }
    const T& operator[](int i) const { return arr[i]; }
    T* data() { return arr; }
    const T* data() const { return arr; }
};

struct IntVect {
    int v[3];
    int& operator[](int i) { return v[i]; }
    const int& operator[](int i) const { return v[i]; }
};

namespace Math {
template <class T> inline T abs(T x) { return std::abs(x); }
inline Real cospi(Real x) { return std::cos(M_PI * x); }
inline Real sinpi(Real x) { return std::sin(M_PI * x); }
}  // namespace Math

template <class T> inline T max(T a, T b) { return a > b ? a : b; }
template <class T> inline T min(T a, T b) { return a < b ? a : b; }

class EBCellFlag {
public:
    uint32_t flag = 0;
    static constexpr int pos(int i, int j, int k) { return 4 + (i + 1) + 3 * (j + 1) + 9 * (k + 1); }
    // The reference asks for offsets of -2 (Source/EB/EBkernels.H:22,43,64), which
    // lie outside the 3x3x3 neighbour table.  We pin that to the linear bit
    // position (aliasing another neighbour's bit) and to "not connected" when the
    // position falls outside the 32-bit word.
    bool isConnected(int i, int j, int k) const {
        int p = pos(i, j, k);
        return p >= 0 && p < 32 && ((flag >> p) & 1u);
    }
    bool isRegular() const { return (flag & 3u) == 0u; }
    bool isSingleValued() const { return (flag & 3u) == 1u; }
    bool isCovered() const { return (flag & 3u) == 3u; }
};

// Pieces of AMReX's memory API used by Source/Constants.cpp.
namespace Gpu {
template <class T> using HostVector = std::vector<T>;
struct HostToDevice {};
static constexpr HostToDevice hostToDevice{};
template <class It, class T>
inline void copyAsync(HostToDevice, It first, It last, T* dst) { std::copy(first, last, dst); }
inline void streamSynchronize() {}
}  // namespace Gpu

struct HostArena {
    void* alloc(std::size_t n) { return std::malloc(n); }
    void free(void* p) { std::free(p); }
};
inline HostArena* The_Arena() { static HostArena a; return &a; }

}  // namespace amrex

#endif
