// Shared device/host helpers for the MPDO engine: complex arithmetic on
// float2/double2, strided matrix views, launch bookkeeping.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <set>
#include <utility>

namespace mpdo {

template <typename T> struct CT;
template <> struct CT<float> { using type = float2; };
template <> struct CT<double> { using type = double2; };
template <typename T> using cx = typename CT<T>::type;

template <typename T> __host__ __device__ __forceinline__ cx<T> cmk(T x, T y) {
  cx<T> r; r.x = x; r.y = y; return r;
}
template <typename T> __host__ __device__ __forceinline__ cx<T> czero() { return cmk<T>(T(0), T(0)); }
template <typename T> __host__ __device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) {
  return cmk<T>(a.x + b.x, a.y + b.y);
}
template <typename T> __host__ __device__ __forceinline__ cx<T> csub(cx<T> a, cx<T> b) {
  return cmk<T>(a.x - b.x, a.y - b.y);
}
template <typename T> __host__ __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
  return cmk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
template <typename T> __host__ __device__ __forceinline__ cx<T> cmulc(cx<T> a, cx<T> b) {
  return cmk<T>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename T> __host__ __device__ __forceinline__ cx<T> cconj(cx<T> a) { return cmk<T>(a.x, -a.y); }
template <typename T> __host__ __device__ __forceinline__ cx<T> cscale(cx<T> a, T s) {
  return cmk<T>(a.x * s, a.y * s);
}
template <typename T> __host__ __device__ __forceinline__ T cabs2(cx<T> a) { return a.x * a.x + a.y * a.y; }
// acc += a * b
template <typename T> __host__ __device__ __forceinline__ void cfma(cx<T> &acc, cx<T> a, cx<T> b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename T> __host__ __device__ __forceinline__ void cfmac(cx<T> &acc, cx<T> a, cx<T> b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
}

// A strided (optionally conjugated) batched matrix view:
//   element (b, i, j) = conj?( p[b*bs + (i / n1)*s0 + (i % n1)*s1 + j*cs] )
// A plain matrix uses n1 = 1 and s0 = row stride.  The two-level row index
// lets one view walk rows that are a product of two tensor legs with
// unrelated strides (e.g. rows (l,s) x r of an [l][s][a][r] site).
template <typename T> struct View {
  const cx<T> *p;
  int64_t bs;
  int64_t n1;
  int64_t s0, s1;
  int64_t cs;
  int conj;
};

template <typename T> __host__ __device__ __forceinline__ int64_t view_off(const View<T> &v, int64_t b,
                                                                           int64_t i, int64_t j) {
  return b * v.bs + (i / v.n1) * v.s0 + (i % v.n1) * v.s1 + j * v.cs;
}
template <typename T> __device__ __forceinline__ cx<T> view_ld(const View<T> &v, int64_t b, int64_t i,
                                                              int64_t j) {
  cx<T> x = v.p[view_off(v, b, i, j)];
  if (v.conj) x.y = -x.y;
  return x;
}

template <typename T> inline View<T> view_rowmajor(const cx<T> *p, int64_t ld, int64_t bs = 0, int conj = 0) {
  return View<T>{p, bs, 1, ld, 0, 1, conj};
}
template <typename T> inline View<T> view_colmajor(const cx<T> *p, int64_t ld, int64_t bs = 0, int conj = 0) {
  return View<T>{p, bs, 1, 1, 0, ld, conj};
}
// (op(M))(i,j) = conj(M(j,i)) for a row-major M with leading dimension ld.
template <typename T> inline View<T> view_adjoint_of_rowmajor(const cx<T> *p, int64_t ld, int64_t bs = 0) {
  return View<T>{p, bs, 1, 1, 0, ld, 1};
}

// Device status words written by factorisation kernels.
enum DevStatus : int { DEV_OK = 0, DEV_NOT_CONVERGED = 1, DEV_NONFINITE = 2 };

// Dynamic shared memory: every kernel that takes more than the default 48 KB
// is opted in once per device to the one ceiling all its launches stay under
// (200 KB), so host threads launching concurrently never change the limit
// under each other's launches.
constexpr int kSmemCeiling = 200 * 1024;
inline void smem_optin_raw(const void *kernel) {
  static std::mutex mu;
  static std::set<std::pair<const void *, int>> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  if (done.insert({kernel, dev}).second)
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemCeiling);
}
template <typename F> inline void smem_optin(F *kernel) { smem_optin_raw(reinterpret_cast<const void *>(kernel)); }

// Launch counter (all kernels of this library go through count_launch(),
// which also keeps a count per launcher function).
void count_launch(const char *fn = __builtin_FUNCTION());
uint64_t launch_count();
// (launcher name, launches) pairs so far; returns how many were written.
int launch_histogram(const char **names, uint64_t *counts, int cap);

}  // namespace mpdo

#define MPDO_CUDA_CHECK(expr)                                                      \
  do {                                                                             \
    cudaError_t _e = (expr);                                                       \
    if (_e != cudaSuccess) throw mpdo::CudaError(_e, #expr, __FILE__, __LINE__);   \
  } while (0)

namespace mpdo {
struct CudaError {
  cudaError_t err;
  const char *expr, *file;
  int line;
  CudaError(cudaError_t e, const char *x, const char *f, int l) : err(e), expr(x), file(f), line(l) {}
};
}  // namespace mpdo
