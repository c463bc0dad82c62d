// Engine internals shared by the engine (engine.cu) and its adjoint
// (adjoint.cu): the engine handle with its device-memory cache and
// per-kernel-class profiling, the chain of site tensors, scoped device
// buffers, the GEMM wrapper and the factorisation steps every sweep uses.
#pragma once

#include "kernels.cuh"
#include "mpdo_gb300.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

namespace mpdo {

// ------------------------------------------------------------ errors ----
struct Error {
  mpdo_status st;
  std::string msg;
};
[[noreturn]] inline void fail(mpdo_status s, const std::string &m) { throw Error{s, m}; }


// ------------------------------------------------------------ engine ----
struct Engine {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaMemPool_t pool = nullptr;
  int *d_status = nullptr;
  int status_cap = 8192;
  int status_used = 0;
  bool fuse_2q = true;
  bool defer_1q = true;              // trace-preserving 1q channels deferred past the truncate sweeps
  int wide_range = -1;              // verified range finder on wide bonds: 1 on, 0 off, -1 complex128 only
  int wide_eig = -1;                // wide-bond Gram: tridiagonal (1), block Jacobi (0), -1: by precision
  int wide_eig_from = 257;          // (-1, complex64) Grams at least this wide take the tridiagonal route
  long long wide_eig_calls = 0;
  long long wide_range_hits = 0, wide_exact_calls = 0;
  double wide_resid_max = 0;        // largest accepted |Y - Q Q^H Y|_F / |Y|_F
  double wide_range_tol = 8.0;      // acceptance: residual <= tol * eps * sqrt(p) * |Y|_F
  int max_sweeps = 60;
  int wide_oversample = 16;          // wide bonds: Rayleigh-Ritz space = leading (want + this) directions
  // TSQR chunk rows: a shared-memory chunk is used only when it holds at least
  // tsqr_ratio x n rows, else chunks of ceil(tsqr_ratio n) rows in global memory
  // (every level shrinks the stack by about that factor)
  double tsqr_ratio = 3.0;
  int bjacobi_bs = 0;               // block-Jacobi block width (columns); 0: from the shared-memory cap
  bool bjacobi_fused = true;        // block Jacobi as one thread-block-cluster launch (else one launch per round)
  int first_status = 0;
  // per-kernel-class profiling (CUDA events around each launch)
  struct ProfRec { int cls; cudaEvent_t a, b; double flops, bytes; };
  bool profiling = false;
  std::vector<ProfRec> recs;
  double acc_ms[14] = {0}, acc_flops[14] = {0}, acc_bytes[14] = {0};
  long long acc_n[14] = {0};
  // Freed device blocks kept for reuse, by rounded size.  Every block of an
  // engine is used on the engine's one stream, so a block freed after its
  // last use was enqueued can serve the next allocation at once (stream order
  // separates the uses); the driver's allocator is then off the hot path.
  std::unordered_map<size_t, std::vector<void *>> cache;
  std::unordered_map<void *, size_t> live;
  size_t cached_bytes = 0;
};

// kernel classes reported by mpdo_engine_profile_read
enum KClass {
  K_GEMM = 0, K_QR_FACTOR = 1, K_QR_APPLY = 2, K_JACOBI = 3, K_KRAUS1Q = 4, K_MIX2Q = 5, K_OTHER = 6,
  K_BJACOBI = 8,  // (7 reports the wide-bond counters)
  // phases (spans of many launches, overlapping the kernel classes)
  P_QR_SWEEP = 9, P_SVD_SWEEP = 10, P_KAPPA = 11, P_WIDE_SVD = 12,
  K_HETRD = 13     // cluster tridiagonalisation of wide-bond Gram matrices
};
constexpr int kProfClasses = 14;

// Launch wrapper: when profiling, bracket the launch with events and keep the
// algorithmic flop/byte count of the call.
template <class F> inline void prof(Engine &e, int cls, double flops, double bytes, F &&launch) {
  if (!e.profiling) { launch(); return; }
  Engine::ProfRec r{cls, nullptr, nullptr, flops, bytes};
  cudaEventCreate(&r.a);
  cudaEventCreate(&r.b);
  cudaEventRecord(r.a, e.stream);
  launch();
  cudaEventRecord(r.b, e.stream);
  e.recs.push_back(r);
}
inline void prof_flush(Engine &e) {
  if (e.recs.empty()) return;
  cudaStreamSynchronize(e.stream);
  for (auto &r : e.recs) {
    float ms = 0;
    cudaEventElapsedTime(&ms, r.a, r.b);
    e.acc_ms[r.cls] += ms;
    e.acc_flops[r.cls] += r.flops;
    e.acc_bytes[r.cls] += r.bytes;
    e.acc_n[r.cls] += 1;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  e.recs.clear();
}

// Phase span (profiling only): events around a block of launches.
struct Phase {
  Engine &e;
  Engine::ProfRec r;
  Phase(Engine &eng, int cls) : e(eng), r{cls, nullptr, nullptr, 0, 0} {
    if (!e.profiling) return;
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, e.stream);
  }
  ~Phase() {
    if (!e.profiling || !r.a) return;
    cudaEventRecord(r.b, e.stream);
    e.recs.push_back(r);
  }
};

// Allocation size classes: multiples of 256 B up to 64 KiB, then eight steps
// per power of two (at most 12.5% slack).
inline size_t size_class(size_t bytes) {
  if (bytes <= 65536) return (bytes + 255) / 256 * 256;
  int k = 63 - __builtin_clzll((unsigned long long)(bytes - 1));   // 2^k < bytes <= 2^(k+1)
  const size_t step = size_t(1) << (k - 2);
  return (bytes + step - 1) / step * step;
}

constexpr size_t kCacheCapBytes = size_t(16) << 30;   // per engine

inline void release_cache(Engine &e) {
  for (auto &kv : e.cache)
    for (void *q : kv.second) cudaFreeAsync(q, e.stream);
  e.cache.clear();
  e.cached_bytes = 0;
}

inline void *dalloc(Engine &e, size_t bytes) {
  if (bytes == 0) bytes = 16;
  const size_t sz = size_class(bytes);
  auto it = e.cache.find(sz);
  if (it != e.cache.end() && !it->second.empty()) {
    void *p = it->second.back();
    it->second.pop_back();
    e.cached_bytes -= sz;
    e.live[p] = sz;
    return p;
  }
  void *p = nullptr;
  cudaError_t err = cudaMallocFromPoolAsync(&p, sz, e.pool, e.stream);
  if (err != cudaSuccess) {
    cudaGetLastError();
    release_cache(e);                        // give cached blocks back and retry once
    err = cudaMallocFromPoolAsync(&p, sz, e.pool, e.stream);
    if (err != cudaSuccess) {
      cudaGetLastError();
      fail(MPDO_ERR_OOM, "device allocation of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(err));
    }
  }
  e.live[p] = sz;
  return p;
}
inline void dfree(Engine &e, void *p) {
  if (!p) return;
  auto it = e.live.find(p);
  if (it == e.live.end()) {                  // not from dalloc: hand straight back
    cudaFreeAsync(p, e.stream);
    return;
  }
  const size_t sz = it->second;
  e.live.erase(it);
  e.cache[sz].push_back(p);
  e.cached_bytes += sz;
  if (e.cached_bytes > kCacheCapBytes) release_cache(e);
}

// Scoped device buffer
template <typename X> struct DBuf {
  Engine *e = nullptr;
  X *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(Engine &eng, size_t count) : e(&eng), n(count) { p = static_cast<X *>(dalloc(eng, count * sizeof(X))); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : e(o.e), p(o.p), n(o.n) { o.p = nullptr; }
  DBuf &operator=(DBuf &&o) noexcept {
    reset();
    e = o.e; p = o.p; n = o.n; o.p = nullptr;
    return *this;
  }
  X *release() { X *q = p; p = nullptr; return q; }
  void reset() { if (p && e) dfree(*e, p); p = nullptr; }
  ~DBuf() { if (p && e) dfree(*e, p); }
};

int *status_slot(Engine &e, int count);
void check_status(Engine &e);

// ------------------------------------------------------------- chain ----
struct Site {
  void *p = nullptr;
  int l = 1, a = 1, r = 1;
  size_t elems() const { return (size_t)l * 2 * a * r; }
};
struct Pend {
  bool on = false;
  std::vector<double> t;
  int K = 1;
  double cutoff = 0;
};
}  // namespace mpdo

struct mpdo_engine_s {
  mpdo::Engine e;
};
struct mpdo_chain_s {
  mpdo_engine_s *eng = nullptr;
  int n = 0;
  int dtype = MPDO_C64;
  std::vector<mpdo::Site> s;
  std::vector<char> bond;
  std::vector<mpdo::Pend> pend;
  std::vector<mpdo::Pend> pend1;     // deferred trace-preserving 1q Kraus maps, per site
};

namespace mpdo {

// ---------------------------------------------------------- helpers -----
template <typename T> inline View<T> RM(const cx<T> *p, int64_t ld, int conj = 0, int64_t bs = 0) {
  return View<T>{p, bs, 1, ld, 0, 1, conj};
}
template <typename T> inline View<T> CM(const cx<T> *p, int64_t ld, int conj = 0, int64_t bs = 0) {
  return View<T>{p, bs, 1, 1, 0, ld, conj};
}

template <typename T>
inline void gemm(Engine &e, int M, int N, int K, const View<T> &A, const View<T> &B, cx<T> *C, int64_t ldc,
                 int batch = 1, int64_t cbs = 0, cx<T> beta = czero<T>(), cx<T> alpha = cmk<T>(T(1), T(0))) {
  const double fl = 8.0 * M * N * K * batch;
  const double by = (double)sizeof(cx<T>) * batch * ((double)M * K + (double)K * N + (double)M * N);
  // split-K workspace for small-output long-K products
  const int64_t tiles = (int64_t)((M + 63) / 64) * ((N + 63) / 64) * batch;
  if (K >= 512 && tiles < 148) {
    const int nsplit = (int)std::min<int64_t>(std::max<int64_t>(1, 296 / tiles), K / 128);
    if (nsplit > 1) {
      const size_t ws = (size_t)nsplit * batch * M * N;
      DBuf<cx<T>> w(e, ws);
      prof(e, K_GEMM, fl, by, [&] {
        cgemm<T>(e.stream, M, N, K, batch, alpha, A, B, beta, C, ldc, 1, cbs, w.p, ws);
      });
      return;
    }
  }
  prof(e, K_GEMM, fl, by, [&] { cgemm<T>(e.stream, M, N, K, batch, alpha, A, B, beta, C, ldc, 1, cbs); });
}

template <typename T> inline cx<T> *site_ptr(mpdo_chain_s *ch, int i) { return static_cast<cx<T> *>(ch->s[i].p); }

template <typename T> inline void set_site(mpdo_chain_s *ch, int i, cx<T> *p, int l, int a, int r) {
  Engine &e = ch->eng->e;
  if (ch->s[i].p) dfree(e, ch->s[i].p);
  ch->s[i].p = p;
  ch->s[i].l = l; ch->s[i].a = a; ch->s[i].r = r;
}

// ---------------------------------------------- shared factorisations ----
// (defined in engine.cu, instantiated for float and double)
template <typename T> void qr(Engine &e, int m, int n, const View<T> &in, cx<T> *Q, cx<T> *R);
template <typename T> void qr_r_batched(Engine &e, int batch, int m, int n, const View<T> &in, cx<T> *R);
template <typename T> void right_svd(Engine &e, int m, int n, const View<T> &in, DBuf<cx<T>> &W, DBuf<T> &sigma);
template <typename T>
int error_rule_keep(const std::vector<T> &s_in, int nsv, int max_sv, double err, bool relative,
                    double total_sq = -1.0);
bool connected(mpdo_chain_s *ch);
template <typename T> void materialize_all(mpdo_chain_s *ch);

// C-ABI guard: runs f, maps exceptions to a status and the thread's last
// error message.
template <typename F> inline mpdo_status guard(F &&f) {
  try {
    f();
    return MPDO_OK;
  } catch (const Error &err) {
    set_last_error(err.msg);
    return err.st;
  } catch (const CudaError &ce) {
    set_last_error(std::string(ce.expr) + ": " + cudaGetErrorString(ce.err) + " (" + ce.file + ":" +
                   std::to_string(ce.line) + ")");
    return MPDO_ERR_CUDA;
  } catch (const std::exception &ex) {
    set_last_error(ex.what());
    return MPDO_ERR_INVALID;
  }
}

}  // namespace mpdo
