// Allocation-free right-SVD entry point.
//
// Some callers cannot allocate device memory: a serving process whose memory
// is carved up in advance by its own allocator (a cudaMalloc behind its back
// breaks its accounting or fails on a full device), code running under an
// allocation hook that forbids growth, or a host loop that must not take the
// driver's allocation locks.  For them mpdo_right_svd_noalloc computes the
// same decomposition as the engine's SVD step (Householder TSQR, then
// one-sided Jacobi on R with the rotations accumulated) with every workspace
// carved out of one file-scope device array of fixed size.
//
// The array (kScratchBytes) exists once per device that loads this library and
// stays allocated until the process exits.  Host code must not use its name as
// an address: the first call on a device (with that device current) resolves
// the device address with cudaGetSymbolAddress and caches it; make that first
// call before any stream capture.  All calls share the array and it keeps the
// contents of the last call, so two calls whose work overlaps on the GPU (on
// different streams, or different host threads) race; serialise them.
#include "kernels.cuh"
#include "mpdo_gb300.h"

#include <mutex>
#include <string>

namespace mpdo {
namespace {

constexpr size_t kScratchBytes = size_t(8) << 20;   // 8 MiB per device
constexpr int kMaxN = 64;                            // columns
constexpr int kMaxM = 8192;                          // rows
constexpr size_t kSmemCap = 200 * 1024;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 128;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {nullptr};

// Device address of g_scratch for the current device (resolved once per device).
cudaError_t scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_addr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

struct Carve {
  unsigned char *base;
  size_t off = 0, cap;
  template <typename X> X *take(size_t n) {
    off = (off + 255) / 256 * 256;
    X *p = reinterpret_cast<X *>(base + off);
    off += n * sizeof(X);
    return p;
  }
};

struct Level {
  int m, mc, nch;
  cx<float> *v, *tau, *rs;
};

// A TSQR plan in the engine's style (row chunks that fit shared memory,
// compact R stacking), laid out in the scratch array.  Its chunks are sized
// for (n + 1) columns of shared memory where the engine's qr() reserves
// (n + 2), so for tall inputs the chunking -- and with it the rounding -- can
// differ slightly from mpdo_debug_svd.  Returns the bytes needed.
size_t plan(int m, int n, unsigned char *base, Level *lv, int *nlev, cx<float> **U, cx<float> **xws,
            cx<float> **wws, int **status) {
  const size_t esz = sizeof(cx<float>);
  Carve c{base, 0, kScratchBytes};
  int curm = m, L = 0;
  while (true) {
    int mc;
    if ((size_t)curm * n * esz <= kSmemCap) mc = curm;
    else {
      size_t mcs = kSmemCap / ((size_t)(n + 1) * esz) / 32 * 32;
      mc = (mcs > (size_t)n) ? (int)std::min<size_t>(mcs, (size_t)curm) : curm;
    }
    const int nch = (curm + mc - 1) / mc;
    lv[L].m = curm; lv[L].mc = mc; lv[L].nch = nch;
    lv[L].v = c.take<cx<float>>((size_t)nch * mc * n);
    lv[L].tau = c.take<cx<float>>((size_t)nch * n);
    lv[L].rs = c.take<cx<float>>((size_t)nch * n * n);
    ++L;
    if (nch == 1 || L == 16) break;
    curm = (nch - 1) * n + std::min(n, curm - (nch - 1) * mc);
  }
  *nlev = L;
  const int k = std::min(m, n);
  *U = c.take<cx<float>>((size_t)k * n);
  *xws = c.take<cx<float>>((size_t)k * n);
  *wws = c.take<cx<float>>((size_t)n * n);
  *status = c.take<int>(1);
  return c.off;
}

}  // namespace
}  // namespace mpdo

using namespace mpdo;

extern "C" mpdo_status mpdo_right_svd_noalloc(int m, int n, const void *a, void *w, void *sigma, int *status,
                                              void *stream) {
  if (!a || !w || !sigma) {
    set_last_error("mpdo_right_svd_noalloc: a, w and sigma must be device pointers");
    return MPDO_ERR_INVALID;
  }
  if (m < 1 || n < 1 || n > kMaxN || m > kMaxM) {
    set_last_error("mpdo_right_svd_noalloc: m=" + std::to_string(m) + ", n=" + std::to_string(n) +
            " is outside the allocation-free limits (1 <= m <= 8192, 1 <= n <= 64; 8 MiB static scratch)");
    return MPDO_ERR_INVALID;
  }
  void *addr = nullptr;
  cudaError_t ce = scratch_address(&addr);
  if (ce != cudaSuccess) {
    set_last_error(std::string("mpdo_right_svd_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(ce));
    return MPDO_ERR_CUDA;
  }
  Level lv[16];
  int nlev = 0;
  cx<float> *U = nullptr, *xws = nullptr, *wws = nullptr;
  int *st_scratch = nullptr;
  const size_t need = plan(m, n, static_cast<unsigned char *>(addr), lv, &nlev, &U, &xws, &wws, &st_scratch);
  if (need > kScratchBytes) {
    set_last_error("mpdo_right_svd_noalloc: needs " + std::to_string(need) + " bytes of scratch, more than the " +
            std::to_string(kScratchBytes) + "-byte static array");
    return MPDO_ERR_INVALID;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int *st_word = status ? status : st_scratch;
  // every kernel below writes its whole output region; only the status word
  // is cleared explicitly so that a stale value from the last call never shows
  ce = cudaMemsetAsync(st_word, 0, sizeof(int), st);
  if (ce == cudaSuccess) {
    View<float> cur = View<float>{static_cast<const cx<float> *>(a), 0, 1, n, 0, 1, 0};
    for (int L = 0; L < nlev; ++L) {
      qr_factor_chunks<float>(st, lv[L].m, n, lv[L].mc, lv[L].nch, cur, lv[L].v, lv[L].tau, lv[L].rs);
      cur = View<float>{lv[L].rs, 0, 1, n, 0, 1, 0};
    }
    const int k = std::min(m, n);
    // R is the first k rows of the top level's stack
    jacobi_svd<float>(st, 1, k, n, View<float>{lv[nlev - 1].rs, 0, 1, n, 0, 1, 0}, U, static_cast<float *>(sigma),
                      static_cast<cx<float> *>(w), xws, wws, 60, st_word);
    ce = cudaGetLastError();
  }
  if (ce != cudaSuccess) {
    set_last_error(std::string("mpdo_right_svd_noalloc: ") + cudaGetErrorString(ce));
    return MPDO_ERR_CUDA;
  }
  return MPDO_OK;
}
