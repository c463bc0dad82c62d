// Memory-bound site-tensor kernels: Kraus application, the two-site gate/Kraus
// mix, layout copies, diagonal scalings and small reductions.
#include "kernels.cuh"

#include <algorithm>
#include <atomic>

namespace mpdo {

static std::atomic<uint64_t> g_launches{0};
// Per-launcher counts: a lock-free open-addressing table keyed by the
// launcher's function-name literal (pointer identity).
constexpr int kHistSlots = 128;
static std::atomic<const char *> g_hist_key[kHistSlots];
static std::atomic<uint64_t> g_hist_count[kHistSlots];

void count_launch(const char *fn) {
  // a launch that could not start (shared memory, grid or argument limits)
  // must not leave its output unwritten silently
  const cudaError_t err = cudaPeekAtLastError();
  if (err != cudaSuccess) {
    cudaGetLastError();
    throw CudaError(err, fn, __FILE__, __LINE__);
  }
  g_launches.fetch_add(1, std::memory_order_relaxed);
  const uintptr_t h = reinterpret_cast<uintptr_t>(fn);
  for (int i = 0; i < kHistSlots; ++i) {
    const int slot = (int)((h / 8 + (uintptr_t)i) % kHistSlots);
    const char *k = g_hist_key[slot].load(std::memory_order_acquire);
    if (k == nullptr) {
      const char *expected = nullptr;
      if (g_hist_key[slot].compare_exchange_strong(expected, fn) || expected == fn) {
        g_hist_count[slot].fetch_add(1, std::memory_order_relaxed);
        return;
      }
      continue;
    }
    if (k == fn) {
      g_hist_count[slot].fetch_add(1, std::memory_order_relaxed);
      return;
    }
  }
}
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }
int launch_histogram(const char **names, uint64_t *counts, int cap) {
  int n = 0;
  for (int i = 0; i < kHistSlots && n < cap; ++i) {
    const char *k = g_hist_key[i].load(std::memory_order_acquire);
    if (k) {
      names[n] = k;
      counts[n] = g_hist_count[i].load(std::memory_order_relaxed);
      ++n;
    }
  }
  return n;
}

namespace {
inline int nblocks(int64_t n, int t = 256) { return (int)std::min<int64_t>((n + t - 1) / t, 152 * 32); }

template <typename T> struct Gate1 { cx<T> g[2 * 2 * 16]; };
template <typename T> struct Gate2 { cx<T> t[16 * 16]; };

// V consecutive complex values moved as one access (16 bytes for complex64
// pairs and single complex128 values)
template <typename T, int V> struct alignas(sizeof(cx<T>) * V) CVec { cx<T> v[V]; };

// out[l][x][a*K + k][r] = sum_s g[x][s][k] A[l][s][a][r].  Each thread owns
// V consecutive r of one (l, a): two 16-byte loads, 2 K 16-byte stores, all
// coalesced across the warp; index arithmetic in I (32-bit unless the output
// has 2^31 elements or more).
template <typename T, int V, typename I>
__global__ void k_kraus1q(const cx<T> *__restrict__ A, cx<T> *__restrict__ out, int L, int Aa, int R, int K,
                          const Gate1<T> G) {
  const I Rv = R / V;
  const I total = (I)L * Aa * Rv;
  const I aK = (I)Aa * K;
  for (I t = blockIdx.x * (I)blockDim.x + threadIdx.x; t < total; t += (I)gridDim.x * blockDim.x) {
    const I rv = t % Rv, la = t / Rv, a = la % Aa, l = la / Aa;
    const I r = rv * V;
    const CVec<T, V> a0 = *reinterpret_cast<const CVec<T, V> *>(A + ((l * 2 + 0) * Aa + a) * R + r);
    const CVec<T, V> a1 = *reinterpret_cast<const CVec<T, V> *>(A + ((l * 2 + 1) * Aa + a) * R + r);
#pragma unroll
    for (int x = 0; x < 2; ++x) {
      cx<T> *o = out + ((l * 2 + x) * aK + a * K) * R + r;
      for (int k = 0; k < K; ++k) {
        const cx<T> g0 = G.g[(x * 2 + 0) * K + k], g1 = G.g[(x * 2 + 1) * K + k];
        CVec<T, V> v;
#pragma unroll
        for (int q = 0; q < V; ++q) {
          v.v[q] = cmul<T>(g0, a0.v[q]);
          cfma<T>(v.v[q], g1, a1.v[q]);
        }
        *reinterpret_cast<CVec<T, V> *>(o + (I)k * R) = v;
      }
    }
  }
}

// W: [nb][2 s][kr][2 t][C][R]  ->  Z: [nb][2 x][kr][2 y][C*K][R]
template <typename T>
__global__ void k_mix2q(const cx<T> *__restrict__ W, cx<T> *__restrict__ Z, int nb, int kr, int Cc, int R, int K,
                        const Gate2<T> G) {
  const int64_t CR = (int64_t)Cc * R;
  const int64_t total = (int64_t)nb * kr * CR;
  const int64_t blkW = 2 * (int64_t)kr * 2 * CR;     // per nb slice
  const int64_t blkZ = 2 * (int64_t)kr * 2 * CR * K;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cr = t % CR, kk = (t / CR) % kr, b = t / (CR * kr);
    const int64_t c = cr / R, r = cr % R;
    const cx<T> *w = W + b * blkW;
    cx<T> in[2][2];
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int tt = 0; tt < 2; ++tt) in[s][tt] = w[((s * (int64_t)kr + kk) * 2 + tt) * CR + cr];
    cx<T> *z = Z + b * blkZ;
    for (int x = 0; x < 2; ++x)
      for (int y = 0; y < 2; ++y) {
        cx<T> *zo = z + ((x * (int64_t)kr + kk) * 2 + y) * (CR * K) + (c * K) * R + r;
        for (int q = 0; q < K; ++q) {
          cx<T> v = czero<T>();
#pragma unroll
          for (int s = 0; s < 2; ++s)
#pragma unroll
            for (int tt = 0; tt < 2; ++tt) cfma<T>(v, G.t[(((x * 2 + y) * 2 + s) * 2 + tt) * K + q], in[s][tt]);
          zo[(int64_t)q * R] = v;
        }
      }
  }
}

template <typename T>
__global__ void k_copy4d(cx<T> *dst, const cx<T> *src, int64_t d0, int64_t d1, int64_t d2, int64_t d3, int64_t s0,
                         int64_t s1, int64_t s2, int64_t s3, int conj) {
  const int64_t total = d0 * d1 * d2 * d3;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t;
    const int64_t i3 = r % d3; r /= d3;
    const int64_t i2 = r % d2; r /= d2;
    const int64_t i1 = r % d1; r /= d1;
    const int64_t i0 = r;
    cx<T> v = src[i0 * s0 + i1 * s1 + i2 * s2 + i3 * s3];
    if (conj) v.y = -v.y;
    dst[t] = v;
  }
}

struct Perm6 { int64_t d[6], s[6]; };

// dst (contiguous in the order of d) = conj?(src at sum_k i_k s[k]); unused
// leading axes have d = 1
template <typename T>
__global__ void k_permute6(cx<T> *__restrict__ dst, const cx<T> *__restrict__ src, int64_t total, Perm6 P,
                           int conj) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t, off = 0;
#pragma unroll
    for (int k = 5; k >= 0; --k) {
      const int64_t i = r % P.d[k];
      r /= P.d[k];
      off += i * P.s[k];
    }
    cx<T> v = src[off];
    if (conj) v.y = -v.y;
    dst[t] = v;
  }
}

template <typename T>
__device__ __forceinline__ T scale_of(T s, int mode, T thr) {
  switch (mode) {
    case 0: return s;
    case 1: return s > T(0) ? sqrt(s) : T(0);
    case 2: return s > thr ? T(1) / sqrt(s) : T(0);
    default: return s > thr ? T(1) / s : T(0);
  }
}

template <typename T>
__global__ void k_scale(cx<T> *X, int M, int N, int64_t ld, const T *s, int by_row, int mode, T thr_rel) {
  const int64_t total = (int64_t)M * N;
  const T thr = thr_rel * s[0];
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / N, j = t % N;
    const T f = scale_of<T>(s[by_row ? i : j], mode, thr);
    cx<T> &x = X[i * ld + j];
    x = cscale<T>(x, f);
  }
}

template <typename T>
__global__ void k_blockdiag2(cx<T> *dst, const cx<T> *Q, int B, int Aa, int kr) {
  // dst[b][x][a][x'*kr + k]
  const int64_t total = (int64_t)B * 2 * Aa * 2 * kr;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t;
    const int64_t k = r % kr; r /= kr;
    const int64_t xp = r % 2; r /= 2;
    const int64_t a = r % Aa; r /= Aa;
    const int64_t x = r % 2; r /= 2;
    const int64_t b = r;
    dst[t] = (x == xp) ? Q[(b * Aa + a) * kr + k] : czero<T>();
  }
}

template <typename T>
__global__ void k_fill0(cx<T> *p, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    p[t] = czero<T>();
}

template <typename T>
__global__ void k_sigma_weights(const T *sigma, int n, int keep, double *out) {
  __shared__ double sk[256], st[256];
  double a = 0, b = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = (double)sigma[i] * (double)sigma[i];
    b += v;
    if (i < keep) a += v;
  }
  sk[threadIdx.x] = a; st[threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) { sk[threadIdx.x] += sk[threadIdx.x + o]; st[threadIdx.x] += st[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[0] = sk[0]; out[1] = st[0]; }
}

template <typename T>
__global__ void k_sqrt_inplace(T *s, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s[i] = s[i] > T(0) ? sqrt(s[i]) : T(0);
}

template <typename T>
__global__ void k_apply_op(const cx<T> *A, cx<T> *out, int L, int Aa, int R, cx<T> o00, cx<T> o01, cx<T> o10,
                           cx<T> o11) {
  const int64_t total = (int64_t)L * Aa * R;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % R, la = t / R, a = la % Aa, l = la / Aa;
    const cx<T> a0 = A[((l * 2 + 0) * Aa + a) * R + r];
    const cx<T> a1 = A[((l * 2 + 1) * Aa + a) * R + r];
    cx<T> v0 = cmul<T>(o00, a0); cfma<T>(v0, o01, a1);
    cx<T> v1 = cmul<T>(o10, a0); cfma<T>(v1, o11, a1);
    out[((l * 2 + 0) * Aa + a) * R + r] = v0;
    out[((l * 2 + 1) * Aa + a) * R + r] = v1;
  }
}

// Deterministic Gaussian test matrix: splitmix64 counter hash -> two uniforms
// -> Box-Muller; real and imaginary parts N(0, 1/2).
__device__ __forceinline__ uint64_t smix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
template <typename T>
__global__ void k_gauss(cx<T> *out, size_t n, uint64_t seed) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = smix(seed ^ (2 * t)), h2 = smix(seed ^ (2 * t + 1));
    const double u1 = ((h1 >> 11) + 1.0) * (1.0 / 9007199254740993.0);   // (0, 1]
    const double u2 = (h2 >> 11) * (1.0 / 9007199254740992.0);
    const double r = sqrt(-log(u1)), th = 6.283185307179586 * u2;
    out[t] = cmk<T>((T)(r * cos(th)), (T)(r * sin(th)));
  }
}
template <typename T>
__global__ void k_sumsq(const cx<T> *x, size_t n, double *out) {
  __shared__ double red[256];
  double a = 0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    a += (double)x[t].x * x[t].x + (double)x[t].y * x[t].y;
  red[threadIdx.x] = a;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(out, red[0]);
}

template <typename T>
__global__ void k_trace(const cx<T> *M, int n, int64_t ld, int64_t bs, int batch, double2 *out) {
  for (int b = blockIdx.x; b < batch; b += gridDim.x) {
    __shared__ double re[256], im[256];
    double a = 0, c = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const cx<T> v = M[b * bs + (int64_t)i * ld + i];
      a += v.x; c += v.y;
    }
    re[threadIdx.x] = a; im[threadIdx.x] = c;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) { re[threadIdx.x] += re[threadIdx.x + o]; im[threadIdx.x] += im[threadIdx.x + o]; }
      __syncthreads();
    }
    if (threadIdx.x == 0) out[b] = make_double2(re[0], im[0]);
    __syncthreads();
  }
}
// out[b] = Re sum_i E[b][i] R[i]  (the full contraction of a left and a
// right environment, both indexed [ket][bra])
template <typename T>
__global__ void k_env_dot(const cx<T> *E, const cx<T> *R, int64_t msize, int batch, double *out) {
  for (int b = blockIdx.x; b < batch; b += gridDim.x) {
    __shared__ double red[256];
    double a = 0;
    const cx<T> *Eb = E + (int64_t)b * msize;
    for (int64_t i = threadIdx.x; i < msize; i += blockDim.x) a += (double)Eb[i].x * R[i].x - (double)Eb[i].y * R[i].y;
    red[threadIdx.x] = a;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[b] = red[0];
    __syncthreads();
  }
}

// dst[b] = src[idx[b]] for msize-element matrices
template <typename T>
__global__ void k_gather_mats(const cx<T> *src, cx<T> *dst, const int *idx, int64_t msize, int batch) {
  const int64_t total = (int64_t)batch * msize;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / msize, i = t % msize;
    dst[t] = src[(int64_t)idx[b] * msize + i];
  }
}
}  // namespace

template <typename T>
void env_dot(cudaStream_t st, const cx<T> *E, const cx<T> *R, int64_t msize, int batch, double *out) {
  k_env_dot<T><<<std::min(batch, 4096), 256, 0, st>>>(E, R, msize, batch, out);
  count_launch();
}

template <typename T>
void gather_mats(cudaStream_t st, const cx<T> *src, cx<T> *dst, const int *idx, int64_t msize, int batch) {
  k_gather_mats<T><<<nblocks((int64_t)batch * msize), 256, 0, st>>>(src, dst, idx, msize, batch);
  count_launch();
}

template <typename T>
void kraus1q(cudaStream_t st, const cx<T> *A, cx<T> *out, int L, int Aa, int R, const double *g, int K) {
  Gate1<T> G;
  for (int i = 0; i < 4 * K; ++i) G.g[i] = cmk<T>((T)g[2 * i], (T)g[2 * i + 1]);
  const int64_t nout = (int64_t)L * 2 * Aa * K * R;
  const bool pair = sizeof(T) == 4 && R % 2 == 0 && ((uintptr_t)A % 16) == 0 && ((uintptr_t)out % 16) == 0;
  const int64_t threads = (int64_t)L * Aa * (pair ? R / 2 : R);
  if (nout < ((int64_t)1 << 31)) {
    if (pair) k_kraus1q<T, 2, int><<<nblocks(threads), 256, 0, st>>>(A, out, L, Aa, R, K, G);
    else k_kraus1q<T, 1, int><<<nblocks(threads), 256, 0, st>>>(A, out, L, Aa, R, K, G);
  } else {
    if (pair) k_kraus1q<T, 2, int64_t><<<nblocks(threads), 256, 0, st>>>(A, out, L, Aa, R, K, G);
    else k_kraus1q<T, 1, int64_t><<<nblocks(threads), 256, 0, st>>>(A, out, L, Aa, R, K, G);
  }
  count_launch();
}

template <typename T>
void mix2q(cudaStream_t st, const cx<T> *W, cx<T> *Z, int kr, int Cc, int R, const double *t, int K) {
  // nb folded into kr by the caller when the leading legs are contiguous; see engine
  Gate2<T> G;
  for (int i = 0; i < 16 * K; ++i) G.t[i] = cmk<T>((T)t[2 * i], (T)t[2 * i + 1]);
  k_mix2q<T><<<nblocks((int64_t)kr * Cc * R), 256, 0, st>>>(W, Z, 1, kr, Cc, R, K, G);
  count_launch();
}

template <typename T>
void mix2q_batched(cudaStream_t st, const cx<T> *W, cx<T> *Z, int nb, int kr, int Cc, int R, const double *t, int K) {
  Gate2<T> G;
  for (int i = 0; i < 16 * K; ++i) G.t[i] = cmk<T>((T)t[2 * i], (T)t[2 * i + 1]);
  k_mix2q<T><<<nblocks((int64_t)nb * kr * Cc * R), 256, 0, st>>>(W, Z, nb, kr, Cc, R, K, G);
  count_launch();
}

template <typename T>
void copy4d(cudaStream_t st, cx<T> *dst, const cx<T> *src, const int64_t d[4], const int64_t s[4], int conj) {
  const int64_t total = d[0] * d[1] * d[2] * d[3];
  if (total <= 0) return;
  k_copy4d<T><<<nblocks(total), 256, 0, st>>>(dst, src, d[0], d[1], d[2], d[3], s[0], s[1], s[2], s[3], conj);
  count_launch();
}

template <typename T>
void permute(cudaStream_t st, cx<T> *dst, const cx<T> *src, int nd, const int64_t *d, const int64_t *s, int conj) {
  Perm6 P;
  int64_t total = 1;
  for (int k = 0; k < 6; ++k) {
    const int j = k - (6 - nd);
    P.d[k] = j >= 0 ? d[j] : 1;
    P.s[k] = j >= 0 ? s[j] : 0;
    total *= P.d[k];
  }
  if (total <= 0) return;
  k_permute6<T><<<nblocks(total), 256, 0, st>>>(dst, src, total, P, conj);
  count_launch();
}

template <typename T>
void scale_matrix(cudaStream_t st, cx<T> *X, int M, int N, int64_t ld, const T *s, int by_row, int mode) {
  if ((int64_t)M * N <= 0) return;
  const T thr_rel = sizeof(T) == 4 ? T(1e-6) : T(1e-14);
  k_scale<T><<<nblocks((int64_t)M * N), 256, 0, st>>>(X, M, N, ld, s, by_row, mode, thr_rel);
  count_launch();
}

template <typename T>
void blockdiag2(cudaStream_t st, cx<T> *dst, const cx<T> *Q, int B, int Aa, int kr) {
  k_blockdiag2<T><<<nblocks((int64_t)B * 4 * Aa * kr), 256, 0, st>>>(dst, Q, B, Aa, kr);
  count_launch();
}

template <typename T>
void fill_zero(cudaStream_t st, cx<T> *p, size_t n) {
  if (n == 0) return;
  k_fill0<T><<<nblocks((int64_t)n), 256, 0, st>>>(p, n);
  count_launch();
}

template <typename T>
void sigma_weights(cudaStream_t st, const T *sigma, int n, int keep, double *out) {
  k_sigma_weights<T><<<1, 256, 0, st>>>(sigma, n, keep, out);
  count_launch();
}

template <typename T>
void sqrt_inplace(cudaStream_t st, T *s, int n) {
  k_sqrt_inplace<T><<<(n + 255) / 256, 256, 0, st>>>(s, n);
  count_launch();
}

template <typename T>
void apply_op_site(cudaStream_t st, const cx<T> *A, cx<T> *out, int L, int Aa, int R, const double *o) {
  k_apply_op<T><<<nblocks((int64_t)L * Aa * R), 256, 0, st>>>(A, out, L, Aa, R, cmk<T>((T)o[0], (T)o[1]),
                                                               cmk<T>((T)o[2], (T)o[3]), cmk<T>((T)o[4], (T)o[5]),
                                                               cmk<T>((T)o[6], (T)o[7]));
  count_launch();
}

template <typename T>
void batched_trace(cudaStream_t st, const cx<T> *M, int n, int64_t ld, int64_t bs, int batch, double2 *out) {
  k_trace<T><<<std::min(batch, 4096), 256, 0, st>>>(M, n, ld, bs, batch, out);
  count_launch();
}

template <typename T>
void gaussian(cudaStream_t st, cx<T> *out, size_t n, uint64_t seed) {
  k_gauss<T><<<nblocks((int64_t)n), 256, 0, st>>>(out, n, seed);
  count_launch();
}

template <typename T>
void sumsq(cudaStream_t st, const cx<T> *x, size_t n, double *out) {
  cudaMemsetAsync(out, 0, sizeof(double), st);
  k_sumsq<T><<<std::min<int64_t>(nblocks((int64_t)n), 1024), 256, 0, st>>>(x, n, out);
  count_launch();
}

#define INST(T)                                                                                             \
  template void kraus1q<T>(cudaStream_t, const cx<T> *, cx<T> *, int, int, int, const double *, int);      \
  template void mix2q<T>(cudaStream_t, const cx<T> *, cx<T> *, int, int, int, const double *, int);        \
  template void mix2q_batched<T>(cudaStream_t, const cx<T> *, cx<T> *, int, int, int, int, const double *, \
                                 int);                                                                      \
  template void copy4d<T>(cudaStream_t, cx<T> *, const cx<T> *, const int64_t *, const int64_t *, int);     \
  template void permute<T>(cudaStream_t, cx<T> *, const cx<T> *, int, const int64_t *, const int64_t *, int); \
  template void scale_matrix<T>(cudaStream_t, cx<T> *, int, int, int64_t, const T *, int, int);             \
  template void blockdiag2<T>(cudaStream_t, cx<T> *, const cx<T> *, int, int, int);                        \
  template void fill_zero<T>(cudaStream_t, cx<T> *, size_t);                                               \
  template void sigma_weights<T>(cudaStream_t, const T *, int, int, double *);                             \
  template void sqrt_inplace<T>(cudaStream_t, T *, int);                                                   \
  template void apply_op_site<T>(cudaStream_t, const cx<T> *, cx<T> *, int, int, int, const double *);      \
  template void batched_trace<T>(cudaStream_t, const cx<T> *, int, int64_t, int64_t, int, double2 *);       \
  template void gaussian<T>(cudaStream_t, cx<T> *, size_t, uint64_t);                                     \
  template void sumsq<T>(cudaStream_t, const cx<T> *, size_t, double *);                                  \
  template void env_dot<T>(cudaStream_t, const cx<T> *, const cx<T> *, int64_t, int, double *);            \
  template void gather_mats<T>(cudaStream_t, const cx<T> *, cx<T> *, const int *, int64_t, int);
INST(float)
INST(double)
#undef INST

}  // namespace mpdo
