// Kernels of the adjoint (reverse-mode) sweep: transposed Kraus / two-site
// mixes with their gate-tensor reductions, the right-side triangular solve of
// the QR adjoint, the Hermitian "copy lower to upper" step, the eigenvector
// adjoint coefficients of the truncated splits and the kappa pass, and the
// matrix-product-operator mixes of the readout environments.
//
// Cotangents follow one convention throughout: for a real loss L and a complex
// tensor X, Xbar = dL/dRe(X) + i dL/dIm(X), so that for a real parameter p,
// dL/dp = Re sum conj(Xbar) dX/dp.
#include "kernels.cuh"

#include <algorithm>
#include <stdexcept>

namespace mpdo {

namespace {
inline int nblk(int64_t n, int t = 256) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + t - 1) / t, 152 * 16)); }

template <typename T> struct G1 { cx<T> g[2 * 2 * 16]; };
template <typename T> struct G2 { cx<T> t[16 * 16]; };

template <typename T> __device__ __forceinline__ T wred(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Abar[l][s][a][r] = sum_{x,k} conj(G[x][s][k]) Obar[l][x][a K + k][r]
template <typename T>
__global__ void k_kraus1q_bwd(const cx<T> *__restrict__ Ob, cx<T> *__restrict__ Ab, int L, int Aa, int R, int K,
                              const G1<T> G) {
  const int64_t total = (int64_t)L * Aa * R;
  const int64_t aK = (int64_t)Aa * K;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % R, la = t / R, a = la % Aa, l = la / Aa;
    cx<T> acc[2] = {czero<T>(), czero<T>()};
    for (int x = 0; x < 2; ++x) {
      const cx<T> *o = Ob + ((l * 2 + x) * aK + a * K) * R + r;
      for (int k = 0; k < K; ++k) {
        const cx<T> v = o[(int64_t)k * R];
#pragma unroll
        for (int s = 0; s < 2; ++s) cfmac<T>(acc[s], G.g[(x * 2 + s) * K + k], v);
      }
    }
    Ab[((l * 2 + 0) * Aa + a) * R + r] = acc[0];
    Ab[((l * 2 + 1) * Aa + a) * R + r] = acc[1];
  }
}

// acc[(x*2+s)*K + k] += sum_{l,a,r} Obar[l][x][aK+k][r] conj(A[l][s][a][r]); grid.y = k
template <typename T>
__global__ void k_kraus1q_grad(const cx<T> *__restrict__ Ob, const cx<T> *__restrict__ A, int L, int Aa, int R,
                               int K, double2 *acc) {
  __shared__ double red[32][8];
  const int k = blockIdx.y;
  const int64_t total = (int64_t)L * Aa * R;
  const int64_t aK = (int64_t)Aa * K;
  cx<T> s4[4] = {czero<T>(), czero<T>(), czero<T>(), czero<T>()};
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % R, la = t / R, a = la % Aa, l = la / Aa;
    const cx<T> a0 = A[((l * 2 + 0) * Aa + a) * R + r], a1 = A[((l * 2 + 1) * Aa + a) * R + r];
#pragma unroll
    for (int x = 0; x < 2; ++x) {
      const cx<T> o = Ob[((l * 2 + x) * aK + a * K + k) * R + r];
      cfmac<T>(s4[x * 2 + 0], a0, o);      // conj(a0) * o
      cfmac<T>(s4[x * 2 + 1], a1, o);
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const T re = wred<T>(s4[q].x), im = wred<T>(s4[q].y);
    if (lane == 0) { red[w][2 * q] = re; red[w][2 * q + 1] = im; }
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    double v = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) v += red[i][threadIdx.x];
    const int q = threadIdx.x >> 1;
    double *dst = reinterpret_cast<double *>(acc + q * K + k) + (threadIdx.x & 1);
    atomicAdd(dst, v);
  }
}

// Zbar: [2 x][kr][2 y][C*K][R] -> Wbar: [2 s][kr][2 t][C][R]
// Wbar[s][k][t][c][r] = sum_{x,y,q} conj(T[x][y][s][t][q]) Zbar[x][k][y][c K + q][r]
template <typename T>
__global__ void k_mix2q_bwd(const cx<T> *__restrict__ Zb, cx<T> *__restrict__ Wb, int kr, int Cc, int R, int K,
                            const G2<T> G) {
  const int64_t CR = (int64_t)Cc * R;
  const int64_t total = (int64_t)kr * CR;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cr = t % CR, kk = t / CR;
    const int64_t c = cr / R, r = cr % R;
    cx<T> out[2][2];
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int u = 0; u < 2; ++u) out[s][u] = czero<T>();
    for (int x = 0; x < 2; ++x)
      for (int y = 0; y < 2; ++y) {
        const cx<T> *z = Zb + ((x * (int64_t)kr + kk) * 2 + y) * (CR * K) + (c * K) * R + r;
        for (int q = 0; q < K; ++q) {
          const cx<T> v = z[(int64_t)q * R];
#pragma unroll
          for (int s = 0; s < 2; ++s)
#pragma unroll
            for (int u = 0; u < 2; ++u) cfmac<T>(out[s][u], G.t[(((x * 2 + y) * 2 + s) * 2 + u) * K + q], v);
        }
      }
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int u = 0; u < 2; ++u) Wb[((s * (int64_t)kr + kk) * 2 + u) * CR + cr] = out[s][u];
  }
}

// acc[(((x*2+y)*2+s)*2+u)*K + q] += sum_{k,c,r} Zbar[x][k][y][cK+q][r] conj(W[s][k][u][c][r]); grid.y = q
template <typename T>
__global__ void k_mix2q_grad(const cx<T> *__restrict__ Zb, const cx<T> *__restrict__ W, int kr, int Cc, int R, int K,
                             double2 *acc) {
  __shared__ double red[32][32];
  const int q = blockIdx.y;
  const int64_t CR = (int64_t)Cc * R;
  const int64_t total = (int64_t)kr * CR;
  cx<T> s16[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) s16[i] = czero<T>();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cr = t % CR, kk = t / CR;
    const int64_t c = cr / R, r = cr % R;
    cx<T> z[4], w[4];
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int y = 0; y < 2; ++y) z[x * 2 + y] = Zb[((x * (int64_t)kr + kk) * 2 + y) * (CR * K) + (c * K + q) * R + r];
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int u = 0; u < 2; ++u) w[s * 2 + u] = W[((s * (int64_t)kr + kk) * 2 + u) * CR + cr];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) cfmac<T>(s16[i * 4 + j], w[j], z[i]);
  }
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const T re = wred<T>(s16[i].x), im = wred<T>(s16[i].y);
    if (lane == 0) { red[wi][2 * i] = re; red[wi][2 * i + 1] = im; }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) v += red[i][threadIdx.x];
    const int e = threadIdx.x >> 1;    // (x*2+y)*4 + (s*2+u)
    double *dst = reinterpret_cast<double *>(acc + e * K + q) + (threadIdx.x & 1);
    atomicAdd(dst, v);
  }
}

// B (m x k, row-major, ld ldb) <- B R^-H for R upper triangular (k x k,
// row-major, ld ldr).  One warp per row; lane j%32 holds entry j.  Solves
// b_i = sum_{j >= i} z_j conj(R_ij) from the last column; a diagonal entry
// below tiny * max|R_jj| gives z_j = 0 (rank-deficient factor).
template <typename T, int NREG, bool SM>
__global__ void k_trsm_rh(cx<T> *B, int m, int k, int64_t ldb, const cx<T> *R, int64_t ldr, T tiny) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cx<T> *St = reinterpret_cast<cx<T> *>(smraw);        // St[j][i] = conj(R[i][j])
  __shared__ T dmax;
  if (SM) {
    for (int64_t e = threadIdx.x; e < (int64_t)k * k; e += blockDim.x) {
      const int j = (int)(e / k), i = (int)(e % k);
      const cx<T> v = R[(int64_t)i * ldr + j];
      St[e] = cmk<T>(v.x, -v.y);
    }
  }
  if (threadIdx.x == 0) {
    T mx = T(0);
    for (int j = 0; j < k; ++j) mx = fmax(mx, sqrt(cabs2<T>(R[(int64_t)j * ldr + j])));
    dmax = mx;
  }
  __syncthreads();
  const T thr = tiny * dmax;
  const int lane = threadIdx.x & 31;
  const int warps = blockDim.x >> 5;
  for (int row = blockIdx.x * warps + (threadIdx.x >> 5); row < m; row += gridDim.x * warps) {
    cx<T> *b = B + (int64_t)row * ldb;
    cx<T> v[NREG];
#pragma unroll
    for (int q = 0; q < NREG; ++q) {
      const int i = lane + 32 * q;
      v[q] = i < k ? b[i] : czero<T>();
    }
    for (int j = k - 1; j >= 0; --j) {
      cx<T> bj = czero<T>();
#pragma unroll
      for (int q = 0; q < NREG; ++q)
        if (q == (j >> 5)) bj = v[q];
      bj.x = __shfl_sync(0xffffffffu, bj.x, j & 31);
      bj.y = __shfl_sync(0xffffffffu, bj.y, j & 31);
      const cx<T> rjj = R[(int64_t)j * ldr + j];
      const T a2 = cabs2<T>(rjj);
      cx<T> z = czero<T>();
      if (sqrt(a2) > thr && a2 > T(0)) {
        // z = bj / conj(rjj) = bj * rjj / |rjj|^2
        z = cscale<T>(cmul<T>(bj, rjj), T(1) / a2);
      }
#pragma unroll
      for (int q = 0; q < NREG; ++q) {
        const int i = lane + 32 * q;
        if (i == j) v[q] = z;
        else if (i < j) {
          const cx<T> c = SM ? St[(int64_t)j * k + i] : cconj<T>(R[(int64_t)i * ldr + j]);
          v[q] = csub<T>(v[q], cmul<T>(z, c));
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NREG; ++q) {
      const int i = lane + 32 * q;
      if (i < k) b[i] = v[q];
    }
  }
}

// M (n x n row-major) <- lower triangle of M mirrored: M_ij = conj(M_ji) for
// i < j, real diagonal
template <typename T>
__global__ void k_copyltu(cx<T> *M, int n) {
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / n), j = (int)(t % n);
    if (i < j) M[t] = cconj<T>(M[(int64_t)j * n + i]);
    else if (i == j) M[t].y = T(0);
  }
}

template <typename T>
__device__ __forceinline__ T broadened_inv(T d, T eta) {
  return eta > T(0) ? d / (d * d + eta) : (d != T(0) ? T(1) / d : T(0));
}

// Split adjoint coefficients: K (b x k, row-major) from UhUb = U^H Ubar_k,
// lam = s^2 (b values), dl[j] = Re<Lbar_j, L_j>, dr[j] = Re<Rbar_j, R_j>:
// K_ij = F_ij UhUb_ij (i != j), K_jj = lambar_j = (dl_j - dr_j) / (4 s_j^2),
// F_ij = 1 / (lam_j - lam_i) broadened by eta = (beta lam_0)^2.
template <typename T>
__global__ void k_split_K(const cx<T> *UhUb, const T *s, int b, int k, const double *dl, const double *dr, T beta,
                          cx<T> *Kout) {
  const int64_t total = (int64_t)b * k;
  const T l0 = s[0] * s[0];
  const T eta = (beta * l0) * (beta * l0);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / k), j = (int)(t % k);
    const T lj = s[j] * s[j], li = s[i] * s[i];
    if (i == j) {
      Kout[t] = cmk<T>(lj > T(0) ? (T)((dl[j] - dr[j]) / (4.0 * (double)lj)) : T(0), T(0));
    } else {
      const T f = broadened_inv<T>(lj - li, eta);
      Kout[t] = cscale<T>(UhUb[t], f);
    }
  }
}

// Kappa-pass adjoint coefficients: C (a x k, row-major) = F o VhX on the
// discarded rows i >= k (zero on the kept block), F_ij = 1/(lam_j - lam_i).
template <typename T>
__global__ void k_kappa_C(const cx<T> *VhX, const T *s, int a, int k, T beta, cx<T> *C) {
  const int64_t total = (int64_t)a * k;
  const T l0 = s[0] * s[0];
  const T eta = (beta * l0) * (beta * l0);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / k), j = (int)(t % k);
    if (i < k) { C[t] = czero<T>(); continue; }
    const T lj = s[j] * s[j], li = s[i] * s[i];
    C[t] = cscale<T>(VhX[t], broadened_inv<T>(lj - li, eta));
  }
}

// out[j] = Re sum_i conj(A[i*si + j*sj]) B[i*si + j*sj], i < len, j < n (one block per j)
template <typename T>
__global__ void k_redot(const cx<T> *A, const cx<T> *B, int n, int64_t len, int64_t si, int64_t sj, double *out) {
  __shared__ double red[32];
  const int j = blockIdx.x;
  double acc = 0;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
    const cx<T> a = A[i * si + j * sj], b = B[i * si + j * sj];
    acc += (double)a.x * b.x + (double)a.y * b.y;
  }
  acc = wred<double>(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
    out[j] = v;
  }
}

// Qbar[(b a)][k] = sum_x Sbar[b][x][a][x kq + k]   (adjoint of blockdiag2)
template <typename T>
__global__ void k_blockdiag2_bwd(const cx<T> *Sb, cx<T> *Qb, int B, int Aa, int kq) {
  const int64_t total = (int64_t)B * Aa * kq;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = t % kq, ba = t / kq, a = ba % Aa, b = ba / Aa;
    const cx<T> v0 = Sb[((b * 2 + 0) * Aa + a) * (2 * (int64_t)kq) + k];
    const cx<T> v1 = Sb[((b * 2 + 1) * Aa + a) * (2 * (int64_t)kq) + kq + k];
    Qb[t] = cadd<T>(v0, v1);
  }
}

// out[o][l][x][rest] = sum_{i < Din, y} W[i*wi + o*wo + x*2 + y] in[i][l][y][rest]
// (W: Din x Dout blocks of 2 x 2 operators, element [x][y] = W[.. + x*2 + y])
template <typename T>
__global__ void k_mpo_mix(const cx<T> *in, cx<T> *out, const cx<T> *W, int Din, int Dout, int64_t wi, int64_t wo,
                          int64_t L, int64_t rest) {
  const int64_t total = (int64_t)Dout * L * 2 * rest;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = t % rest;
    const int64_t x = (t / rest) % 2;
    const int64_t l = (t / (rest * 2)) % L;
    const int64_t o = t / (rest * 2 * L);
    cx<T> acc = czero<T>();
    for (int i = 0; i < Din; ++i) {
      const cx<T> *w = W + i * wi + o * wo + x * 2;
      const cx<T> *src = in + ((int64_t)i * L + l) * 2 * rest + q;
      cfma<T>(acc, w[0], src[0]);
      cfma<T>(acc, w[1], src[rest]);
    }
    out[t] = acc;
  }
}

// y[i] += alpha x[i]
template <typename T>
__global__ void k_axpy(cx<T> *y, const cx<T> *x, int64_t n, T alpha) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    y[t].x += alpha * x[t].x;
    y[t].y += alpha * x[t].y;
  }
}
}  // namespace

template <typename T>
void kraus1q_bwd(cudaStream_t st, const cx<T> *Ob, cx<T> *Ab, int L, int Aa, int R, const double *g_host, int K) {
  G1<T> G;
  for (int i = 0; i < 4 * K; ++i) G.g[i] = cmk<T>((T)g_host[2 * i], (T)g_host[2 * i + 1]);
  k_kraus1q_bwd<T><<<nblk((int64_t)L * Aa * R), 256, 0, st>>>(Ob, Ab, L, Aa, R, K, G);
  count_launch();
}

template <typename T>
void kraus1q_grad(cudaStream_t st, const cx<T> *Ob, const cx<T> *A, int L, int Aa, int R, int K, double2 *acc) {
  const int64_t total = (int64_t)L * Aa * R;
  dim3 grid(std::min(nblk(total), 256), K);
  k_kraus1q_grad<T><<<grid, 256, 0, st>>>(Ob, A, L, Aa, R, K, acc);
  count_launch();
}

template <typename T>
void mix2q_bwd(cudaStream_t st, const cx<T> *Zb, cx<T> *Wb, int kr, int Cc, int R, const double *t_host, int K) {
  G2<T> G;
  for (int i = 0; i < 16 * K; ++i) G.t[i] = cmk<T>((T)t_host[2 * i], (T)t_host[2 * i + 1]);
  k_mix2q_bwd<T><<<nblk((int64_t)kr * Cc * R), 256, 0, st>>>(Zb, Wb, kr, Cc, R, K, G);
  count_launch();
}

template <typename T>
void mix2q_grad(cudaStream_t st, const cx<T> *Zb, const cx<T> *W, int kr, int Cc, int R, int K, double2 *acc) {
  const int64_t total = (int64_t)kr * Cc * R;
  dim3 grid(std::min(nblk(total), 256), K);
  k_mix2q_grad<T><<<grid, 256, 0, st>>>(Zb, W, kr, Cc, R, K, acc);
  count_launch();
}

template <typename T>
void trsm_rh(cudaStream_t st, cx<T> *B, int m, int k, int64_t ldb, const cx<T> *R, int64_t ldr) {
  if (m <= 0 || k <= 0) return;
  const T tiny = sizeof(T) == 4 ? T(1e-6) : T(1e-14);
  const size_t bytes = (size_t)k * k * sizeof(cx<T>);
  const bool sm = bytes <= (size_t)kSmemCeiling;
  const int warps = 8;
  const int grid = std::max(1, std::min((m + warps - 1) / warps, 152 * 4));
#define MPDO_TRSM(NR)                                                                                        \
  if (k <= 32 * NR) {                                                                                        \
    if (sm) {                                                                                                \
      smem_optin(k_trsm_rh<T, NR, true>);                                                                    \
      k_trsm_rh<T, NR, true><<<grid, 32 * warps, bytes, st>>>(B, m, k, ldb, R, ldr, tiny);                   \
    } else {                                                                                                 \
      k_trsm_rh<T, NR, false><<<grid, 32 * warps, 0, st>>>(B, m, k, ldb, R, ldr, tiny);                      \
    }                                                                                                        \
    count_launch();                                                                                          \
    return;                                                                                                  \
  }
  MPDO_TRSM(1)
  MPDO_TRSM(2)
  MPDO_TRSM(4)
  MPDO_TRSM(8)
  MPDO_TRSM(16)
#undef MPDO_TRSM
  throw std::runtime_error("trsm_rh: factor wider than 512 columns");
}

template <typename T>
void copyltu(cudaStream_t st, cx<T> *M, int n) {
  k_copyltu<T><<<nblk((int64_t)n * n), 256, 0, st>>>(M, n);
  count_launch();
}

template <typename T>
void split_K(cudaStream_t st, const cx<T> *UhUb, const T *s, int b, int k, const double *dl, const double *dr,
             double beta, cx<T> *Kout) {
  k_split_K<T><<<nblk((int64_t)b * k), 256, 0, st>>>(UhUb, s, b, k, dl, dr, (T)beta, Kout);
  count_launch();
}

template <typename T>
void kappa_C(cudaStream_t st, const cx<T> *VhX, const T *s, int a, int k, double beta, cx<T> *C) {
  k_kappa_C<T><<<nblk((int64_t)a * k), 256, 0, st>>>(VhX, s, a, k, (T)beta, C);
  count_launch();
}

template <typename T>
void redot(cudaStream_t st, const cx<T> *A, const cx<T> *B, int n, int64_t len, int64_t si, int64_t sj, double *out) {
  if (n <= 0) return;
  k_redot<T><<<n, 256, 0, st>>>(A, B, n, len, si, sj, out);
  count_launch();
}

template <typename T>
void blockdiag2_bwd(cudaStream_t st, const cx<T> *Sb, cx<T> *Qb, int B, int Aa, int kq) {
  k_blockdiag2_bwd<T><<<nblk((int64_t)B * Aa * kq), 256, 0, st>>>(Sb, Qb, B, Aa, kq);
  count_launch();
}

template <typename T>
void mpo_mix(cudaStream_t st, const cx<T> *in, cx<T> *out, const cx<T> *W, int Din, int Dout, int64_t wi, int64_t wo,
             int64_t L, int64_t rest) {
  k_mpo_mix<T><<<nblk((int64_t)Dout * L * 2 * rest), 256, 0, st>>>(in, out, W, Din, Dout, wi, wo, L, rest);
  count_launch();
}

template <typename T>
void axpy(cudaStream_t st, cx<T> *y, const cx<T> *x, int64_t n, double alpha) {
  if (n <= 0) return;
  k_axpy<T><<<nblk(n), 256, 0, st>>>(y, x, n, (T)alpha);
  count_launch();
}

#define INST_ADJ(T)                                                                                              \
  template void kraus1q_bwd<T>(cudaStream_t, const cx<T> *, cx<T> *, int, int, int, const double *, int);        \
  template void kraus1q_grad<T>(cudaStream_t, const cx<T> *, const cx<T> *, int, int, int, int, double2 *);      \
  template void mix2q_bwd<T>(cudaStream_t, const cx<T> *, cx<T> *, int, int, int, const double *, int);          \
  template void mix2q_grad<T>(cudaStream_t, const cx<T> *, const cx<T> *, int, int, int, int, double2 *);        \
  template void trsm_rh<T>(cudaStream_t, cx<T> *, int, int, int64_t, const cx<T> *, int64_t);                     \
  template void copyltu<T>(cudaStream_t, cx<T> *, int);                                                          \
  template void split_K<T>(cudaStream_t, const cx<T> *, const T *, int, int, const double *, const double *,      \
                           double, cx<T> *);                                                                     \
  template void kappa_C<T>(cudaStream_t, const cx<T> *, const T *, int, int, double, cx<T> *);                  \
  template void redot<T>(cudaStream_t, const cx<T> *, const cx<T> *, int, int64_t, int64_t, int64_t, double *);  \
  template void blockdiag2_bwd<T>(cudaStream_t, const cx<T> *, cx<T> *, int, int, int);                          \
  template void mpo_mix<T>(cudaStream_t, const cx<T> *, cx<T> *, const cx<T> *, int, int, int64_t, int64_t,      \
                           int64_t, int64_t);                                                                    \
  template void axpy<T>(cudaStream_t, cx<T> *, const cx<T> *, int64_t, double);
INST_ADJ(float)
INST_ADJ(double)

}  // namespace mpdo
