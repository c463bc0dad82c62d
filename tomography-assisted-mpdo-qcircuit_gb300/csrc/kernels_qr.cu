// Householder QR of row blocks ("chunks") -- the building block of a
// tall-skinny QR (TSQR) -- and the matching explicit-Q construction.
//
// One CTA per chunk.  The chunk (rows_c x n, column-major) lives in shared
// memory when it fits, otherwise in its global workspace slot (L2 resident).
// Reflectors follow LAPACK's zlarfg convention (real beta, H = I - tau v v^H,
// v(0) = 1), so R has a real diagonal of sign -sign(Re alpha); the trailing
// update applies H^H (zgeqr2), Q is accumulated backwards with H (zungqr).
#include "kernels.cuh"

#include <algorithm>
#include <cfloat>

namespace mpdo {

namespace {
constexpr int QR_NT = 1024;
constexpr size_t SMEM_CAP = 200 * 1024;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ T block_sum(T v, T *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T s = T(0);
  if (threadIdx.x < 32) {
    s = (lane < nw) ? red[lane] : T(0);
    s = warp_sum(s);
    if (lane == 0) red[32] = s;
  }
  __syncthreads();
  return red[32];
}

template <typename T> struct NormalMin;
template <> struct NormalMin<float> { static constexpr float v = FLT_MIN; };
template <> struct NormalMin<double> { static constexpr double v = DBL_MIN; };

template <typename T>
__device__ T block_max(T v, T *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    T s = (lane < nw) ? red[lane] : T(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
    if (lane == 0) red[32] = s;
  }
  __syncthreads();
  return red[32];
}

// Scaled 2-norm parts of x[i0..rows) by one warp: amax = max |re|, |im|
// and q = sum |x_i / amax|^2 (q = 0 when amax is below the smallest normal).
template <typename T>
__device__ __forceinline__ void warp_col_norm(const cx<T> *x, int i0, int rows, int lane, T &amax, T &q) {
  T pmax = T(0);
  for (int i = i0 + lane; i < rows; i += 32) pmax = fmax(pmax, fmax(fabs(x[i].x), fabs(x[i].y)));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) pmax = fmax(pmax, __shfl_xor_sync(0xffffffffu, pmax, o));
  T part = T(0);
  if (pmax >= NormalMin<T>::v) {
    const T inv = T(1) / pmax;
    for (int i = i0 + lane; i < rows; i += 32) part += cabs2<T>(cscale<T>(x[i], inv));
  }
  amax = pmax;
  q = warp_sum(part);
}

template <typename T, bool SMEM>
__global__ void __launch_bounds__(QR_NT) k_qr_factor(int m, int n, int mc, View<T> in, cx<T> *vws,
                                                     cx<T> *tau_out, cx<T> *rstack) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ cx<T> hh[2];  // tau, scale
  __shared__ T cn[4];      // scaled norm parts of the next column, by parity
  // blockIdx.y: matrix of a batch (input at batch stride in.bs; each
  // matrix's reflectors, tau and R stack in consecutive slots)
  const int bb = blockIdx.y;
  const int nchunks = gridDim.x;
  vws += (int64_t)bb * nchunks * mc * n;
  tau_out += (int64_t)bb * nchunks * n;
  rstack += (int64_t)bb * nchunks * n * n;
  const int c = blockIdx.x;
  const int r0 = c * mc;
  const int rows = min(mc, m - r0);
  const int kc = min(rows, n);
  cx<T> *Wg = vws + (int64_t)c * mc * n;
  cx<T> *W = SMEM ? reinterpret_cast<cx<T> *>(smem_raw) : Wg;
  const int64_t ld = mc;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;

  for (int64_t idx = tid; idx < (int64_t)rows * n; idx += blockDim.x) {
    const int i = (int)(idx % rows), j = (int)(idx / rows);
    W[j * ld + i] = view_ld(in, bb, r0 + i, j);
  }
  __syncthreads();

  // Column j's reflector needs the scaled 2-norm of its part below the
  // diagonal (as LAPACK's nrm2: max |x_i|, then sum (|x_i| / max)^2, so that
  // columns near the underflow threshold keep an exact norm and the
  // reflector stays unitary).  The warp that applies reflector j to column
  // j+1 computes that column's norm right after its update (double-buffered
  // by parity), every thread then forms reflector j+1 itself from that norm
  // and the diagonal entry, and the writes that finish reflector j (beta on
  // the diagonal, v = scl * x below it) are deferred to step j+1, where
  // nothing reads column j.  One block barrier per column.
  if (warp == 0 && kc > 0) {
    T a, q;
    warp_col_norm<T>(W + 0 * ld, 1, rows, lane, a, q);
    if (lane == 0) { cn[0] = a; cn[1] = q; }
  }
  __syncthreads();
  cx<T> prev_tau = czero<T>(), prev_scl = czero<T>(), prev_beta = czero<T>();
  bool prev_zero_v = false, prev_set_beta = false;
  auto finish = [&](int jc) {            // deferred writes of reflector jc
    for (int i = jc + 1 + tid; i < rows; i += blockDim.x)
      W[jc * ld + i] = prev_zero_v ? czero<T>() : cmul<T>(W[jc * ld + i], prev_scl);
    if (tid == 0 && prev_set_beta) W[jc * ld + jc] = prev_beta;
  };
  for (int j = 0; j < kc; ++j) {
    if (j > 0) finish(j - 1);
    T amax = cn[2 * (j & 1)];
    const T xs = cn[2 * (j & 1) + 1];
    // entries below the smallest normal number are underflow debris: the
    // column is treated as exactly zero (1/amax would overflow)
    const bool debris = amax < NormalMin<T>::v;
    if (debris) amax = T(0);
    const cx<T> al = W[j * ld + j];
    cx<T> tau = czero<T>(), scl = czero<T>(), beta_c = czero<T>();
    bool set_beta = false;
    {
      const T xnorm = amax * sqrt(xs);
      const T nrm = hypot(hypot(al.x, al.y), xnorm);
      if (!(xnorm == T(0) && al.y == T(0)) && nrm >= NormalMin<T>::v) {
        const T beta = (al.x >= T(0)) ? -nrm : nrm;
        tau = cmk<T>((beta - al.x) / beta, -al.y / beta);
        // scl = 1 / (alpha - beta), scaled complex reciprocal
        const cx<T> d = cmk<T>(al.x - beta, al.y);
        const T sc = fmax(fabs(d.x), fabs(d.y));
        const cx<T> ds = cmk<T>(d.x / sc, d.y / sc);
        const T dd = cabs2<T>(ds);
        scl = cmk<T>(ds.x / (dd * sc), -ds.y / (dd * sc));
        beta_c = cmk<T>(beta, T(0));
        set_beta = true;
      }
    }
    if (tid == 0) tau_out[(int64_t)c * n + j] = tau;
    const bool ident = tau.x == T(0) && tau.y == T(0);
    const cx<T> ctau = cconj<T>(tau), cscl = cconj<T>(scl);
    // two trailing columns per warp and pass (k, k + nw): one read of the
    // reflector serves both, and their dot / reduce / update chains overlap;
    // each column's arithmetic is the same as one at a time
    for (int k = j + 1 + warp; k < n; k += 2 * nw) {
      const int k2 = k + nw;
      const bool two = k2 < n;
      cx<T> *Wk = W + k * ld;
      cx<T> *Wk2 = W + (two ? k2 : k) * ld;
      if (!ident) {
        cx<T> d = czero<T>(), d2 = czero<T>();
        if (!debris) {
          if (two) {
            for (int i = j + 1 + lane; i < rows; i += 32) {
              const cx<T> v = W[j * ld + i];
              cfmac<T>(d, v, Wk[i]);
              cfmac<T>(d2, v, Wk2[i]);
            }
          } else {
            for (int i = j + 1 + lane; i < rows; i += 32) cfmac<T>(d, W[j * ld + i], Wk[i]);
          }
        }
        d.x = warp_sum(d.x); d.y = warp_sum(d.y);
        if (two) { d2.x = warp_sum(d2.x); d2.y = warp_sum(d2.y); }
        // w = tau^H (W[j][k] + v^H W[:, k]) with v = scl x
        const cx<T> w = cmul<T>(ctau, cadd<T>(Wk[j], cmul<T>(cscl, d)));
        const cx<T> g = cmul<T>(scl, w);
        const cx<T> w2 = cmul<T>(ctau, cadd<T>(Wk2[j], cmul<T>(cscl, d2)));
        const cx<T> g2 = cmul<T>(scl, w2);
        __syncwarp();
        if (lane == 0) {
          Wk[j] = csub<T>(Wk[j], w);
          if (two) Wk2[j] = csub<T>(Wk2[j], w2);
        }
        if (!debris) {
          if (two) {
            for (int i = j + 1 + lane; i < rows; i += 32) {
              const cx<T> v = W[j * ld + i];
              Wk[i] = csub<T>(Wk[i], cmul<T>(v, g));
              Wk2[i] = csub<T>(Wk2[i], cmul<T>(v, g2));
            }
          } else {
            for (int i = j + 1 + lane; i < rows; i += 32) Wk[i] = csub<T>(Wk[i], cmul<T>(W[j * ld + i], g));
          }
        }
      }
      if (k == j + 1 && k < kc) {
        __syncwarp();
        T a, q;
        warp_col_norm<T>(Wk, k + 1, rows, lane, a, q);
        if (lane == 0) { cn[2 * (k & 1)] = a; cn[2 * (k & 1) + 1] = q; }
      }
    }
    __syncthreads();
    prev_tau = tau;
    prev_scl = scl;
    prev_beta = beta_c;
    prev_set_beta = set_beta;
    prev_zero_v = ident || debris;
  }
  if (kc > 0) {
    finish(kc - 1);
    __syncthreads();
  }
  for (int j = kc; j < n; ++j) {
    if (tid == 0) tau_out[(int64_t)c * n + j] = czero<T>();
  }

  // R_c into its n-row slot of the stack
  cx<T> *Rs = rstack + (int64_t)c * n * n;
  for (int64_t idx = tid; idx < (int64_t)n * n; idx += blockDim.x) {
    const int i = (int)(idx / n), j = (int)(idx % n);
    Rs[idx] = (i < kc && j >= i) ? W[j * ld + i] : czero<T>();
  }
  if (SMEM) {
    for (int64_t idx = tid; idx < (int64_t)rows * n; idx += blockDim.x) {
      const int i = (int)(idx % rows), j = (int)(idx / rows);
      Wg[j * ld + i] = W[j * ld + i];
    }
  }
}

template <typename T, bool SMEM>
__global__ void __launch_bounds__(QR_NT) k_qr_apply(int m, int n, int mc, const cx<T> *vws, const cx<T> *tau,
                                                    const cx<T> *bin, int64_t ldb, int nq, cx<T> *qout,
                                                    int64_t ldq) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // blockIdx.y selects a group of gridDim.y-way split columns of B (groups
  // sized so that each fits shared memory)
  int q0 = 0;
  {
    const int per = (nq + gridDim.y - 1) / gridDim.y;
    q0 = blockIdx.y * per;
    if (bin) bin += q0;
    qout += q0;
    nq = max(0, min(per, nq - q0));
    if (nq == 0) return;
  }
  const int c = blockIdx.x;
  const int r0 = c * mc;
  const int rows = min(mc, m - r0);
  const int kc = min(rows, n);
  const cx<T> *V = vws + (int64_t)c * mc * n;
  const cx<T> *tc = tau + (int64_t)c * n;
  cx<T> *vcol = reinterpret_cast<cx<T> *>(smem_raw);
  // B: rows x nq; in shared memory column-major (ld = rows), else in place in
  // qout (row-major, leading dimension ldq)
  cx<T> *Bs = vcol + 2 * mc;
  cx<T> *Bg = qout + (int64_t)r0 * ldq;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  auto B = [&](int i, int q) -> cx<T> & { return SMEM ? Bs[(int64_t)q * rows + i] : Bg[(int64_t)i * ldq + q]; };

  for (int64_t idx = tid; idx < (int64_t)rows * nq; idx += blockDim.x) {
    int i, q;
    if (SMEM) { i = (int)(idx % rows); q = (int)(idx / rows); } else { i = (int)(idx / nq); q = (int)(idx % nq); }
    cx<T> v = czero<T>();
    if (i < kc) {
      if (bin) v = bin[(int64_t)(c * n + i) * ldb + q];
      else v = (i == q + q0) ? cmk<T>(T(1), T(0)) : czero<T>();
    }
    B(i, q) = v;
  }
  __syncthreads();
  // reflector j's vector is staged in vcol[j & 1] while reflector j+1 is
  // being applied from the other buffer: one block barrier per reflector
  auto stage = [&](int jj) {
    cx<T> *vb = vcol + (jj & 1) * mc;
    for (int i = jj + 1 + tid; i < rows; i += blockDim.x) vb[i] = V[(int64_t)jj * mc + i];
  };
  if (kc > 0) stage(kc - 1);
  __syncthreads();
  for (int j = kc - 1; j >= 0; --j) {
    if (j > 0) stage(j - 1);
    const cx<T> tj = tc[j];
    const cx<T> *vj = vcol + (j & 1) * mc;
    if (!(tj.x == T(0) && tj.y == T(0))) {
      // each warp takes up to QB columns at a time, so every v_i read from
      // shared memory serves QB products
      constexpr int QB = 4;
      for (int q0 = warp * QB; q0 < nq; q0 += nw * QB) {
        const int nb = min(QB, nq - q0);
        cx<T> w[QB];
#pragma unroll
        for (int b = 0; b < QB; ++b) w[b] = (lane == 0 && b < nb) ? B(j, q0 + b) : czero<T>();
        for (int i = j + 1 + lane; i < rows; i += 32) {
          const cx<T> v = vj[i];
#pragma unroll
          for (int b = 0; b < QB; ++b)
            if (b < nb) cfmac<T>(w[b], v, B(i, q0 + b));
        }
#pragma unroll
        for (int b = 0; b < QB; ++b) {
          w[b].x = warp_sum(w[b].x);
          w[b].y = warp_sum(w[b].y);
          w[b] = cmul<T>(tj, w[b]);
        }
        __syncwarp();
        if (lane == 0)
          for (int b = 0; b < nb; ++b) B(j, q0 + b) = csub<T>(B(j, q0 + b), w[b]);
        for (int i = j + 1 + lane; i < rows; i += 32) {
          const cx<T> v = vj[i];
#pragma unroll
          for (int b = 0; b < QB; ++b)
            if (b < nb) B(i, q0 + b) = csub<T>(B(i, q0 + b), cmul<T>(v, w[b]));
        }
      }
    }
    __syncthreads();
  }
  if (SMEM) {
    for (int64_t idx = tid; idx < (int64_t)rows * nq; idx += blockDim.x) {
      const int i = (int)(idx / nq), q = (int)(idx % nq);
      Bg[(int64_t)i * ldq + q] = Bs[(int64_t)q * rows + i];
    }
  }
}
}  // namespace

template <typename T>
void qr_factor_chunks(cudaStream_t st, int m, int n, int mc, int nchunks, const View<T> &in, cx<T> *vws,
                      cx<T> *tau, cx<T> *rstack, int batch) {
  const size_t bytes = (size_t)mc * n * sizeof(cx<T>);
  const dim3 grid(nchunks, std::max(batch, 1));
  if (bytes <= SMEM_CAP) {
    smem_optin(k_qr_factor<T, true>);
    k_qr_factor<T, true><<<grid, QR_NT, bytes, st>>>(m, n, mc, in, vws, tau, rstack);
  } else {
    k_qr_factor<T, false><<<grid, QR_NT, 0, st>>>(m, n, mc, in, vws, tau, rstack);
  }
  count_launch();
}

template <typename T>
void qr_apply_chunks(cudaStream_t st, int m, int n, int mc, int nchunks, const cx<T> *vws, const cx<T> *tau,
                     const cx<T> *bin, int64_t ldb, int nq, cx<T> *qout, int64_t ldq) {
  // columns of B are split into groups that fit shared memory next to the
  // two reflector buffers, one CTA per (chunk, group)
  const size_t esz = sizeof(cx<T>);
  const int64_t fit = ((int64_t)(SMEM_CAP / esz) - 2 * (int64_t)mc) / std::max(mc, 1);
  const int groups = fit >= 1 ? (int)((nq + fit - 1) / fit) : 0;
  if (groups >= 1 && groups <= 64) {
    const int per = (nq + groups - 1) / groups;
    const size_t bytes = ((size_t)2 * mc + (size_t)mc * per) * esz;
    smem_optin(k_qr_apply<T, true>);
    k_qr_apply<T, true><<<dim3(nchunks, groups), QR_NT, bytes, st>>>(m, n, mc, vws, tau, bin, ldb, nq, qout, ldq);
  } else {
    const size_t vb = (size_t)2 * mc * sizeof(cx<T>);
    smem_optin(k_qr_apply<T, false>);
    k_qr_apply<T, false><<<nchunks, QR_NT, vb, st>>>(m, n, mc, vws, tau, bin, ldb, nq, qout, ldq);
  }
  count_launch();
}

template void qr_factor_chunks<float>(cudaStream_t, int, int, int, int, const View<float> &, cx<float> *,
                                      cx<float> *, cx<float> *, int);
template void qr_factor_chunks<double>(cudaStream_t, int, int, int, int, const View<double> &, cx<double> *,
                                       cx<double> *, cx<double> *, int);
template void qr_apply_chunks<float>(cudaStream_t, int, int, int, int, const cx<float> *, const cx<float> *,
                                     const cx<float> *, int64_t, int, cx<float> *, int64_t);
template void qr_apply_chunks<double>(cudaStream_t, int, int, int, int, const cx<double> *,
                                      const cx<double> *, const cx<double> *, int64_t, int, cx<double> *,
                                      int64_t);

}  // namespace mpdo
