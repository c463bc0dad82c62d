// One-sided (Hestenes) Jacobi SVD, one CTA per matrix.
//
// Columns are orthogonalised pairwise with complex Jacobi rotations (Golub &
// Van Loan, sec. 8.5 symmetric Schur step applied to the 2x2 Gram block
// [[alpha, gamma], [conj(gamma), beta]] after removing gamma's phase).  Pairs
// follow the round-robin (circle) ordering so that every round holds n/2
// disjoint pairs, one warp per pair.  The sweep count is bounded; the status
// word reports non-convergence or non-finite input instead of spinning.
// The matrix lives in shared memory when it fits, otherwise in its global
// workspace slot (L2 resident).
#include "kernels.cuh"

#include <algorithm>
#include <cfloat>

namespace mpdo {

namespace {
constexpr int JT = 1024;
constexpr size_t SMEM_CAP = 200 * 1024;

template <typename T>
__device__ __forceinline__ T wsum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T> struct Eps;
template <> struct Eps<float> { static constexpr float v = FLT_EPSILON; static constexpr float tiny = 1e-30f; };
template <> struct Eps<double> { static constexpr double v = DBL_EPSILON; static constexpr double tiny = 1e-290; };

template <typename T, bool SMEM>
__global__ void __launch_bounds__(JT) k_jacobi(int m, int n, View<T> in, cx<T> *uout, T *sigma, cx<T> *wout,
                                               cx<T> *xws, cx<T> *wws, int max_sweeps, T tol, int *status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int rot_count;
  __shared__ int bad;
  const int b = blockIdx.x;
  const bool wantW = (wout != nullptr);
  cx<T> *X = SMEM ? reinterpret_cast<cx<T> *>(smem_raw) : xws + (int64_t)b * m * n;
  cx<T> *W = wantW ? (SMEM ? X + (int64_t)m * n : wws + (int64_t)b * n * n) : nullptr;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;

  if (tid == 0) bad = 0;
  for (int64_t idx = tid; idx < (int64_t)m * n; idx += blockDim.x) {
    const int i = (int)(idx % m), j = (int)(idx / m);
    cx<T> v = view_ld(in, b, i, j);
    if (!isfinite(v.x) || !isfinite(v.y)) bad = 1;
    X[(int64_t)j * m + i] = v;
  }
  if (wantW)
    for (int64_t idx = tid; idx < (int64_t)n * n; idx += blockDim.x) {
      const int i = (int)(idx % n), j = (int)(idx / n);
      W[idx] = (i == j) ? cmk<T>(T(1), T(0)) : czero<T>();
    }
  __syncthreads();

  __shared__ T nrm[1024];
  const int ne = n + (n & 1);
  const int npairs = ne / 2;
  int sweep = 0;
  bool converged = (n < 2) || bad;
  __shared__ T colmax;
  const T floor_rel = T(16) * T(n) * Eps<T>::v * Eps<T>::v;
  for (; sweep < max_sweeps && !converged; ++sweep) {
    // noise floor: columns whose squared norm is below floor_rel * max_j |x_j|^2
    // are at rounding level; rotating them cannot converge and is skipped
    if (tid == 0) rot_count = 0;
    for (int j = warp; j < n; j += nw) {
      T sq = T(0);
      for (int i = lane; i < m; i += 32) sq += cabs2<T>(X[(int64_t)j * m + i]);
      sq = wsum(sq);
      if (lane == 0) nrm[j] = sq;
    }
    __syncthreads();
    if (warp == 0) {
      T mx = T(0);
      for (int j = lane; j < n; j += 32) mx = fmax(mx, nrm[j]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (lane == 0) colmax = mx;
    }
    __syncthreads();
    const T floor_abs = colmax * floor_rel;
    for (int r = 0; r < ne - 1; ++r) {
      for (int p = warp; p < npairs; p += nw) {
        int a, c;
        if (p == 0) { a = ne - 1; c = r; }
        else { a = (r + p) % (ne - 1); c = (r - p + ne - 1) % (ne - 1); }
        if (a >= n || c >= n) continue;
        const int pc = min(a, c), qc = max(a, c);
        cx<T> *xp = X + (int64_t)pc * m, *xq = X + (int64_t)qc * m;
        T al = T(0), be = T(0);
        cx<T> ga = czero<T>();
        for (int i = lane; i < m; i += 32) {
          const cx<T> u = xp[i], v = xq[i];
          al += cabs2<T>(u);
          be += cabs2<T>(v);
          cfmac<T>(ga, u, v);
        }
        al = wsum(al); be = wsum(be); ga.x = wsum(ga.x); ga.y = wsum(ga.y);
        const T g = sqrt(cabs2<T>(ga));
        if (!(g > tol * sqrt(al * be)) || al <= floor_abs || be <= floor_abs || al <= Eps<T>::tiny ||
            be <= Eps<T>::tiny || g <= Eps<T>::tiny)
          continue;
        const T zeta = (be - al) / (T(2) * g);
        const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
        const T cs = T(1) / sqrt(T(1) + t * t);
        const T sn = cs * t;
        // e = gamma/|gamma|; x_p' = c x_p - s conj(e) x_q ; x_q' = s x_p + c conj(e) x_q
        const cx<T> ec = cmk<T>(ga.x / g, -ga.y / g);
        const cx<T> sec = cscale<T>(ec, sn), cec = cscale<T>(ec, cs);
        for (int i = lane; i < m; i += 32) {
          const cx<T> u = xp[i], v = xq[i];
          const cx<T> ev_s = cmul<T>(sec, v), ev_c = cmul<T>(cec, v);
          xp[i] = cmk<T>(cs * u.x - ev_s.x, cs * u.y - ev_s.y);
          xq[i] = cmk<T>(sn * u.x + ev_c.x, sn * u.y + ev_c.y);
        }
        if (wantW) {
          cx<T> *wp = W + (int64_t)pc * n, *wq = W + (int64_t)qc * n;
          for (int i = lane; i < n; i += 32) {
            const cx<T> u = wp[i], v = wq[i];
            const cx<T> ev_s = cmul<T>(sec, v), ev_c = cmul<T>(cec, v);
            wp[i] = cmk<T>(cs * u.x - ev_s.x, cs * u.y - ev_s.y);
            wq[i] = cmk<T>(sn * u.x + ev_c.x, sn * u.y + ev_c.y);
          }
        }
        if (lane == 0) atomicAdd(&rot_count, 1);
      }
      __syncthreads();
    }
    converged = (rot_count == 0);
    __syncthreads();
  }

  // column norms
  for (int j = warp; j < n; j += nw) {
    T s = T(0);
    for (int i = lane; i < m; i += 32) s += cabs2<T>(X[(int64_t)j * m + i]);
    s = wsum(s);
    if (lane == 0) nrm[j] = sqrt(s);
  }
  __syncthreads();
  // rank by descending norm (ties by index), then scatter
  for (int j = warp; j < n; j += nw) {
    const T sj = nrm[j];
    int rank = 0;
    for (int i = lane; i < n; i += 32) {
      const T si = nrm[i];
      rank += (si > sj || (si == sj && i < j)) ? 1 : 0;
    }
    rank = (int)wsum((T)rank);
    const T inv = (sj > T(0)) ? T(1) / sj : T(0);
    cx<T> *uo = uout + (int64_t)b * m * n + (int64_t)rank * m;
    for (int i = lane; i < m; i += 32) uo[i] = cscale<T>(X[(int64_t)j * m + i], inv);
    if (wantW) {
      cx<T> *wo = wout + (int64_t)b * n * n + (int64_t)rank * n;
      for (int i = lane; i < n; i += 32) wo[i] = W[(int64_t)j * n + i];
    }
    if (lane == 0) {
      sigma[(int64_t)b * n + rank] = sj;
      if (!isfinite(sj)) bad = 1;
    }
  }
  __syncthreads();
  if (tid == 0 && status) status[b] = bad ? DEV_NONFINITE : (converged ? DEV_OK : DEV_NOT_CONVERGED);
}
}  // namespace

template <typename T>
void jacobi_svd(cudaStream_t st, int batch, int m, int n, const View<T> &in, cx<T> *uout, T *sigma, cx<T> *wout,
                cx<T> *xws, cx<T> *wws, int max_sweeps, int *status) {
  if (batch <= 0 || n <= 0) return;
  const T tol = T(4) * sqrt(T(std::max(m, 1))) * Eps<T>::v;
  if (n > 1024) return;  // callers never ask for more columns
  size_t bytes = ((size_t)m * n + (wout ? (size_t)n * n : 0)) * sizeof(cx<T>);
  if (bytes <= SMEM_CAP) {
    cudaFuncSetAttribute(k_jacobi<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    k_jacobi<T, true><<<batch, JT, bytes, st>>>(m, n, in, uout, sigma, wout, xws, wws, max_sweeps, tol, status);
  } else {
    k_jacobi<T, false><<<batch, JT, 0, st>>>(m, n, in, uout, sigma, wout, xws, wws, max_sweeps, tol, status);
  }
  count_launch();
}

template void jacobi_svd<float>(cudaStream_t, int, int, int, const View<float> &, cx<float> *, float *,
                                cx<float> *, cx<float> *, cx<float> *, int, int *);
template void jacobi_svd<double>(cudaStream_t, int, int, int, const View<double> &, cx<double> *, double *,
                                 cx<double> *, cx<double> *, cx<double> *, int, int *);

}  // namespace mpdo
