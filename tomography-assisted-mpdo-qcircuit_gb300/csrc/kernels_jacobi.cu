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
#include <cooperative_groups.h>
#include <mutex>
#include <set>
#include <tuple>

namespace cg = cooperative_groups;

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

// One Hestenes rotation of the column pair (xp, xq) (m entries each) by one
// warp, given their squared norms.  Returns false when the pair is already
// orthogonal to tolerance (or at the rounding floor); otherwise rotates and
// gives t and |g| for the norm update (alpha' = alpha - t|g|,
// beta' = beta + t|g|) and the rotation (cs, sec, cec) for accumulating W.
// With m <= 32 * RMAX the columns stay in registers between the inner
// product and the rotation (one shared-memory read of each entry).
template <typename T, int RMAX>
__device__ __forceinline__ bool hestenes_pair(cx<T> *xp, cx<T> *xq, int m, int lane, T al, T be, T tol,
                                              T floor_abs, T &t, T &g, T &cs, T &sn, cx<T> &sec, cx<T> &cec) {
  const bool cached = m <= 32 * RMAX;
  cx<T> up[RMAX], vq[RMAX];
  cx<T> ga = czero<T>();
  if (cached) {
#pragma unroll
    for (int r = 0; r < RMAX; ++r) {
      const int i = lane + 32 * r;
      if (i < m) {
        up[r] = xp[i];
        vq[r] = xq[i];
        cfmac<T>(ga, up[r], vq[r]);
      }
    }
  } else {
    for (int i = lane; i < m; i += 32) cfmac<T>(ga, xp[i], xq[i]);
  }
  ga.x = wsum(ga.x); ga.y = wsum(ga.y);
  g = sqrt(cabs2<T>(ga));
  if (!(g > tol * sqrt(al * be)) || al <= floor_abs || be <= floor_abs || al <= Eps<T>::tiny ||
      be <= Eps<T>::tiny || g <= Eps<T>::tiny)
    return false;
  const T zeta = (be - al) / (T(2) * g);
  t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
  cs = T(1) / sqrt(T(1) + t * t);
  sn = cs * t;
  // e = gamma/|gamma|; x_p' = c x_p - s conj(e) x_q ; x_q' = s x_p + c conj(e) x_q
  const cx<T> ec = cmk<T>(ga.x / g, -ga.y / g);
  sec = cscale<T>(ec, sn);
  cec = cscale<T>(ec, cs);
  if (cached) {
#pragma unroll
    for (int r = 0; r < RMAX; ++r) {
      const int i = lane + 32 * r;
      if (i < m) {
        const cx<T> u = up[r], v = vq[r];
        const cx<T> ev_s = cmul<T>(sec, v), ev_c = cmul<T>(cec, v);
        xp[i] = cmk<T>(cs * u.x - ev_s.x, cs * u.y - ev_s.y);
        xq[i] = cmk<T>(sn * u.x + ev_c.x, sn * u.y + ev_c.y);
      }
    }
  } else {
    __syncwarp();
    for (int i = lane; i < m; i += 32) {
      const cx<T> u = xp[i], v = xq[i];
      const cx<T> ev_s = cmul<T>(sec, v), ev_c = cmul<T>(cec, v);
      xp[i] = cmk<T>(cs * u.x - ev_s.x, cs * u.y - ev_s.y);
      xq[i] = cmk<T>(sn * u.x + ev_c.x, sn * u.y + ev_c.y);
    }
  }
  return true;
}

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
  // max_sweeps == 0: the caller only wants the columns normalised and sorted
  bool converged = (n < 2) || bad || max_sweeps == 0;
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
        // squared norms carried from the sweep start through the rotations
        const T al = nrm[pc], be = nrm[qc];
        T t, g, cs, sn;
        cx<T> sec, cec;
        if (!hestenes_pair<T, sizeof(T) == 4 ? 4 : 2>(xp, xq, m, lane, al, be, tol, floor_abs, t, g, cs, sn, sec, cec)) continue;
        if (lane == 0) {
          nrm[pc] = fmax(al - t * g, T(0));
          nrm[qc] = be + t * g;
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

  // column norms.  A rotation whose 1 + t^2 rounds to 1 (single precision,
  // t^2 < eps) scales both of its columns by sqrt(1 + t^2), in X and in the
  // accumulated W alike (X W stays A W): with W accumulated, sigma_j =
  // |X_j| / |W_j| removes that growth from the singular values.
  for (int j = warp; j < n; j += nw) {
    T s = T(0);
    for (int i = lane; i < m; i += 32) s += cabs2<T>(X[(int64_t)j * m + i]);
    s = wsum(s);
    T g = T(1);
    if (wantW) {
      T w2 = T(0);
      for (int i = lane; i < n; i += 32) w2 += cabs2<T>(W[(int64_t)j * n + i]);
      w2 = wsum(w2);
      if (w2 > T(0)) g = sqrt(w2);
    }
    if (lane == 0) nrm[j] = sqrt(s) / g;
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
    // U_j = X_j / |X_j| (from the column itself, whatever the sigma correction)
    T xs = T(0);
    for (int i = lane; i < m; i += 32) xs += cabs2<T>(X[(int64_t)j * m + i]);
    xs = wsum(xs);
    const T inv = (xs > T(0) && sj > T(0)) ? T(1) / sqrt(xs) : T(0);
    cx<T> *uo = uout + (int64_t)b * m * n + (int64_t)rank * m;
    for (int i = lane; i < m; i += 32) uo[i] = cscale<T>(X[(int64_t)j * m + i], inv);
    if (wantW) {
      // the accumulated rotations leave each column's norm off 1 by the
      // rounding of every rotation applied to it (in single precision a
      // bias of ~2e-7 per kappa pass that the site norms would inherit):
      // the columns are written unit-normalised
      T wn = T(0);
      for (int i = lane; i < n; i += 32) wn += cabs2<T>(W[(int64_t)j * n + i]);
      wn = wsum(wn);
      const T winv = wn > T(0) ? T(1) / sqrt(wn) : T(0);
      cx<T> *wo = wout + (int64_t)b * n * n + (int64_t)rank * n;
      for (int i = lane; i < n; i += 32) wo[i] = cscale<T>(W[(int64_t)j * n + i], winv);
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
    smem_optin(k_jacobi<T, true>);
    k_jacobi<T, true><<<batch, JT, bytes, st>>>(m, n, in, uout, sigma, wout, xws, wws, max_sweeps, tol, status);
  } else {
    k_jacobi<T, false><<<batch, JT, 0, st>>>(m, n, in, uout, sigma, wout, xws, wws, max_sweeps, tol, status);
  }
  count_launch();
}

namespace {
// ------------------------------------------------------ block Jacobi -----
// a complex load that bypasses L1 (data another SM wrote since this SM last
// read the line must come from L2)
template <typename T> __device__ __forceinline__ cx<T> ldcg_cx(const cx<T> *p) { return __ldcg(p); }

// The columns of X (m x n, column-major in global memory) are cut into blocks
// of bs columns (nblk blocks; an id >= nblk is an empty block).  An outer
// sweep visits every pair of blocks once in nb - 1 tournament rounds of nb / 2
// disjoint pairs (nb = nblk rounded up to even).  Pair p of round r is
// (a, c) = (nb - 1, r) for p = 0, else ((r + p) mod (nb - 1), (r - p) mod (nb - 1)).
__device__ __forceinline__ void bj_pair_of(int nb, int r, int p, int &a, int &c) {
  if (p == 0) { a = nb - 1; c = r; }
  else { a = (r + p) % (nb - 1); c = (r - p + nb - 1) % (nb - 1); }
}

// Orthogonalises the two blocks held in shared memory S (columns [0, w0) of
// the first block, [w0, w0 + w1) of the second; m rows, column-major) against
// each other with up to inner_sweeps one-sided Jacobi sweeps (no vector
// accumulation).  Every thread of the CTA calls it; the result (whether any
// rotation happened) is the same in all threads.  nrm2 holds >= w0 + w1
// entries of shared memory.
template <typename T>
__device__ __forceinline__ bool bj_pair_sweeps(cx<T> *S, int m, int w0, int w1, T tol, T floor_abs,
                                               int inner_sweeps, T *nrm2, int *rot_count) {
  const int nc = w0 + w1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int ne = nc + (nc & 1);
  const int npairs = ne / 2;
  bool any = false;
  // squared column norms, recomputed at the start of every inner sweep and
  // carried through rotations exactly as the 2 x 2 Gram's diagonal moves
  // (alpha' = alpha - t|g|, beta' = beta + t|g|), so a pair costs one
  // reduction (its inner product) instead of three
  auto rotate_pair = [&](int pc, int qc) -> bool {
    const T al = nrm2[pc], be = nrm2[qc];
    T t, g, cs, sn;
    cx<T> sec, cec;
    if (!hestenes_pair<T, sizeof(T) == 4 ? 8 : 4>(S + (int64_t)pc * m, S + (int64_t)qc * m, m, lane, al, be, tol, floor_abs, t, g, cs,
                              sn, sec, cec))
      return false;
    if (lane == 0) {
      nrm2[pc] = fmax(al - t * g, T(0));
      nrm2[qc] = be + t * g;
    }
    return true;
  };
  // after the first inner sweep (all pairs) only the pairs that straddle the
  // two blocks are revisited: bs steps of bs disjoint pairs
  const bool cross_only_ok = (w0 == w1) && w0 > 0;
  for (int sw = 0; sw < inner_sweeps && nc >= 2; ++sw) {
    if (tid == 0) *rot_count = 0;
    for (int j = warp; j < nc; j += nw) {
      T sq = T(0);
      for (int i = lane; i < m; i += 32) sq += cabs2<T>(S[(int64_t)j * m + i]);
      sq = wsum(sq);
      if (lane == 0) nrm2[j] = sq;
    }
    __syncthreads();
    if (sw == 0 || !cross_only_ok) {
      for (int r = 0; r < ne - 1; ++r) {
        for (int p = warp; p < npairs; p += nw) {
          int a, c;
          bj_pair_of(ne, r, p, a, c);
          if (a >= nc || c >= nc) continue;
          if (rotate_pair(min(a, c), max(a, c)) && lane == 0) atomicAdd(rot_count, 1);
        }
        __syncthreads();
      }
    } else {
      for (int st = 0; st < w0; ++st) {
        for (int i = warp; i < w0; i += nw)
          if (rotate_pair(i, w0 + (i + st) % w0) && lane == 0) atomicAdd(rot_count, 1);
        __syncthreads();
      }
    }
    const int rc = *rot_count;
    __syncthreads();
    if (rc == 0) break;
    any = true;
  }
  __syncthreads();
  return any;
}

// One tournament round of a one-sided block-Jacobi sweep.  CTA p loads the
// column blocks pairs[2p], pairs[2p+1] into shared memory, orthogonalises them
// against each other (bj_pair_sweeps), writes them back, and sets *flag when
// it rotated anything.  gmax2: the largest squared column norm, for the
// rounding-level floor.
template <typename T>
__global__ void __launch_bounds__(512) k_bjacobi(int m, int n, int bs, int nblk, cx<T> *X, const int *pairs,
                                                 T tol, const T *gmax2, int inner_sweeps, int *flag) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int rot_count;
  __shared__ T nrm2[64];
  cx<T> *S = reinterpret_cast<cx<T> *>(smem_raw);
  const int b0 = pairs[2 * blockIdx.x], b1 = pairs[2 * blockIdx.x + 1];
  const int c0 = b0 * bs, c1 = b1 * bs;
  const int w0 = (b0 < nblk) ? min(bs, n - c0) : 0;
  const int w1 = (b1 < nblk) ? min(bs, n - c1) : 0;
  const int nc = w0 + w1;
  const int tid = threadIdx.x;
  for (int64_t idx = tid; idx < (int64_t)m * nc; idx += blockDim.x) {
    const int i = (int)(idx % m), j = (int)(idx / m);
    const int col = j < w0 ? c0 + j : c1 + (j - w0);
    S[(int64_t)j * m + i] = X[(int64_t)col * m + i];
  }
  __syncthreads();
  const T floor_abs = (*gmax2) * T(16) * T(n) * Eps<T>::v * Eps<T>::v;
  const bool any_rot = bj_pair_sweeps<T>(S, m, w0, w1, tol, floor_abs, inner_sweeps, nrm2, &rot_count);
  for (int64_t idx = tid; idx < (int64_t)m * nc; idx += blockDim.x) {
    const int i = (int)(idx % m), j = (int)(idx / m);
    const int col = j < w0 ? c0 + j : c1 + (j - w0);
    X[(int64_t)col * m + i] = S[(int64_t)j * m + i];
  }
  if (tid == 0 && any_rot) atomicOr(flag, 1);
}

// The whole block-Jacobi iteration in one launch on one thread-block cluster
// of nb / 2 CTAs: CTA p takes pair p of every round (bj_pair_of), loads its two
// blocks from X, orthogonalises them and writes them back; a cluster barrier
// separates the rounds (the blocks a CTA loads were written by other CTAs of
// the cluster in the round before; loads bypass L1).  After each outer sweep
// every CTA reads the rotation flags of all CTAs of the cluster (distributed
// shared memory) and the cluster stops once a sweep rotated nothing, or after
// max_outer sweeps.  The arithmetic per round is k_bjacobi's, in the same
// order, so both paths give the same columns.  *sweeps_out (nullable): outer
// sweeps run.
template <typename T>
__global__ void __launch_bounds__(512) k_bjacobi_cl(int m, int n, int bs, int nblk, cx<T> *X, T tol,
                                                    const T *gmax2, int inner_sweeps, int max_outer,
                                                    int *sweeps_out) {
  cg::cluster_group cl = cg::this_cluster();
  const int p = (int)cl.block_rank();
  const int np = (int)cl.num_blocks();
  const int nb = 2 * np, rounds = nb - 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int rot_count;
  __shared__ T nrm2[64];
  // rotflag[s & 1]: this CTA rotated something in outer sweep s.  Cleared for
  // sweep s + 1 after the first barrier of sweep s, when every CTA has read
  // the flags of sweep s - 1 (same slot)
  __shared__ int rotflag[2];
  cx<T> *S = reinterpret_cast<cx<T> *>(smem_raw);
  const int tid = threadIdx.x;
  if (tid == 0) rotflag[0] = rotflag[1] = 0;
  const T floor_abs = (*gmax2) * T(16) * T(n) * Eps<T>::v * Eps<T>::v;
  cl.sync();
  int outer = 0;
  while (outer < max_outer) {
    for (int r = 0; r < rounds; ++r) {
      int b0, b1;
      bj_pair_of(nb, r, p, b0, b1);
      const int c0 = b0 * bs, c1 = b1 * bs;
      const int w0 = (b0 < nblk) ? min(bs, n - c0) : 0;
      const int w1 = (b1 < nblk) ? min(bs, n - c1) : 0;
      const int nc = w0 + w1;
      for (int64_t idx = tid; idx < (int64_t)m * nc; idx += blockDim.x) {
        const int i = (int)(idx % m), j = (int)(idx / m);
        const int col = j < w0 ? c0 + j : c1 + (j - w0);
        S[(int64_t)j * m + i] = ldcg_cx<T>(X + (int64_t)col * m + i);
      }
      __syncthreads();
      const bool any = bj_pair_sweeps<T>(S, m, w0, w1, tol, floor_abs, inner_sweeps, nrm2, &rot_count);
      for (int64_t idx = tid; idx < (int64_t)m * nc; idx += blockDim.x) {
        const int i = (int)(idx % m), j = (int)(idx / m);
        const int col = j < w0 ? c0 + j : c1 + (j - w0);
        X[(int64_t)col * m + i] = S[(int64_t)j * m + i];
      }
      if (tid == 0 && any) rotflag[outer & 1] = 1;
      __threadfence();
      cl.sync();
      if (r == 0 && tid == 0) rotflag[(outer + 1) & 1] = 0;
    }
    int v = 0;
    for (int q = 0; q < np; ++q) v |= *cl.map_shared_rank(&rotflag[outer & 1], q);
    ++outer;
    if (!v) break;
  }
  // no CTA leaves while another may still read its flags
  cl.sync();
  if (sweeps_out && p == 0 && tid == 0) *sweeps_out = outer;
}

template <typename T>
__global__ void k_colmax2(int m, int n, const cx<T> *X, T *out) {
  __shared__ T red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T mx = T(0);
  for (int j = warp; j < n; j += nw) {
    T s = T(0);
    for (int i = lane; i < m; i += 32) s += cabs2<T>(X[(int64_t)j * m + i]);
    s = wsum(s);
    mx = fmax(mx, s);
  }
  if (lane == 0) red[warp] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    T v = T(0);
    for (int w = 0; w < nw; ++w) v = fmax(v, red[w]);
    *out = v;
  }
}
}  // namespace

template <typename T>
void bjacobi_round(cudaStream_t st, int m, int n, int bs, int nblk, cx<T> *X, const int *pairs_round,
                   int npairs, const T *gmax2, int inner_sweeps, int *flag) {
  const T tol = T(4) * sqrt(T(std::max(m, 1))) * Eps<T>::v;
  const size_t bytes = (size_t)m * 2 * bs * sizeof(cx<T>);
  smem_optin(k_bjacobi<T>);
  k_bjacobi<T><<<npairs, 512, bytes, st>>>(m, n, bs, nblk, X, pairs_round, tol, gmax2, inner_sweeps, flag);
  count_launch();
}

template <typename T>
bool bjacobi_cluster_fits(int m, int n, int bs) {
  const int nblk = (n + bs - 1) / bs;
  const int np = (nblk + (nblk & 1)) / 2;
  return np >= 1 && np <= 16 && 2 * bs <= 64 && (size_t)m * 2 * bs * sizeof(cx<T>) <= SMEM_CAP;
}

template <typename T>
cudaError_t bjacobi_cluster(cudaStream_t st, int m, int n, int bs, int nblk, cx<T> *X, const T *gmax2,
                            int inner_sweeps, int max_outer, int *sweeps_out) {
  const T tol = T(4) * sqrt(T(std::max(m, 1))) * Eps<T>::v;
  const size_t bytes = (size_t)m * 2 * bs * sizeof(cx<T>);
  const int np = (nblk + (nblk & 1)) / 2;
  if (!bjacobi_cluster_fits<T>(m, n, bs)) return cudaErrorInvalidValue;
  smem_optin(k_bjacobi_cl<T>);
  // clusters above 8 CTAs need the non-portable opt-in, which CUDA keeps per
  // device: set once per (kernel, device)
  if (np > 8) {
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    std::lock_guard<std::mutex> lk(mu);
    if (!done.count(dev)) {
      err = cudaFuncSetAttribute(k_bjacobi_cl<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if (err != cudaSuccess) return err;
      done.insert(dev);
    }
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(np, 1, 1);
  cfg.blockDim = dim3(512, 1, 1);
  cfg.dynamicSmemBytes = bytes;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = np;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (np > 8) {
    // a non-portable cluster must fit one GPC of this device: ask once per
    // (device, cluster size, shared memory) and leave the per-round launches
    // to the caller when it does not
    static std::mutex mu;
    static std::set<std::tuple<int, int, size_t>> ok, refused;
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    const auto key = std::make_tuple(dev, np, bytes);
    std::lock_guard<std::mutex> lk(mu);
    if (refused.count(key)) return cudaErrorInvalidClusterSize;
    if (!ok.count(key)) {
      int nclusters = 0;
      err = cudaOccupancyMaxActiveClusters(&nclusters, k_bjacobi_cl<T>, &cfg);
      if (err != cudaSuccess || nclusters < 1) {
        cudaGetLastError();
        refused.insert(key);
        return cudaErrorInvalidClusterSize;
      }
      ok.insert(key);
    }
  }
  cudaError_t err = cudaLaunchKernelEx(&cfg, k_bjacobi_cl<T>, m, n, bs, nblk, X, tol, gmax2, inner_sweeps, max_outer,
                                       sweeps_out);
  if (err != cudaSuccess) {
    cudaGetLastError();          // not placed: the caller runs the per-round launches, nothing ran
    return err;
  }
  count_launch();
  return err;
}

template <typename T>
void colmax2(cudaStream_t st, int m, int n, const cx<T> *X, T *out) {
  k_colmax2<T><<<1, 1024, 0, st>>>(m, n, X, out);
  count_launch();
}

template void bjacobi_round<float>(cudaStream_t, int, int, int, int, cx<float> *, const int *, int, const float *,
                                   int, int *);
template void bjacobi_round<double>(cudaStream_t, int, int, int, int, cx<double> *, const int *, int,
                                    const double *, int, int *);
template bool bjacobi_cluster_fits<float>(int, int, int);
template bool bjacobi_cluster_fits<double>(int, int, int);
template cudaError_t bjacobi_cluster<float>(cudaStream_t, int, int, int, int, cx<float> *, const float *, int, int,
                                            int *);
template cudaError_t bjacobi_cluster<double>(cudaStream_t, int, int, int, int, cx<double> *, const double *, int,
                                             int, int *);
template void colmax2<float>(cudaStream_t, int, int, const cx<float> *, float *);
template void colmax2<double>(cudaStream_t, int, int, const cx<double> *, double *);

template void jacobi_svd<float>(cudaStream_t, int, int, int, const View<float> &, cx<float> *, float *,
                                cx<float> *, cx<float> *, cx<float> *, int, int *);
template void jacobi_svd<double>(cudaStream_t, int, int, int, const View<double> &, cx<double> *, double *,
                                 cx<double> *, cx<double> *, cx<double> *, int, int *);

}  // namespace mpdo
