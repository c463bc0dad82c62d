// Hermitian eigensolver for the Gram matrix of a wide bond.
//
// A wide pair bond (Mr rows, 113 < Mr <= 512) needs the leading kr
// eigenvectors of G = Y Y^H (Mr x Mr).  Instead of sweeping Jacobi rotations
// over G, the matrix is reduced to real symmetric tridiagonal form by
// Householder reflections (as LAPACK's zhetd2: T = Q^H G Q), the top kr
// eigenpairs of T are found by bisection and inverse iteration, and the
// eigenvectors are brought back with the reflectors (U = Q Z, by the
// explicit-Q kernel of kernels_qr.cu).  The caller re-orthonormalises U and
// refines it by a Rayleigh-Ritz step on Y, exactly as after the Jacobi path.
//
// The reduction runs on one thread-block cluster: CTA r holds columns
// [32 r, 32 r + 32) of G in shared memory, the owner of column k forms
// reflector k, and the matrix-vector product and the rank-2 update are split
// by columns, partial products being summed across the cluster through
// distributed shared memory.  Three cluster barriers per column.
#include "kernels.cuh"

#include <cfloat>
#include <cooperative_groups.h>

namespace cg = cooperative_groups;

namespace mpdo {

namespace {
constexpr int EIG_NT = 512;
constexpr int EIG_NC = 32;   // columns per CTA

template <typename T> struct EigEps;
template <> struct EigEps<float> { static constexpr float eps = FLT_EPSILON; static constexpr float tiny = FLT_MIN; };
template <> struct EigEps<double> { static constexpr double eps = DBL_EPSILON; static constexpr double tiny = DBL_MIN; };

template <typename T>
__device__ __forceinline__ T e_wsum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T e_wmax(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// block-wide sum / max (all threads of the CTA call it; red holds >= 33)
template <typename T>
__device__ T e_bsum(T v, T *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = e_wsum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    T s = lane < nw ? red[lane] : T(0);
    s = e_wsum(s);
    if (lane == 0) red[32] = s;
  }
  __syncthreads();
  return red[32];
}
template <typename T>
__device__ T e_bmax(T v, T *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = e_wmax(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    T s = lane < nw ? red[lane] : T(0);
    s = e_wmax(s);
    if (lane == 0) red[32] = s;
  }
  __syncthreads();
  return red[32];
}

// G: n x n Hermitian, column-major (ld n), global.  Outputs: d[n], e[n-1]
// (T = Q^H G Q, real), the reflectors of Q as an (n-1) x (n-1) column-major
// block (reflector k in column k, rows k.. relative to row 1 of G, unit
// leading entry implied) and their tau.
template <typename T>
__global__ void __launch_bounds__(EIG_NT) k_hetrd(int n, const cx<T> *G, T *d_out, T *e_out, cx<T> *vref,
                                                  cx<T> *tau_out) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int csz = (int)cl.num_blocks();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T> *Gs = reinterpret_cast<cx<T> *>(smem_raw);   // n x EIG_NC, column-major
  cx<T> *vloc = Gs + (size_t)n * EIG_NC;            // reflector (absolute rows)
  cx<T> *xpart = vloc + n;                          // this CTA's part of G v
  cx<T> *wful = xpart + n;                          // w (absolute rows)
  __shared__ cx<T> sc[2];                           // tau, scl of the current reflector
  __shared__ T red[33];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int c0 = rank * EIG_NC;
  const int ncl = max(0, min(EIG_NC, n - c0));
  for (int64_t idx = tid; idx < (int64_t)n * ncl; idx += nt) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    Gs[(size_t)j * n + i] = G[(size_t)(c0 + j) * n + i];
  }
  __syncthreads();
  const int m1 = n - 1;
  for (int k = 0; k < n - 1; ++k) {
    const int owner = k / EIG_NC;
    // ---- reflector k from column k below the subdiagonal (zlarfg convention)
    if (rank == owner) {
      const cx<T> *col = Gs + (size_t)(k - c0) * n;
      T pmax = T(0);
      for (int i = k + 2 + tid; i < n; i += nt) pmax = fmax(pmax, fmax(fabs(col[i].x), fabs(col[i].y)));
      T amax = e_bmax(pmax, red);
      const bool debris = amax < EigEps<T>::tiny;
      T part = T(0);
      if (!debris) {
        const T inv = T(1) / amax;
        for (int i = k + 2 + tid; i < n; i += nt) part += cabs2<T>(cscale<T>(col[i], inv));
      }
      const T xs = e_bsum(part, red);
      if (tid == 0) {
        const cx<T> al = col[k + 1];
        cx<T> tau = czero<T>(), scl = czero<T>();
        T sub = al.x;
        const T xnorm = debris ? T(0) : amax * sqrt(xs);
        const T nrm = hypot(hypot(al.x, al.y), xnorm);
        if (!(xnorm == T(0) && al.y == T(0)) && nrm >= EigEps<T>::tiny) {
          const T beta = (al.x >= T(0)) ? -nrm : nrm;
          tau = cmk<T>((beta - al.x) / beta, -al.y / beta);
          const cx<T> dd = cmk<T>(al.x - beta, al.y);
          const T s = fmax(fabs(dd.x), fabs(dd.y));
          const cx<T> ds = cmk<T>(dd.x / s, dd.y / s);
          const T q = cabs2<T>(ds);
          scl = cmk<T>(ds.x / (q * s), -ds.y / (q * s));
          sub = beta;
        }
        sc[0] = tau;
        sc[1] = (debris || (tau.x == T(0) && tau.y == T(0))) ? czero<T>() : scl;
        d_out[k] = col[k].x;
        e_out[k] = sub;
        tau_out[k] = tau;
      }
      __syncthreads();
      const cx<T> s1 = sc[1];
      for (int i = k + 1 + tid; i < n; i += nt) {
        const cx<T> v = (i == k + 1) ? cmk<T>(T(1), T(0)) : cmul<T>(col[i], s1);
        vloc[i] = v;
        vref[(size_t)k * m1 + (i - 1)] = v;
      }
    }
    cl.sync();
    // ---- every CTA: the reflector
    cx<T> tau;
    if (rank == owner) {
      tau = sc[0];
    } else {
      const cx<T> *ov = cl.map_shared_rank(vloc, owner);
      for (int i = k + 1 + tid; i < n; i += nt) vloc[i] = ov[i];
      tau = *cl.map_shared_rank(&sc[0], owner);
    }
    const bool ident = tau.x == T(0) && tau.y == T(0);
    __syncthreads();
    // ---- x = A v over this CTA's columns (A = G[k+1:, k+1:])
    const int jlo = max(k + 1, c0) - c0;
    if (!ident)
      for (int i = k + 1 + tid; i < n; i += nt) {
        cx<T> acc = czero<T>();
        for (int j = jlo; j < ncl; ++j) acc = cadd<T>(acc, cmul<T>(Gs[(size_t)j * n + i], vloc[c0 + j]));
        xpart[i] = acc;
      }
    cl.sync();
    // ---- full x, s = v^H x (real), w = tau x - (|tau|^2 s / 2) v
    T sp = T(0);
    if (!ident)
      for (int i = k + 1 + tid; i < n; i += nt) {
        cx<T> acc = czero<T>();
        for (int r = 0; r < csz; ++r) acc = cadd<T>(acc, cl.map_shared_rank(xpart, r)[i]);
        wful[i] = acc;
        const cx<T> v = vloc[i];
        sp += v.x * acc.x + v.y * acc.y;
      }
    const T s = e_bsum(sp, red);
    if (!ident) {
      const T h = T(0.5) * cabs2<T>(tau) * s;
      for (int i = k + 1 + tid; i < n; i += nt) {
        const cx<T> x = wful[i], v = vloc[i];
        const cx<T> tx = cmul<T>(tau, x);
        wful[i] = cmk<T>(tx.x - h * v.x, tx.y - h * v.y);
      }
    }
    __syncthreads();
    // ---- A -= v w^H + w v^H on this CTA's columns
    if (!ident) {
      const int nj = ncl - jlo, ni = n - (k + 1);
      for (int64_t idx = tid; idx < (int64_t)nj * ni; idx += nt) {
        const int i = k + 1 + (int)(idx % ni), j = jlo + (int)(idx / ni);
        const int ja = c0 + j;
        const cx<T> vi = vloc[i], wi = wful[i], vj = vloc[ja], wj = wful[ja];
        cx<T> &a = Gs[(size_t)j * n + i];
        // v_i conj(w_j) + w_i conj(v_j)
        const cx<T> t1 = cmk<T>(vi.x * wj.x + vi.y * wj.y, vi.y * wj.x - vi.x * wj.y);
        const cx<T> t2 = cmk<T>(wi.x * vj.x + wi.y * vj.y, wi.y * vj.x - wi.x * vj.y);
        a = cmk<T>(a.x - t1.x - t2.x, a.y - t1.y - t2.y);
      }
    }
    __syncthreads();
    cl.sync();
  }
  if (n >= 1 && rank == (n - 1) / EIG_NC && tid == 0) d_out[n - 1] = Gs[(size_t)(n - 1 - c0) * n + (n - 1)].x;
  cl.sync();
}

// Number of eigenvalues of the symmetric tridiagonal (d, e) below x.
template <typename T>
__device__ int sturm_count(int n, const T *d, const T *e, T x, T pivmin) {
  int cnt = 0;
  T q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < T(0)) ++cnt;
  for (int i = 1; i < n; ++i) {
    q = d[i] - x - e[i - 1] * e[i - 1] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < T(0)) ++cnt;
  }
  return cnt;
}

// Top kr eigenpairs of the symmetric tridiagonal (d, e): thread t finds the
// t-th largest eigenvalue by bisection on the Sturm count and its vector by
// inverse iteration (three solves with L D L^T of T - lambda I, tiny pivots
// replaced), written as column t of Z (n x kr, row-major, complex with zero
// imaginary part).  work: 2 n scalars per thread.  tail_out: the trace of T
// minus the sum of the kr eigenvalues (the energy of the rest of the
// spectrum), clamped at zero.
template <typename T>
__global__ void k_tridiag_top(int n, const T *d, const T *e, int kr, T *lam_out, cx<T> *Z, T *work, T *tail_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ T red[33];
  T tnorm = T(0), lo = T(0), hi = T(0);
  for (int i = 0; i < n; ++i) {
    const T r = (i > 0 ? fabs(e[i - 1]) : T(0)) + (i < n - 1 ? fabs(e[i]) : T(0));
    lo = (i == 0) ? d[i] - r : fmin(lo, d[i] - r);
    hi = (i == 0) ? d[i] + r : fmax(hi, d[i] + r);
    tnorm = fmax(tnorm, fabs(d[i]) + r);
  }
  const T pivmin = fmax(EigEps<T>::tiny, tnorm * EigEps<T>::eps * EigEps<T>::eps);
  T lam = T(0);
  if (t < kr) {
    const int idx = n - 1 - t;   // ascending index of the t-th largest
    T a = lo - tnorm * EigEps<T>::eps - pivmin, b = hi + tnorm * EigEps<T>::eps + pivmin;
    for (int it = 0; it < 200; ++it) {
      const T mid = T(0.5) * (a + b);
      if (b - a <= T(2) * EigEps<T>::eps * fmax(fabs(a), fabs(b)) + pivmin || mid == a || mid == b) break;
      if (sturm_count(n, d, e, mid, pivmin) > idx) b = mid;
      else a = mid;
    }
    lam = T(0.5) * (a + b);
    lam_out[t] = lam;
    // inverse iteration
    T *q = work + (size_t)t * 2 * n, *y = q + n;
    const T guard = fmax(pivmin, tnorm * EigEps<T>::eps);
    T qq = d[0] - lam;
    if (fabs(qq) < guard) qq = qq < T(0) ? -guard : guard;
    q[0] = qq;
    for (int i = 1; i < n; ++i) {
      qq = d[i] - lam - e[i - 1] * e[i - 1] / q[i - 1];
      if (fabs(qq) < guard) qq = qq < T(0) ? -guard : guard;
      q[i] = qq;
    }
    // deterministic start vector (distinct per eigenvalue)
    uint32_t h = 2166136261u ^ (uint32_t)(t * 16777619u);
    for (int i = 0; i < n; ++i) {
      h = h * 1664525u + 1013904223u;
      y[i] = T(0.5) + T((h >> 8) & 0xffff) / T(65536);
    }
    if (!(tnorm > T(0)))        // zero matrix: any orthonormal set will do
      for (int i = 0; i < n; ++i) y[i] = (i == t) ? T(1) : T(0);
    for (int pass = 0; pass < 3 && tnorm > T(0); ++pass) {
      // L D L^T x = y: L unit lower bidiagonal with l_i = e_i / q_i
      for (int i = 1; i < n; ++i) y[i] -= (e[i - 1] / q[i - 1]) * y[i - 1];
      for (int i = 0; i < n; ++i) y[i] /= q[i];
      for (int i = n - 2; i >= 0; --i) y[i] -= (e[i] / q[i]) * y[i + 1];
      T mx = T(0);
      for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(y[i]));
      const T inv = mx > T(0) ? T(1) / mx : T(1);
      for (int i = 0; i < n; ++i) y[i] *= inv;
    }
    T s2 = T(0);
    for (int i = 0; i < n; ++i) s2 += y[i] * y[i];
    const T inv = s2 > T(0) ? T(1) / sqrt(s2) : T(0);
    for (int i = 0; i < n; ++i) Z[(size_t)i * kr + t] = cmk<T>(y[i] * inv, T(0));
  }
  if (gridDim.x == 1) {
    const T tot = e_bsum(t < kr ? lam : T(0), red);
    if (threadIdx.x == 0) {
      T tr = T(0);
      for (int i = 0; i < n; ++i) tr += d[i];
      *tail_out = fmax(tr - tot, T(0));
    }
  }
}
}  // namespace

template <typename T>
bool hetrd_cluster_fits(int n) {
  if (n < 2 || n > 16 * EIG_NC) return false;
  const size_t bytes = ((size_t)n * EIG_NC + 3 * (size_t)n) * sizeof(cx<T>);
  return bytes <= 200 * 1024;
}

template <typename T>
cudaError_t hetrd_cluster(cudaStream_t st, int n, const cx<T> *G, T *d, T *e, cx<T> *vref, cx<T> *tau) {
  const int csz = (n + EIG_NC - 1) / EIG_NC;
  const size_t bytes = ((size_t)n * EIG_NC + 3 * (size_t)n) * sizeof(cx<T>);
  smem_optin(k_hetrd<T>);
  // cluster sizes above 8 need the non-portable opt-in, which CUDA keeps per
  // device: set once per (kernel, device), like the shared-memory ceiling
  {
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    std::lock_guard<std::mutex> lk(mu);
    if (!done.count(dev)) {
      err = cudaFuncSetAttribute(k_hetrd<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if (err != cudaSuccess) return err;
      done.insert(dev);
    }
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(csz, 1, 1);
  cfg.blockDim = dim3(EIG_NT, 1, 1);
  cfg.dynamicSmemBytes = bytes;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csz;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t err = cudaLaunchKernelEx(&cfg, k_hetrd<T>, n, G, d, e, vref, tau);
  if (err != cudaSuccess) {
    cudaGetLastError();          // not placed: the caller falls back, nothing ran
    return err;
  }
  count_launch();
  return err;
}

template <typename T>
void tridiag_top(cudaStream_t st, int n, const T *d, const T *e, int kr, T *lam, cx<T> *Z, T *work, T *tail) {
  const int threads = ((kr + 31) / 32) * 32;
  k_tridiag_top<T><<<1, threads, 0, st>>>(n, d, e, kr, lam, Z, work, tail);
  count_launch();
}

#define INST_EIG(T)                                                                                              \
  template bool hetrd_cluster_fits<T>(int);                                                                      \
  template cudaError_t hetrd_cluster<T>(cudaStream_t, int, const cx<T> *, T *, T *, cx<T> *, cx<T> *);            \
  template void tridiag_top<T>(cudaStream_t, int, const T *, const T *, int, T *, cx<T> *, T *, T *);
INST_EIG(float)
INST_EIG(double)

}  // namespace mpdo
