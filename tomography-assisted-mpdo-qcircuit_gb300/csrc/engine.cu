// MPDO engine: chain state on the device, the hot-path operations and the
// C ABI declared in include/mpdo_gb300.h.
//
// Reference operations restated here (paths relative to the reference root):
//   Circuit.py:138-178  single-qubit (noisy) gate         -> apply_1q
//   Circuit.py:74-136   two-qubit gate + SVD split         -> apply_2q / materialize_pair
//   TNNOptimizer.py:87-108  qr_left2right                  -> qr_sweep
//   TNNOptimizer.py:111-134 svd_right2left                 -> svd_sweep
//   TNNOptimizer.py:164-197 svdKappa_left2right            -> kappa_pass
//   Circuit.py:226-295, dmOperations.py:135-201 readout    -> env_* / reduced_dm / expect
//
// Deferred two-qubit gates.  A 2q gate is recorded on its pair and applied
// lazily.  If the next operation touching the pair is a truncate() that runs,
// the gate is fused into the QR left-to-right sweep: the reference would split
// theta by an SVD (Circuit.py:116-126) and immediately re-orthogonalise the
// left factor by QR (TNNOptimizer.py:98-106), which leaves the state equal to
// theta up to the split's cutoff (tail weight below GLOBAL_MINIMUM-level).
// The fused step factors the left site directly by Householder QR and pushes
// the gate into the right site, so no SVD of theta is needed.  Any other
// operation on the pair (another gate, readout, a skipped truncate followed
// by readout) materialises the gate with the reference's SVD split and its
// cutoff rule.
#include "kernels.cuh"
#include "mpdo_gb300.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>

#include "engine_core.cuh"

namespace mpdo {

static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }

// ---------------------------------------------------------------- QR ----
// Rows per TSQR chunk of an m x n level: the whole level if it fits shared
// memory; else the largest multiple of 32 that fits (with the explicit-Q
// pass and its two reflector buffers) and exceeds n, so that every level
// shrinks the stacked R; and when no shared-memory chunk can exceed n (wide
// factors, n > ~100 in complex64), chunks of 2n rows factored in global
// memory (L2 resident), so that the level still splits across CTAs instead of
// one CTA sweeping all m rows.
static int tsqr_chunk_rows(int m, int n, size_t esz, size_t cap, double ratio) {
  if ((size_t)m * (n + 2) * esz <= cap) return m;
  size_t mcs = cap / ((size_t)(n + 2) * esz);
  mcs = mcs / 32 * 32;
  if (mcs > (size_t)n && (double)mcs >= ratio * n) return (int)std::min<size_t>(mcs, (size_t)m);
  const int g = ((int)std::ceil(std::max(ratio, 2.0) * n) + 31) / 32 * 32;
  return m > g ? g : m;
}

// Householder QR of an m x n matrix (view `in`): Q (m x k, row-major, ld k),
// R (k x n row-major), k = min(m, n).  Tall-skinny inputs go through TSQR
// levels of shared-memory-resident chunks.
template <typename T>
void qr(Engine &e, int m, int n, const View<T> &in, cx<T> *Q, cx<T> *R) {
  const size_t esz = sizeof(cx<T>);
  const size_t cap = 200 * 1024;
  struct Level {
    int m, mc, nch;
    DBuf<cx<T>> v, tau, rs;
  };
  std::vector<Level> lv;
  View<T> cur = in;
  int curm = m;
  while (true) {
    // chunk rows: the whole matrix if it fits in shared memory, else the
    // largest multiple of 32 that fits (with the explicit-Q pass and its two
    // reflector buffers) and exceeds
    // n, so that every level shrinks the stacked R; else one global chunk
    int mc = tsqr_chunk_rows(curm, n, esz, cap, e.tsqr_ratio);
    const int nch = (curm + mc - 1) / mc;
    Level L;
    L.m = curm; L.mc = mc; L.nch = nch;
    L.v = DBuf<cx<T>>(e, (size_t)nch * mc * n);
    L.tau = DBuf<cx<T>>(e, (size_t)nch * n);
    L.rs = DBuf<cx<T>>(e, (size_t)nch * n * n);
    {
      const double mm = (double)std::min(mc, curm), nn = n, kk = std::min(mm, nn);
      const double fl = nch * 4.0 * (2.0 * mm * nn * kk - (mm + nn) * kk * kk + 2.0 / 3.0 * kk * kk * kk);
      const double by = (double)sizeof(cx<T>) * ((double)curm * n + (double)nch * n * n);
      prof(e, K_QR_FACTOR, fl, by, [&] { qr_factor_chunks<T>(e.stream, curm, n, mc, nch, cur, L.v.p, L.tau.p, L.rs.p); });
    }
    lv.push_back(std::move(L));
    if (nch == 1) break;
    // compact stack: full chunks give n rows each, the last min(rows, n)
    cur = RM<T>(lv.back().rs.p, n);
    curm = (nch - 1) * n + std::min(n, curm - (nch - 1) * mc);
  }
  const int k = std::min(m, n);
  const Level &top = lv.back();
  const int ktop = std::min(top.m, n);
  if (ktop != k) fail(MPDO_ERR_BAD_SHAPE, "internal TSQR rank mismatch");
  MPDO_CUDA_CHECK(cudaMemcpyAsync(R, top.rs.p, (size_t)k * n * esz, cudaMemcpyDeviceToDevice, e.stream));
  if (Q == nullptr) return;
  // Q top-down
  DBuf<cx<T>> qa, qb;
  const cx<T> *bin = nullptr;
  for (int li = (int)lv.size() - 1; li >= 0; --li) {
    const Level &L = lv[li];
    cx<T> *out;
    if (li == 0) out = Q;
    else {
      DBuf<cx<T>> nb(e, (size_t)L.m * k);
      out = nb.p;
      if (li % 2) { qa = std::move(nb); } else { qb = std::move(nb); }
    }
    {
      const double mm = (double)std::min(L.mc, L.m), kk = std::min<double>(mm, n);
      const double fl = L.nch * 4.0 * (4.0 * mm * k * kk - 2.0 * k * kk * kk);
      const double by = (double)sizeof(cx<T>) * ((double)L.m * n + (double)L.m * k);
      prof(e, K_QR_APPLY, fl, by, [&] { qr_apply_chunks<T>(e.stream, L.m, n, L.mc, L.nch, L.v.p, L.tau.p, bin, k, k, out, k); });
    }
    bin = out;
  }
}

// ------------------------------------------------------------ SVD -----
// Right singular vectors of an m x n matrix given by a view: Householder QR
// (R is k x n, k = min(m, n)), then one-sided Jacobi on the columns of R with
// the rotations accumulated: R W = U diag(sigma).  W (n x n, column-major,
// columns sorted by sigma descending) is unitary to rounding whatever the
// rank; sigma has n entries (zeros beyond the rank).
// R factors of a batch of equally shaped m x n matrices (input b at in.bs*b):
// R (batch x k x n, row-major, k = min(m, n)), by the same TSQR levels as qr().
template <typename T>
void qr_r_batched(Engine &e, int batch, int m, int n, const View<T> &in, cx<T> *R) {
  const size_t esz = sizeof(cx<T>);
  const size_t cap = 200 * 1024;
  DBuf<cx<T>> v, tau, rs, rs_prev;
  View<T> cur = in;
  int curm = m, last_nch = 1;
  while (true) {
    int mc = tsqr_chunk_rows(curm, n, esz, cap, e.tsqr_ratio);
    const int nch = (curm + mc - 1) / mc;
    v = DBuf<cx<T>>(e, (size_t)batch * nch * mc * n);
    tau = DBuf<cx<T>>(e, (size_t)batch * nch * n);
    rs = DBuf<cx<T>>(e, (size_t)batch * nch * n * n);
    {
      const double mm = (double)std::min(mc, curm), nn = n, kk = std::min(mm, nn);
      const double fl = batch * nch * 4.0 * (2.0 * mm * nn * kk - (mm + nn) * kk * kk + 2.0 / 3.0 * kk * kk * kk);
      const double by = (double)esz * batch * ((double)curm * n + (double)nch * n * n);
      prof(e, K_QR_FACTOR, fl, by,
           [&] { qr_factor_chunks<T>(e.stream, curm, n, mc, nch, cur, v.p, tau.p, rs.p, batch); });
    }
    last_nch = nch;
    if (nch == 1) break;
    rs_prev = std::move(rs);
    cur = View<T>{rs_prev.p, (int64_t)nch * n * n, 1, n, 0, 1, 0};
    curm = (nch - 1) * n + std::min(n, curm - (nch - 1) * mc);
  }
  (void)last_nch;
  const int k = std::min(m, n);
  if (std::min(curm, n) != k) fail(MPDO_ERR_BAD_SHAPE, "internal TSQR rank mismatch");
  MPDO_CUDA_CHECK(cudaMemcpy2DAsync(R, (size_t)k * n * esz, rs.p, (size_t)n * n * esz, (size_t)k * n * esz, batch,
                                    cudaMemcpyDeviceToDevice, e.stream));
}

template <typename T>
void right_svd(Engine &e, int m, int n, const View<T> &in, DBuf<cx<T>> &W, DBuf<T> &sigma) {
  const int k = std::min(m, n);
  DBuf<cx<T>> R(e, (size_t)k * n);
  qr<T>(e, m, n, in, nullptr, R.p);
  W = DBuf<cx<T>>(e, (size_t)n * n);
  sigma = DBuf<T>(e, n);
  DBuf<cx<T>> U(e, (size_t)k * n), xws(e, (size_t)k * n), wws(e, (size_t)n * n);
  {
    // algorithmic count of a thin SVD of the k x n factor with vectors
    const double mm = std::max(k, n), nn = std::min(k, n);
    const double fl = 4.0 * (4.0 * mm * nn * nn + 22.0 * nn * nn * nn);
    const double by = (double)sizeof(cx<T>) * ((double)k * n * 2 + (double)n * n);
    int *slot = status_slot(e, 1);
    prof(e, K_JACOBI, fl, by, [&] {
      jacobi_svd<T>(e.stream, 1, k, n, RM<T>(R.p, n), U.p, sigma.p, W.p, xws.p, wws.p, e.max_sweeps, slot);
    });
  }
}

// --------------------------------------------------- wide-bond SVD ----
// One-sided block Jacobi on the columns of X (m x n, column-major, in place):
// tournament ordering over column blocks, one CTA per block pair per round,
// repeated until an outer sweep makes no rotation (at most 40 sweeps).  By
// default the whole iteration is one launch on a thread-block cluster that
// decides convergence on the device; where the cluster does not fit (more
// than 32 blocks, or the device refuses it) every round is its own launch and
// the host reads the rotation flag after each sweep.  Both give the same
// columns.
template <typename T>
static void block_jacobi(Engine &e, int m, int n, cx<T> *X) {
  const size_t esz = sizeof(cx<T>), cap = 200 * 1024;
  int bs = (int)std::min<size_t>(cap / (2 * (size_t)m * esz), 32);
  bs = e.bjacobi_bs > 0 ? std::max(4, std::min(bs, e.bjacobi_bs)) : std::max(4, std::min(bs, std::max(8, n / 16)));
  // a block pair (2 bs columns of m rows) lives in shared memory
  if (2 * (size_t)bs * m * esz > cap)
    fail(MPDO_ERR_INVALID, "a wide split of " + std::to_string(m) + " rows exceeds the block-Jacobi shared-memory "
                           "limit (" + std::to_string(cap / (8 * esz)) + " rows at this precision); truncate the "
                           "Kraus legs (kappa) or the bonds (chi) before the gate");
  const int nblk = (n + bs - 1) / bs;
  const int nb = nblk + (nblk & 1);
  const int rounds = nb - 1, np = nb / 2;
  constexpr int kMaxOuter = 40;
  DBuf<T> gmax(e, 1);
  colmax2<T>(e.stream, m, n, X, gmax.p);
  // algorithmic work: one thin SVD of the m x n matrix (4 (4 m n^2 + 22 n^3)),
  // booked once; repeated sweeps add none
  const double fl = 4.0 * (4.0 * m * (double)n * n + 22.0 * (double)n * n * n);
  if (e.bjacobi_fused && bjacobi_cluster_fits<T>(m, n, bs)) {
    cudaError_t err = cudaSuccess;
    prof(e, K_BJACOBI, fl, (double)esz * m * n * 2, [&] {
      err = bjacobi_cluster<T>(e.stream, m, n, bs, nblk, X, gmax.p, 2, kMaxOuter, nullptr);
    });
    if (err == cudaSuccess) return;
  }
  std::vector<int> pairs((size_t)rounds * np * 2);
  for (int r = 0; r < rounds; ++r)
    for (int p = 0; p < np; ++p) {
      int a, c;
      if (p == 0) { a = nb - 1; c = r; }
      else { a = (r + p) % (nb - 1); c = (r - p + nb - 1) % (nb - 1); }
      pairs[((size_t)r * np + p) * 2] = a;
      pairs[((size_t)r * np + p) * 2 + 1] = c;
    }
  DBuf<int> dp(e, pairs.size()), flag(e, 1);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(dp.p, pairs.data(), pairs.size() * sizeof(int), cudaMemcpyHostToDevice, e.stream));
  int hflag = 1;
  for (int outer = 0; outer < kMaxOuter && hflag; ++outer) {
    MPDO_CUDA_CHECK(cudaMemsetAsync(flag.p, 0, sizeof(int), e.stream));
    for (int r = 0; r < rounds; ++r)
      prof(e, K_BJACOBI, (outer == 0 && r == 0) ? fl : 0.0, (double)esz * m * n * 2, [&] {
        bjacobi_round<T>(e.stream, m, n, bs, nblk, X, dp.p + (size_t)r * np * 2, np, gmax.p, 2, flag.p);
      });
    MPDO_CUDA_CHECK(cudaMemcpyAsync(&hflag, flag.p, sizeof(int), cudaMemcpyDeviceToHost, e.stream));
    MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  }
}

// Leading left singular vectors of a wide-bond Y (Mr x Nc): eigenvectors of
// the Gram matrix Y Y^H (Householder tridiagonalisation on a thread-block
// cluster + bisection / inverse iteration for the top kr; block Jacobi where
// the cluster does not fit), then a Rayleigh-Ritz refinement in
// the leading kr = min(Mr, want + 16) directions (QR + one-sided Jacobi of
// Z = U^H Y), which restores the accuracy of the small singular values.
// U: Mr x kr column-major; s: Mr values (kr refined, the rest from the Gram).
template <typename T>
static void left_svd_wide_exact(Engine &e, const cx<T> *Y, int Mr, int Nc, int want, DBuf<cx<T>> &U, DBuf<T> &s,
                                int &kr) {
  DBuf<cx<T>> G(e, (size_t)Mr * Mr), X(e, (size_t)Mr * Mr);
  gemm<T>(e, Mr, Mr, Nc, RM<T>(Y, Nc), CM<T>(Y, Nc, 1), G.p, Mr);
  {  // X (column-major) = G^T = conj(G) for a Hermitian G stored row-major
    const int64_t d[4] = {1, 1, 1, (int64_t)Mr * Mr};
    const int64_t st[4] = {0, 0, 0, 1};
    copy4d<T>(e.stream, X.p, G.p, d, st, 1);
  }
  G.reset();
  kr = std::min(Mr, want + e.wide_oversample);
  // leading kr eigenvectors of the Gram: U_a (Mr x kr, as a view) and the
  // eigenvalue tail beyond them
  DBuf<cx<T>> Ua;
  View<T> ua_view{};
  DBuf<T> lam, tail;
  bool have = false;
  // Default: tridiagonal for complex128 (1.8x faster than block Jacobi,
  // both at the oracle to 1e-14); in complex64 block Jacobi up to Grams of
  // 256 (chi <= 64 at kappa 4) and tridiagonal from wide_eig_from = 257.
  // Measured in complex64 on the n=32, chi=64, kappa=4 circuit against the
  // complex128 oracle: with the error rule 1e-6 (well conditioned) both reach
  // ~2e-5, the floor that single-precision storage of the state sets there;
  // on the chi-capped benchmark form (ill-conditioned: complex128 runs that
  // differ only in rounding spread by 3e-3 at depth 8) Jacobi lands inside
  // the spread and the tridiagonal route at twice it.  On 512-wide Grams
  // (chi = 128) the Jacobi rounds cost 8x the tridiagonal route.  Jacobi also
  // remains where the cluster does not fit or cannot be placed.
  const bool use_eig = e.wide_eig > 0 || (e.wide_eig < 0 && (sizeof(T) == 8 || Mr >= e.wide_eig_from));
  if (use_eig && hetrd_cluster_fits<T>(Mr)) {
    DBuf<T> dd(e, Mr), ee(e, Mr), work(e, (size_t)kr * 2 * Mr);
    DBuf<cx<T>> vref(e, (size_t)(Mr - 1) * (Mr - 1)), tau(e, Mr), Zt(e, (size_t)Mr * kr);
    lam = DBuf<T>(e, kr);
    tail = DBuf<T>(e, 1);
    cudaError_t err;
    prof(e, K_HETRD, 16.0 / 3.0 * 4.0 * (double)Mr * Mr * Mr, (double)sizeof(cx<T>) * Mr * Mr * 2, [&] {
      err = hetrd_cluster<T>(e.stream, Mr, X.p, dd.p, ee.p, vref.p, tau.p);
    });
    if (err == cudaSuccess) {
      tridiag_top<T>(e.stream, Mr, dd.p, ee.p, kr, lam.p, Zt.p, work.p, tail.p);
      const cx<T> *vr = vref.p, *ta = tau.p, *zt = Zt.p;
      Ua = DBuf<cx<T>>(e, (size_t)Mr * kr);
      // U = Q Z: row 0 is untouched by the reflectors, rows 1.. get Q'
      MPDO_CUDA_CHECK(cudaMemcpyAsync(Ua.p, zt, kr * sizeof(cx<T>), cudaMemcpyDeviceToDevice, e.stream));
      prof(e, K_QR_APPLY, 8.0 * (double)Mr * Mr * kr, (double)sizeof(cx<T>) * ((double)Mr * Mr / 2 + 2.0 * Mr * kr), [&] {
        qr_apply_chunks<T>(e.stream, Mr - 1, Mr - 1, Mr - 1, 1, vr, ta, zt + kr, kr, kr, Ua.p + kr, kr);
      });
      {  // to column-major, so the QR below reads it coalesced
        DBuf<cx<T>> Uc(e, (size_t)Mr * kr);
        const int64_t dd4[4] = {1, 1, kr, Mr};
        const int64_t st4[4] = {0, 0, 1, kr};
        copy4d<T>(e.stream, Uc.p, Ua.p, dd4, st4, 0);
        Ua = std::move(Uc);
      }
      ua_view = CM<T>(Ua.p, Mr);
      have = true;
      e.wide_eig_calls++;
    } else {
      cudaGetLastError();          // the cluster could not be placed: Jacobi path
    }
  }
  if (!have) {
    block_jacobi<T>(e, Mr, Mr, X.p);
    Ua = DBuf<cx<T>>(e, (size_t)Mr * Mr);
    DBuf<cx<T>> xws(e, (size_t)Mr * Mr);
    lam = DBuf<T>(e, Mr);
    jacobi_svd<T>(e.stream, 1, Mr, Mr, CM<T>(X.p, Mr), Ua.p, lam.p, nullptr, xws.p, nullptr, 0, status_slot(e, 1));
    ua_view = CM<T>(Ua.p, Mr);
  }
  X.reset();
  // Orthonormal basis of the leading kr eigenvector columns: directions with
  // rounding-level eigenvalues come out of the normalisation as arbitrary,
  // non-orthogonal vectors; Householder QR keeps the leading span and replaces
  // them by an orthonormal completion.
  DBuf<cx<T>> Qb(e, (size_t)Mr * kr), Rb(e, (size_t)kr * kr);
  qr<T>(e, Mr, kr, ua_view, Qb.p, Rb.p);                         // Qb row-major Mr x kr
  Ua.reset();
  Rb.reset();
  DBuf<cx<T>> Z(e, (size_t)kr * Nc);
  gemm<T>(e, kr, Nc, Mr, CM<T>(Qb.p, kr, 1), RM<T>(Y, Nc), Z.p, Nc);   // Qb^H Y
  DBuf<cx<T>> Wz;
  DBuf<T> sz;
  right_svd<T>(e, Nc, kr, CM<T>(Z.p, Nc, 1), Wz, sz);          // left singular vectors of Z
  U = DBuf<cx<T>>(e, (size_t)Mr * kr);
  gemm<T>(e, Mr, kr, kr, RM<T>(Qb.p, kr), CM<T>(Wz.p, kr), U.p, kr);   // row-major Mr x kr
  {  // to column-major
    DBuf<cx<T>> Uc(e, (size_t)Mr * kr);
    const int64_t d[4] = {1, 1, kr, Mr};
    const int64_t st[4] = {0, 0, 1, kr};
    copy4d<T>(e.stream, Uc.p, U.p, d, st, 0);
    U = std::move(Uc);
  }
  s = DBuf<T>(e, Mr);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(s.p, sz.p, kr * sizeof(T), cudaMemcpyDeviceToDevice, e.stream));
  if (Mr > kr) {
    if (have) {
      // only the energy of the rest of the spectrum is known: it goes to the
      // first slot past kr (what the discarded-weight sums use)
      MPDO_CUDA_CHECK(cudaMemsetAsync(s.p + kr, 0, (Mr - kr) * sizeof(T), e.stream));
      sqrt_inplace<T>(e.stream, tail.p, 1);
      MPDO_CUDA_CHECK(cudaMemcpyAsync(s.p + kr, tail.p, sizeof(T), cudaMemcpyDeviceToDevice, e.stream));
    } else {
      sqrt_inplace<T>(e.stream, lam.p, Mr);
      MPDO_CUDA_CHECK(cudaMemcpyAsync(s.p + kr, lam.p + kr, (Mr - kr) * sizeof(T), cudaMemcpyDeviceToDevice, e.stream));
    }
  }
}

// Verified randomized range finder for a wide bond: Q = orth(Y Omega) with
// p = want + 32 columns (optionally one power step Q <- orth(Y Y^H Q)), then the
// exact SVD of B = Q^H Y (QR + one-sided Jacobi).  The result is accepted only
// if the residual |Y - Q B|_F is below working precision relative to |Y|_F:
// then span(Q) holds the whole numerical range of Y and the singular triplets
// equal those of an exact SVD to rounding.  Returns false (caller falls back
// to the exact block-Jacobi path) otherwise.
template <typename T>
static bool left_svd_wide_range(Engine &e, const cx<T> *Y, int Mr, int Nc, int want, DBuf<cx<T>> &U, DBuf<T> &s,
                                int &kr) {
  const int p = std::min(Mr, std::min(Nc, want + 32));
  if (p >= Mr) return false;
  const T eps = sizeof(T) == 4 ? T(1.1920929e-7) : T(2.220446049250313e-16);
  // rounding level of the residual itself: |fl(Y - Q (Q^H Y))|_F ~ eps sqrt(p) |Y|_F
  const double tol = e.wide_range_tol * eps * std::sqrt((double)p);
  DBuf<double> nrm(e, 2);
  sumsq<T>(e.stream, Y, (size_t)Mr * Nc, nrm.p);
  DBuf<cx<T>> Z(e, (size_t)Mr * p), Q(e, (size_t)Mr * p), Rq(e, (size_t)p * p), B(e, (size_t)p * Nc),
      E(e, (size_t)Mr * Nc);
  {
    DBuf<cx<T>> Om(e, (size_t)Nc * p);
    gaussian<T>(e.stream, Om.p, (size_t)Nc * p, 0x5eed5eedull + (uint64_t)Nc * 131 + p);
    gemm<T>(e, Mr, p, Nc, RM<T>(Y, Nc), RM<T>(Om.p, p), Z.p, p);
  }
  bool ok = false;
  for (int it = 0; it < 2 && !ok; ++it) {
    qr<T>(e, Mr, p, RM<T>(Z.p, p), Q.p, Rq.p);
    gemm<T>(e, p, Nc, Mr, CM<T>(Q.p, p, 1), RM<T>(Y, Nc), B.p, Nc);          // B = Q^H Y
    MPDO_CUDA_CHECK(cudaMemcpyAsync(E.p, Y, (size_t)Mr * Nc * sizeof(cx<T>), cudaMemcpyDeviceToDevice, e.stream));
    prof(e, K_GEMM, 8.0 * Mr * Nc * p, (double)sizeof(cx<T>) * ((double)Mr * p + (double)p * Nc + 2.0 * Mr * Nc), [&] {
      cgemm<T>(e.stream, Mr, Nc, p, 1, cmk<T>(T(-1), T(0)), RM<T>(Q.p, p), RM<T>(B.p, Nc), cmk<T>(T(1), T(0)), E.p,
               Nc, 1, 0);                                                  // E = Y - Q B
    });
    sumsq<T>(e.stream, E.p, (size_t)Mr * Nc, nrm.p + 1);
    double h[2];
    MPDO_CUDA_CHECK(cudaMemcpyAsync(h, nrm.p, sizeof(h), cudaMemcpyDeviceToHost, e.stream));
    MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
    const double ratio = h[0] > 0.0 ? std::sqrt(h[1] / h[0]) : 0.0;
    ok = ratio <= tol;
    if (ok) {
      e.wide_resid_max = std::max(e.wide_resid_max, ratio);
      break;
    }
    // one power step squares the captured/missed ratio; beyond reach of one
    // step (a heavy tail past p) go straight to the exact path
    if (it == 1 || ratio > 1e3 * tol) break;
    gemm<T>(e, Mr, p, Nc, RM<T>(Y, Nc), CM<T>(B.p, Nc, 1), Z.p, p);      // Z = Y B^H = Y Y^H Q
  }
  if (!ok) return false;
  E.reset();
  DBuf<cx<T>> Wb;
  DBuf<T> sb;
  right_svd<T>(e, Nc, p, CM<T>(B.p, Nc, 1), Wb, sb);             // left singular vectors of B
  DBuf<cx<T>> Urm(e, (size_t)Mr * p);
  gemm<T>(e, Mr, p, p, RM<T>(Q.p, p), CM<T>(Wb.p, p), Urm.p, p);
  U = DBuf<cx<T>>(e, (size_t)Mr * p);
  {
    const int64_t d[4] = {1, 1, p, Mr};
    const int64_t st[4] = {0, 0, 1, p};
    copy4d<T>(e.stream, U.p, Urm.p, d, st, 0);
  }
  s = DBuf<T>(e, Mr);
  MPDO_CUDA_CHECK(cudaMemsetAsync(s.p, 0, Mr * sizeof(T), e.stream));
  MPDO_CUDA_CHECK(cudaMemcpyAsync(s.p, sb.p, p * sizeof(T), cudaMemcpyDeviceToDevice, e.stream));
  kr = p;
  return true;
}

template <typename T>
static void left_svd_wide(Engine &e, const cx<T> *Y, int Mr, int Nc, int want, DBuf<cx<T>> &U, DBuf<T> &s,
                          int &kr) {
  Phase ph(e, P_WIDE_SVD);
  const bool try_range = e.wide_range > 0 || (e.wide_range < 0 && sizeof(T) == 8);
  if (try_range && left_svd_wide_range<T>(e, Y, Mr, Nc, want, U, s, kr)) {
    e.wide_range_hits++;
    return;
  }
  e.wide_exact_calls++;
  left_svd_wide_exact<T>(e, Y, Mr, Nc, want, U, s, kr);
}

// --------------------------------------------------------- SVD split ----
// Y (Mr x Nc, row-major) = L R with L = U_k sqrt(S_k) (Mr x keep, ld keep)
// and R = sqrt(S_k) V_k^H (keep x Nc), keep chosen by keep_fn(s_dev, nsv).
// The left singular vectors of Y are the right singular vectors of Y^H:
// QR of Y^H, one-sided Jacobi on R.  R_out is formed as s^-1/2 U_k^H Y.
// When keep exceeds min(Mr, Nc) the extra columns/rows are zero (the
// reference's SVD returns (near-)zero singular values there).
// wsum (nullable): device double[2] = {kept, total} sum s^2.
template <typename T, typename KeepFn>
static void svd_split(Engine &e, const cx<T> *Y, int Mr, int Nc, KeepFn keep_fn, DBuf<cx<T>> &Lout,
                      DBuf<cx<T>> &Rout, int &keep_out, double *wsum, int want = -1) {
  DBuf<cx<T>> W;
  DBuf<T> sg;
  const int nsv_ref = std::min(Mr, Nc);
  const size_t esz = sizeof(cx<T>);
  int kr = Mr;   // number of computed singular vectors
  if (2 * (size_t)Mr * Mr * esz <= 200 * 1024) {
    right_svd<T>(e, Nc, Mr, CM<T>(Y, Nc, 1), W, sg);       // view of Y^H (Nc x Mr)
  } else {
    left_svd_wide<T>(e, Y, Mr, Nc, want < 0 ? nsv_ref : std::min(want, nsv_ref), W, sg, kr);
  }
  int keep = keep_fn(sg.p, nsv_ref);
  if (std::min(keep, nsv_ref) > kr) fail(MPDO_ERR_BAD_SHAPE, "internal: kept more vectors than refined");
  keep_out = keep;
  if (wsum) {
    // kept weight from the (refined) kept singular values; the total from
    // |Y|_F^2 accumulated in double, so that total - kept does not depend on
    // how accurately the discarded values themselves were computed (the wide
    // path only estimates them from the Gram matrix)
    sigma_weights<T>(e.stream, sg.p, Mr, keep, wsum);
    sumsq<T>(e.stream, Y, (size_t)Mr * Nc, wsum + 1);
  }
  const int kk = std::min(keep, nsv_ref);
  (void)kr;
  Lout = DBuf<cx<T>>(e, (size_t)Mr * std::max(keep, 1));
  Rout = DBuf<cx<T>>(e, (size_t)std::max(keep, 1) * Nc);
  if (keep > kk) {
    fill_zero<T>(e.stream, Lout.p, (size_t)Mr * keep);
    fill_zero<T>(e.stream, Rout.p, (size_t)keep * Nc);
  }
  if (kk <= 0) return;
  // L = W[:, :kk] sqrt(s)  (W column-major: element (i, j) at j*Mr + i)
  {
    const int64_t d[4] = {1, 1, Mr, kk};
    const int64_t st[4] = {0, 0, 1, Mr};
    if (keep == kk) {
      copy4d<T>(e.stream, Lout.p, W.p, d, st, 0);
    } else {
      DBuf<cx<T>> Lk(e, (size_t)Mr * kk);
      copy4d<T>(e.stream, Lk.p, W.p, d, st, 0);
      MPDO_CUDA_CHECK(cudaMemcpy2DAsync(Lout.p, keep * sizeof(cx<T>), Lk.p, kk * sizeof(cx<T>), kk * sizeof(cx<T>),
                                        Mr, cudaMemcpyDeviceToDevice, e.stream));
    }
  }
  scale_matrix<T>(e.stream, Lout.p, Mr, kk, keep, sg.p, 0, 1);
  // R = s^-1/2 W[:, :kk]^H Y
  gemm<T>(e, kk, Nc, Mr, RM<T>(W.p, Mr, 1), RM<T>(Y, Nc), Rout.p, Nc);
  scale_matrix<T>(e.stream, Rout.p, kk, Nc, Nc, sg.p, 1, 2);
}

// decompositions.py:121-134 truncation rule on host singular values.  The
// reference decomposes a matrix with nsv singular values; entries beyond the
// computed spectrum are zero.
template <typename T>
int error_rule_keep(const std::vector<T> &s_in, int nsv, int max_sv, double err, bool relative, double total_sq) {
  // evaluated in double whatever T: in single precision the cumulative
  // norms' rounding (~6e-8 s_0) is a tenth of a 1e-6 relative threshold.
  // total_sq >= 0 gives the matrix's |Y|_F^2 for the full norm (when the
  // trailing singular values are only estimated, as on wide bonds)
  int n_err = max_sv;
  if (err >= 0 && nsv > 0) {
    std::vector<double> te(nsv);
    double acc = 0.0;
    for (int i = 0; i < nsv; ++i) {
      const double v = i < (int)s_in.size() ? (double)s_in[i] : 0.0;
      acc += v * v;
      te[i] = std::sqrt(acc);
    }
    if (total_sq >= 0) te[nsv - 1] = std::sqrt(total_sq);
    const double s0 = s_in.empty() ? 0.0 : (double)s_in[0];
    const double thr = relative ? err * s0 : err;
    for (int idx = 0; idx < nsv - 1; ++idx)
      if (te[nsv - 1] - te[idx] <= thr) { n_err = idx + 1; break; }
  }
  return std::min(max_sv, n_err);
}

// -------------------------------------------------------------- ops -----
template <typename T> static void materialize_pair(mpdo_chain_s *ch, int i);

// Deferred single-qubit gates.  A 1q Kraus map with sum_k K_k^H K_k = I
// (trace preserving) acts on a site's physical and Kraus legs as an isometry
// B (I_l (x) G (x) I_r with G^H G = I on the (s, a) legs): the QR factor R of
// B A equals that of A, and the left singular vectors and values of a bond
// matrix B Y equal those of Y.  A truncate that follows a 1q sublayer
// therefore runs its QR and SVD sweeps on the pre-gate sites (K times fewer
// rows or columns) and applies the Kraus maps afterwards, before the kappa
// pass; the keep counts use the post-gate dimensions (the extra singular
// values are exact zeros and are zero-padded as the reference keeps them).
// Any other operation on the site applies the map first.
static bool trace_preserving(const double *g, int K, double tol) {
  for (int s = 0; s < 2; ++s)
    for (int t = 0; t < 2; ++t) {
      double re = 0, im = 0;
      for (int x = 0; x < 2; ++x)
        for (int k = 0; k < K; ++k) {
          const double *a = g + 2 * ((x * 2 + s) * K + k), *b = g + 2 * ((x * 2 + t) * K + k);
          re += a[0] * b[0] + a[1] * b[1];       // conj(a) b
          im += a[0] * b[1] - a[1] * b[0];
        }
      if (std::fabs(re - (s == t ? 1.0 : 0.0)) > tol || std::fabs(im) > tol) return false;
    }
  return true;
}

template <typename T> static void kraus_site(mpdo_chain_s *ch, int site, const double *kraus, int K) {
  Engine &e = ch->eng->e;
  const Site s = ch->s[site];
  DBuf<cx<T>> out(e, (size_t)s.l * 2 * s.a * K * s.r);
  prof(e, K_KRAUS1Q, 8.0 * 2 * 2 * K * s.elems(), (double)sizeof(cx<T>) * s.elems() * (1 + K),
       [&] { kraus1q<T>(e.stream, site_ptr<T>(ch, site), out.p, s.l, s.a, s.r, kraus, K); });
  set_site<T>(ch, site, out.release(), s.l, s.a * K, s.r);
}

template <typename T> static void materialize_1q(mpdo_chain_s *ch, int site) {
  Pend &p = ch->pend1[site];
  if (!p.on) return;
  p.on = false;
  kraus_site<T>(ch, site, p.t.data(), p.K);
}
template <typename T> static void materialize_1q_all(mpdo_chain_s *ch) {
  for (int i = 0; i < ch->n; ++i) materialize_1q<T>(ch, i);
}
// Kraus-leg dimension of a site once its deferred map is applied
static int a_eff(const mpdo_chain_s *ch, int i) { return ch->s[i].a * (ch->pend1[i].on ? ch->pend1[i].K : 1); }

template <typename T> static void materialize_touching(mpdo_chain_s *ch, int site) {
  if (site - 1 >= 0 && ch->pend[site - 1].on) materialize_pair<T>(ch, site - 1);
  if (site < ch->n - 1 && ch->pend[site].on) materialize_pair<T>(ch, site);
  materialize_1q<T>(ch, site);
}
template <typename T> void materialize_all(mpdo_chain_s *ch) {
  for (int i = 0; i + 1 < ch->n; ++i)
    if (ch->pend[i].on) materialize_pair<T>(ch, i);
  materialize_1q_all<T>(ch);
}

template <typename T> static void apply_1q(mpdo_chain_s *ch, int site, const double *kraus, int K) {
  Engine &e = ch->eng->e;
  // pending pairs on this site are older than the gate
  if (site - 1 >= 0 && ch->pend[site - 1].on) materialize_pair<T>(ch, site - 1);
  if (site < ch->n - 1 && ch->pend[site].on) materialize_pair<T>(ch, site);
  const double tol = sizeof(T) == 4 ? 1e-6 : 1e-12;
  Pend &p = ch->pend1[site];
  if (e.defer_1q && trace_preserving(kraus, K, tol)) {
    if (p.on && p.K * K <= 16) {
      // compose: G[x][s][k1 K + k2] = sum_y G2[x][y][k2] G1[y][s][k1] (old Kraus index first)
      const int K1 = p.K, KK = K1 * K;
      std::vector<double> g(2 * 4 * KK, 0.0);
      for (int x = 0; x < 2; ++x)
        for (int s = 0; s < 2; ++s)
          for (int k1 = 0; k1 < K1; ++k1)
            for (int k2 = 0; k2 < K; ++k2) {
              double re = 0, im = 0;
              for (int y = 0; y < 2; ++y) {
                const double *a = kraus + 2 * ((x * 2 + y) * K + k2), *b = p.t.data() + 2 * ((y * 2 + s) * K1 + k1);
                re += a[0] * b[0] - a[1] * b[1];
                im += a[0] * b[1] + a[1] * b[0];
              }
              double *o = g.data() + 2 * ((x * 2 + s) * KK + k1 * K + k2);
              o[0] = re;
              o[1] = im;
            }
      p.t.swap(g);
      p.K = KK;
      return;
    }
    materialize_1q<T>(ch, site);
    p.on = true;
    p.t.assign(kraus, kraus + 8 * K);
    p.K = K;
    return;
  }
  materialize_1q<T>(ch, site);
  kraus_site<T>(ch, site, kraus, K);
}

template <typename T> static void materialize_pair(mpdo_chain_s *ch, int i) {
  Engine &e = ch->eng->e;
  Pend pd = ch->pend[i];
  ch->pend[i].on = false;
  const Site A = ch->s[i], B = ch->s[i + 1];
  const int l = A.l, a = A.a, m = A.r, c = B.a, r = B.r, K = pd.K;
  const int Mr = l * 2 * a, Nc = 2 * c * K * r;
  DBuf<cx<T>> P(e, (size_t)Mr * 2 * c * r);
  gemm<T>(e, Mr, 2 * c * r, m, RM<T>(site_ptr<T>(ch, i), m), RM<T>(site_ptr<T>(ch, i + 1), 2 * c * r), P.p,
          2 * c * r);
  DBuf<cx<T>> th(e, (size_t)Mr * Nc);
  mix2q_batched<T>(e.stream, P.p, th.p, l, a, c, r, pd.t.data(), K);
  P.reset();
  // Circuit.py:116-126: exact SVD, absolute cutoff, no cap
  const double cutoff = pd.cutoff;
  auto keep_fn = [&](const T *s_dev, int nsv) -> int {
    std::vector<T> s(std::min(Mr, Nc));
    MPDO_CUDA_CHECK(cudaMemcpyAsync(s.data(), s_dev, s.size() * sizeof(T), cudaMemcpyDeviceToHost, e.stream));
    MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
    return error_rule_keep<T>(s, nsv, nsv, cutoff, false);
  };
  DBuf<cx<T>> Lf, Rf;
  int keep = 0;
  svd_split<T>(e, th.p, Mr, Nc, keep_fn, Lf, Rf, keep, nullptr);
  set_site<T>(ch, i, Lf.release(), l, a, keep);
  set_site<T>(ch, i + 1, Rf.release(), keep, c * K, r);
}

template <typename T> static void apply_2q(mpdo_chain_s *ch, int i, const double *t, int K, double cutoff) {
  for (int j = std::max(0, i - 1); j <= std::min(ch->n - 2, i + 1); ++j)
    if (ch->pend[j].on) materialize_pair<T>(ch, j);
  materialize_1q<T>(ch, i);
  materialize_1q<T>(ch, i + 1);
  Pend &p = ch->pend[i];
  p.on = true;
  p.t.assign(t, t + 32 * K);
  p.K = K;
  p.cutoff = cutoff;
  ch->bond[i] = 1;
}

// TNNOptimizer.py:87-108, with pending pairs fused (see file header)
template <typename T> static void qr_sweep(mpdo_chain_s *ch) {
  Engine &e = ch->eng->e;
  Phase ph(e, P_QR_SWEEP);
  const int n = ch->n;
  DBuf<cx<T>> Rprev;
  int Rrows = 0, Rcols = 0;
  auto absorb = [&](int i) -> DBuf<cx<T>> {
    // returns R_prev . A_i as a new buffer (b x 2 a r)
    const Site s = ch->s[i];
    DBuf<cx<T>> X(e, (size_t)Rrows * 2 * s.a * s.r);
    gemm<T>(e, Rrows, 2 * s.a * s.r, s.l, RM<T>(Rprev.p, Rcols), RM<T>(site_ptr<T>(ch, i), 2 * s.a * s.r), X.p,
            2 * s.a * s.r);
    return X;
  };
  for (int i = 0; i < n - 1; ++i) {
    if (ch->pend[i].on) {
      Pend pd = ch->pend[i];
      ch->pend[i].on = false;
      int b = ch->s[i].l;
      const int a = ch->s[i].a, m = ch->s[i].r;
      if (Rprev.p) {
        DBuf<cx<T>> X = absorb(i);
        set_site<T>(ch, i, X.release(), Rrows, a, m);
        b = Rrows;
        Rprev.reset();
      }
      // At[(b,a)][(s,m)]
      DBuf<cx<T>> At(e, (size_t)b * a * 2 * m);
      {
        const int64_t d[4] = {b, a, 2, m};
        const int64_t st[4] = {(int64_t)2 * a * m, m, (int64_t)a * m, 1};
        copy4d<T>(e.stream, At.p, site_ptr<T>(ch, i), d, st, 0);
      }
      const int mr = b * a, nc = 2 * m, kq = std::min(mr, nc);
      DBuf<cx<T>> Qp(e, (size_t)mr * kq), Rp(e, (size_t)kq * nc);
      qr<T>(e, mr, nc, RM<T>(At.p, nc), Qp.p, Rp.p);
      At.reset();
      DBuf<cx<T>> Si(e, (size_t)b * 2 * a * 2 * kq);
      blockdiag2<T>(e.stream, Si.p, Qp.p, b, a, kq);
      set_site<T>(ch, i, Si.release(), b, a, 2 * kq);
      // W[s][k][t][c][r] = sum_m R'[k][s*m + m'] A_{i+1}[m'][t][c][r]
      const Site B = ch->s[i + 1];
      const int c = B.a, r = B.r, K = pd.K;
      const int ncol = 2 * c * r;
      DBuf<cx<T>> W(e, (size_t)2 * kq * ncol);
      gemm<T>(e, kq, ncol, m, View<T>{Rp.p, (int64_t)m, 1, nc, 0, 1, 0}, RM<T>(site_ptr<T>(ch, i + 1), ncol), W.p,
              ncol, 2, (int64_t)kq * ncol);
      DBuf<cx<T>> Z(e, (size_t)2 * kq * 2 * c * K * r);
      prof(e, K_MIX2Q, 8.0 * 16 * K * (double)kq * c * r, (double)sizeof(cx<T>) * 4.0 * kq * c * r * (1 + K),
           [&] { mix2q<T>(e.stream, W.p, Z.p, kq, c, r, pd.t.data(), K); });
      set_site<T>(ch, i + 1, Z.release(), 2 * kq, c * K, r);
      continue;
    }
    if (Rprev.p) {
      const Site s = ch->s[i];
      DBuf<cx<T>> X = absorb(i);
      set_site<T>(ch, i, X.release(), Rrows, s.a, s.r);
      Rprev.reset();
    }
    const Site s = ch->s[i];
    const int mr = s.l * 2 * s.a, nc = s.r, kq = std::min(mr, nc);
    DBuf<cx<T>> Q(e, (size_t)mr * kq), R(e, (size_t)kq * nc);
    qr<T>(e, mr, nc, RM<T>(site_ptr<T>(ch, i), nc), Q.p, R.p);
    set_site<T>(ch, i, Q.release(), s.l, s.a, kq);
    Rprev = std::move(R);
    Rrows = kq; Rcols = nc;
  }
  if (Rprev.p) {
    const Site s = ch->s[n - 1];
    DBuf<cx<T>> X = absorb(n - 1);
    set_site<T>(ch, n - 1, X.release(), Rrows, s.a, s.r);
  }
}

// TNNOptimizer.py:111-134
template <typename T> static void svd_sweep(mpdo_chain_s *ch, int chi, double max_err, double *wdev) {
  Engine &e = ch->eng->e;
  Phase ph(e, P_SVD_SWEEP);
  for (int idx = ch->n - 1; idx >= 1; --idx) {
    const Site P = ch->s[idx - 1], S = ch->s[idx];
    const int b = S.l, Nc = 2 * S.a * S.r;
    // the reference's keep rule sees the post-gate dimensions of deferred sites
    const int rows_prev = P.l * 2 * a_eff(ch, idx - 1);
    const int Nc_eff = 2 * a_eff(ch, idx) * S.r;
    auto keep_fn = [&](const T *s_dev, int) -> int {
      const int nsv = std::min(rows_prev, Nc_eff);
      const int cap = chi > 0 ? std::min(chi, nsv) : nsv;
      if (max_err < 0) return cap;
      std::vector<T> s(std::min(b, Nc));
      DBuf<double> tot(e, 1);
      sumsq<T>(e.stream, site_ptr<T>(ch, idx), (size_t)b * Nc, tot.p);
      double htot = 0;
      MPDO_CUDA_CHECK(cudaMemcpyAsync(s.data(), s_dev, s.size() * sizeof(T), cudaMemcpyDeviceToHost, e.stream));
      MPDO_CUDA_CHECK(cudaMemcpyAsync(&htot, tot.p, sizeof(double), cudaMemcpyDeviceToHost, e.stream));
      MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
      return error_rule_keep<T>(s, nsv, cap, max_err, true, htot);
    };
    DBuf<cx<T>> Lf, Rf;
    int keep = 0;
    const int want = chi > 0 ? std::min(chi, std::min(rows_prev, Nc_eff)) : -1;
    // under the chi cap alone a wide bond refines its leading want + 16
    // directions (Rayleigh-Ritz); under an error rule, whose cut is decided by
    // the smallest kept values, all of them (measured on the n=32, chi=64,
    // kappa=4 circuit with max_err = 1e-6, complex64: 2e-6 against the
    // complex128 oracle with the full space, 2e-5 with want + 16)
    svd_split<T>(e, site_ptr<T>(ch, idx), b, Nc, keep_fn, Lf, Rf, keep, wdev ? wdev + 2 * (idx - 1) : nullptr,
                 max_err < 0 ? want : -1);
    const int prow = P.l * 2 * P.a;
    DBuf<cx<T>> NP(e, (size_t)prow * keep);
    gemm<T>(e, prow, keep, b, RM<T>(site_ptr<T>(ch, idx - 1), b), RM<T>(Lf.p, keep), NP.p, keep);
    set_site<T>(ch, idx - 1, NP.release(), P.l, P.a, keep);
    set_site<T>(ch, idx, Rf.release(), keep, S.a, S.r);
  }
}

// ------------------------------------------------ standalone sweeps ----
// The reference's sweeps called one at a time on an arbitrary chain
// (TNNOptimizer.py:87-161).  The SVD sweeps decompose the contracted pair
// M = A_{idx-1} A_idx exactly without forming it: the neighbour that the
// step does not keep is factored first (QR of the left site for the
// right-to-left sweep, LQ of the right site for the left-to-right one), and
// only the small remainder is decomposed.  Keep counts follow the pair's
// shape (min(chi, rows, cols) including zero singular values, the relative
// error rule), sqrt(S) goes on both factors.

// TNNOptimizer.py:87-108
template <typename T> static void qr_left2right_only(mpdo_chain_s *ch) {
  materialize_all<T>(ch);
  qr_sweep<T>(ch);
}

template <typename T>
static int sweep_keep(Engine &e, const T *s_dev, int len, int nsv, int chi, double max_err, const cx<T> *Y,
                      size_t ny) {
  const int cap = chi > 0 ? std::min(chi, nsv) : nsv;
  if (max_err < 0) return cap;
  std::vector<T> s(len);
  DBuf<double> tot(e, 1);
  sumsq<T>(e.stream, Y, ny, tot.p);
  double htot = 0;
  MPDO_CUDA_CHECK(cudaMemcpyAsync(s.data(), s_dev, s.size() * sizeof(T), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaMemcpyAsync(&htot, tot.p, sizeof(double), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  return error_rule_keep<T>(s, nsv, cap, max_err, true, htot);
}

static void discarded_to_host(Engine &e, const DBuf<double> &w, int nb, double *out) {
  if (!out) return;
  std::vector<double> h(2 * (size_t)nb);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(h.data(), w.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  for (int i = 0; i < nb; ++i)
    out[i] = h[2 * i + 1] > 0 ? std::max(0.0, (h[2 * i + 1] - h[2 * i]) / h[2 * i + 1]) : 0.0;
}

// TNNOptimizer.py:111-134: for idx = n-1 .. 1, A_{idx-1} = Q R, Y = R A_idx,
// Y = U S V^H: A_{idx-1} := Q U sqrt(S), A_idx := sqrt(S) V^H
template <typename T> static void svd_right2left_only(mpdo_chain_s *ch, int chi, double max_err, double *disc) {
  Engine &e = ch->eng->e;
  materialize_all<T>(ch);
  const int n = ch->n;
  DBuf<double> w(e, (size_t)2 * std::max(1, n - 1));
  MPDO_CUDA_CHECK(cudaMemsetAsync(w.p, 0, sizeof(double) * 2 * std::max(1, n - 1), e.stream));
  for (int idx = n - 1; idx >= 1; --idx) {
    const Site P = ch->s[idx - 1], S = ch->s[idx];
    const int rows = P.l * 2 * P.a, m = P.r, Nc = 2 * S.a * S.r, kq = std::min(rows, m);
    DBuf<cx<T>> Q(e, (size_t)rows * kq), R(e, (size_t)kq * m), Y(e, (size_t)kq * Nc);
    qr<T>(e, rows, m, RM<T>(site_ptr<T>(ch, idx - 1), m), Q.p, R.p);
    gemm<T>(e, kq, Nc, m, RM<T>(R.p, m), RM<T>(site_ptr<T>(ch, idx), Nc), Y.p, Nc);
    const int nsv = std::min(rows, Nc);
    auto keep_fn = [&](const T *s_dev, int) -> int {
      return sweep_keep<T>(e, s_dev, std::min(kq, Nc), nsv, chi, max_err, Y.p, (size_t)kq * Nc);
    };
    DBuf<cx<T>> Lf, Rf;
    int keep = 0;
    svd_split<T>(e, Y.p, kq, Nc, keep_fn, Lf, Rf, keep, w.p + 2 * (idx - 1),
                 max_err < 0 && chi > 0 ? std::min(chi, nsv) : -1);
    DBuf<cx<T>> NP(e, (size_t)rows * keep);
    gemm<T>(e, rows, keep, kq, RM<T>(Q.p, kq), RM<T>(Lf.p, keep), NP.p, keep);
    set_site<T>(ch, idx - 1, NP.release(), P.l, P.a, keep);
    set_site<T>(ch, idx, Rf.release(), keep, S.a, S.r);
  }
  discarded_to_host(e, w, n - 1, disc);
}

// TNNOptimizer.py:137-161: for idx = 0 .. n-2, A_{idx+1} = L Q (LQ: QR of
// its adjoint), Y = A_idx L, Y = U S V^H: A_idx := U sqrt(S),
// A_{idx+1} := sqrt(S) V^H Q
template <typename T> static void svd_left2right_only(mpdo_chain_s *ch, int chi, double max_err, double *disc) {
  Engine &e = ch->eng->e;
  materialize_all<T>(ch);
  const int n = ch->n;
  DBuf<double> w(e, (size_t)2 * std::max(1, n - 1));
  MPDO_CUDA_CHECK(cudaMemsetAsync(w.p, 0, sizeof(double) * 2 * std::max(1, n - 1), e.stream));
  for (int idx = 0; idx + 1 < n; ++idx) {
    const Site A = ch->s[idx], B = ch->s[idx + 1];
    const int rows = A.l * 2 * A.a, m = A.r, cols = 2 * B.a * B.r, kq = std::min(cols, m);
    // B (m x cols) = Lq Qh with B^H = Q0 R0: Lq = R0^H (m x kq), Qh = Q0^H (kq x cols)
    DBuf<cx<T>> Q0(e, (size_t)cols * kq), R0(e, (size_t)kq * m);
    qr<T>(e, cols, m, CM<T>(site_ptr<T>(ch, idx + 1), cols, 1), Q0.p, R0.p);
    DBuf<cx<T>> Y(e, (size_t)rows * kq);
    gemm<T>(e, rows, kq, m, RM<T>(site_ptr<T>(ch, idx), m), CM<T>(R0.p, m, 1), Y.p, kq);   // A_idx R0^H
    const int nsv = std::min(rows, cols);
    // Y is tall (rows >= kq in practice): its right singular vectors by QR +
    // one-sided Jacobi, then L = U sqrt(S) = Y V S^-1/2, R = sqrt(S) V^H
    DBuf<cx<T>> W;
    DBuf<T> sg;
    right_svd<T>(e, rows, kq, RM<T>(Y.p, kq), W, sg);                 // W: kq x kq column-major
    const int keep = sweep_keep<T>(e, sg.p, kq, nsv, chi, max_err, Y.p, (size_t)rows * kq);
    const int kk = std::min(keep, std::min(rows, kq));
    sigma_weights<T>(e.stream, sg.p, kq, keep, w.p + 2 * idx);
    sumsq<T>(e.stream, Y.p, (size_t)rows * kq, w.p + 2 * idx + 1);
    DBuf<cx<T>> Lf(e, (size_t)rows * std::max(keep, 1)), Rf(e, (size_t)std::max(keep, 1) * kq);
    if (keep > kk) {
      fill_zero<T>(e.stream, Lf.p, (size_t)rows * keep);
      fill_zero<T>(e.stream, Rf.p, (size_t)keep * kq);
    }
    if (kk > 0) {
      gemm<T>(e, rows, kk, kq, RM<T>(Y.p, kq), CM<T>(W.p, kq), Lf.p, keep);              // Y V_k
      scale_matrix<T>(e.stream, Lf.p, rows, kk, keep, sg.p, 0, 2);
      const int64_t d[4] = {1, 1, kk, kq};
      const int64_t st[4] = {0, 0, kq, 1};
      copy4d<T>(e.stream, Rf.p, W.p, d, st, 1);                                            // V_k^H
      scale_matrix<T>(e.stream, Rf.p, kk, kq, kq, sg.p, 1, 1);
    }
    DBuf<cx<T>> NB(e, (size_t)keep * cols);
    gemm<T>(e, keep, cols, kq, RM<T>(Rf.p, kq), CM<T>(Q0.p, kq, 1), NB.p, cols);             // Rf Q0^H
    set_site<T>(ch, idx, Lf.release(), A.l, A.a, keep);
    set_site<T>(ch, idx + 1, NB.release(), keep, B.a, B.r);
  }
  discarded_to_host(e, w, n - 1, disc);
}

// TNNOptimizer.py:164-197: per site, SVD of (l,s,r) x a keeping kappa; the
// site becomes U S = A V[:, :keep].  V comes from QR of A and one-sided
// Jacobi on R.
template <typename T> static void kappa_pass(mpdo_chain_s *ch, int kappa, double max_err) {
  Engine &e = ch->eng->e;
  Phase ph(e, P_KAPPA);
  if (kappa <= 0 && max_err < 0) return;
  // sites that need the pass, grouped by shape: without an error rule the
  // kept count is known on the host, so each group runs as one batch
  std::vector<int> todo;
  for (int i = 0; i < ch->n; ++i) {
    const Site s = ch->s[i];
    if (s.a == 1 || (kappa > 0 && s.a <= kappa)) continue;
    todo.push_back(i);
  }
  std::vector<bool> done(ch->n, false);
  for (size_t t = 0; t < todo.size(); ++t) {
    const int i0 = todo[t];
    if (done[i0]) continue;
    const Site s0 = ch->s[i0];
    std::vector<int> grp{i0};
    if (max_err < 0)
      for (size_t u = t + 1; u < todo.size(); ++u) {
        const Site su = ch->s[todo[u]];
        if (!done[todo[u]] && su.l == s0.l && su.r == s0.r && su.a == s0.a) grp.push_back(todo[u]);
      }
    for (int i : grp) done[i] = true;
    const int B = (int)grp.size();
    const int rows = s0.l * 2 * s0.r, a = s0.a;
    const int nsv = std::min(rows, a);
    // (l, s, r) x a per site, consecutive
    DBuf<cx<T>> Am(e, (size_t)B * rows * a);
    for (int b = 0; b < B; ++b) {
      const int64_t d[4] = {s0.l, 2, s0.r, a};
      const int64_t st[4] = {(int64_t)2 * a * s0.r, (int64_t)a * s0.r, 1, s0.r};
      copy4d<T>(e.stream, Am.p + (size_t)b * rows * a, site_ptr<T>(ch, grp[b]), d, st, 0);
    }
    // right singular vectors: R of each (QR), then one-sided Jacobi with V
    const int k = nsv;
    DBuf<cx<T>> R(e, (size_t)B * k * a), V(e, (size_t)B * a * a), Ub(e, (size_t)B * k * a),
        xws(e, (size_t)B * k * a), wws(e, (size_t)B * a * a);
    DBuf<T> sg(e, (size_t)B * a);
    qr_r_batched<T>(e, B, rows, a, View<T>{Am.p, (int64_t)rows * a, 1, a, 0, 1, 0}, R.p);
    {
      const double mm = std::max(k, a), nn = std::min(k, a);
      const double fl = B * 4.0 * (4.0 * mm * nn * nn + 22.0 * nn * nn * nn);
      int *slot = status_slot(e, B);
      prof(e, K_JACOBI, fl, (double)sizeof(cx<T>) * B * ((double)k * a * 2 + (double)a * a), [&] {
        jacobi_svd<T>(e.stream, B, k, a, View<T>{R.p, (int64_t)k * a, 1, a, 0, 1, 0}, Ub.p, sg.p, V.p, xws.p,
                      wws.p, e.max_sweeps, slot);
      });
    }
    int keep = kappa > 0 ? std::min(kappa, nsv) : nsv;
    if (max_err >= 0) {            // (B == 1 here)
      std::vector<T> sv(nsv);
      MPDO_CUDA_CHECK(cudaMemcpyAsync(sv.data(), sg.p, nsv * sizeof(T), cudaMemcpyDeviceToHost, e.stream));
      MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
      keep = error_rule_keep<T>(sv, nsv, keep, max_err, true);
    }
    // site := U S = A V[:, :keep]
    DBuf<cx<T>> NM(e, (size_t)B * rows * keep);
    gemm<T>(e, rows, keep, a, View<T>{Am.p, (int64_t)rows * a, 1, a, 0, 1, 0},
            View<T>{V.p, (int64_t)a * a, 1, 1, 0, a, 0}, NM.p, keep, B, (int64_t)rows * keep);
    for (int b = 0; b < B; ++b) {
      DBuf<cx<T>> NS(e, (size_t)rows * keep);
      const int64_t d[4] = {s0.l, 2, keep, s0.r};
      const int64_t st[4] = {(int64_t)2 * s0.r * keep, (int64_t)s0.r * keep, 1, keep};
      copy4d<T>(e.stream, NS.p, NM.p + (size_t)b * rows * keep, d, st, 0);
      set_site<T>(ch, grp[b], NS.release(), s0.l, keep, s0.r);
    }
  }
}

bool connected(mpdo_chain_s *ch) {
  for (int i = 0; i + 1 < ch->n; ++i)
    if (!ch->bond[i]) return false;
  return true;
}

template <typename T>
static void truncate_layer(mpdo_chain_s *ch, int chi, int kappa, double max_err, int noisy, double *disc_out) {
  Engine &e = ch->eng->e;
  if (!connected(ch)) return;  // Circuit.py:477 checkConnectivity
  DBuf<double> w;
  if (chi > 0 || max_err >= 0) {
    if (disc_out && ch->n > 1) w = DBuf<double>(e, (size_t)2 * (ch->n - 1));
    if (!e.fuse_2q) materialize_all<T>(ch);
    // a deferred site whose QR would keep fewer columns before the gate than
    // after it (rows < right bond, the chain ends) is applied first
    for (int i = 0; i + 1 < ch->n; ++i)
      if (ch->pend1[i].on && ch->s[i].l * 2 * ch->s[i].a < ch->s[i].r) materialize_1q<T>(ch, i);
    qr_sweep<T>(ch);
    svd_sweep<T>(ch, chi, max_err, w.p);
    materialize_1q_all<T>(ch);
  }
  if (noisy) {
    materialize_all<T>(ch);
    kappa_pass<T>(ch, kappa, max_err);
  }
  if (disc_out && ch->n > 1) {
    if (w.p) {
      std::vector<double> h(2 * (ch->n - 1));
      MPDO_CUDA_CHECK(cudaMemcpyAsync(h.data(), w.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, e.stream));
      MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
      for (int i = 0; i < ch->n - 1; ++i)
        disc_out[i] = h[2 * i + 1] > 0 ? std::max(0.0, (h[2 * i + 1] - h[2 * i]) / h[2 * i + 1]) : 0.0;
    } else {
      for (int i = 0; i < ch->n - 1; ++i) disc_out[i] = 0.0;
    }
  }
}

// ------------------------------------------------------------ readout ---
// Environment E[P][r][r'] sweeping left to right.  P enumerates, per kept
// site, the (ket x, bra y) pair (interleaved) -- or just x for diagonal
// readouts.
template <typename T> struct Env {
  DBuf<cx<T>> E;
  int64_t P = 1;
  int r = 1;
};

// one site of an environment sweep.  mode 0: trace (optionally with op on the
// ket side), 1: open (x, y), 2: open diagonal (x = y).
template <typename T>
static void env_step(Engine &e, Env<T> &env, const cx<T> *A, const Site &s, int mode, const double *op) {
  const int l = s.l, a = s.a, R = s.r;
  if (l != env.r) fail(MPDO_ERR_BAD_SHAPE, "bond mismatch in readout");
  const int64_t P = env.P;
  const cx<T> *Aket = A;
  DBuf<cx<T>> Aop;
  if (op) {
    Aop = DBuf<cx<T>>(e, s.elems());
    apply_op_site<T>(e.stream, A, Aop.p, l, a, R, op);
    Aket = Aop.p;
  }
  // F[P][x][l'][a][r] = sum_l E[P][l][l'] Aket[l][x][a][r]
  DBuf<cx<T>> F(e, (size_t)P * 2 * l * a * R);
  const int64_t aR = (int64_t)a * R;
  for (int x = 0; x < 2; ++x)
    gemm<T>(e, l, (int)aR, l, CM<T>(env.E.p, l, 0, (int64_t)l * l), RM<T>(Aket + x * aR, 2 * aR), F.p + x * l * aR,
            aR, (int)P, (int64_t)2 * l * aR);
  // Ap[y][l'][a][r'] (bra side, conjugated in the product)
  DBuf<cx<T>> Ap(e, s.elems());
  {
    const int64_t d[4] = {2, l, a, R};
    const int64_t st[4] = {aR, 2 * aR, R, 1};
    copy4d<T>(e.stream, Ap.p, A, d, st, 0);
  }
  const int64_t kdim = (int64_t)l * a;
  if (mode == 0) {
    DBuf<cx<T>> En(e, (size_t)P * R * R);
    // E'[P][r][r'] = sum_{(x,l',a)} F[P][(x,l',a)][r] conj(Ap[(x,l',a)][r'])
    gemm<T>(e, R, R, (int)(2 * kdim), CM<T>(F.p, R, 0, (int64_t)2 * l * aR), RM<T>(Ap.p, R, 1), En.p, R, (int)P,
            (int64_t)R * R);
    env.E = std::move(En);
  } else if (mode == 1) {
    DBuf<cx<T>> En(e, (size_t)P * 4 * R * R);
    for (int x = 0; x < 2; ++x)
      for (int y = 0; y < 2; ++y)
        gemm<T>(e, R, R, (int)kdim, CM<T>(F.p + x * l * aR, R, 0, (int64_t)2 * l * aR),
                RM<T>(Ap.p + y * l * aR, R, 1), En.p + (x * 2 + y) * (int64_t)R * R, R, (int)P, (int64_t)4 * R * R);
    env.E = std::move(En);
    env.P = P * 4;
  } else {
    DBuf<cx<T>> En(e, (size_t)P * 2 * R * R);
    for (int x = 0; x < 2; ++x)
      gemm<T>(e, R, R, (int)kdim, CM<T>(F.p + x * l * aR, R, 0, (int64_t)2 * l * aR),
              RM<T>(Ap.p + x * l * aR, R, 1), En.p + x * (int64_t)R * R, R, (int)P, (int64_t)2 * R * R);
    env.E = std::move(En);
    env.P = P * 2;
  }
  env.r = R;
}

template <typename T> static Env<T> env_start(Engine &e) {
  Env<T> env;
  env.E = DBuf<cx<T>>(e, 1);
  std::vector<cx<T>> one(1, cmk<T>(T(1), T(0)));
  MPDO_CUDA_CHECK(cudaMemcpyAsync(env.E.p, one.data(), sizeof(cx<T>), cudaMemcpyHostToDevice, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  return env;
}

template <typename T> static std::vector<cx<T>> env_fetch(Engine &e, Env<T> &env) {
  std::vector<cx<T>> h((size_t)env.P * env.r * env.r);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(h.data(), env.E.p, h.size() * sizeof(cx<T>), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  return h;
}

static void check_keep(mpdo_chain_s *ch, const int *keep, int m, int maxm) {
  if (m < 0 || m > maxm) fail(MPDO_ERR_INVALID, "too many kept qubits for a dense readout");
  for (int j = 0; j < m; ++j) {
    if (keep[j] < 0 || keep[j] >= ch->n) fail(MPDO_ERR_INVALID, "qubit index out of range");
    if (j && keep[j] <= keep[j - 1]) fail(MPDO_ERR_INVALID, "kept qubits must be strictly ascending");
  }
}

template <typename T> static void reduced_dm(mpdo_chain_s *ch, const int *keep, int m, double *out) {
  Engine &e = ch->eng->e;
  check_keep(ch, keep, m, 14);
  materialize_all<T>(ch);
  Env<T> env = env_start<T>(e);
  int j = 0;
  for (int k = 0; k < ch->n; ++k) {
    const bool open = (j < m && keep[j] == k);
    if (open) ++j;
    env_step<T>(e, env, site_ptr<T>(ch, k), ch->s[k], open ? 1 : 0, nullptr);
  }
  std::vector<cx<T>> h = env_fetch<T>(e, env);
  const int64_t D = (int64_t)1 << m;
  // P index = interleaved (x0, y0, x1, y1, ...) with x0 most significant
  for (int64_t p = 0; p < D * D; ++p) {
    int64_t row = 0, col = 0;
    for (int q = 0; q < m; ++q) {
      const int64_t bits = (p >> (2 * (m - 1 - q))) & 3;
      row = (row << 1) | (bits >> 1);
      col = (col << 1) | (bits & 1);
    }
    out[2 * (row * D + col)] = (double)h[p].x;
    out[2 * (row * D + col) + 1] = (double)h[p].y;
  }
}

template <typename T> static void probs(mpdo_chain_s *ch, const int *keep, int m, double *out) {
  Engine &e = ch->eng->e;
  check_keep(ch, keep, m, 24);
  materialize_all<T>(ch);
  Env<T> env = env_start<T>(e);
  int j = 0;
  for (int k = 0; k < ch->n; ++k) {
    const bool open = (j < m && keep[j] == k);
    if (open) ++j;
    env_step<T>(e, env, site_ptr<T>(ch, k), ch->s[k], open ? 2 : 0, nullptr);
  }
  std::vector<cx<T>> h = env_fetch<T>(e, env);
  for (int64_t p = 0; p < ((int64_t)1 << m); ++p) out[p] = (double)h[p].x;
}

template <typename T> static double expect_ops(mpdo_chain_s *ch, const int *sites, const double *ops, int m) {
  Engine &e = ch->eng->e;
  materialize_all<T>(ch);
  std::vector<const double *> opat(ch->n, nullptr);
  for (int j = 0; j < m; ++j) {
    if (sites[j] < 0 || sites[j] >= ch->n) fail(MPDO_ERR_INVALID, "qubit index out of range");
    if (opat[sites[j]]) fail(MPDO_ERR_INVALID, "operator sites must be distinct");
    opat[sites[j]] = ops + 8 * j;
  }
  Env<T> env = env_start<T>(e);
  for (int k = 0; k < ch->n; ++k) env_step<T>(e, env, site_ptr<T>(ch, k), ch->s[k], 0, opat[k]);
  std::vector<cx<T>> h = env_fetch<T>(e, env);
  return (double)h[0].x;
}

// dmOperations.py:51-66 trace_rho_rho: Tr(rho_0 rho_1), both states traced
// over the qubits not in `keep` (ascending), for any number of kept qubits.
// A left-to-right sweep of the four-layer environment E[p][q][s][t] (ket and
// bra bonds of rho_0, ket and bra bonds of rho_1): per site four GEMMs, each
// contracting one layer, with strided permutations between them.  A kept
// qubit joins rho_0's ket leg with rho_1's bra leg and rho_0's bra leg with
// rho_1's ket leg; a traced qubit joins ket and bra within each state.  The
// largest intermediate holds bond^3 x 2 x Kraus x bond elements.
template <typename T>
static double trace_rho_rho(mpdo_chain_s *c0, mpdo_chain_s *c1, const int *keep, int m) {
  Engine &e = c0->eng->e;
  check_keep(c0, keep, m, c0->n);
  materialize_all<T>(c0);
  if (c1 != c0) {
    materialize_all<T>(c1);
    MPDO_CUDA_CHECK(cudaStreamSynchronize(c1->eng->e.stream));   // its sites are read on c0's stream
  }
  const int n = c0->n;
  DBuf<cx<T>> E(e, 1);
  {
    const cx<T> one = cmk<T>(T(1), T(0));
    MPDO_CUDA_CHECK(cudaMemcpyAsync(E.p, &one, sizeof(one), cudaMemcpyHostToDevice, e.stream));
    MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  }
  int64_t p = 1, s = 1;   // E[p][q = p][s][t = s]
  auto perm = [&](int64_t elems, const cx<T> *src, std::initializer_list<int64_t> d,
                  std::initializer_list<int64_t> st) {
    DBuf<cx<T>> out(e, (size_t)elems);
    permute<T>(e.stream, out.p, src, (int)d.size(), d.begin(), st.begin(), 0);
    return out;
  };
  int j = 0;
  for (int k = 0; k < n; ++k) {
    const bool kept = j < m && keep[j] == k;
    if (kept) ++j;
    const Site S0 = c0->s[k], S1 = c1->s[k];
    if (S0.l != p || S1.l != s) fail(MPDO_ERR_BAD_SHAPE, "bond mismatch in readout");
    const cx<T> *A0 = site_ptr<T>(c0, k), *A1 = site_ptr<T>(c1, k);
    const int64_t q = p, t = s, a = S0.a, P = S0.r, b = S1.a, R = S1.r;
    // F1[q s t][x a P] = sum_p E[p][q s t] A0[p][x a P]
    const int64_t qst = q * s * t, xaP = 2 * a * P;
    DBuf<cx<T>> F1(e, (size_t)(qst * xaP));
    gemm<T>(e, (int)qst, (int)xaP, (int)p, CM<T>(E.p, qst), RM<T>(A0, xaP), F1.p, xaP);
    E.reset();
    DBuf<cx<T>> En(e, (size_t)(P * P * R * R));
    if (kept) {
      // F2[q s a P][b T] = sum_{t x} F1[q s a P][t x] conj(A1)[t x][b T]
      DBuf<cx<T>> G = perm(qst * xaP, F1.p, {q, s, a, P, t, 2}, {s * t * xaP, t * xaP, P, 1, xaP, a * P});
      F1.reset();
      DBuf<cx<T>> F2(e, (size_t)(q * s * a * P * b * R));
      gemm<T>(e, (int)(q * s * a * P), (int)(b * R), (int)(2 * t), RM<T>(G.p, 2 * t), RM<T>(A1, b * R, 1), F2.p,
              b * R);
      G.reset();
      // F4[q a P T][y S] = sum_{s b} F2[q a P T][s b] A1[s b][y S]
      DBuf<cx<T>> F3 = perm(q * s * a * P * b * R, F2.p, {q, a, P, R, s, b},
                            {s * a * P * b * R, P * b * R, b * R, 1, a * P * b * R, R});
      F2.reset();
      DBuf<cx<T>> A1p = perm(s * 2 * b * R, A1, {s, b, 2, R}, {2 * b * R, R, b * R, 1});
      DBuf<cx<T>> F4(e, (size_t)(q * a * P * R * 2 * R));
      gemm<T>(e, (int)(q * a * P * R), (int)(2 * R), (int)(s * b), RM<T>(F3.p, s * b), RM<T>(A1p.p, 2 * R), F4.p,
              2 * R);
      F3.reset();
      // F6[P T S][Q] = sum_{q y a} F4[P T S][q y a] conj(A0)[q y a][Q]
      DBuf<cx<T>> F5 = perm(q * a * P * R * 2 * R, F4.p, {P, R, R, q, 2, a},
                            {R * 2 * R, 2 * R, 1, a * P * R * 2 * R, R, P * R * 2 * R});
      F4.reset();
      DBuf<cx<T>> F6(e, (size_t)(P * R * R * P));
      gemm<T>(e, (int)(P * R * R), (int)P, (int)(q * 2 * a), RM<T>(F5.p, q * 2 * a), RM<T>(A0, P, 1), F6.p, P);
      F5.reset();
      // E[P][Q][S][T] from F6[P][T][S][Q]
      const int64_t d[4] = {P, P, R, R}, st[4] = {R * R * P, 1, P, R * P};
      copy4d<T>(e.stream, En.p, F6.p, d, st, 0);
    } else {
      // G2[s t P][Q] = sum_{q x a} F1[s t P][q x a] conj(A0)[q x a][Q]
      DBuf<cx<T>> G1 = perm(qst * xaP, F1.p, {s, t, P, q, 2, a}, {t * xaP, xaP, 1, s * t * xaP, a * P, P});
      F1.reset();
      DBuf<cx<T>> G2(e, (size_t)(s * t * P * P));
      gemm<T>(e, (int)(s * t * P), (int)P, (int)(q * 2 * a), RM<T>(G1.p, q * 2 * a), RM<T>(A0, P, 1), G2.p, P);
      G1.reset();
      // G4[t P Q][z b S] = sum_s G2[t P Q][s] A1[s][z b S]
      DBuf<cx<T>> G3 = perm(s * t * P * P, G2.p, {t, P, P, s}, {P * P, P, 1, t * P * P});
      G2.reset();
      const int64_t zbS = 2 * b * R;
      DBuf<cx<T>> G4(e, (size_t)(t * P * P * zbS));
      gemm<T>(e, (int)(t * P * P), (int)zbS, (int)s, RM<T>(G3.p, s), RM<T>(A1, zbS), G4.p, zbS);
      G3.reset();
      // E[P Q S][T] = sum_{t z b} G4[P Q S][t z b] conj(A1)[t z b][T]
      DBuf<cx<T>> G5 = perm(t * P * P * zbS, G4.p, {P, P, R, t, 2, b}, {P * zbS, zbS, 1, P * P * zbS, b * R, R});
      G4.reset();
      gemm<T>(e, (int)(P * P * R), (int)R, (int)(t * 2 * b), RM<T>(G5.p, t * 2 * b), RM<T>(A1, R, 1), En.p, R);
    }
    E = std::move(En);
    p = P;
    s = R;
  }
  cx<T> h;
  MPDO_CUDA_CHECK(cudaMemcpyAsync(&h, E.p, sizeof(h), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  return (double)h.x;
}

// Circuit.py:297-466 sample / randomSample: conditional sampling of the
// qubits `order` (ascending; the other qubits traced) in S measurement
// schemes at once, shots split into groups that share a scheme and a
// measured prefix.  Scheme s measures order[j] in basis schemes[s*L + j]
// (0: X, 1: Y, 2: Z); X and Y rotate the site by the 2 x 2 gate rot[0] or
// rot[1] first (MeasureX / MeasureY), with the same kernel as a 1q gate.
// The right environments (everything to the right traced) depend neither on
// the prefix nor on the scheme -- a unitary on a traced leg leaves the trace
// unchanged -- and are built once.  The left environment of every group
// advances one site per step, in one batched step per basis in use (mode 2
// gives the x = 0 / 1 projections of all groups), and p(x | prefix) is the
// full contraction with the right environment, plus the floor `pfloor` on
// both outcomes as in the reference.  Splits draw binomials from one seeded
// host generator per scheme, groups in order, so scheme s gives the same bits
// as a single-scheme call with seeds[s]; bit rows of a group's 1-branch come
// first.  Schemes run in chunks whose group environments fit 2 GiB.
template <typename T>
static void sample_schemes(mpdo_chain_s *ch, const int *order, int L, const int *schemes, int S, int64_t shots,
                           const uint64_t *seeds, double pfloor, const double *rot, int8_t *out) {
  Engine &e = ch->eng->e;
  check_keep(ch, order, L, ch->n);
  if (L < 1 || shots < 1 || S < 1) fail(MPDO_ERR_INVALID, "need at least one qubit, one shot and one scheme");
  for (int64_t q = 0; q < (int64_t)S * L; ++q) {
    if (schemes[q] < 0 || schemes[q] > 2) fail(MPDO_ERR_INVALID, "measurement basis must be 0 (X), 1 (Y) or 2 (Z)");
    if (schemes[q] < 2 && !rot) fail(MPDO_ERR_INVALID, "X or Y measurement without rotation gates");
  }
  materialize_all<T>(ch);
  const int n = ch->n;
  std::memset(out, 0, (size_t)S * shots * L);
  // right environments R[k] (l_k x l_k), R[n] = [1]; only R[k + 1] of
  // measured sites k is read
  std::vector<DBuf<cx<T>>> R(n + 1);
  R[n] = DBuf<cx<T>>(e, 1);
  {
    const cx<T> one = cmk<T>(T(1), T(0));
    MPDO_CUDA_CHECK(cudaMemcpyAsync(R[n].p, &one, sizeof(one), cudaMemcpyHostToDevice, e.stream));
    MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  }
  for (int k = n - 1; k > order[0]; --k) {
    const Site s = ch->s[k];
    const int rows = s.l * 2 * s.a, ar = 2 * s.a * s.r;
    DBuf<cx<T>> G(e, (size_t)rows * s.r);
    gemm<T>(e, rows, s.r, s.r, RM<T>(site_ptr<T>(ch, k), s.r), RM<T>(R[k + 1].p, s.r), G.p, s.r);
    R[k] = DBuf<cx<T>>(e, (size_t)s.l * s.l);
    gemm<T>(e, s.l, s.l, ar, RM<T>(G.p, ar), CM<T>(site_ptr<T>(ch, k), ar, 1), R[k].p, s.l);
  }
  // device bytes one group holds at once (environment, the step's
  // intermediate and its projections) at the widest site
  double per_group = 1;
  for (int k = 0; k < n; ++k) {
    const Site s = ch->s[k];
    per_group = std::max(per_group, (double)sizeof(cx<T>) *
                                        ((double)s.l * s.l + 2.0 * s.l * s.a * s.r + 4.0 * s.r * s.r));
  }
  const double budget = 2.0 * (1 << 30);
  const double groups_per_scheme = (double)(L >= 62 ? shots : std::min<int64_t>(shots, (int64_t)1 << L));
  const int chunk = (int)std::max(1.0, std::min((double)S, std::floor(budget / (per_group * groups_per_scheme))));

  struct Grp { int s; int64_t start, len; };
  for (int s0 = 0; s0 < S; s0 += chunk) {
    const int s1 = std::min(S, s0 + chunk);
    std::vector<Grp> groups;
    std::vector<int> genv;                                   // environment of each group
    std::vector<std::mt19937_64> rng;
    for (int s = s0; s < s1; ++s) {
      groups.push_back({s, (int64_t)s * shots, shots});
      genv.push_back(0);
      rng.emplace_back(seeds[s]);
    }
    Env<T> env = env_start<T>(e);
    int j = 0;
    for (int k = 0; k < n && j < L; ++k) {
      const Site st = ch->s[k];
      if (order[j] != k) {
        env_step<T>(e, env, site_ptr<T>(ch, k), st, 0, nullptr);
        continue;
      }
      const int G = (int)groups.size();
      std::vector<int> by[3];
      for (int g = 0; g < G; ++g) by[schemes[(size_t)groups[g].s * L + j]].push_back(g);
      const int64_t msz = (int64_t)st.r * st.r;
      const int64_t esz = (int64_t)env.r * env.r;
      DBuf<cx<T>> proj(e, (size_t)2 * G * msz);              // per group (in basis order): x = 0, 1
      std::vector<int> pos(G);
      int off = 0;
      for (int b = 0; b < 3; ++b) {
        if (by[b].empty()) continue;
        const int Gb = (int)by[b].size();
        Env<T> sub;
        sub.r = env.r;
        sub.P = Gb;
        bool ident = Gb == G && Gb == (int)env.P;   // every group, in environment order
        for (int i = 0; i < Gb && ident; ++i) ident = genv[by[b][i]] == i;
        if (ident) {
          sub.E = std::move(env.E);
        } else {
          std::vector<int> src(Gb);
          for (int i = 0; i < Gb; ++i) src[i] = genv[by[b][i]];
          DBuf<int> idx(e, Gb);
          MPDO_CUDA_CHECK(cudaMemcpyAsync(idx.p, src.data(), Gb * sizeof(int), cudaMemcpyHostToDevice, e.stream));
          sub.E = DBuf<cx<T>>(e, (size_t)Gb * esz);
          gather_mats<T>(e.stream, env.E.p, sub.E.p, idx.p, esz, Gb);
          MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));   // (src is pageable host data)
        }
        DBuf<cx<T>> Ar;
        const cx<T> *A = site_ptr<T>(ch, k);
        if (b < 2) {
          Ar = DBuf<cx<T>>(e, st.elems());
          prof(e, K_KRAUS1Q, 8.0 * 2 * 2 * st.elems(), (double)sizeof(cx<T>) * st.elems() * 2,
               [&] { kraus1q<T>(e.stream, A, Ar.p, st.l, st.a, st.r, rot + 8 * b, 1); });
          A = Ar.p;
        }
        env_step<T>(e, sub, A, st, 2, nullptr);
        MPDO_CUDA_CHECK(cudaMemcpyAsync(proj.p + (size_t)2 * off * msz, sub.E.p, sizeof(cx<T>) * 2 * Gb * msz,
                                        cudaMemcpyDeviceToDevice, e.stream));
        for (int i = 0; i < Gb; ++i) pos[by[b][i]] = off + i;
        off += Gb;
      }
      DBuf<double> pr(e, 2 * G);
      env_dot<T>(e.stream, proj.p, R[k + 1].p, msz, 2 * G, pr.p);
      std::vector<double> hp(2 * G);
      MPDO_CUDA_CHECK(cudaMemcpyAsync(hp.data(), pr.p, 2 * G * sizeof(double), cudaMemcpyDeviceToHost, e.stream));
      MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
      std::vector<Grp> next;
      std::vector<int> parent;
      for (int g = 0; g < G; ++g) {
        const int pg = pos[g];
        const double p0 = hp[2 * pg] + pfloor, p1 = hp[2 * pg + 1] + pfloor;
        if (!(p0 >= 0) || !(p1 >= 0))
          fail(MPDO_ERR_NONFINITE, "State is illegal: conditional probabilities " + std::to_string(p0) + ", " +
                                       std::to_string(p1));
        const double q = p1 / (p0 + p1);
        const int64_t len = groups[g].len;
        int64_t k1;
        if (q < pfloor) k1 = 0;
        else if (q > 1 - pfloor) k1 = len;
        else k1 = std::binomial_distribution<int64_t>(len, q)(rng[groups[g].s - s0]);
        for (int64_t r = 0; r < k1; ++r) out[(size_t)(groups[g].start + r) * L + j] = 1;
        if (k1 > 0) { next.push_back({groups[g].s, groups[g].start, k1}); parent.push_back(2 * pg + 1); }
        if (len - k1 > 0) { next.push_back({groups[g].s, groups[g].start + k1, len - k1}); parent.push_back(2 * pg); }
      }
      ++j;
      if (j == L) break;
      DBuf<int> idx(e, parent.size());
      MPDO_CUDA_CHECK(cudaMemcpyAsync(idx.p, parent.data(), parent.size() * sizeof(int), cudaMemcpyHostToDevice,
                                      e.stream));
      DBuf<cx<T>> En(e, (size_t)parent.size() * msz);
      gather_mats<T>(e.stream, proj.p, En.p, idx.p, msz, (int)parent.size());
      MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));   // (parent is pageable host data)
      env.E = std::move(En);
      env.P = (int64_t)parent.size();
      env.r = st.r;
      groups.swap(next);
      genv.resize(groups.size());
      for (size_t g = 0; g < groups.size(); ++g) genv[g] = (int)g;
    }
  }
}

template <typename T>
static void sample_chain(mpdo_chain_s *ch, const int *order, int L, int64_t shots, uint64_t seed, double pfloor,
                         int8_t *out) {
  std::vector<int> z((size_t)std::max(L, 1), 2);
  sample_schemes<T>(ch, order, L, z.data(), 1, shots, &seed, pfloor, nullptr, out);
}

// ------------------------------------------------------------ status ----
int *status_slot(Engine &e, int count) {
  if (e.status_used + count > e.status_cap) check_status(e);
  int *p = e.d_status + e.status_used;
  e.status_used += count;
  return p;
}
void check_status(Engine &e) {
  if (e.status_used == 0) return;
  std::vector<int> h(e.status_used);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(h.data(), e.d_status, h.size() * sizeof(int), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  for (int v : h)
    if (v != 0 && e.first_status == 0) e.first_status = v;
  MPDO_CUDA_CHECK(cudaMemsetAsync(e.d_status, 0, e.status_cap * sizeof(int), e.stream));
  e.status_used = 0;
}

// instantiations of the factorisation steps shared with the adjoint
#define MPDO_INST_CORE(T)                                                                                 \
  template void qr<T>(Engine &, int, int, const View<T> &, cx<T> *, cx<T> *);                            \
  template void qr_r_batched<T>(Engine &, int, int, int, const View<T> &, cx<T> *);                      \
  template void right_svd<T>(Engine &, int, int, const View<T> &, DBuf<cx<T>> &, DBuf<T> &);            \
  template int error_rule_keep<T>(const std::vector<T> &, int, int, double, bool, double);               \
  template void materialize_all<T>(mpdo_chain_s *);
MPDO_INST_CORE(float)
MPDO_INST_CORE(double)

}  // namespace mpdo

// ================================================================ C ABI ====
using namespace mpdo;

#define DISPATCH(ch, FN, ...)                        \
  do {                                               \
    if ((ch)->dtype == MPDO_C64) FN<float>(__VA_ARGS__); \
    else FN<double>(__VA_ARGS__);                    \
  } while (0)

static void need(bool c, const char *msg) {
  if (!c) fail(MPDO_ERR_INVALID, msg);
}
static void set_device(mpdo_engine_s *eng) { MPDO_CUDA_CHECK(cudaSetDevice(eng->e.device)); }

template <typename T>
static void chain_init(mpdo_chain_s *ch, const double *vec) {
  Engine &e = ch->eng->e;
  for (int i = 0; i < ch->n; ++i) {
    cx<T> h[2] = {cmk<T>((T)vec[4 * i], (T)vec[4 * i + 1]), cmk<T>((T)vec[4 * i + 2], (T)vec[4 * i + 3])};
    cx<T> *p = static_cast<cx<T> *>(dalloc(e, 2 * sizeof(cx<T>)));
    MPDO_CUDA_CHECK(cudaMemcpyAsync(p, h, sizeof(h), cudaMemcpyHostToDevice, e.stream));
    ch->s[i] = Site{p, 1, 1, 1};
  }
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
}

template <typename T> static void read_site(mpdo_chain_s *ch, int site, double *out) {
  Engine &e = ch->eng->e;
  materialize_touching<T>(ch, site);
  const size_t n = ch->s[site].elems();
  std::vector<cx<T>> h(n);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(h.data(), ch->s[site].p, n * sizeof(cx<T>), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  for (size_t i = 0; i < n; ++i) { out[2 * i] = h[i].x; out[2 * i + 1] = h[i].y; }
}

template <typename T> static void write_site(mpdo_chain_s *ch, int site, const int dims[4], const double *in) {
  Engine &e = ch->eng->e;
  ch->pend1[site].on = false;                 // replaced by the written tensor
  materialize_touching<T>(ch, site);
  const size_t n = (size_t)dims[0] * 2 * dims[2] * dims[3];
  std::vector<cx<T>> h(n);
  for (size_t i = 0; i < n; ++i) h[i] = cmk<T>((T)in[2 * i], (T)in[2 * i + 1]);
  cx<T> *p = static_cast<cx<T> *>(dalloc(e, n * sizeof(cx<T>)));
  MPDO_CUDA_CHECK(cudaMemcpyAsync(p, h.data(), n * sizeof(cx<T>), cudaMemcpyHostToDevice, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  set_site<T>(ch, site, p, dims[0], dims[2], dims[3]);
}

// A caller's buffer for the device-memory site copies must be device (or
// managed) memory that the engine's device can address.
static void need_device_buffer(const Engine &e, const void *p) {
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    fail(MPDO_ERR_INVALID, "the site buffer is not device memory");
  }
  if (attr.type == cudaMemoryTypeManaged) return;
  if (attr.type != cudaMemoryTypeDevice)
    fail(MPDO_ERR_INVALID, "the site buffer is not device memory (host or unregistered pointer)");
  if (attr.device != e.device)
    fail(MPDO_ERR_INVALID, "the site buffer is on device " + std::to_string(attr.device) + ", the chain on device " +
                               std::to_string(e.device));
}

template <typename T> static void read_site_device(mpdo_chain_s *ch, int site, void *out) {
  Engine &e = ch->eng->e;
  need_device_buffer(e, out);
  materialize_touching<T>(ch, site);
  const size_t n = ch->s[site].elems();
  MPDO_CUDA_CHECK(cudaMemcpyAsync(out, ch->s[site].p, n * sizeof(cx<T>), cudaMemcpyDeviceToDevice, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
}

template <typename T>
static void write_site_device(mpdo_chain_s *ch, int site, const int dims[4], const void *in) {
  Engine &e = ch->eng->e;
  need_device_buffer(e, in);
  ch->pend1[site].on = false;                 // replaced by the written tensor
  materialize_touching<T>(ch, site);
  const size_t n = (size_t)dims[0] * 2 * dims[2] * dims[3];
  cx<T> *p = static_cast<cx<T> *>(dalloc(e, n * sizeof(cx<T>)));
  MPDO_CUDA_CHECK(cudaMemcpyAsync(p, in, n * sizeof(cx<T>), cudaMemcpyDeviceToDevice, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  set_site<T>(ch, site, p, dims[0], dims[2], dims[3]);
}

// ------------------------------------------------------- test hooks -----
template <typename T> static std::vector<cx<T>> to_cx(const double *h, size_t n) {
  std::vector<cx<T>> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = cmk<T>((T)h[2 * i], (T)h[2 * i + 1]);
  return v;
}
template <typename T> static void from_cx(const std::vector<cx<T>> &v, double *h) {
  for (size_t i = 0; i < v.size(); ++i) { h[2 * i] = v[i].x; h[2 * i + 1] = v[i].y; }
}
template <typename T>
static void debug_qr(Engine &e, int m, int n, const double *a, double *q, double *r) {
  const int k = std::min(m, n);
  std::vector<cx<T>> ha = to_cx<T>(a, (size_t)m * n);
  DBuf<cx<T>> A(e, ha.size()), Q(e, (size_t)m * k), R(e, (size_t)k * n);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(A.p, ha.data(), ha.size() * sizeof(cx<T>), cudaMemcpyHostToDevice, e.stream));
  qr<T>(e, m, n, RM<T>(A.p, n), Q.p, R.p);
  std::vector<cx<T>> hq((size_t)m * k), hr((size_t)k * n);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(hq.data(), Q.p, hq.size() * sizeof(cx<T>), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaMemcpyAsync(hr.data(), R.p, hr.size() * sizeof(cx<T>), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  from_cx<T>(hq, q);
  from_cx<T>(hr, r);
}
template <typename T>
static void debug_split(Engine &e, int Mr, int Nc, int keep, const double *y, double *l, double *r) {
  std::vector<cx<T>> hy = to_cx<T>(y, (size_t)Mr * Nc);
  DBuf<cx<T>> Y(e, hy.size()), Lf, Rf;
  MPDO_CUDA_CHECK(cudaMemcpyAsync(Y.p, hy.data(), hy.size() * sizeof(cx<T>), cudaMemcpyHostToDevice, e.stream));
  int kept = 0;
  svd_split<T>(e, Y.p, Mr, Nc, [&](const T *, int) { return keep; }, Lf, Rf, kept, nullptr, keep);
  std::vector<cx<T>> hl((size_t)Mr * keep), hr((size_t)keep * Nc);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(hl.data(), Lf.p, hl.size() * sizeof(cx<T>), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaMemcpyAsync(hr.data(), Rf.p, hr.size() * sizeof(cx<T>), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  from_cx<T>(hl, l);
  from_cx<T>(hr, r);
}
template <typename T>
static void debug_svd(Engine &e, int m, int n, const double *a, double *w, double *sv) {
  std::vector<cx<T>> ha = to_cx<T>(a, (size_t)m * n);
  DBuf<cx<T>> A(e, ha.size()), W;
  DBuf<T> S;
  MPDO_CUDA_CHECK(cudaMemcpyAsync(A.p, ha.data(), ha.size() * sizeof(cx<T>), cudaMemcpyHostToDevice, e.stream));
  right_svd<T>(e, m, n, RM<T>(A.p, n), W, S);
  std::vector<cx<T>> hw((size_t)n * n);
  std::vector<T> hs(n);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(hw.data(), W.p, hw.size() * sizeof(cx<T>), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaMemcpyAsync(hs.data(), S.p, n * sizeof(T), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  from_cx<T>(hw, w);
  for (int i = 0; i < n; ++i) sv[i] = hs[i];
}

extern "C" {

int mpdo_abi_version(void) { return MPDO_ABI_VERSION; }

const char *mpdo_status_string(mpdo_status s) {
  switch (s) {
    case MPDO_OK: return "ok";
    case MPDO_ERR_INVALID: return "invalid argument";
    case MPDO_ERR_BAD_SHAPE: return "bad shape";
    case MPDO_ERR_OOM: return "out of device memory";
    case MPDO_ERR_CUDA: return "CUDA error";
    case MPDO_ERR_NOT_CONVERGED: return "Jacobi iteration did not converge";
    case MPDO_ERR_NONFINITE: return "non-finite value in a factorisation";
    case MPDO_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

const char *mpdo_last_error(void) { return g_last_error.c_str(); }

mpdo_status mpdo_engine_create(int device, mpdo_engine_t *out) {
  return guard([&] {
    need(out != nullptr, "out is NULL");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      fail(MPDO_ERR_NO_DEVICE, "no CUDA device available");
    }
    need(device >= 0 && device < ndev, "device index out of range");
    auto eng = std::make_unique<mpdo_engine_s>();
    Engine &e = eng->e;
    e.device = device;
    MPDO_CUDA_CHECK(cudaSetDevice(device));
    MPDO_CUDA_CHECK(cudaStreamCreateWithFlags(&e.own_stream, cudaStreamNonBlocking));
    e.stream = e.own_stream;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    MPDO_CUDA_CHECK(cudaMemPoolCreate(&e.pool, &props));
    uint64_t thr = UINT64_MAX;
    MPDO_CUDA_CHECK(cudaMemPoolSetAttribute(e.pool, cudaMemPoolAttrReleaseThreshold, &thr));
    MPDO_CUDA_CHECK(cudaMalloc(&e.d_status, e.status_cap * sizeof(int)));
    MPDO_CUDA_CHECK(cudaMemsetAsync(e.d_status, 0, e.status_cap * sizeof(int), e.stream));
    *out = eng.release();
  });
}

mpdo_status mpdo_engine_destroy(mpdo_engine_t eng) {
  return guard([&] {
    if (!eng) return;
    Engine &e = eng->e;
    cudaSetDevice(e.device);
    release_cache(e);
    cudaStreamSynchronize(e.stream);
    if (e.d_status) cudaFree(e.d_status);
    if (e.pool) cudaMemPoolDestroy(e.pool);
    if (e.own_stream) cudaStreamDestroy(e.own_stream);
    delete eng;
  });
}

mpdo_status mpdo_engine_set_stream(mpdo_engine_t eng, void *stream) {
  return guard([&] {
    need(eng != nullptr, "engine is NULL");
    Engine &e = eng->e;
    MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
    e.stream = stream ? static_cast<cudaStream_t>(stream) : e.own_stream;
  });
}

mpdo_status mpdo_engine_set_option(mpdo_engine_t eng, const char *name, double value) {
  return guard([&] {
    need(eng && name, "NULL argument");
    const std::string k(name);
    Engine &e = eng->e;
    if (k == "fuse_2q") e.fuse_2q = value != 0;
    else if (k == "defer_1q") e.defer_1q = value != 0;
    else if (k == "wide_range") e.wide_range = value > 0 ? 1 : (value < 0 ? -1 : 0);
    else if (k == "wide_eig") e.wide_eig = value > 0 ? 1 : (value < 0 ? -1 : 0);
    else if (k == "wide_eig_from") {
      need(value >= 2 && value <= 1e9, "wide_eig_from out of range");
      e.wide_eig_from = (int)value;
    }
    else if (k == "wide_range_tol") {
      need(value > 0, "wide_range_tol must be positive");
      e.wide_range_tol = value;
    }
    else if (k == "bjacobi_bs") {
      need(value >= 0 && value <= 64, "bjacobi_bs out of range");
      e.bjacobi_bs = (int)value;
    }
    else if (k == "bjacobi_fused") e.bjacobi_fused = value != 0;
    else if (k == "tsqr_ratio") {
      need(value >= 1.0 && value <= 64.0, "tsqr_ratio out of range");
      e.tsqr_ratio = value;
    }
    else if (k == "wide_oversample") {
      need(value >= 0 && value <= 256, "wide_oversample out of range");
      e.wide_oversample = (int)value;
    }
    else if (k == "max_sweeps") { need(value >= 1 && value <= 1000, "max_sweeps out of range"); e.max_sweeps = (int)value; }
    else fail(MPDO_ERR_INVALID, "unknown option: " + k);
  });
}

mpdo_status mpdo_engine_profile(mpdo_engine_t eng, int enable) {
  return guard([&] {
    need(eng != nullptr, "engine is NULL");
    Engine &e = eng->e;
    prof_flush(e);
    for (int c = 0; c < kProfClasses; ++c) { e.acc_ms[c] = e.acc_flops[c] = e.acc_bytes[c] = 0; e.acc_n[c] = 0; }
    e.wide_range_hits = e.wide_exact_calls = e.wide_eig_calls = 0;
    e.wide_resid_max = 0;
    e.profiling = enable != 0;
  });
}

mpdo_status mpdo_engine_profile_read(mpdo_engine_t eng, int kclass, long long *launches, double *ms, double *flops,
                                     double *bytes) {
  return guard([&] {
    need(eng && launches && ms && flops && bytes, "NULL argument");
    need(kclass >= 0 && kclass < kProfClasses, "kernel class out of range");
    Engine &e = eng->e;
    prof_flush(e);
    if (kclass == 7) {   // wide-bond SVD path counters: range finder accepted / exact block Jacobi
      *launches = e.wide_range_hits;
      *ms = (double)e.wide_eig_calls;
      *flops = (double)e.wide_exact_calls;
      *bytes = e.wide_resid_max;
      return;
    }
    *launches = e.acc_n[kclass];
    *ms = e.acc_ms[kclass];
    *flops = e.acc_flops[kclass];
    *bytes = e.acc_bytes[kclass];
  });
}

mpdo_status mpdo_engine_sync(mpdo_engine_t eng) {
  mpdo_status st = guard([&] {
    need(eng != nullptr, "engine is NULL");
    set_device(eng);
    check_status(eng->e);
    MPDO_CUDA_CHECK(cudaStreamSynchronize(eng->e.stream));
    MPDO_CUDA_CHECK(cudaGetLastError());
  });
  if (st != MPDO_OK) return st;
  const int fs = eng->e.first_status;
  eng->e.first_status = 0;
  if (fs == DEV_NOT_CONVERGED) { g_last_error = "Jacobi sweep limit reached"; return MPDO_ERR_NOT_CONVERGED; }
  if (fs == DEV_NONFINITE) { g_last_error = "non-finite value met in a factorisation"; return MPDO_ERR_NONFINITE; }
  return MPDO_OK;
}

mpdo_status mpdo_engine_launch_count(mpdo_engine_t eng, uint64_t *count) {
  return guard([&] {
    need(eng != nullptr && count != nullptr, "NULL argument");
    *count = launch_count();
  });
}

mpdo_status mpdo_launch_histogram(char *buf, int len) {
  return guard([&] {
    need(buf != nullptr && len > 0, "buffer is NULL");
    const char *names[128];
    uint64_t counts[128];
    const int n = launch_histogram(names, counts, 128);
    std::string out;
    for (int i = 0; i < n; ++i) out += std::string(names[i]) + " " + std::to_string(counts[i]) + "\n";
    std::strncpy(buf, out.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  });
}


mpdo_status mpdo_chain_create(mpdo_engine_t eng, int n, int dtype, const double *vectors, int connected_,
                              mpdo_chain_t *out) {
  return guard([&] {
    need(eng && vectors && out, "NULL argument");
    need(n >= 1, "n must be >= 1");
    need(dtype == MPDO_C64 || dtype == MPDO_C128, "dtype must be MPDO_C64 or MPDO_C128");
    set_device(eng);
    auto ch = std::make_unique<mpdo_chain_s>();
    ch->eng = eng;
    ch->n = n;
    ch->dtype = dtype;
    ch->s.assign(n, Site{});
    ch->bond.assign(std::max(0, n - 1), connected_ ? 1 : 0);
    ch->pend.assign(std::max(0, n - 1), Pend{});
    ch->pend1.assign(n, Pend{});
    if (dtype == MPDO_C64) chain_init<float>(ch.get(), vectors);
    else chain_init<double>(ch.get(), vectors);
    *out = ch.release();
  });
}

mpdo_status mpdo_chain_destroy(mpdo_chain_t ch) {
  return guard([&] {
    if (!ch) return;
    set_device(ch->eng);
    for (auto &s : ch->s)
      if (s.p) dfree(ch->eng->e, s.p);
    delete ch;
  });
}

mpdo_status mpdo_chain_clone(mpdo_chain_t src, mpdo_chain_t *out) {
  return guard([&] {
    need(src && out, "NULL argument");
    set_device(src->eng);
    Engine &e = src->eng->e;
    auto ch = std::make_unique<mpdo_chain_s>(*src);
    const size_t esz = src->dtype == MPDO_C64 ? 8 : 16;
    for (int i = 0; i < ch->n; ++i) {
      void *p = dalloc(e, src->s[i].elems() * esz);
      MPDO_CUDA_CHECK(cudaMemcpyAsync(p, src->s[i].p, src->s[i].elems() * esz, cudaMemcpyDeviceToDevice, e.stream));
      ch->s[i].p = p;
    }
    *out = ch.release();
  });
}

mpdo_status mpdo_chain_num_sites(mpdo_chain_t ch, int *n) {
  return guard([&] {
    need(ch && n, "NULL argument");
    *n = ch->n;
  });
}

mpdo_status mpdo_chain_site_dims(mpdo_chain_t ch, int site, int dims[4]) {
  return guard([&] {
    need(ch && dims, "NULL argument");
    need(site >= 0 && site < ch->n, "site out of range");
    set_device(ch->eng);
    DISPATCH(ch, materialize_touching, ch, site);
    dims[0] = ch->s[site].l; dims[1] = 2; dims[2] = ch->s[site].a; dims[3] = ch->s[site].r;
  });
}

mpdo_status mpdo_chain_bond_present(mpdo_chain_t ch, int bond, int *present) {
  return guard([&] {
    need(ch && present, "NULL argument");
    need(bond >= 0 && bond < ch->n - 1, "bond out of range");
    *present = ch->bond[bond] ? 1 : 0;
  });
}


mpdo_status mpdo_chain_read_site(mpdo_chain_t ch, int site, double *host_out) {
  return guard([&] {
    need(ch && host_out, "NULL argument");
    need(site >= 0 && site < ch->n, "site out of range");
    set_device(ch->eng);
    DISPATCH(ch, read_site, ch, site, host_out);
  });
}


mpdo_status mpdo_chain_write_site(mpdo_chain_t ch, int site, const int dims[4], const double *host_in) {
  return guard([&] {
    need(ch && dims && host_in, "NULL argument");
    need(site >= 0 && site < ch->n, "site out of range");
    need(dims[0] >= 1 && dims[1] == 2 && dims[2] >= 1 && dims[3] >= 1, "bad site dims");
    set_device(ch->eng);
    DISPATCH(ch, write_site, ch, site, dims, host_in);
  });
}

mpdo_status mpdo_chain_read_site_device(mpdo_chain_t ch, int site, void *dev_out) {
  return guard([&] {
    need(ch && dev_out, "NULL argument");
    need(site >= 0 && site < ch->n, "site out of range");
    set_device(ch->eng);
    DISPATCH(ch, read_site_device, ch, site, dev_out);
  });
}

mpdo_status mpdo_chain_write_site_device(mpdo_chain_t ch, int site, const int dims[4], const void *dev_in) {
  return guard([&] {
    need(ch && dims && dev_in, "NULL argument");
    need(site >= 0 && site < ch->n, "site out of range");
    need(dims[0] >= 1 && dims[1] == 2 && dims[2] >= 1 && dims[3] >= 1, "bad site dims");
    set_device(ch->eng);
    DISPATCH(ch, write_site_device, ch, site, dims, dev_in);
  });
}

mpdo_status mpdo_apply_1q(mpdo_chain_t ch, int site, const double *kraus, int K) {
  return guard([&] {
    need(ch && kraus, "NULL argument");
    need(site >= 0 && site < ch->n, "Qubit index out of range");
    need(K >= 1 && K <= 16, "K must be in [1, 16]");
    set_device(ch->eng);
    DISPATCH(ch, apply_1q, ch, site, kraus, K);
  });
}

mpdo_status mpdo_apply_2q(mpdo_chain_t ch, int site_min, const double *kraus, int K, double abs_cutoff) {
  return guard([&] {
    need(ch && kraus, "NULL argument");
    need(ch->n >= 2 && site_min >= 0 && site_min < ch->n - 1, "Qubit index out of range");
    need(K >= 1 && K <= 16, "K must be in [1, 16]");
    set_device(ch->eng);
    DISPATCH(ch, apply_2q, ch, site_min, kraus, K, abs_cutoff);
  });
}

mpdo_status mpdo_truncate(mpdo_chain_t ch, int chi, int kappa, double max_err, int noisy, double *discarded_out) {
  return guard([&] {
    need(ch != nullptr, "NULL argument");
    set_device(ch->eng);
    DISPATCH(ch, truncate_layer, ch, chi, kappa, max_err, noisy, discarded_out);
  });
}

mpdo_status mpdo_kappa_truncate(mpdo_chain_t ch, int kappa, double max_err) {
  return guard([&] {
    need(ch != nullptr, "NULL argument");
    set_device(ch->eng);
    DISPATCH(ch, materialize_all, ch);
    DISPATCH(ch, kappa_pass, ch, kappa, max_err);
  });
}

mpdo_status mpdo_qr_left2right(mpdo_chain_t ch) {
  return guard([&] {
    need(ch != nullptr, "NULL argument");
    need(connected(ch), "qr_left2right needs every neighbouring pair to share a bond");
    set_device(ch->eng);
    DISPATCH(ch, qr_left2right_only, ch);
  });
}

mpdo_status mpdo_svd_right2left(mpdo_chain_t ch, int chi, double max_err, double *discarded_out) {
  return guard([&] {
    need(ch != nullptr, "NULL argument");
    need(connected(ch), "svd_right2left needs every neighbouring pair to share a bond");
    set_device(ch->eng);
    DISPATCH(ch, svd_right2left_only, ch, chi, max_err, discarded_out);
  });
}

mpdo_status mpdo_svd_left2right(mpdo_chain_t ch, int chi, double max_err, double *discarded_out) {
  return guard([&] {
    need(ch != nullptr, "NULL argument");
    need(connected(ch), "svd_left2right needs every neighbouring pair to share a bond");
    set_device(ch->eng);
    DISPATCH(ch, svd_left2right_only, ch, chi, max_err, discarded_out);
  });
}

mpdo_status mpdo_reduced_dm(mpdo_chain_t ch, const int *keep, int m, double *host_out) {
  return guard([&] {
    need(ch && host_out && (keep || m == 0), "NULL argument");
    set_device(ch->eng);
    DISPATCH(ch, reduced_dm, ch, keep, m, host_out);
  });
}

mpdo_status mpdo_trace_rho_rho(mpdo_chain_t a, mpdo_chain_t b, const int *keep, int m, double *out) {
  return guard([&] {
    need(a && b && out && (keep || m == 0), "NULL argument");
    need(a->n == b->n && a->dtype == b->dtype, "the two states need the same qubit count and precision");
    set_device(a->eng);
    *out = a->dtype == MPDO_C64 ? trace_rho_rho<float>(a, b, keep, m) : trace_rho_rho<double>(a, b, keep, m);
  });
}

mpdo_status mpdo_probs(mpdo_chain_t ch, const int *keep, int m, double *host_out) {
  return guard([&] {
    need(ch && host_out && (keep || m == 0), "NULL argument");
    set_device(ch->eng);
    DISPATCH(ch, probs, ch, keep, m, host_out);
  });
}

mpdo_status mpdo_expect_ops(mpdo_chain_t ch, const int *sites, const double *ops, int m, double *out) {
  return guard([&] {
    need(ch && out && ((sites && ops) || m == 0), "NULL argument");
    set_device(ch->eng);
    if (ch->dtype == MPDO_C64) *out = expect_ops<float>(ch, sites, ops, m);
    else *out = expect_ops<double>(ch, sites, ops, m);
  });
}

mpdo_status mpdo_sample(mpdo_chain_t ch, const int *order, int L, int64_t shots, uint64_t seed, double pfloor,
                        int8_t *bits_out) {
  return guard([&] {
    need(ch && order && bits_out, "NULL argument");
    set_device(ch->eng);
    if (ch->dtype == MPDO_C64) sample_chain<float>(ch, order, L, shots, seed, pfloor, bits_out);
    else sample_chain<double>(ch, order, L, shots, seed, pfloor, bits_out);
  });
}

mpdo_status mpdo_sample_schemes(mpdo_chain_t ch, const int *order, int L, const int *schemes, int S, int64_t shots,
                                const uint64_t *seeds, double pfloor, const double *rot, int8_t *bits_out) {
  return guard([&] {
    need(ch && order && schemes && seeds && bits_out, "NULL argument");
    set_device(ch->eng);
    if (ch->dtype == MPDO_C64) sample_schemes<float>(ch, order, L, schemes, S, shots, seeds, pfloor, rot, bits_out);
    else sample_schemes<double>(ch, order, L, schemes, S, shots, seeds, pfloor, rot, bits_out);
  });
}

mpdo_status mpdo_expect_pauli_batch(mpdo_chain_t ch, const int8_t *paulis, int nterms, double *out) {
  static const double PM[4][8] = {{1, 0, 0, 0, 0, 0, 1, 0},
                                  {0, 0, 1, 0, 1, 0, 0, 0},
                                  {0, 0, 0, -1, 0, 1, 0, 0},
                                  {1, 0, 0, 0, 0, 0, -1, 0}};
  return guard([&] {
    need(ch && out && (paulis || nterms == 0), "NULL argument");
    set_device(ch->eng);
    for (int t = 0; t < nterms; ++t) {
      std::vector<int> sites;
      std::vector<double> ops;
      for (int q = 0; q < ch->n; ++q) {
        const int p = paulis[(size_t)t * ch->n + q];
        need(p >= 0 && p <= 3, "Pauli code must be 0..3");
        if (p == 0) continue;
        sites.push_back(q);
        ops.insert(ops.end(), PM[p], PM[p] + 8);
      }
      if (ch->dtype == MPDO_C64) out[t] = expect_ops<float>(ch, sites.data(), ops.data(), (int)sites.size());
      else out[t] = expect_ops<double>(ch, sites.data(), ops.data(), (int)sites.size());
    }
  });
}

mpdo_status mpdo_debug_qr(mpdo_engine_t eng, int dtype, int m, int n, const double *a, double *q, double *r) {
  return guard([&] {
    need(eng && a && q && r && m > 0 && n > 0, "bad argument");
    set_device(eng);
    if (dtype == MPDO_C64) debug_qr<float>(eng->e, m, n, a, q, r);
    else debug_qr<double>(eng->e, m, n, a, q, r);
  });
}

mpdo_status mpdo_debug_split(mpdo_engine_t eng, int dtype, int m, int n, int keep, const double *y, double *l,
                             double *r) {
  return guard([&] {
    need(eng && y && l && r && m > 0 && n > 0 && keep > 0, "bad argument");
    set_device(eng);
    if (dtype == MPDO_C64) debug_split<float>(eng->e, m, n, keep, y, l, r);
    else debug_split<double>(eng->e, m, n, keep, y, l, r);
  });
}

mpdo_status mpdo_keep_count(const double *s, int len, int nsv, int max_sv, double err, int relative, int *keep) {
  return guard([&] {
    need(keep != nullptr && (s != nullptr || len == 0) && len >= 0 && nsv >= 0 && max_sv >= 0, "bad argument");
    const std::vector<double> v(s, s + len);
    *keep = error_rule_keep<double>(v, nsv, max_sv, err, relative != 0);
  });
}

mpdo_status mpdo_debug_svd(mpdo_engine_t eng, int dtype, int m, int n, const double *a, double *w,
                           double *sigma) {
  return guard([&] {
    need(eng && a && w && sigma && m > 0 && n > 0 && n <= 1024, "bad argument");
    set_device(eng);
    if (dtype == MPDO_C64) debug_svd<float>(eng->e, m, n, a, w, sigma);
    else debug_svd<double>(eng->e, m, n, a, w, sigma);
  });
}

}  // extern "C"
