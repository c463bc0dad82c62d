// Host-side launchers of the engine's CUDA kernels.  All launchers enqueue on
// the given stream and never synchronise.
#pragma once

#include "common.cuh"

#include <string>

namespace mpdo {

// ---------------------------------------------------------------- GEMM ----
// C[b](i,j) = alpha * sum_k A[b](i,k) B[b](k,j) + beta * C[b](i,j)
// for i < M, j < N, b < batch; A, B are strided (optionally conjugated) views;
// C is written with strides (c_rs, c_cs, c_bs).  beta == 0 never reads C.
template <typename T>
void cgemm(cudaStream_t st, int M, int N, int K, int batch, cx<T> alpha, const View<T> &A,
           const View<T> &B, cx<T> beta, cx<T> *C, int64_t c_rs, int64_t c_cs, int64_t c_bs,
           cx<T> *splitk_ws = nullptr, size_t splitk_ws_elems = 0);

// -------------------------------------------------- Householder QR (TSQR) --
// Factor nchunks independent row blocks of an m x n matrix given by `in`
// (chunk c holds rows [c*mc, min(m, (c+1)*mc))).  Per chunk: the Householder
// vectors and tau are kept in `vws` (mc x n column-major per chunk) and `tau`
// (n per chunk); R_c (kc x n, kc = min(rows_c, n)) is written row-major into
// `rstack` at row offset c*n (rows kc..n-1 of the slot are zero-filled).
// batch > 1 factors that many matrices (input b at in.bs * b), each with its
// own consecutive nchunks slots of vws / tau / rstack.
template <typename T>
void qr_factor_chunks(cudaStream_t st, int m, int n, int mc, int nchunks, const View<T> &in, cx<T> *vws,
                      cx<T> *tau, cx<T> *rstack, int batch = 1);

// Q_c = H_c(0) ... H_c(kc-1) [B_c; 0] for every chunk, where B_c is the
// kc x nq block of `bin` (row-major, leading dimension ldb) starting at row
// c*n, or the identity when bin == nullptr.  Q_c is written into `qout`
// (row-major m x nq, leading dimension ldq) at rows [c*mc, c*mc + rows_c).
template <typename T>
void qr_apply_chunks(cudaStream_t st, int m, int n, int mc, int nchunks, const cx<T> *vws, const cx<T> *tau,
                     const cx<T> *bin, int64_t ldb, int nq, cx<T> *qout, int64_t ldq);

// ------------------------------------------------- one-sided Jacobi SVD ---
// For each of `batch` matrices X_b (m x n, given by `in`), orthogonalise the
// columns by Hestenes-Jacobi rotations: X W = U diag(sigma).  Outputs, sorted
// by sigma descending: U (m x n column-major per batch in `uout`, zero columns
// where sigma == 0), sigma (n per batch) and, when wout != nullptr, W
// (n x n column-major per batch).  xws: workspace m x n per batch (distinct
// from uout).  wws: workspace n x n per batch when W is wanted.  status[b]
// gets a DevStatus.  max_sweeps = 0 only normalises and sorts the columns.
template <typename T>
void jacobi_svd(cudaStream_t st, int batch, int m, int n, const View<T> &in, cx<T> *uout, T *sigma,
                cx<T> *wout, cx<T> *xws, cx<T> *wws, int max_sweeps, int *status);

// One tournament round of a one-sided block-Jacobi sweep on the columns of X
// (m x n column-major, in place, bs-column blocks, nblk blocks; pairs_round:
// npairs block-id pairs, ids >= nblk are empty).  Several CTAs, one per pair.
// *flag |= 1 when any rotation happened.  gmax2: max squared column norm.
template <typename T>
void bjacobi_round(cudaStream_t st, int m, int n, int bs, int nblk, cx<T> *X, const int *pairs_round, int npairs,
                   const T *gmax2, int inner_sweeps, int *flag);
// All outer sweeps of the same block Jacobi in one launch on a thread-block
// cluster of ceil(nblk / 2) CTAs (at most 16), stopping after the first sweep
// without a rotation or after max_outer sweeps; the per-round arithmetic is
// bjacobi_round's.  Returns the launch status: an error means nothing ran (the
// cluster does not fit this device or shape) and the caller uses the
// per-round launches.  sweeps_out (nullable, device): outer sweeps run.
template <typename T> bool bjacobi_cluster_fits(int m, int n, int bs);
template <typename T>
cudaError_t bjacobi_cluster(cudaStream_t st, int m, int n, int bs, int nblk, cx<T> *X, const T *gmax2,
                            int inner_sweeps, int max_outer, int *sweeps_out);
// *out = max_j |X[:, j]|^2 for an m x n column-major X
template <typename T>
void colmax2(cudaStream_t st, int m, int n, const cx<T> *X, T *out);

// --------------------------------------------------- site-tensor kernels --
// out[l][x][a*K+k][r] = sum_s G[x][s][k] A[l][s][a][r]     (K <= 16)
template <typename T>
void kraus1q(cudaStream_t st, const cx<T> *A, cx<T> *out, int L, int Aa, int R, const double *g_host, int K);

// Z[(x,k)][y][(c,kk)][r] = sum_{s,t} Tg[x][y][s][t][kk] W[s][k][t][c][r]
// W: [2][kr][2][C][R]; Z: [2][kr][2][C*K][R].  (K <= 16)
template <typename T>
void mix2q(cudaStream_t st, const cx<T> *W, cx<T> *Z, int kr, int Cc, int R, const double *t_host, int K);
// Same with a leading batch leg: W [nb][2][kr][2][C][R] -> Z [nb][2][kr][2][C*K][R]
template <typename T>
void mix2q_batched(cudaStream_t st, const cx<T> *W, cx<T> *Z, int nb, int kr, int Cc, int R, const double *t_host,
                   int K);

// Generic strided 4-D copy: dst[i0][i1][i2][i3] (contiguous) = conj?(src[...strided...])
template <typename T>
void copy4d(cudaStream_t st, cx<T> *dst, const cx<T> *src, const int64_t dims[4], const int64_t sstr[4],
            int conj);

// Strided permutation of up to 6 axes: dst (contiguous, axis order of d) =
// conj?(src[sum_k i_k s[k]]), nd <= 6 axes
template <typename T>
void permute(cudaStream_t st, cx<T> *dst, const cx<T> *src, int nd, const int64_t *d, const int64_t *s, int conj);

// X[i][j] *= f(s[j]) (col scaling) or f(s[i]) (row scaling) for a row-major
// M x N matrix with leading dimension ld.  mode: 0 = s, 1 = sqrt(s),
// 2 = 1/sqrt(s), 3 = 1/s; modes 2 and 3 give 0 where s <= rel * s[0]
// (rel = 1e-6 for fp32, 1e-14 for fp64: singular values at rounding level,
// whose directions are noise, are dropped instead of amplified).
template <typename T>
void scale_matrix(cudaStream_t st, cx<T> *X, int M, int N, int64_t ld, const T *s, int by_row, int mode);

// Block-diagonal embedding: dst[b][x][a][x'*kr + k] = (x == x') * Q[(b*A + a)][k]
// Q row-major ((B*A) x kr).
template <typename T>
void blockdiag2(cudaStream_t st, cx<T> *dst, const cx<T> *Q, int B, int Aa, int kr);

template <typename T>
void fill_zero(cudaStream_t st, cx<T> *p, size_t n);

// Sum of squares of sigma[0..n) in double; out[0] = kept sum, out[1] = total
// (kept = first `keep` entries).  Used for the discarded-weight report.
template <typename T>
void sigma_weights(cudaStream_t st, const T *sigma, int n, int keep, double *out);

// s[i] = sqrt(max(s[i], 0))
template <typename T>
void sqrt_inplace(cudaStream_t st, T *s, int n);

// Readout: E'[D][x][D'][y][r][r'] style environment steps are expressed via
// cgemm; this kernel contracts a single-site operator into a site:
// out[l][y][a][r] = sum_x O[y][x] A[l][x][a][r]   (O 2x2 host complex)
template <typename T>
void apply_op_site(cudaStream_t st, const cx<T> *A, cx<T> *out, int L, int Aa, int R, const double *o_host);

// Trace of a batch of square matrices: out[b] = sum_i M_b[i][i]  (complex, double accum)
template <typename T>
void batched_trace(cudaStream_t st, const cx<T> *M, int n, int64_t ld, int64_t bs, int batch, double2 *out);

// Deterministic complex Gaussian test matrix (re, im ~ N(0, 1/2)).
template <typename T>
void gaussian(cudaStream_t st, cx<T> *out, size_t n, uint64_t seed);
// *out = sum |x_i|^2 (double accumulation; *out is cleared first)
template <typename T>
void sumsq(cudaStream_t st, const cx<T> *x, size_t n, double *out);

// Hermitian eigensolver pieces for wide-bond Gram matrices (kernels_eig.cu):
// Householder tridiagonalisation of G (n x n, column-major) on one
// thread-block cluster (T = Q^H G Q; d, e real; reflectors of Q as an
// (n-1) x (n-1) column-major block with their tau), and the top kr eigenpairs
// of the tridiagonal by bisection + inverse iteration (Z: n x kr row-major;
// *tail = trace minus their sum).  hetrd_cluster returns the launch status
// (a cluster that cannot be placed reports an error and launches nothing).
template <typename T> bool hetrd_cluster_fits(int n);
template <typename T>
cudaError_t hetrd_cluster(cudaStream_t st, int n, const cx<T> *G, T *d, T *e, cx<T> *vref, cx<T> *tau);
template <typename T>
void tridiag_top(cudaStream_t st, int n, const T *d, const T *e, int kr, T *lam, cx<T> *Z, T *work, T *tail);

// out[b] = Re sum_i E[b*msize + i] R[i] (left/right environment contraction)
template <typename T>
void env_dot(cudaStream_t st, const cx<T> *E, const cx<T> *R, int64_t msize, int batch, double *out);
// dst[b] = src[idx[b]] (msize-element blocks)
template <typename T>
void gather_mats(cudaStream_t st, const cx<T> *src, cx<T> *dst, const int *idx, int64_t msize, int batch);

// ------------------------------------------------- adjoint (kernels_adj.cu) --
// Cotangent convention: Xbar = dL/dRe X + i dL/dIm X for a real loss L.
// Abar[l][s][a][r] = sum_{x,k} conj(G[x][s][k]) Obar[l][x][aK+k][r]
template <typename T>
void kraus1q_bwd(cudaStream_t st, const cx<T> *Ob, cx<T> *Ab, int L, int Aa, int R, const double *g_host, int K);
// acc[(x*2+s)*K + k] += sum_{l,a,r} Obar[l][x][aK+k][r] conj(A[l][s][a][r])   (double accumulators)
template <typename T>
void kraus1q_grad(cudaStream_t st, const cx<T> *Ob, const cx<T> *A, int L, int Aa, int R, int K, double2 *acc);
// Wbar[s][k][t][c][r] = sum_{x,y,q} conj(Tg[x][y][s][t][q]) Zbar[x][k][y][cK+q][r]
template <typename T>
void mix2q_bwd(cudaStream_t st, const cx<T> *Zb, cx<T> *Wb, int kr, int Cc, int R, const double *t_host, int K);
// acc[(((x*2+y)*2+s)*2+t)*K + q] += sum_{k,c,r} Zbar[x][k][y][cK+q][r] conj(W[s][k][t][c][r])
template <typename T>
void mix2q_grad(cudaStream_t st, const cx<T> *Zb, const cx<T> *W, int kr, int Cc, int R, int K, double2 *acc);
// B (m x k, ld ldb) <- B R^-H, R upper triangular k x k (ld ldr); rank-deficient columns give zeros
template <typename T>
void trsm_rh(cudaStream_t st, cx<T> *B, int m, int k, int64_t ldb, const cx<T> *R, int64_t ldr);
// M (n x n) <- lower triangle mirrored to the upper one, real diagonal
template <typename T>
void copyltu(cudaStream_t st, cx<T> *M, int n);
// truncated-split adjoint coefficients (b x k) from U^H Ubar_k, s and the L / R dot products
template <typename T>
void split_K(cudaStream_t st, const cx<T> *UhUb, const T *s, int b, int k, const double *dl, const double *dr,
             double beta, cx<T> *Kout);
// kappa-pass adjoint coefficients (a x k): F o (V^H X) on discarded rows, zero on the kept block
template <typename T>
void kappa_C(cudaStream_t st, const cx<T> *VhX, const T *s, int a, int k, double beta, cx<T> *C);
// out[j] = Re sum_i conj(A[i si + j sj]) B[i si + j sj]
template <typename T>
void redot(cudaStream_t st, const cx<T> *A, const cx<T> *B, int n, int64_t len, int64_t si, int64_t sj, double *out);
// adjoint of blockdiag2: Qbar[(b a)][k] = sum_x Sbar[b][x][a][x kq + k]
template <typename T>
void blockdiag2_bwd(cudaStream_t st, const cx<T> *Sb, cx<T> *Qb, int B, int Aa, int kq);
// out[o][l][x][rest] = sum_{i, y} W[i wi + o wo + 2x + y] in[i][l][y][rest]  (MPO environment mix)
template <typename T>
void mpo_mix(cudaStream_t st, const cx<T> *in, cx<T> *out, const cx<T> *W, int Din, int Dout, int64_t wi, int64_t wo,
             int64_t L, int64_t rest);
// y += alpha x
template <typename T>
void axpy(cudaStream_t st, cx<T> *y, const cx<T> *x, int64_t n, double alpha);

// Message returned by mpdo_last_error() on the calling thread.
void set_last_error(const std::string &msg);

}  // namespace mpdo
