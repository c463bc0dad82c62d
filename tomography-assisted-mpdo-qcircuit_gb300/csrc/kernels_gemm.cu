// Batched strided complex GEMM (fp32 or fp64 complex, FMA pipe).
//
// 64x64 output tile per CTA, 256 threads, each thread owns a 4x4 block of
// outputs interleaved with stride 16 so that shared-memory reads and global
// stores of consecutive threads hit consecutive addresses.  Operands are
// read through strided views (any transpose / conjugation / leg
// permutation), staged in shared memory per 16-deep K slice.  Small-output,
// long-K products (Gram matrices) are split along K into a workspace and
// reduced by a second kernel.
#include "kernels.cuh"

#include <algorithm>

namespace mpdo {

namespace {
constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

template <typename T>
__global__ void __launch_bounds__(NT) k_cgemm(int M, int N, int K, int kslice, cx<T> alpha, View<T> A,
                                              View<T> B, cx<T> beta, cx<T> *C, int64_t crs, int64_t ccs,
                                              int64_t cbs, int a_kfast, int b_kfast, int nsplit,
                                              int64_t ws_bs) {
  __shared__ cx<T> As[BK][BM + 1];
  __shared__ cx<T> Bs[BK][BN + 1];
  const int zb = blockIdx.z;
  const int b = zb / nsplit, split = zb % nsplit;
  const int i0 = blockIdx.y * BM, j0 = blockIdx.x * BN;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int kbeg = split * kslice, kend = min(K, kbeg + kslice);

  cx<T> acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = czero<T>();

  for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int e0 = 0; e0 < BM * BK; e0 += NT) {
      const int e = e0 + tid;
      int i, k;
      if (a_kfast) { i = e / BK; k = e % BK; } else { i = e % BM; k = e / BM; }
      const int gi = i0 + i, gk = k0 + k;
      As[k][i] = (gi < M && gk < kend) ? view_ld(A, b, gi, gk) : czero<T>();
    }
#pragma unroll
    for (int e0 = 0; e0 < BN * BK; e0 += NT) {
      const int e = e0 + tid;
      int j, k;
      if (b_kfast) { j = e / BK; k = e % BK; } else { j = e % BN; k = e / BN; }
      const int gj = j0 + j, gk = k0 + k;
      Bs[k][j] = (gj < N && gk < kend) ? view_ld(B, b, gk, gj) : czero<T>();
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      cx<T> av[4], bv[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) av[r] = As[k][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) bv[c] = Bs[k][tx + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) cfma<T>(acc[r][c], av[r], bv[c]);
    }
    __syncthreads();
  }

  if (nsplit > 1) {
    // partial sums into the workspace: [b][split][M][N]
    cx<T> *W = C + (int64_t)zb * ws_bs;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int gi = i0 + ty + 16 * r;
      if (gi >= M) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int gj = j0 + tx + 16 * c;
        if (gj < N) W[(int64_t)gi * N + gj] = acc[r][c];
      }
    }
    return;
  }
  const bool use_beta = (beta.x != T(0) || beta.y != T(0));
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int gi = i0 + ty + 16 * r;
    if (gi >= M) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int gj = j0 + tx + 16 * c;
      if (gj >= N) continue;
      cx<T> *dst = C + (int64_t)b * cbs + (int64_t)gi * crs + (int64_t)gj * ccs;
      cx<T> v = cmul<T>(alpha, acc[r][c]);
      if (use_beta) cfma<T>(v, beta, *dst);
      *dst = v;
    }
  }
}

template <typename T>
__global__ void k_splitk_reduce(int M, int N, int nsplit, const cx<T> *ws, cx<T> alpha, cx<T> beta, cx<T> *C,
                                int64_t crs, int64_t ccs, int64_t cbs, int batch) {
  const int64_t total = (int64_t)batch * M * N;
  const bool use_beta = (beta.x != T(0) || beta.y != T(0));
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / ((int64_t)M * N);
    const int64_t rem = t % ((int64_t)M * N);
    const int64_t i = rem / N, j = rem % N;
    cx<T> s = czero<T>();
    for (int q = 0; q < nsplit; ++q) {
      const cx<T> w = ws[((b * nsplit + q) * M + i) * N + j];
      s.x += w.x; s.y += w.y;
    }
    cx<T> *dst = C + b * cbs + i * crs + j * ccs;
    cx<T> v = cmul<T>(alpha, s);
    if (use_beta) cfma<T>(v, beta, *dst);
    *dst = v;
  }
}
}  // namespace

template <typename T>
void cgemm(cudaStream_t st, int M, int N, int K, int batch, cx<T> alpha, const View<T> &A, const View<T> &B,
           cx<T> beta, cx<T> *C, int64_t c_rs, int64_t c_cs, int64_t c_bs, cx<T> *ws, size_t ws_elems) {
  if (M <= 0 || N <= 0 || batch <= 0) return;
  // k-fast staging when the K direction is the contiguous one
  const int a_kfast = (A.n1 == 1 && A.cs == 1 && A.s0 != 1) ? 1 : 0;
  const int b_kfast = (B.n1 == 1 && B.s0 == 1 && B.cs != 1) ? 1 : 0;
  const int gx = (N + BN - 1) / BN, gy = (M + BM - 1) / BM;
  int nsplit = 1;
  const int64_t tiles = (int64_t)gx * gy * batch;
  if (ws != nullptr && K >= 4 * BK * 8 && tiles < 148) {
    nsplit = (int)std::min<int64_t>(std::max<int64_t>(1, 296 / tiles), K / (BK * 8));
    while (nsplit > 1 && (size_t)nsplit * batch * M * N > ws_elems) --nsplit;
  }
  int kslice = K;
  if (nsplit > 1) {
    kslice = ((K + nsplit - 1) / nsplit + BK - 1) / BK * BK;
    nsplit = (K + kslice - 1) / kslice;
  }
  if (K <= 0) {
    // C = beta * C only; reuse the reduce kernel with zero partials
    nsplit = 1;
  }
  const int maxz = 65535 / nsplit;
  for (int b0 = 0; b0 < batch; b0 += maxz) {
    const int nb = std::min(maxz, batch - b0);
    View<T> Ab = A, Bb = B;
    Ab.p = A.p + (int64_t)b0 * A.bs;
    Bb.p = B.p + (int64_t)b0 * B.bs;
    cx<T> *Cb = C + (int64_t)b0 * c_bs;
    dim3 grid(gx, gy, nb * nsplit);
    if (nsplit > 1) {
      k_cgemm<T><<<grid, NT, 0, st>>>(M, N, K, kslice, alpha, Ab, Bb, beta, ws, 0, 0, 0, a_kfast, b_kfast,
                                      nsplit, (int64_t)M * N);
      count_launch();
      const int64_t total = (int64_t)nb * M * N;
      const int rb = (int)std::min<int64_t>((total + 255) / 256, 4096);
      k_splitk_reduce<T><<<rb, 256, 0, st>>>(M, N, nsplit, ws, alpha, beta, Cb, c_rs, c_cs, c_bs, nb);
      count_launch();
    } else {
      k_cgemm<T><<<grid, NT, 0, st>>>(M, N, K, std::max(K, 1), alpha, Ab, Bb, beta, Cb, c_rs, c_cs, c_bs,
                                      a_kfast, b_kfast, 1, 0);
      count_launch();
    }
  }
}

template void cgemm<float>(cudaStream_t, int, int, int, int, cx<float>, const View<float> &,
                           const View<float> &, cx<float>, cx<float> *, int64_t, int64_t, int64_t,
                           cx<float> *, size_t);
template void cgemm<double>(cudaStream_t, int, int, int, int, cx<double>, const View<double> &,
                            const View<double> &, cx<double>, cx<double> *, int64_t, int64_t, int64_t,
                            cx<double> *, size_t);

}  // namespace mpdo
