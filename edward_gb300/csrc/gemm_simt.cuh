// Batched FP32 SIMT GEMM with fused epilogues, shared by the Bayesian NN and
// sigmoid belief network steps:
//   C[b](m, n) = epi(b, m, n, sum_k A[b](m, k) B[b](k, n))
// with A(m, k) = A[b*sA + m*lda + k] (A[b*sA + k*lda + m] when TA) and
// B(k, n) = B[b*sB + k*ldb + n] (B[b*sB + n*ldb + k] when TB).
// 64 x 64 x 16 tiles, 256 threads with 4 x 4 outputs each, double-buffered
// shared memory.
#pragma once

#include "edg_common.cuh"

namespace edg {
namespace simt {

constexpr int BM = 64, BN = 64, BK = 16, kT = 256;

template <bool TA, bool TB, class Epi>
__global__ void __launch_bounds__(kT) bgemm_kernel(const float* __restrict__ A,
                                                   const float* __restrict__ B, float* C, int M,
                                                   int N, int K, int lda, int ldb, int ldc,
                                                   int64_t sA, int64_t sB, int64_t sC, Epi epi) {
  __shared__ __align__(16) float As[2][BK][BM + 4];
  __shared__ __align__(16) float Bs[2][BK][BN + 4];
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const float* Ab = A + b * sA;
  const float* Bb = B + b * sB;
  const int tid = threadIdx.x;
  const int tm = tid / 16, tn = tid % 16;  // 16 x 16 threads, 4 x 4 outputs each
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;

  auto load = [&](int buf, int k0) {
    // 64 x 16 elements of A and of B, 4 per thread
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + r * kT;
      // A tile: As[k][m]
      int mm, kk;
      if (TA) {
        kk = e / BM;
        mm = e % BM;
      } else {
        mm = e / BK;
        kk = e % BK;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      float va = 0.0f;
      if (gm < M && gk < K) va = TA ? Ab[(int64_t)gk * lda + gm] : Ab[(int64_t)gm * lda + gk];
      As[buf][kk][mm] = va;
      // B tile: Bs[k][n]
      int nn, kb;
      if (TB) {
        nn = e / BK;
        kb = e % BK;
      } else {
        kb = e / BN;
        nn = e % BN;
      }
      const int gn = n0 + nn, gk2 = k0 + kb;
      float vb = 0.0f;
      if (gn < N && gk2 < K) vb = TB ? Bb[(int64_t)gn * ldb + gk2] : Bb[(int64_t)gk2 * ldb + gn];
      Bs[buf][kb][nn] = vb;
    }
  };

  const int nk = (K + BK - 1) / BK;
  load(0, 0);
  __syncthreads();
  for (int t = 0; t < nk; ++t) {
    const int buf = t & 1;
    if (t + 1 < nk) load(buf ^ 1, (t + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      const float4 a4 = *reinterpret_cast<const float4*>(&As[buf][kk][tm * 4]);
      const float4 b4 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tn * 4]);
      const float av[4] = {a4.x, a4.y, a4.z, a4.w};
      const float bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
  float* Cb = C + b * sC;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + tm * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tn * 4 + j;
      if (n < N) Cb[(int64_t)m * ldc + n] = epi(b, m, n, acc[i][j]);
    }
  }
}

struct EpiIdentity {
  __device__ float operator()(int, int, int, float v) const { return v; }
};
// tanh(v + bias[b][n])
struct EpiBiasTanh {
  const float* bias;
  int64_t sBias;
  __device__ float operator()(int b, int, int n, float v) const {
    return tanhf(v + bias[b * sBias + n]);
  }
};
// tanh(v) (the bias is folded into an augmented weight block)
struct EpiTanh {
  __device__ float operator()(int, int, int, float v) const { return tanhf(v); }
};
// v * (1 - h^2) with h = H[b][m][n] (the tanh output being differentiated)
struct EpiTanhGrad {
  const float* H;
  int64_t sH;
  int ldh;
  __device__ float operator()(int b, int m, int n, float v) const {
    const float h = H[b * sH + (int64_t)m * ldh + n];
    return v * (1.0f - h * h);
  }
};

template <bool TA, bool TB, class Epi>
static int bgemm(const float* A, const float* B, float* C, int M, int N, int K, int lda, int ldb,
                 int ldc, int64_t sA, int64_t sB, int64_t sC, int batch, Epi epi,
                 cudaStream_t st) {
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
  bgemm_kernel<TA, TB, Epi><<<grid, kT, 0, st>>>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, epi);
  return check_launch("simt bgemm_kernel");
}

}  // namespace simt
}  // namespace edg
