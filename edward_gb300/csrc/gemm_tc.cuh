// Batched tensor-core GEMM (tcgen05.mma kind::tf32, 3xTF32) with fused epilogues:
//   C[b](m, n) = epi(b, m, n, sum_k A[b](m, k) B[b](k, n))
// with A(m, k) = A[b*sA + m*lda + k] (A[b*sA + k*lda + m] when TA) and
// B(k, n) = B[b*sB + k*ldb + n] (B[b*sB + n*ldb + k] when TB), FP32 in and out.
//
// 3xTF32: every operand element is split in flight, a = hi + lo with
// hi = tf32_rna(a) and lo = a - hi, and each product is lo*hi + hi*lo + hi*hi
// (small terms first) accumulated in FP32 in tensor memory.
//
// Persistent kernel, one CTA per SM, 416 threads:
//   warps 0-7   producers: global -> registers (float4), hi/lo split, st.shared
//               into the canonical K-major no-swizzle layout of both operands
//               (K-contiguous sources store one 16-byte core-matrix row per
//               float4; MN-contiguous sources are transposed 4 x 4 in registers);
//   warps 8-11  epilogue: tcgen05.ld of the accumulator (row m = TMEM lane),
//               epilogue functor, stores to C;
//   warp 12     TMEM owner and MMA issuer (one elected lane).
// Tiles are 128 (M) x 256 (N) x 16 (K) with 3 shared-memory stages and two
// TMEM accumulators (2 x 256 columns), so the epilogue of one tile overlaps the
// main loop of the next.  The core-matrix strides (LBO = 160 B between K groups,
// SBO = 656 B between 8-row groups) make both producer store patterns free of
// shared-memory bank conflicts.
//
// Long reductions are split over K (kchunk rows per split, partial tiles
// summed in FP32 with round-to-nearest by a reduce kernel): the tensor core's
// accumulation truncates, and bounding the number of MMAs per accumulator
// bounds that error.
//
// Every mbarrier wait is bounded (~1 s); on timeout the kernel records
// EDG_E_TIMEOUT in *err and runs to completion.
#pragma once

#include <algorithm>

#include "edg_common.cuh"
#include "tc_common.cuh"

namespace edg {
namespace tcg {

using namespace ptx;

constexpr int BM = 128, BN = 256, BK = 16, kStages = 3;
constexpr int kProdWarps = 8, kEpiWarps = 4;
constexpr int kProdThreads = kProdWarps * 32;
constexpr int kThreads = (kProdWarps + kEpiWarps + 1) * 32;
constexpr int kMmaWarp = kProdWarps + kEpiWarps;
constexpr uint32_t kLBO = 160, kSBO = 656;
constexpr uint32_t kABytes = (BM / 8) * kSBO;  // one plane (hi or lo) of the A tile
constexpr uint32_t kBBytes = (BN / 8) * kSBO;
constexpr uint32_t kStageBytes = 2 * kABytes + 2 * kBBytes;
constexpr uint32_t kTmemCols = 2 * BN;
constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + 256;

static_assert(kABytes % 16 == 0 && kBBytes % 16 == 0, "16-byte aligned planes");

__device__ __forceinline__ uint32_t soff(int row, int kk) {
  return (uint32_t)(row >> 3) * kSBO + (uint32_t)(kk >> 2) * kLBO + (uint32_t)(row & 7) * 16u +
         (uint32_t)(kk & 3) * 4u;
}

__device__ __forceinline__ void st_split4(uint32_t hi_addr, uint32_t lo_addr, float4 v) {
  float4 h, l;
  h.x = tf32_rna(v.x);
  h.y = tf32_rna(v.y);
  h.z = tf32_rna(v.z);
  h.w = tf32_rna(v.w);
  l.x = v.x - h.x;
  l.y = v.y - h.y;
  l.z = v.z - h.z;
  l.w = v.w - h.w;
  asm volatile("st.shared.v4.f32 [%0], {%1,%2,%3,%4};" ::"r"(hi_addr), "f"(h.x), "f"(h.y),
               "f"(h.z), "f"(h.w)
               : "memory");
  asm volatile("st.shared.v4.f32 [%0], {%1,%2,%3,%4};" ::"r"(lo_addr), "f"(l.x), "f"(l.y),
               "f"(l.z), "f"(l.w)
               : "memory");
}

struct Operand {
  const float* p;
  int ld;
  int64_t sb;  // batch stride
  int rows;    // extent along M (A) or N (B)
  bool kcontig;
  bool vec;    // float4 loads allowed (16-byte aligned base, ld and batch stride)
};

// Loads a float4 along K (K-contiguous source) at (row, k..k+3), masked.
__device__ __forceinline__ float4 load_k4(const Operand& o, const float* base, int row, int k,
                                          int K) {
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (row >= o.rows || k >= K) return v;
  const float* q = base + (int64_t)row * o.ld + k;
  if (o.vec && k + 3 < K) return __ldg(reinterpret_cast<const float4*>(q));
  v.x = __ldg(q);
  if (k + 1 < K) v.y = __ldg(q + 1);
  if (k + 2 < K) v.z = __ldg(q + 2);
  if (k + 3 < K) v.w = __ldg(q + 3);
  return v;
}

// Loads a float4 along the row dimension (MN-contiguous source) at (row..row+3, k), masked.
__device__ __forceinline__ float4 load_mn4(const Operand& o, const float* base, int row, int k,
                                           int K) {
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (row >= o.rows || k >= K) return v;
  const float* q = base + (int64_t)k * o.ld + row;
  if (o.vec && row + 3 < o.rows) return __ldg(reinterpret_cast<const float4*>(q));
  v.x = __ldg(q);
  if (row + 1 < o.rows) v.y = __ldg(q + 1);
  if (row + 2 < o.rows) v.z = __ldg(q + 2);
  if (row + 3 < o.rows) v.w = __ldg(q + 3);
  return v;
}

// One operand tile (R rows x BK) of one stage: producer thread tp of kProdThreads.
template <int R>
__device__ __forceinline__ void load_tile(const Operand& o, const float* base, int r0, int k0,
                                          int K, uint32_t hi, uint32_t lo, int tp) {
  if (o.kcontig) {
    // R * BK / 4 float4 chunks; chunk c: row c / 4, K group c % 4
    constexpr int kChunks = R * BK / 4;
#pragma unroll
    for (int c = tp; c < kChunks; c += kProdThreads) {
      const int row = c >> 2, kg = c & 3;
      const float4 v = load_k4(o, base, r0 + row, k0 + 4 * kg, K);
      const uint32_t off = soff(row, 4 * kg);
      st_split4(hi + off, lo + off, v);
    }
  } else {
    // (R / 4) row groups x 4 K groups; each task loads a 4 x 4 block and transposes it
    constexpr int kTasks = (R / 4) * 4;
#pragma unroll
    for (int t = tp; t < kTasks; t += kProdThreads) {
      const int rg = t % (R / 4), kg = t / (R / 4);
      float4 v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = load_mn4(o, base, r0 + 4 * rg, k0 + 4 * kg + j, K);
      const float4 c0 = make_float4(v[0].x, v[1].x, v[2].x, v[3].x);
      const float4 c1 = make_float4(v[0].y, v[1].y, v[2].y, v[3].y);
      const float4 c2 = make_float4(v[0].z, v[1].z, v[2].z, v[3].z);
      const float4 c3 = make_float4(v[0].w, v[1].w, v[2].w, v[3].w);
      const int row = 4 * rg;
      st_split4(hi + soff(row + 0, 4 * kg), lo + soff(row + 0, 4 * kg), c0);
      st_split4(hi + soff(row + 1, 4 * kg), lo + soff(row + 1, 4 * kg), c1);
      st_split4(hi + soff(row + 2, 4 * kg), lo + soff(row + 2, 4 * kg), c2);
      st_split4(hi + soff(row + 3, 4 * kg), lo + soff(row + 3, 4 * kg), c3);
    }
  }
}

struct Problem {
  Operand A, B;
  float* C;
  int ldc;
  int64_t sC;
  int M, N, K;
  int batch, splits, kchunk;
  int tiles_m, tiles_n;
  int64_t total;
  float* part;  // [splits][batch][M][N] when splits > 1
  unsigned* err;
};

struct Tile {
  int b, ks, mt, nt;
};

__device__ __forceinline__ Tile tile_of(const Problem& p, int64_t t) {
  Tile x;
  x.mt = (int)(t % p.tiles_m);
  t /= p.tiles_m;
  x.nt = (int)(t % p.tiles_n);
  t /= p.tiles_n;
  x.ks = (int)(t % p.splits);
  x.b = (int)(t / p.splits);
  return x;
}

template <class Epi>
__global__ void __launch_bounds__(kThreads, 1) gemm_tc_kernel(Problem p, Epi epi) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t sbase = smem_u32(smem);
  const uint32_t bar0 = sbase + kStages * kStageBytes;
  // barriers: full[kStages], empty[kStages], accfull[2], accempty[2], drain
  auto full = [&](int s) { return bar0 + 8u * s; };
  auto empty = [&](int s) { return bar0 + 8u * (kStages + s); };
  auto accfull = [&](int i) { return bar0 + 8u * (2 * kStages + i); };
  auto accempty = [&](int i) { return bar0 + 8u * (2 * kStages + 2 + i); };
  const uint32_t drain = bar0 + 8u * (2 * kStages + 4);
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(smem + kStages * kStageBytes + 128);
  __shared__ volatile int s_err;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    s_err = 0;
    for (int s = 0; s < kStages; ++s) {
      mbar_init(full(s), kProdThreads);
      mbar_init(empty(s), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(accfull(i), 1);
      mbar_init(accempty(i), kEpiWarps * 32);
    }
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     sbase + kStages * kStageBytes + 128),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int nk_full = (p.kchunk + BK - 1) / BK;

  if (warp < kProdWarps) {
    // ---------------------------------------------------------------- producers
    const int tp = threadIdx.x;
    uint32_t it = 0;
    for (int64_t t = blockIdx.x; t < p.total && !s_err; t += gridDim.x) {
      const Tile x = tile_of(p, t);
      const int kb = x.ks * p.kchunk, ke = min(p.K, kb + p.kchunk);
      const int nk = (ke - kb + BK - 1) / BK;
      const float* Ab = p.A.p + x.b * p.A.sb;
      const float* Bb = p.B.p + x.b * p.B.sb;
      for (int kt = 0; kt < nk && !s_err; ++kt, ++it) {
        const int s = (int)(it % kStages);
        if (it >= (uint32_t)kStages) mbar_wait(empty(s), ((it / kStages) - 1) & 1, &s_err);
        const uint32_t st = sbase + s * kStageBytes;
        const int k0 = kb + kt * BK;
        load_tile<BM>(p.A, Ab, x.mt * BM, k0, ke, st, st + kABytes, tp);
        load_tile<BN>(p.B, Bb, x.nt * BN, k0, ke, st + 2 * kABytes, st + 2 * kABytes + kBBytes, tp);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(full(s));
      }
    }
  } else if (warp == kMmaWarp) {
    // ---------------------------------------------------------------- MMA issuer
    constexpr uint32_t idesc = idesc_tf32(BM, BN);
    uint32_t it = 0, tcount = 0;
    for (int64_t t = blockIdx.x; t < p.total && !s_err; t += gridDim.x, ++tcount) {
      const Tile x = tile_of(p, t);
      const int kb = x.ks * p.kchunk, ke = min(p.K, kb + p.kchunk);
      const int nk = (ke - kb + BK - 1) / BK;
      const int ab = (int)(tcount & 1);
      if (tcount >= 2) mbar_wait(accempty(ab), ((tcount >> 1) - 1) & 1, &s_err);
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(ab * BN);
      for (int kt = 0; kt < nk && !s_err; ++kt, ++it) {
        const int s = (int)(it % kStages);
        mbar_wait(full(s), (it / kStages) & 1, &s_err);
        tc_fence_after();
        if (lane == 0) {
          const uint32_t st = sbase + s * kStageBytes;
#pragma unroll
          for (int j = 0; j < BK / 8; ++j) {
            const uint32_t ko = (uint32_t)j * 2u * kLBO;
            const uint64_t ahi = sdesc(st + ko, kLBO, kSBO);
            const uint64_t alo = sdesc(st + kABytes + ko, kLBO, kSBO);
            const uint64_t bhi = sdesc(st + 2 * kABytes + ko, kLBO, kSBO);
            const uint64_t blo = sdesc(st + 2 * kABytes + kBBytes + ko, kLBO, kSBO);
            const uint32_t acc0 = (kt > 0 || j > 0) ? 1u : 0u;
            mma_ss(d, alo, bhi, idesc, acc0);
            mma_ss(d, ahi, blo, idesc, 1u);
            mma_ss(d, ahi, bhi, idesc, 1u);
          }
          mma_commit(empty(s));
          if (kt == nk - 1) mma_commit(accfull(ab));
        }
        __syncwarp();
      }
    }
    // every MMA this thread issued has completed before TMEM is released
    // (also after a timeout, when nobody else waited for them)
    if (lane == 0) mma_commit(drain);
    __syncwarp();
    volatile int drain_err = 0;
    mbar_wait(drain, 0, &drain_err);
  } else {
    // ---------------------------------------------------------------- epilogue
    const int q = warp & 3;  // TMEM lane quarter of this warp
    const int row = q * 32 + lane;
    uint32_t tcount = 0;
    for (int64_t t = blockIdx.x; t < p.total && !s_err; t += gridDim.x, ++tcount) {
      const Tile x = tile_of(p, t);
      const int ab = (int)(tcount & 1);
      mbar_wait(accfull(ab), (tcount >> 1) & 1, &s_err);
      tc_fence_after();
      const int m = x.mt * BM + row;
      const int nbase = x.nt * BN;
      float* out;
      int64_t ldo;
      bool direct = p.splits == 1;
      if (direct) {
        out = p.C + x.b * p.sC + (int64_t)m * p.ldc;
        ldo = p.ldc;
      } else {
        out = p.part + (((int64_t)x.ks * p.batch + x.b) * p.M + m) * p.N;
        ldo = p.N;
      }
      (void)ldo;
      const bool vec_out = ((reinterpret_cast<uintptr_t>(out) & 15) == 0) && ((nbase & 3) == 0);
#pragma unroll 1
      for (int c = 0; c < BN / 32; ++c) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(ab * BN + c * 32), v);
        if (m < p.M) {
          const int n0 = nbase + c * 32;
#pragma unroll
          for (int i = 0; i < 32; ++i)
            v[i] = direct ? epi(x.b, m, n0 + i, v[i]) : v[i];
          if (vec_out && n0 + 32 <= p.N) {
#pragma unroll
            for (int i = 0; i < 32; i += 4)
              *reinterpret_cast<float4*>(out + n0 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
          } else {
#pragma unroll
            for (int i = 0; i < 32; ++i)
              if (n0 + i < p.N) out[n0 + i] = v[i];
          }
        }
      }
      tc_fence_before();
      mbar_arrive(accempty(ab));
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols));
  }
  if (threadIdx.x == 0 && s_err) atomicExch(p.err, (unsigned)(-EDG_E_TIMEOUT));
}

// C[m][n] = epi(b, m, n, sum_s part[s][b][m][n])
template <class Epi>
__global__ void splitk_sum_kernel(const float* __restrict__ part, int splits, int batch, int M,
                                  int N, float* C, int ldc, int64_t sC, Epi epi) {
  const int64_t MN = (int64_t)M * N, total = MN * batch;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(i / MN);
    const int64_t r = i % MN;
    const int m = (int)(r / N), n = (int)(r % N);
    float acc = 0.0f;
    for (int s = 0; s < splits; ++s) acc += part[(int64_t)s * total + i];
    C[b * sC + (int64_t)m * ldc + n] = epi(b, m, n, acc);
  }
}

__device__ unsigned g_gemm_err;

inline int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

inline bool aligned16(const void* p, int ld, int64_t sb) {
  return (reinterpret_cast<uintptr_t>(p) & 15) == 0 && (ld & 3) == 0 && (sb & 3) == 0;
}

// Partial-sum floats gemm() needs for this problem (0 without a K split).
inline size_t part_floats(int M, int N, int K, int batch, int kchunk) {
  const int splits = kchunk > 0 ? (K + kchunk - 1) / kchunk : 1;
  return splits > 1 ? (size_t)splits * batch * M * N : 0;
}

// Host launcher.  kchunk > 0 splits K into chunks of kchunk rows (multiple of
// BK), reduced by splitk_sum_kernel from `part` (part_floats() floats).
template <bool TA, bool TB, class Epi>
int gemm(const float* A, const float* B, float* C, int M, int N, int K, int lda, int ldb, int ldc,
         int64_t sA, int64_t sB, int64_t sC, int batch, Epi epi, int kchunk, float* part,
         unsigned* err, cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0 || batch <= 0) return EDG_OK;
  Problem p;
  p.A = Operand{A, lda, sA, M, !TA, aligned16(A, lda, sA)};
  p.B = Operand{B, ldb, sB, N, TB, aligned16(B, ldb, sB)};
  p.C = C;
  p.ldc = ldc;
  p.sC = sC;
  p.M = M;
  p.N = N;
  p.K = K;
  p.batch = batch;
  p.kchunk = (kchunk > 0 && kchunk < K) ? (kchunk + BK - 1) / BK * BK : K;
  p.splits = (K + p.kchunk - 1) / p.kchunk;
  p.tiles_m = (M + BM - 1) / BM;
  p.tiles_n = (N + BN - 1) / BN;
  p.total = (int64_t)p.tiles_m * p.tiles_n * p.splits * batch;
  p.part = part;
  if (p.splits > 1 && !part) return EDG_E_NULL;
  if (!err) {
    void* a = nullptr;
    cudaGetSymbolAddress(&a, g_gemm_err);
    err = reinterpret_cast<unsigned*>(a);
  }
  p.err = err;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(gemm_tc_kernel<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmemBytes);
    attr_set = true;
  }
  const int grid = (int)std::min<int64_t>(p.total, sm_count());
  gemm_tc_kernel<Epi><<<grid, kThreads, kSmemBytes, st>>>(p, epi);
  int rc = check_launch("gemm_tc_kernel");
  if (rc || p.splits == 1) return rc;
  const int64_t total = (int64_t)M * N * batch;
  splitk_sum_kernel<<<(int)std::min<int64_t>((total + 255) / 256, 8 * sm_count()), 256, 0, st>>>(
      part, p.splits, batch, M, N, C, ldc, sC, epi);
  return check_launch("splitk_sum_kernel");
}

}  // namespace tcg
}  // namespace edg
