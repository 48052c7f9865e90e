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

#include <cstddef>
#include <cstdint>

#include <algorithm>

#include "edg_common.cuh"
#include "tc_common.cuh"

namespace edg {
namespace tcg {

constexpr int kBK = 16;  // K rows per pipeline stage

// Partial-sum floats gemm() needs for this problem (0 without a K split).
inline size_t part_floats(int M, int N, int K, int batch, int kchunk) {
  const int splits = kchunk > 0 ? (K + kchunk - 1) / kchunk : 1;
  return splits > 1 ? (size_t)splits * batch * M * N : 0;
}

// C[b] = epi(op(A[b]) op(B[b])) on the tensor cores.  kchunk > 0 splits K into
// chunks of kchunk rows (rounded up to a multiple of 16) whose partials are
// summed in FP32 from `part` (part_floats() floats); err (device, may be NULL)
// receives EDG_E_TIMEOUT if a bounded wait gave up.  Instantiated in gemm.cu
// for the (TA, TB, Epi) combinations the library uses.
template <bool TA, bool TB, class Epi>
int gemm(const float* A, const float* B, float* C, int M, int N, int K, int lda, int ldb, int ldc,
         int64_t sA, int64_t sB, int64_t sC, int batch, Epi epi, int kchunk, float* part,
         unsigned* err, cudaStream_t st);

// C[b][m][n] (+)= sum over splits of part[s][b][m][n] (C row stride ldc, batch stride sC).
int sum_partials(const float* part, int splits, int batch, int M, int N, float* C, int ldc,
                 int64_t sC, cudaStream_t st);

}  // namespace tcg
}  // namespace edg

#ifdef EDG_GEMM_TC_IMPL
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

// One operand tile (R rows x BK) of one stage is fetched into four float4
// registers per producer thread and then split and stored, so that the
// global loads of the next stage are in flight while this one is stored.
// K-contiguous source: float4 chunk c = tp + 256 i holds row c / 4, K group c % 4.
// MN-contiguous source: task tp (< R) loads the 4 x 4 block of rows
// 4 (tp % (R / 4)) .. + 3 and K group tp / (R / 4), transposed when stored.
template <int R>
__device__ __forceinline__ void fetch_tile(const Operand& o, const float* base, int r0, int k0,
                                           int K, int tp, float4 (&r)[4]) {
  if (o.kcontig) {
    constexpr int kPer = R * BK / 4 / kProdThreads;  // 2 (R = 128) or 4 (R = 256)
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int c = tp + i * kProdThreads;
      r[i] = load_k4(o, base, r0 + (c >> 2), k0 + 4 * (c & 3), K);
    }
  } else if (tp < R) {
    const int rg = tp % (R / 4), kg = tp / (R / 4);
#pragma unroll
    for (int j = 0; j < 4; ++j) r[j] = load_mn4(o, base, r0 + 4 * rg, k0 + 4 * kg + j, K);
  }
}

template <int R>
__device__ __forceinline__ void put_tile(const Operand& o, int tp, const float4 (&r)[4],
                                         uint32_t hi, uint32_t lo) {
  if (o.kcontig) {
    constexpr int kPer = R * BK / 4 / kProdThreads;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int c = tp + i * kProdThreads;
      const uint32_t off = soff(c >> 2, 4 * (c & 3));
      st_split4(hi + off, lo + off, r[i]);
    }
  } else if (tp < R) {
    const int rg = tp % (R / 4), kg = tp / (R / 4);
    const int row = 4 * rg;
    st_split4(hi + soff(row + 0, 4 * kg), lo + soff(row + 0, 4 * kg),
              make_float4(r[0].x, r[1].x, r[2].x, r[3].x));
    st_split4(hi + soff(row + 1, 4 * kg), lo + soff(row + 1, 4 * kg),
              make_float4(r[0].y, r[1].y, r[2].y, r[3].y));
    st_split4(hi + soff(row + 2, 4 * kg), lo + soff(row + 2, 4 * kg),
              make_float4(r[0].z, r[1].z, r[2].z, r[3].z));
    st_split4(hi + soff(row + 3, 4 * kg), lo + soff(row + 3, 4 * kg),
              make_float4(r[0].w, r[1].w, r[2].w, r[3].w));
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
    // Stages are produced in one flat sequence over this CTA's tiles; the
    // loads of stage i + 1 are issued before stage i is stored.
    const int tp = threadIdx.x;
    struct Job {
      int64_t t;
      int kt, nk, kb, ke, r0a, r0b;
      const float* Ab;
      const float* Bb;
    };
    auto make_job = [&](int64_t t, Job& j) {
      const Tile x = tile_of(p, t);
      j.t = t;
      j.kt = 0;
      j.kb = x.ks * p.kchunk;
      j.ke = min(p.K, j.kb + p.kchunk);
      j.nk = (j.ke - j.kb + BK - 1) / BK;
      j.r0a = x.mt * BM;
      j.r0b = x.nt * BN;
      j.Ab = p.A.p + x.b * p.A.sb;
      j.Bb = p.B.p + x.b * p.B.sb;
    };
    float4 ca[4], cb[4], na[4], nb[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) ca[i] = cb[i] = na[i] = nb[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    Job cur;
    bool have = blockIdx.x < p.total;
    if (have) {
      make_job(blockIdx.x, cur);
      fetch_tile<BM>(p.A, cur.Ab, cur.r0a, cur.kb, cur.ke, tp, ca);
      fetch_tile<BN>(p.B, cur.Bb, cur.r0b, cur.kb, cur.ke, tp, cb);
    }
    for (uint32_t it = 0; have && !s_err; ++it) {
      Job nxt = cur;
      bool have_next = true;
      if (++nxt.kt == cur.nk) {
        const int64_t t2 = cur.t + gridDim.x;
        have_next = t2 < p.total;
        if (have_next) make_job(t2, nxt);
      }
      if (have_next) {
        const int k0 = nxt.kb + nxt.kt * BK;
        fetch_tile<BM>(p.A, nxt.Ab, nxt.r0a, k0, nxt.ke, tp, na);
        fetch_tile<BN>(p.B, nxt.Bb, nxt.r0b, k0, nxt.ke, tp, nb);
      }
      const int s = (int)(it % kStages);
      if (it >= (uint32_t)kStages) mbar_wait(empty(s), ((it / kStages) - 1) & 1, &s_err);
      const uint32_t st = sbase + s * kStageBytes;
      put_tile<BM>(p.A, tp, ca, st, st + kABytes);
      put_tile<BN>(p.B, tp, cb, st + 2 * kABytes, st + 2 * kABytes + kBBytes);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(full(s));
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        ca[i] = na[i];
        cb[i] = nb[i];
      }
      cur = nxt;
      have = have_next;
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
  static bool attr_set = false;  // one kernel per Epi, owned by this translation unit
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

#endif  // EDG_GEMM_TC_IMPL
