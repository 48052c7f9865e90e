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
//   warps 0-7   producers: cp.async of 16-byte chunks into a per-thread raw
//               ring (3 stages in flight), then hi/lo split and st.shared into
//               the canonical K-major no-swizzle layout of both operands
//               (K-contiguous sources give one 16-byte core-matrix row per
//               chunk; MN-contiguous sources are transposed 4 x 4 in registers);
//   warps 8-11  epilogue: tcgen05.ld of the accumulator (row m = TMEM lane),
//               epilogue functor, stores to C;
//   warp 12     TMEM owner and MMA issuer (one elected lane).
// Tiles are 128 (M) x 256 (N) x 16 (K) with 2 split (hi/lo) shared-memory
// stages, 3 raw stages and two TMEM accumulators (2 x 256 columns), so the
// epilogue of one tile overlaps the main loop of the next.  The core-matrix
// strides (LBO = 160 B between K groups, SBO = 656 B between 8-row groups)
// make both producer store patterns free of shared-memory bank conflicts.
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

constexpr int BM = 128, BN = 256, BK = 16, kStages = 2, kRaw = 3;
constexpr int kProdWarps = 8, kEpiWarps = 4;
constexpr int kProdThreads = kProdWarps * 32;
constexpr int kThreads = (kProdWarps + kEpiWarps + 1) * 32;
constexpr int kMmaWarp = kProdWarps + kEpiWarps;
constexpr uint32_t kLBO = 160, kSBO = 656;
constexpr uint32_t kABytes = (BM / 8) * kSBO;  // one plane (hi or lo) of the A tile
constexpr uint32_t kBBytes = (BN / 8) * kSBO;
constexpr uint32_t kStageBytes = 2 * kABytes + 2 * kBBytes;
// Raw (unsplit) copies in flight: per slot, 8 16-byte chunks per producer thread
// ([chunk][thread], so that a warp's chunk i is one contiguous 512-byte run).
constexpr uint32_t kRawSlot = 8u * kProdThreads * 16u;
constexpr uint32_t kRawBase = kStages * kStageBytes;
constexpr uint32_t kBarBase = kRawBase + kRaw * kRawSlot;
constexpr uint32_t kTmemCols = 2 * BN;
constexpr size_t kSmemBytes = (size_t)kBarBase + 256;

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

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ float4 ld_shared4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr)
               : "memory");
  return v;
}

// 16 bytes of a K-contiguous source at (row, k .. k + 3) into dst; elements
// outside the rows or beyond K are zero-filled.
__device__ __forceinline__ void copy_k4(const Operand& o, const float* base, int row, int k, int K,
                                        uint32_t dst) {
  const int nv = row < o.rows ? max(0, min(4, K - k)) : 0;
  const float* q = base + (int64_t)row * o.ld + k;
  if (o.vec) {
    cp_async16(dst, nv ? q : base, 4u * nv);
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) cp_async4(dst + 4 * e, e < nv ? q + e : base, e < nv ? 4u : 0u);
  }
}

// 16 bytes of an MN-contiguous source at (rows row .. row + 3, k) into dst.
__device__ __forceinline__ void copy_mn4(const Operand& o, const float* base, int row, int k, int K,
                                         uint32_t dst) {
  const int nr = k < K ? max(0, min(4, o.rows - row)) : 0;
  const float* q = base + (int64_t)k * o.ld + row;
  if (o.vec) {
    cp_async16(dst, nr ? q : base, 4u * nr);
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) cp_async4(dst + 4 * e, e < nr ? q + e : base, e < nr ? 4u : 0u);
  }
}

// Raw copy of one operand tile (R rows x BK) of one stage: this thread's chunks
// go to raw + (c0 + i) * kProdThreads * 16 + tp * 16.
// K-contiguous source: chunk i is float4 number tp + 256 i (row / 4, K group % 4).
// MN-contiguous source: thread tp < R owns the 4 x 4 block of rows
// 4 (tp % (R / 4)) .. + 3 and K group tp / (R / 4); chunk j = K row j of it.
template <int R>
__device__ __forceinline__ void fetch_tile(const Operand& o, const float* base, int r0, int k0,
                                           int K, int tp, uint32_t raw, int c0) {
  if (o.kcontig) {
    constexpr int kPer = R * BK / 4 / kProdThreads;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int c = tp + i * kProdThreads;
      copy_k4(o, base, r0 + (c >> 2), k0 + 4 * (c & 3), K,
              raw + (uint32_t)((c0 + i) * kProdThreads + tp) * 16u);
    }
  } else if (tp < R) {
    const int rg = tp % (R / 4), kg = tp / (R / 4);
#pragma unroll
    for (int j = 0; j < 4; ++j)
      copy_mn4(o, base, r0 + 4 * rg, k0 + 4 * kg + j, K,
               raw + (uint32_t)((c0 + j) * kProdThreads + tp) * 16u);
  }
}

// Splits this thread's raw chunks of one operand tile into the hi / lo planes.
template <int R>
__device__ __forceinline__ void convert_tile(const Operand& o, int tp, uint32_t raw, int c0,
                                             uint32_t hi, uint32_t lo) {
  if (o.kcontig) {
    constexpr int kPer = R * BK / 4 / kProdThreads;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int c = tp + i * kProdThreads;
      const float4 v = ld_shared4(raw + (uint32_t)((c0 + i) * kProdThreads + tp) * 16u);
      const uint32_t off = soff(c >> 2, 4 * (c & 3));
      st_split4(hi + off, lo + off, v);
    }
  } else if (tp < R) {
    const int rg = tp % (R / 4), kg = tp / (R / 4);
    float4 r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
      r[j] = ld_shared4(raw + (uint32_t)((c0 + j) * kProdThreads + tp) * 16u);
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
  const uint32_t bar0 = sbase + kBarBase;
  // barriers: full[kStages], empty[kStages], accfull[2], accempty[2], drain
  auto full = [&](int s) { return bar0 + 8u * s; };
  auto empty = [&](int s) { return bar0 + 8u * (kStages + s); };
  auto accfull = [&](int i) { return bar0 + 8u * (2 * kStages + i); };
  auto accempty = [&](int i) { return bar0 + 8u * (2 * kStages + 2 + i); };
  const uint32_t drain = bar0 + 8u * (2 * kStages + 4);
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(smem + kBarBase + 128);
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
                     sbase + kBarBase + 128),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < kProdWarps) {
    // ---------------------------------------------------------------- producers
    // Stages form one flat sequence over this CTA's tiles.  Each thread keeps
    // kRaw - 1 stages of its own raw 16-byte chunks in flight (cp.async), and
    // converts a stage once its own copies have landed -- no barrier between
    // copy and conversion, since every thread converts exactly what it copied.
    const int tp = threadIdx.x;
    struct Job {
      int64_t t;
      int kt, nk, kb, ke, r0a, r0b;
      const float* Ab;
      const float* Bb;
      bool valid;
    };
    auto start_tile = [&](int64_t t, Job& j) {
      j.valid = t < p.total;
      if (!j.valid) return;
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
    Job f;
    start_tile(blockIdx.x, f);
    uint32_t nfetched = 0;
    auto fetch_next = [&]() {
      if (f.valid) {
        const uint32_t raw = sbase + kRawBase + (nfetched % kRaw) * kRawSlot;
        const int k0 = f.kb + f.kt * BK;
        fetch_tile<BM>(p.A, f.Ab, f.r0a, k0, f.ke, tp, raw, 0);
        fetch_tile<BN>(p.B, f.Bb, f.r0b, k0, f.ke, tp, raw, 4);
        ++nfetched;
        if (++f.kt == f.nk) start_tile(f.t + gridDim.x, f);
      }
      cp_async_commit();
    };
#pragma unroll 1
    for (int i = 0; i < kRaw - 1; ++i) fetch_next();
    for (uint32_t c = 0; c < nfetched && !s_err; ++c) {
      fetch_next();
      cp_async_wait<kRaw - 1>();
      const int s = (int)(c % kStages);
      if (c >= (uint32_t)kStages) mbar_wait(empty(s), ((c / kStages) - 1) & 1, &s_err);
      const uint32_t raw = sbase + kRawBase + (c % kRaw) * kRawSlot;
      const uint32_t st = sbase + s * kStageBytes;
      convert_tile<BM>(p.A, tp, raw, 0, st, st + kABytes);
      convert_tile<BN>(p.B, tp, raw, 4, st + 2 * kABytes, st + 2 * kABytes + kBBytes);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(full(s));
    }
    cp_async_wait<0>();
  } else if (warp == kMmaWarp) {
    // ---------------------------------------------------------------- MMA issuer
    // the whole warp runs the issue loop; one elected lane issues
    constexpr uint32_t idesc = idesc_tf32(BM, BN);
    const uint32_t issue = elect_one();
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
        {
          const uint32_t st = sbase + s * kStageBytes;
#pragma unroll
          for (int j = 0; j < BK / 8; ++j) {
            const uint32_t ko = (uint32_t)j * 2u * kLBO;
            const uint64_t ahi = sdesc(st + ko, kLBO, kSBO);
            const uint64_t alo = sdesc(st + kABytes + ko, kLBO, kSBO);
            const uint64_t bhi = sdesc(st + 2 * kABytes + ko, kLBO, kSBO);
            const uint64_t blo = sdesc(st + 2 * kABytes + kBBytes + ko, kLBO, kSBO);
            const uint32_t acc0 = (kt > 0 || j > 0) ? 1u : 0u;
            mma_ss_if(issue, d, alo, bhi, idesc, acc0);
            mma_ss_if(issue, d, ahi, blo, idesc, 1u);
            mma_ss_if(issue, d, ahi, bhi, idesc, 1u);
          }
          mma_commit_if(issue, empty(s));
          if (kt == nk - 1) mma_commit_if(issue, accfull(ab));
        }
        __syncwarp();
      }
    }
    // every MMA this thread issued has completed before TMEM is released
    // (also after a timeout, when nobody else waited for them)
    mma_commit_if(issue, drain);
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

// Per-device status word of the GEMMs launched without a caller error word
// (edg_gemm): a bounded wait that gives up stores -EDG_E_TIMEOUT here; it stays
// set until edg_gemm_status reads and clears it.
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
    // the calling device's status word (looked up on every call: the address
    // is per device and does not outlive a device reset)
    void* a = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&a, g_gemm_err);
    if (e != cudaSuccess || !a)
      return fail(EDG_E_CUDA, "gemm status word: %s", cudaGetErrorString(e));
    err = reinterpret_cast<unsigned*>(a);
  }
  p.err = err;
  int rc = set_max_dyn_smem(gemm_tc_kernel<Epi>, kSmemBytes, "gemm_tc_kernel");
  if (rc) return rc;
  const int grid = (int)std::min<int64_t>(p.total, sm_count());
  gemm_tc_kernel<Epi><<<grid, kThreads, kSmemBytes, st>>>(p, epi);
  rc = check_launch("gemm_tc_kernel");
  if (rc || p.splits == 1) return rc;
  const int64_t total = (int64_t)M * N * batch;
  splitk_sum_kernel<<<(int)std::min<int64_t>((total + 255) / 256, 8 * sm_count()), 256, 0, st>>>(
      part, p.splits, batch, M, N, C, ldc, sC, epi);
  return check_launch("splitk_sum_kernel");
}

}  // namespace tcg
}  // namespace edg

#endif  // EDG_GEMM_TC_IMPL
