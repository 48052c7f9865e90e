// Tensor-core (tcgen05, 3xTF32) HMC for the GLM family.
//
// Work decomposition
//   * one thread-block CLUSTER per 128 chains (the MMA M dimension); the R CTAs
//     of a cluster split the rows of X; every leapfrog gradient is reduced
//     across the cluster through distributed shared memory (DSMEM);
//   * per CTA and 64-row tile of X, two chained GEMMs on the tensor core:
//       forward   eta^T[c][n] = sum_d Z[c][d] X[n][d]      (SS: A = Z smem, B = X tile)
//       backward  G[c][d]    += sum_n r[c][n] X[n][d]      (TS: A = r in TMEM, B = X^T tile)
//     with r = d log p(y_n | eta) / d eta computed by the epilogue warps from
//     the forward accumulator (TMEM) and written back to TMEM as the backward
//     A operand; eta/r are double-buffered so the epilogue of tile i overlaps
//     the MMAs of tile i+1;
//   * 3xTF32: every operand is split a = hi + lo (hi = tf32(a), lo = tf32(a - hi))
//     and each product is hi*hi + hi*lo + lo*hi with FP32 accumulation;
//   * X is re-laid once per model into 64-row tiles already in the canonical
//     K-major shared-memory layout (hi, lo, transposed hi, transposed lo),
//     so each tile is two cp.async.bulk copies (forward part, backward part),
//     each completing on its own mbarrier; the epilogue reads y straight from
//     the model's array.
//
// Warp roles (608 threads): warp 0 bulk-copy producers, warp 1 forward MMA
// issuer and TMEM owner, warp 18 backward MMA issuer, warps 2-17 epilogue;
// between gradient evaluations warps 2-17 are the "owners" that run the
// leapfrog / Metropolis arithmetic for this CTA's share of the cluster's
// chains, with the chain state in registers.
//
// Every mbarrier wait is bounded (~1 s of clock64): on timeout the kernel
// records EDG_E_TIMEOUT in edg_state_t::error and runs to completion without
// waiting further, so no launch can hang.
#include <algorithm>
#include <cstdio>
#include <type_traits>

#include "edg_common.cuh"
#include "tc_common.cuh"

namespace edg {
namespace tc {

using namespace ptx;

constexpr int kCT = 128;        // chains per cluster = MMA M
constexpr int kNR = 64;         // rows per X tile = forward N = backward K
constexpr int kEpiWarps = 16;
constexpr int kFWarp = 1, kBWarp = 2 + kEpiWarps;  // MMA issuers
constexpr int kThreads = 32 * (3 + kEpiWarps);     // + the bulk-copy warp
constexpr uint32_t kTmemCols = 512;

__host__ __device__ constexpr uint32_t stage_bytes(int PP) { return 1024u * PP; }

// Canonical K-major, no-swizzle layout: 8-row x 16-byte core matrices; core
// matrices adjacent along K are 128 B apart (LBO), 8-row groups are
// (K/4)*128 B apart (SBO).
__host__ __device__ inline uint32_t kmajor_off(int row, int k, int Kext) {
  return (uint32_t)((row >> 3) * (Kext * 32) + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// ------------------------------------------------------------------ tiling
__global__ void prep_tiles_kernel(const float* __restrict__ X, int N,
                                  int D, int bias, int PP, int ntiles,
                                  unsigned char* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t total = (int64_t)ntiles * kNR * PP;
  if (i >= total) return;
  const int tile = (int)(i / (kNR * PP));
  const int rem = (int)(i % (kNR * PP));
  const int n = rem / PP, d = rem % PP;
  const int row = tile * kNR + n;
  float v = 0.0f;
  if (row < N) {
    if (d < D)
      v = X[(size_t)row * D + d];
    else if (d == D && bias)
      v = 1.0f;
  }
  const float hi = tf32_rna(v);
  const float lo = tf32_rna(v - hi);
  unsigned char* base = out + (size_t)tile * stage_bytes(PP);
  float* xhi = reinterpret_cast<float*>(base);
  float* xlo = reinterpret_cast<float*>(base + 256 * PP);
  float* xthi = reinterpret_cast<float*>(base + 512 * PP);
  float* xtlo = reinterpret_cast<float*>(base + 768 * PP);
  const uint32_t o1 = kmajor_off(n, d, PP) / 4;   // X tile: rows n, K = d
  const uint32_t o2 = kmajor_off(d, n, kNR) / 4;  // X^T tile: rows d, K = n
  xhi[o1] = hi;
  xlo[o1] = lo;
  xthi[o2] = hi;
  xtlo[o2] = lo;
}

// ------------------------------------------------------------------ main kernel
struct TcArgs {
  const unsigned char* tiles;
  const float* y;  // the model's observations (the epilogue reads them directly)
  int ntiles, N, P, PP, lik;
  float inv_lik_var, lik_norm;
  float zscale;  // Z is broadcast as zscale * z: -log2(e) for Bernoulli (the MMA gives
                 // -log2(e) eta, the exponent the residual needs), 1 for Normal
  const float* prior_loc;
  const float* prior_scale;
  int C, n_iter, n_steps, cache_valid;
  float step_size;
  uint64_t seed;
  float* z;
  float* grad;
  double* lj;
  int32_t* n_accept;
  edg_state_t* state;
  float* samples;
  int64_t T_cap;
  double* moments;
  const float* r_ovr;
  const double* u_ovr;
  double* ratio_out;
  // stochastic-gradient MCMC (the SG instantiation): EDG_SGMCMC_*, SGHMC
  // friction, the likelihood's data scale, the SGHMC velocity [C, P] and the
  // noise override [n_iter, C, P]
  int sg_method;
  float friction, dscale;
  float* v;
  const float* noise;
  // Metropolis-Hastings (the MH instantiation): proposal location [P] (NULL =
  // random walk) and scale [P]; `noise` then overrides the proposal draws
  const float* mh_loc;
  const float* mh_scale;
};

constexpr int kMaxEPT = 4;  // chain-state elements per owner thread


// Residuals r = d log p(y | eta) / d eta of 8 consecutive rows, split into
// tf32 hi (v) and lo = r - hi.  On entry v holds what the forward MMA gave:
// w = -log2(e) eta for Bernoulli (Z was broadcast scaled), eta for Normal.
// hi keeps r's top 10 mantissa bits (truncation: one logical operation) and
// lo = r - hi is exact; the tensor core's own truncation of lo leaves a
// relative 2^-20 of r.
//   LL (the evaluation also needs the log-likelihood): Bernoulli with
//     e = 2^-|w| = e^-|eta| <= 1 and a = 1 + e: sigmoid(eta) = 1/a
//     (eta >= 0, i.e. w <= 0) or e/a, one reciprocal per pair of rows, and
//     log p(y | eta) = -(max(eta, 0) - eta y + log1p(e))
//                    = -ln 2 (max(-w, 0) + w y + log2(a))
//     (absolute error ~2e-7 per row); the 8 rows' terms are summed in FP32
//     and added to kl (compensated) once.  Rows at or beyond nvalid get r = 0
//     and add nothing to kl.
//   otherwise the short form: Bernoulli sigmoid(eta) = 1 / (1 + 2^w) with one
//     reciprocal per PAIR of rows, 1/a = b / (a b), 1/b = a / (a b); 2^w is
//     capped at e^40 so that a b stays below 2^116 (sigmoid changes by at most
//     e^-40 absolute).  Rows beyond N are not masked: their X rows are zero,
//     so their r only ever multiplies zeros in the backward MMA.
template <bool LL, bool BERN, bool SCALE = false>
__device__ __forceinline__ void residual_block(float (&v)[8], float (&lo)[8], const float (&y)[8],
                                               int nvalid, float inv_var, float lik_norm,
                                               Kahan& kl, float rscale = 1.0f) {
  float r[8];
  if (LL) {
    float part = 0.0f;
    if (BERN) {
      float e[8], a[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        e[k] = ex2_approx(-fabsf(v[k]));
        a[k] = 1.0f + e[k];
      }
#pragma unroll
      for (int k = 0; k < 8; k += 2) {
        const float ir = rcp_approx(a[k] * a[k + 1]);
        const float s0 = a[k + 1] * ir, s1 = a[k] * ir;  // 1/a[k], 1/a[k+1]
        r[k] = y[k] - (v[k] <= 0.0f ? s0 : e[k] * s0);
        r[k + 1] = y[k + 1] - (v[k + 1] <= 0.0f ? s1 : e[k + 1] * s1);
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float l = kLn2 * ((fmaxf(-v[k], 0.0f) + v[k] * y[k]) + lg2_approx(a[k]));
        part -= k < nvalid ? l : 0.0f;
      }
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float diff = y[k] - v[k];
        r[k] = diff * inv_var;
        part += k < nvalid ? -0.5f * diff * diff * inv_var - lik_norm : 0.0f;
      }
    }
    kl.add(part);
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] = k < nvalid ? r[k] : 0.0f;
  } else if (BERN) {
    constexpr float kCap = 57.70780163555854f;  // 40 log2 e
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = 1.0f + ex2_approx(fminf(v[k], kCap));
#pragma unroll
    for (int k = 0; k < 8; k += 2) {
      const float ir = rcp_approx(a[k] * a[k + 1]);
      r[k] = y[k] - a[k + 1] * ir;
      r[k + 1] = y[k + 1] - a[k] * ir;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] = (y[k] - v[k]) * inv_var;
  }
  if (SCALE) {
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] *= rscale;  // the data scale of SG-MCMC
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    v[k] = __uint_as_float(__float_as_uint(r[k]) & 0xFFFFE000u);
    lo[k] = r[k] - v[k];
  }
}

// MODE 0: HMC (leapfrog, Metropolis).  MODE 1: SGLD / SGHMC, one gradient
// evaluation per iteration, each iteration's update made with the cached
// gradient of the current state in the pre phase and every proposal kept
// (sgld.py:52-88, sghmc.py:58-102).  MODE 2: Metropolis-Hastings with Normal
// proposals, one log-joint evaluation per iteration and the FP64 test of
// metropolis_hastings.py:64-156; the backward side keeps its barriers and
// does no work (no X^T copies, residual stores or backward MMAs).
template <int MODE>
__global__ void __launch_bounds__(kThreads, 1) hmc_glm_tc_kernel(const TcArgs a) {
  constexpr bool SG = MODE == 1, MH = MODE == 2;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int PP = a.PP, P = a.P;
  const uint32_t SB = stage_bytes(PP);
  const uint32_t XB = 512u * PP;      // forward part of a tile: X hi, X lo
  const uint32_t TB = SB - XB;        // backward part: X^T hi, X^T lo
  unsigned char* stage0 = smem;
  unsigned char* stage1 = smem + SB;
  float* Zhi = reinterpret_cast<float*>(smem + 2 * SB);
  float* Zlo = Zhi + kCT * PP;
  uint64_t* bars = reinterpret_cast<uint64_t*>(Zlo + kCT * PP);
  // bars: fullx[2] fullt[2] emptyx[2] emptyt[2] eta[2] r[2] gfull[2], 2 spare
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 16);
  volatile int* err = reinterpret_cast<volatile int*>(tmem_slot + 1);
  __shared__ bool s_last;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t R = cluster_size(), rank = cluster_rank();
  const int cluster_id = blockIdx.x / R;
  const int c_base = cluster_id * kCT;
  const int t_begin = (int)((int64_t)a.ntiles * rank / R);
  const int t_end = (int)((int64_t)a.ntiles * (rank + 1) / R);
  const int nt = t_end - t_begin;

  const uint32_t b_fullx = smem_u32(bars + 0), b_fullt = smem_u32(bars + 2);
  const uint32_t b_emptyx = smem_u32(bars + 4), b_emptyt = smem_u32(bars + 6);
  const uint32_t b_eta = smem_u32(bars + 8), b_r = smem_u32(bars + 10);
  const uint32_t b_gfull = smem_u32(bars + 12);

  if (threadIdx.x == 0) {
    for (int i = 0; i < 2; ++i) {
      mbar_init(b_fullx + 8 * i, 1);
      mbar_init(b_fullt + 8 * i, 1);
      mbar_init(b_emptyx + 8 * i, 1);
      mbar_init(b_emptyt + 8 * i, 1);
      mbar_init(b_eta + 8 * i, 1);
      mbar_init(b_r + 8 * i, kEpiWarps);
      mbar_init(b_gfull + 8 * i, 1);
    }
    *err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tmem_slot;
  // TMEM columns, per buffer b: eta, r_hi, r_lo at 192 b + {0, 64, 128}; the
  // per-tile gradient partial at 384 + 64 b.  The tensor core accumulates with
  // truncation, so G is accumulated per tile in TMEM (24 MMAs) and summed
  // across tiles in FP32 registers with round-to-nearest.
#define COL_ETA(b) (192u * (b))
#define COL_RHI(b) (64u + 192u * (b))
#define COL_RLO(b) (128u + 192u * (b))
#define COL_GP(b) (384u + 64u * (b))

  // ---- owner mapping (warps 2-17, 512 threads): 4R threads per chain
  const bool owner = warp >= 2 && warp < 2 + kEpiWarps;
  const int et = threadIdx.x - 64;
  const int TPC = 4 * (int)R;
  const int CPO = kCT / (int)R;
  const int EPT = PP / TPC;
  const int chain_local = owner ? et / TPC : 0;
  const int part = owner ? et % TPC : 0;
  const int d0 = part * EPT;
  const int cc = (int)rank * CPO + chain_local;  // chain within the cluster (MMA row)
  const int cg = c_base + cc;                    // global chain
  const bool cvalid = owner && cg < a.C;
  // Working position / momentum / gradient in registers; the accepted state
  // (z, its gradient and log joint) stays in the caller's z / grad / lj arrays,
  // touched once per iteration, which keeps the epilogue's registers free.
  float zr[kMaxEPT], rr[kMaxEPT], gr[kMaxEPT];
  double kin0 = 0.0;
  float* zg = a.z + (size_t)(cvalid ? cg : 0) * P;
  float* gg = a.grad + (size_t)(cvalid ? cg : 0) * P;
#pragma unroll
  for (int i = 0; i < kMaxEPT; ++i) {
    const int d = d0 + i;
    const bool ok = cvalid && i < EPT && d < P;
    zr[i] = ok ? zg[d] : 0.0f;
    rr[i] = (SG && ok && a.v) ? a.v[(size_t)cg * P + d] : 0.0f;  // SGHMC velocity
    gr[i] = (SG && ok && a.cache_valid) ? gg[d] : 0.0f;
  }
  // prior loc and precision 1/scale^2 per coordinate (zero beyond P), and this
  // thread's share of the log-density normalising constant
  __shared__ float s_ploc[64], s_pprec[64];
  __shared__ double s_logu[kCT];  // log of the Metropolis uniform, per chain of this CTA
  for (int d = threadIdx.x; d < PP; d += kThreads) {
    const bool ok = d < P;
    const float sc = ok ? a.prior_scale[d] : 1.0f;
    s_ploc[d] = ok ? a.prior_loc[d] : 0.0f;
    s_pprec[d] = ok ? 1.0f / (sc * sc) : 0.0f;
  }
  double plogc = 0.0;
  for (int i = 0; i < EPT; ++i) {
    const int d = d0 + i;
    if (owner && d < P) plogc += -(double)logf(a.prior_scale[d]) - kHalfLog2Pi;
  }
  const int64_t t0 = *(volatile int64_t*)&a.state->t;
  const float eps = a.step_size, half = 0.5f * a.step_size;
  const uint32_t zhi_addr = smem_u32(Zhi), zlo_addr = smem_u32(Zlo);
  // end-of-evaluation exchange buffers (alias stage 0, idle between evaluations)
  // Gsum rows are PP + 4 floats apart, so the epilogue's row-per-lane float4
  // stores spread over 8 bank groups
  const int GS = PP + 4;
  float* Gsum = reinterpret_cast<float*>(stage0);                           // [128][PP + 4]
  double* llpart = reinterpret_cast<double*>(stage0 + (size_t)kCT * GS * 4);  // [4][128]
  const uint32_t gsum_addr = smem_u32(Gsum), llpart_addr = smem_u32(llpart);

  // every CTA of the cluster must be running before any DSMEM access
  cluster_sync();

  const int L = a.n_steps;
  const int E = (a.cache_valid ? 0 : 1) + a.n_iter * L;
  uint32_t gt = 0;  // running tile counter (identical in every role)
  for (int e = 0; e < E; ++e) {
    const bool cache_eval = !a.cache_valid && e == 0;
    const int ee = e - (a.cache_valid ? 0 : 1);
    const int it = cache_eval ? 0 : ee / L;
    const int l = cache_eval ? 0 : ee % L;
    const bool need_ll = MH || (!SG && (cache_eval || l == L - 1));
    const int64_t t = t0 + it;
    const uint32_t iter = (uint32_t)t;

    // ================= pre phase: position for this evaluation, broadcast as Z
    if (owner) {
      if (SG) {
        if (!cache_eval) {
          // the update of iteration t from the cached gradient of the current state
          const bool sgld = a.sg_method == EDG_SGMCMC_SGLD;
          const float lr = sgld ? a.step_size / powf((float)(t + 1), 0.55f) : a.step_size * 0.01f;
          const float sq = sqrtf(sgld ? lr : lr * a.friction);
#pragma unroll
          for (int i = 0; i < kMaxEPT; ++i) {
            const int d = d0 + i;
            const bool ok = cvalid && i < EPT && d < P;
            float e = 0.0f;
            if (ok)
              e = a.noise ? a.noise[((size_t)it * a.C + cg) * P + d]
                          : philox_normal(a.seed, 5u, iter, (uint32_t)cg, (uint32_t)d);
            if (sgld) {
              zr[i] = ok ? zr[i] + 0.5f * lr * gr[i] + sq * e : 0.0f;
            } else {
              const float vv = rr[i];
              zr[i] = ok ? zr[i] + vv : 0.0f;
              rr[i] = ok ? (1.0f - 0.5f * a.friction) * vv + lr * gr[i] + sq * e : 0.0f;
            }
          }
        }
      } else if (MH) {
        if (!cache_eval) {
          // the proposal z' = (random walk ? z : loc) + scale e (Philox stream 6)
          // from the accepted state, and log g(z | z') - log g(z' | z) in FP64
          // (zero for the random walk), kept in kin0
          double lq = 0.0;
#pragma unroll
          for (int i = 0; i < kMaxEPT; ++i) {
            const int d = d0 + i;
            const bool ok = cvalid && i < EPT && d < P;
            float zn = 0.0f;
            if (ok) {
              const float e = a.noise ? a.noise[((size_t)it * a.C + cg) * P + d]
                                      : philox_normal(a.seed, 6u, iter, (uint32_t)cg, (uint32_t)d);
              const float s = a.mh_scale[d], zc = zg[d];
              zn = (a.mh_loc ? a.mh_loc[d] : zc) + s * e;
              if (a.mh_loc) {
                const double u0 = ((double)zc - a.mh_loc[d]) / s, u1 = ((double)zn - a.mh_loc[d]) / s;
                lq += -0.5 * u0 * u0 + 0.5 * u1 * u1;
              }
            }
            zr[i] = zn;
          }
          for (int o = TPC >> 1; o > 0; o >>= 1) lq += __shfl_xor_sync(0xffffffffu, lq, o);
          kin0 = lq;
        }
      } else if (!cache_eval) {
        if (l == 0) {
          float kf = 0.0f;
#pragma unroll
          for (int i = 0; i < kMaxEPT; ++i) {
            const int d = d0 + i;
            float r = 0.0f;
            if (cvalid && i < EPT && d < P)
              r = a.r_ovr ? a.r_ovr[((size_t)it * a.C + cg) * P + d]
                          : philox_normal(a.seed, 1u, iter, (uint32_t)cg, (uint32_t)d);
            const bool ok = cvalid && i < EPT && d < P;
            rr[i] = r;
            zr[i] = ok ? zg[d] : 0.0f;
            gr[i] = ok ? gg[d] : 0.0f;
            kf = fmaf(r, r, kf);
          }
          // FP32 over this thread's few elements, FP64 across the chain's
          // threads (GB300's FP64 rate is a small fraction of its FP32 rate)
          double k = (double)kf;
          for (int o = TPC >> 1; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
          kin0 = k;
        }
#pragma unroll
        for (int i = 0; i < kMaxEPT; ++i) {
          rr[i] = rr[i] + half * gr[i];
          zr[i] = zr[i] + eps * rr[i];
        }
      }
      // Z hi/lo into every CTA of the cluster (canonical K-major layout)
#pragma unroll
      for (int i = 0; i < kMaxEPT; i += 4) {
        if (i < EPT) {
          float h[4], lo4[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float v = zr[i + j] * a.zscale;
            h[j] = tf32_rna(v);
            lo4[j] = tf32_rna(v - h[j]);
          }
          const uint32_t off = kmajor_off(cc, d0 + i, PP);
          for (uint32_t q = 0; q < R; ++q) {
            st_dsmem4(mapa(zhi_addr + off, q), make_float4(h[0], h[1], h[2], h[3]));
            st_dsmem4(mapa(zlo_addr + off, q), make_float4(lo4[0], lo4[1], lo4[2], lo4[3]));
          }
        }
      }
      fence_proxy_async();
    }
    __syncwarp();
    cluster_sync();  // Z ready in every CTA

    // ================= gradient evaluation over this CTA's row tiles
    if (warp == 0) {
      // lane 0 streams the forward parts (X hi/lo), lane 1 the backward parts
      // (X^T hi/lo); each part is one bulk copy into a double buffer
      if (lane < 2) {
        const uint32_t part_off = lane == 0 ? 0u : XB;
        const uint32_t bytes = lane == 0 ? XB : TB;
        const uint32_t full = lane == 0 ? b_fullx : b_fullt;
        const uint32_t empty = lane == 0 ? b_emptyx : b_emptyt;
        for (int i = 0; i < nt; ++i) {
          const uint32_t g = gt + i, s = g & 1u;
          if (g >= 2) mbar_wait(empty + 8 * s, ((g >> 1) - 1) & 1u, err);
          if (MH && lane == 1) {
            mbar_arrive(full + 8 * s);  // Metropolis-Hastings reads no X^T
          } else {
            mbar_expect_tx(full + 8 * s, bytes);
            bulk_g2s(smem_u32((s ? stage1 : stage0) + part_off),
                     a.tiles + (size_t)(t_begin + i) * SB + part_off, bytes, full + 8 * s);
          }
        }
      }
      __syncwarp();
    } else if (warp == kFWarp) {
      // forward issuer: the whole warp runs the loop, one elected lane issues
      const uint32_t issue = elect_one();
      fence_proxy_async();
      const uint32_t id_f = idesc_tf32(kCT, kNR);
      // Descriptors are built once; a K step of 8 tf32 elements is 256 bytes,
      // i.e. +16 in the descriptor's start-address field (address >> 4).
      const uint32_t sbo_k = 32u * PP;
      const uint64_t dz_hi = sdesc(zhi_addr, 128, sbo_k), dz_lo = sdesc(zlo_addr, 128, sbo_k);
      const uint32_t st0 = smem_u32(stage0), st1 = smem_u32(stage1);
      const uint64_t dx_hi[2] = {sdesc(st0, 128, sbo_k), sdesc(st1, 128, sbo_k)};
      const uint64_t dx_lo[2] = {sdesc(st0 + 256u * PP, 128, sbo_k),
                                 sdesc(st1 + 256u * PP, 128, sbo_k)};
      // forward K steps: only the 8-wide K blocks that hold a coordinate of z
      // (columns P .. PP-1 of Z and of the X tile are zero), 7 instead of 8
      // for P = 51
      const int KF = (P + 7) / 8;
      for (int i = 0; i < nt; ++i) {
        const uint32_t g = gt + i, s = g & 1u, b = g & 1u;
        mbar_wait(b_fullx + 8 * s, (g >> 1) & 1u, err);
        // eta buffer b is rewritten: the epilogue has read tile g-2's eta once
        // all its warps arrived on r for that tile
        if (g >= 2) mbar_wait(b_r + 8 * b, ((g >> 1) - 1) & 1u, err);
        tc_fence_after();
        const uint32_t dt = tbase + COL_ETA(b);
        const uint64_t xh = s ? dx_hi[1] : dx_hi[0], xl = s ? dx_lo[1] : dx_lo[0];
        // lo products first (small running sum), hi*hi last: fewer
        // truncating additions land on a large accumulator
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          if (kk < KF) {
            mma_ss_if(issue, dt, dz_hi + 16 * kk, xl + 16 * kk, id_f, kk > 0 ? 1u : 0u);
            mma_ss_if(issue, dt, dz_lo + 16 * kk, xh + 16 * kk, id_f, 1u);
          }
        }
#pragma unroll
        for (int kk = 0; kk < 8; ++kk)
          if (kk < KF) mma_ss_if(issue, dt, dz_hi + 16 * kk, xh + 16 * kk, id_f, 1u);
        mma_commit_if(issue, b_emptyx + 8 * s);  // forward operands consumed
        mma_commit_if(issue, b_eta + 8 * b);
      }
      __syncwarp();
    } else if (warp == kBWarp) {
      // backward issuer, concurrent with the forward one: each warp's barrier
      // waits hide behind the other's MMAs in the tensor pipe
      if (!SG && !cache_eval && l == L - 1) {
        // the Metropolis uniforms of this CTA's chains and their FP64 logs,
        // computed here (this warp mostly waits) rather than by the owners
        for (int c = lane; c < CPO; c += 32) {
          const int cgl = c_base + (int)rank * CPO + c;
          double lu = 0.0;
          if (cgl < a.C)
            lu = log(a.u_ovr ? a.u_ovr[(size_t)it * a.C + cgl]
                             : u01d(philox_at(a.seed, MH ? 7u : 2u, iter, (uint32_t)cgl, 0u).x));
          s_logu[c] = lu;
        }
      }
      const uint32_t issue = elect_one();
      fence_proxy_async();
      const uint32_t id_b = idesc_tf32(kCT, PP);
      const uint32_t sbo_t = 32u * kNR;
      const uint32_t st0 = smem_u32(stage0), st1 = smem_u32(stage1);
      const uint64_t dt_hi[2] = {sdesc(st0 + 512u * PP, 128, sbo_t),
                                 sdesc(st1 + 512u * PP, 128, sbo_t)};
      const uint64_t dt_lo[2] = {sdesc(st0 + 768u * PP, 128, sbo_t),
                                 sdesc(st1 + 768u * PP, 128, sbo_t)};
      for (int i = 0; i < nt; ++i) {
        const uint32_t g = gt + i, s = g & 1u, b = g & 1u;
        mbar_wait(b_fullt + 8 * s, (g >> 1) & 1u, err);
        // r of tile g complete also means every epilogue warp has read the
        // gradient partial of tile g-2 (it does so before arriving on r), so
        // the partial buffer b is free
        mbar_wait(b_r + 8 * b, (g >> 1) & 1u, err);
        tc_fence_after();
        if (!MH) {  // Metropolis-Hastings needs no gradient: the commits alone
          const uint32_t dg = tbase + COL_GP(b);
          const uint32_t rh = tbase + COL_RHI(b), rl = tbase + COL_RLO(b);
          const uint64_t th = s ? dt_hi[1] : dt_hi[0], tlo = s ? dt_lo[1] : dt_lo[0];
#pragma unroll
          for (int kk = 0; kk < kNR / 8; ++kk) {
            mma_ts_if(issue, dg, rh + 8u * kk, tlo + 16 * kk, id_b, kk > 0 ? 1u : 0u);
            mma_ts_if(issue, dg, rl + 8u * kk, th + 16 * kk, id_b, 1u);
          }
#pragma unroll
          for (int kk = 0; kk < kNR / 8; ++kk)
            mma_ts_if(issue, dg, rh + 8u * kk, th + 16 * kk, id_b, 1u);
        }
        mma_commit_if(issue, b_emptyt + 8 * s);
        mma_commit_if(issue, b_gfull + 8 * b);
      }
      __syncwarp();
    } else {
      // epilogue: TMEM lane = chain row 32*(warp%4) + lane; the four warps of a
      // lane quarter split the tile's 64 rows (TMEM columns) and the gradient
      // columns into quarters
      const int q = warp & 3;
      const int qs = (warp - 2) >> 2;
      const int row = 32 * q + lane;
      const uint32_t tl = tbase + ((uint32_t)(32 * q) << 16);
      const int gcols = PP >> 2;        // gradient columns of this quarter (4, 8 or 16)
      const int gc0 = qs * gcols;
      float Gacc[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) Gacc[k] = 0.0f;
      Kahan kl;
      const bool y_vec = (reinterpret_cast<uintptr_t>(a.y) & 15u) == 0;
      auto consume_gpart = [&](int i) {
        const uint32_t g = gt + i, b = g & 1u;
        mbar_wait(b_gfull + 8 * b, (g >> 1) & 1u, err);
        tc_fence_after();
        const uint32_t ga = tl + COL_GP(b) + gc0;
        if (MH) {
          // no gradient partial was computed
        } else if (gcols == 16) {
          float v[16];
          tmem_ld16(ga, v);
#pragma unroll
          for (int k = 0; k < 16; ++k) Gacc[k] += v[k];
        } else if (gcols == 8) {
          float v[8];
          tmem_ld8(ga, v);
#pragma unroll
          for (int k = 0; k < 8; ++k) Gacc[k] += v[k];
        } else {
          float v[4];
          tmem_ld4(ga, v);
#pragma unroll
          for (int k = 0; k < 4; ++k) Gacc[k] += v[k];
        }
        tc_fence_before();
        __syncwarp();
      };
      // The tile loop, compiled once per (log-likelihood wanted, likelihood)
      // and selected once per evaluation, so the loop body has no branch on
      // either.
      auto tile_loop = [&](auto ll_tag, auto bern_tag) {
        constexpr bool LL = decltype(ll_tag)::value;
        constexpr bool BERN = decltype(bern_tag)::value;
        for (int i = 0; i < nt; ++i) {
          const uint32_t g = gt + i, b = g & 1u;
          // y of this thread's 16 rows straight from the model (L2-resident;
          // the next tile's rows are prefetched into L1 below, since eta is
          // usually ready when a tile starts and would not hide an L2 latency)
          const int row0 = (t_begin + i) * kNR + 16 * qs;
          const int nvalid = min(kNR, a.N - (t_begin + i) * kNR) - 16 * qs;
          float ye[16];
          if (nvalid >= 16 && y_vec) {
            const float4* y4p = reinterpret_cast<const float4*>(a.y + row0);
#pragma unroll
            for (int k4 = 0; k4 < 4; ++k4) {
              const float4 y4 = __ldg(y4p + k4);
              ye[4 * k4] = y4.x;
              ye[4 * k4 + 1] = y4.y;
              ye[4 * k4 + 2] = y4.z;
              ye[4 * k4 + 3] = y4.w;
            }
          } else {
#pragma unroll
            for (int k = 0; k < 16; ++k) ye[k] = k < nvalid ? __ldg(a.y + row0 + k) : 0.0f;
          }
          if (lane == 0 && i + 1 < nt) prefetch_l1(a.y + min(row0 + kNR, a.N - 1));
          mbar_wait(b_eta + 8 * b, (g >> 1) & 1u, err);
          tc_fence_after();
          // eta of 16 rows in one TMEM load; then two halves of 8 rows:
          // residuals, st hi / lo.  One compact loop per (log-likelihood wanted,
          // likelihood), so the leapfrog's inner evaluations run the short
          // residual-only loop.
          float ve[16];
          tmem_ld16_issue(tl + COL_ETA(b) + 16 * qs, ve);
          tmem_ld_wait(ve);
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            float lo[8];
            float (&v)[8] = *reinterpret_cast<float (*)[8]>(&ve[8 * h]);
            const float (&yh)[8] = *reinterpret_cast<const float (*)[8]>(&ye[8 * h]);
            const uint32_t col = 16 * qs + 8 * h;
            const int nv = nvalid - 8 * h;
            residual_block<LL, BERN, SG>(v, lo, yh, nv, a.inv_lik_var, a.lik_norm, kl, a.dscale);
            if (!MH) {  // Metropolis-Hastings keeps only the log-likelihood
              tmem_st8(tl + COL_RHI(b) + col, v);
              tmem_st8(tl + COL_RLO(b) + col, lo);
            }
          }
          tmem_st_wait();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(b_r + 8 * b);
          if (i >= 1) consume_gpart(i - 1);
        }
      };
      const bool bern = a.lik == EDG_LIK_BERNOULLI;
      if (need_ll) {
        if (bern)
          tile_loop(std::true_type{}, std::true_type{});
        else
          tile_loop(std::true_type{}, std::false_type{});
      } else {
        if (bern)
          tile_loop(std::false_type{}, std::true_type{});
        else
          tile_loop(std::false_type{}, std::false_type{});
      }
      consume_gpart(nt - 1);
      // this CTA's partial gradient and log-likelihood for the owners
#pragma unroll
      for (int c4 = 0; c4 < 4; ++c4)
        if (4 * c4 < gcols)
          *reinterpret_cast<float4*>(Gsum + row * GS + gc0 + 4 * c4) =
              make_float4(Gacc[4 * c4], Gacc[4 * c4 + 1], Gacc[4 * c4 + 2], Gacc[4 * c4 + 3]);
      if (need_ll) llpart[qs * kCT + row] = kl.value();
      tc_fence_before();
    }
    gt += (uint32_t)nt;
    __syncwarp();
    cluster_sync();  // partial gradients of every CTA ready

    // ================= post phase: reduce, leapfrog kick, Metropolis
    if (owner) {
      float G[kMaxEPT];
#pragma unroll
      for (int i = 0; i < kMaxEPT; ++i) G[i] = 0.0f;
      for (uint32_t q = 0; q < R; ++q) {
#pragma unroll
        for (int i = 0; i < kMaxEPT; i += 4) {
          if (i < EPT) {
            const float4 v = ld_dsmem4(mapa(gsum_addr + 4u * (cc * GS + d0 + i), q));
            G[i] += v.x;
            G[i + 1] += v.y;
            G[i + 2] += v.z;
            G[i + 3] += v.w;
          }
        }
      }
      // log-likelihood of the chain: R CTAs x 4 quarter partials, one per
      // thread of the chain (4R threads), reduced across them
      double llsum = 0.0;
      if (need_ll) {
        const uint32_t q = (uint32_t)part >> 2, h = (uint32_t)part & 3u;
        llsum = ld_dsmem_f64(mapa(llpart_addr + 8u * (h * kCT + cc), q));
        for (int o = TPC >> 1; o > 0; o >>= 1) llsum += __shfl_xor_sync(0xffffffffu, llsum, o);
      }
      float lpf = 0.0f;
#pragma unroll
      for (int i = 0; i < kMaxEPT; ++i) {
        const int d = min(d0 + i, PP - 1);
        const float pr = i < EPT ? s_pprec[d] : 0.0f;
        const float dz = zr[i] - s_ploc[d];
        G[i] = (i < EPT && d0 + i < P) ? G[i] - dz * pr : 0.0f;
        if (need_ll) lpf += -0.5f * dz * dz * pr;
      }
      double lp = plogc + (double)lpf;
      if (need_ll)
        for (int o = TPC >> 1; o > 0; o >>= 1) lp += __shfl_xor_sync(0xffffffffu, lp, o);
      if (SG) {
        // the new state's gradient, cached for the next iteration's update;
        // the new state itself is kept (every proposal is accepted)
#pragma unroll
        for (int i = 0; i < kMaxEPT; ++i) gr[i] = G[i];
        if (cvalid) {
#pragma unroll
          for (int i = 0; i < kMaxEPT; ++i) {
            const int d = d0 + i;
            if (i < EPT && d < P) {
              gg[d] = G[i];
              if (!cache_eval) {
                if (!isfinite(zr[i])) atomicAdd(&a.state->nonfinite, 1u);
                zg[d] = zr[i];
                if (a.samples && t < a.T_cap) a.samples[((size_t)t * a.C + cg) * P + d] = zr[i];
              }
            }
          }
          if (!cache_eval && part == 0 && a.n_accept) a.n_accept[cg] += 1;
        }
      } else if (cache_eval) {
        if (cvalid) {
#pragma unroll
          for (int i = 0; i < kMaxEPT; ++i)
            if (i < EPT && d0 + i < P) gg[d0 + i] = G[i];
          if (part == 0) a.lj[cg] = llsum + lp;
        }
      } else if (MH) {
        // ratio = log p(x, z') - log p(x, z) + log g(z | z') - log g(z' | z),
        // accept if log u < ratio (Philox stream 7), on the chain's first thread
        const double lj_new = llsum + lp;
        double ratio = 0.0;
        int acc_lead = 0;
        if (part == 0 && cvalid) {
          ratio = lj_new - a.lj[cg] + kin0;
          acc_lead = s_logu[chain_local] < ratio ? 1 : 0;
        }
        const bool accept = __shfl_sync(0xffffffffu, acc_lead, lane & ~(TPC - 1)) != 0;
        if (cvalid) {
          if (part == 0) {
            if (accept) a.lj[cg] = lj_new;
            if (a.n_accept) a.n_accept[cg] += accept ? 1 : 0;
            if (a.ratio_out) a.ratio_out[(size_t)it * a.C + cg] = ratio;
          }
#pragma unroll
          for (int i = 0; i < kMaxEPT; ++i) {
            const int d = d0 + i;
            if (i < EPT && d < P) {
              const float kept = accept ? zr[i] : zg[d];
              if (accept) zg[d] = zr[i];
              if (a.samples && t < a.T_cap) a.samples[((size_t)t * a.C + cg) * P + d] = kept;
            }
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < kMaxEPT; ++i) {
          gr[i] = G[i];
          rr[i] = rr[i] + half * G[i];
        }
        if (l == L - 1) {
          // Metropolis test in FP64 (hmc.py:100-109), on the chain's first
          // thread; the decision is broadcast to the chain's other threads
          float kf = 0.0f;
#pragma unroll
          for (int i = 0; i < kMaxEPT; ++i) kf = fmaf(rr[i], rr[i], kf);
          double k = (double)kf;
          for (int o = TPC >> 1; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
          const double lj_new = llsum + lp;
          double ratio = 0.0;
          int acc_lead = 0;
          if (part == 0 && cvalid) {
            const double lj0 = a.lj[cg];
            ratio = 0.5 * kin0 - 0.5 * k + lj_new - lj0;
            acc_lead = s_logu[chain_local] < ratio ? 1 : 0;
          }
          const bool accept = __shfl_sync(0xffffffffu, acc_lead, lane & ~(TPC - 1)) != 0;
          if (cvalid) {
            if (part == 0) {
              if (accept) a.lj[cg] = lj_new;
              if (a.n_accept) a.n_accept[cg] += accept ? 1 : 0;
              if (a.ratio_out) a.ratio_out[(size_t)it * a.C + cg] = ratio;
            }
#pragma unroll
            for (int i = 0; i < kMaxEPT; ++i) {
              const int d = d0 + i;
              if (i < EPT && d < P) {
                float kept;
                if (accept) {
                  kept = zr[i];
                  zg[d] = zr[i];
                  gg[d] = gr[i];
                } else {
                  kept = zg[d];
                }
                if (a.samples && t < a.T_cap) a.samples[((size_t)t * a.C + cg) * P + d] = kept;
                if (a.moments) {
                  const size_t gi = (size_t)cg * P + d;
                  a.moments[gi] += (double)kept;
                  a.moments[(size_t)a.C * P + gi] += (double)kept * (double)kept;
                }
              }
            }
          }
        }
      }
    }
  }

  if (SG && cvalid && a.v) {
    // the SGHMC velocity for the next launch
#pragma unroll
    for (int i = 0; i < kMaxEPT; ++i)
      if (i < EPT && d0 + i < P) a.v[(size_t)cg * P + d0 + i] = rr[i];
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                 "r"(kTmemCols));
  }
  cluster_sync();  // no CTA leaves while a peer may still read its shared memory
  if (threadIdx.x == 0) {
    if (*err) atomicExch(&a.state->error, (uint32_t)(-EDG_E_TIMEOUT));
    __threadfence();
    const unsigned prev = atomicAdd(&a.state->done, 1u);
    s_last = (prev == gridDim.x - 1);
    if (s_last) {
      a.state->t = t0 + a.n_iter;
      a.state->done = 0;
      __threadfence();
    }
  }
}

// ------------------------------------------------------------------ host side
// Operand width: 16, 32 or 64 columns (the owner split needs PP / (2R) in {4, 8}).
static int padded_P(int P) { return P <= 16 ? 16 : (P <= 32 ? 32 : round_up(P, 64)); }

// Dynamic shared memory: at least 120 KB so that no two CTAs share an SM
// (each allocates all 512 TMEM columns; a second resident CTA would block in
// tcgen05.alloc while its cluster waits on it).
static size_t smem_bytes(int PP) {
  return std::max<size_t>(2 * (size_t)stage_bytes(PP) + (size_t)1024 * PP + 256, 120 * 1024);
}

static int sm_count() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return v > 0 ? v : 1;
}

// Cluster size: a power of two R <= 8 with R <= ntiles and owner elements per
// thread PP/(4R) equal to 4 (R = PP/16), and clusters * R close to the SM count.
static int choose_R(int PP, int C, int ntiles, int want) {
  const int nclusters = (C + kCT - 1) / kCT;
  int best = 0;
  for (int R = 1; R <= 8; R <<= 1) {
    const int ept = PP / (4 * R);
    if (PP % (4 * R) != 0 || ept > kMaxEPT || ept % 4 != 0 || R > ntiles) continue;
    if (want > 0) {
      if (R == want) return R;
      continue;
    }
    if (nclusters * R <= sm_count() || best == 0) best = R;
  }
  return best;
}

}  // namespace tc
}  // namespace edg

using namespace edg;
using namespace edg::tc;

extern "C" size_t edg_hmc_glm_tc_tiles_bytes(const edg_glm_t* model) {
  GLMDev m;
  if (make_glm(model, &m) != EDG_OK) return 0;
  const int PP = padded_P(m.P);
  if (PP > 64) return 0;
  const int ntiles = (m.N + kNR - 1) / kNR;
  return (size_t)ntiles * stage_bytes(PP);
}

extern "C" int edg_hmc_glm_tc_prepare(const edg_glm_t* model, void* tiles, size_t tiles_bytes,
                                      void* stream) {
  GLMDev m;
  int rc = make_glm(model, &m);
  if (rc) return rc;
  const int PP = padded_P(m.P);
  EDG_REQUIRE(PP <= 64, EDG_E_UNSUPPORTED, "tensor-core HMC supports P <= 64 (got %d)", m.P);
  const int ntiles = (m.N + kNR - 1) / kNR;
  const size_t need = (size_t)ntiles * stage_bytes(PP);
  EDG_REQUIRE(tiles && tiles_bytes >= need, EDG_E_WORKSPACE, "tiles buffer of %zu bytes needed",
              need);
  const int64_t total = (int64_t)ntiles * kNR * PP;
  prep_tiles_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      m.X, m.N, m.D, m.bias, PP, ntiles, reinterpret_cast<unsigned char*>(tiles));
  return check_launch("prep_tiles_kernel");
}

// One launch of the tensor-core kernel: a cluster of R CTAs per 128 chains.
template <int MODE>
static int launch_tc(const TcArgs& a, int PP, int R, void* stream) {
  const size_t sm = smem_bytes(PP);
  int rc = set_max_dyn_smem(hmc_glm_tc_kernel<MODE>, sm, "hmc_glm_tc_kernel");
  if (rc) return rc;
  const int nclusters = (a.C + kCT - 1) / kCT;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(nclusters * R);
  lc.blockDim = dim3(kThreads);
  lc.dynamicSmemBytes = sm;
  lc.stream = (cudaStream_t)stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = R;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&lc, hmc_glm_tc_kernel<MODE>, a);
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "hmc_glm_tc_kernel launch: %s", cudaGetErrorString(e));
  return check_launch("hmc_glm_tc_kernel");
}

extern "C" int edg_hmc_glm_tc_run(const edg_glm_t* model, const edg_hmc_t* cfg, int32_t C,
                                  int32_t n_iter, const void* tiles, float* z, float* grad,
                                  double* lj, int32_t cache_valid, int32_t* n_accept,
                                  edg_state_t* state, float* samples, int64_t T_cap,
                                  double* moments, const float* r_override,
                                  const double* u_override, double* ratio_out, void* stream) {
  GLMDev m;
  int rc = make_glm(model, &m);
  if (rc) return rc;
  EDG_REQUIRE(cfg && tiles, EDG_E_NULL, "cfg and tiles must not be NULL");
  EDG_REQUIRE(z && grad && lj && state, EDG_E_NULL, "z, grad, lj and state must not be NULL");
  EDG_REQUIRE(C > 0 && n_iter >= 0, EDG_E_SHAPE, "C must be positive and n_iter >= 0");
  EDG_REQUIRE(cfg->n_steps > 0, EDG_E_UNSUPPORTED,
              "tensor-core HMC needs n_steps > 0 (use edg_hmc_glm_run)");
  EDG_REQUIRE(!samples || T_cap > 0, EDG_E_SHAPE, "T_cap must be positive when samples is given");
  const int PP = padded_P(m.P);
  EDG_REQUIRE(PP <= 64, EDG_E_UNSUPPORTED, "tensor-core HMC supports P <= 64 (got %d)", m.P);
  if (n_iter == 0 && cache_valid) return EDG_OK;
  const int ntiles = (m.N + kNR - 1) / kNR;
  const int R = choose_R(PP, C, ntiles, cfg->cluster_size);
  EDG_REQUIRE(R > 0, EDG_E_UNSUPPORTED,
              "no cluster size fits P=%d with %d row tiles (requested %d)", m.P, ntiles,
              cfg->cluster_size);
  TcArgs a;
  a.tiles = reinterpret_cast<const unsigned char*>(tiles);
  a.y = m.y;
  a.ntiles = ntiles;
  a.N = m.N;
  a.P = m.P;
  a.PP = PP;
  a.lik = m.lik;
  a.zscale = m.lik == EDG_LIK_BERNOULLI ? -kLog2e : 1.0f;
  a.inv_lik_var = m.inv_lik_var;
  a.lik_norm = m.lik_norm;
  a.prior_loc = m.prior_loc;
  a.prior_scale = m.prior_scale;
  a.C = C;
  a.n_iter = n_iter;
  a.n_steps = cfg->n_steps;
  a.cache_valid = cache_valid;
  a.step_size = cfg->step_size;
  a.seed = cfg->seed;
  a.z = z;
  a.grad = grad;
  a.lj = lj;
  a.n_accept = n_accept;
  a.state = state;
  a.samples = samples;
  a.T_cap = T_cap;
  a.moments = moments;
  a.r_ovr = r_override;
  a.u_ovr = u_override;
  a.ratio_out = ratio_out;
  a.sg_method = -1;
  a.friction = 0.0f;
  a.dscale = 1.0f;
  a.v = nullptr;
  a.noise = nullptr;
  a.mh_loc = nullptr;
  a.mh_scale = nullptr;
  return launch_tc<0>(a, PP, R, stream);
}

extern "C" int edg_sgmcmc_glm_tc_run(const edg_glm_t* model, const edg_sgmcmc_t* cfg, int32_t C,
                                     int32_t n_iter, const void* tiles, float* z, float* v,
                                     float* grad, int32_t cache_valid, int32_t* n_accept,
                                     edg_state_t* state, float* samples, int64_t T_cap,
                                     const float* noise_override, void* stream) {
  GLMDev m;
  int rc = make_glm(model, &m);
  if (rc) return rc;
  EDG_REQUIRE(cfg && tiles, EDG_E_NULL, "cfg and tiles must not be NULL");
  EDG_REQUIRE(z && grad && state, EDG_E_NULL, "z, grad and state must not be NULL");
  EDG_REQUIRE(cfg->method == EDG_SGMCMC_SGLD || cfg->method == EDG_SGMCMC_SGHMC, EDG_E_VALUE,
              "unknown SG-MCMC method %d", cfg->method);
  EDG_REQUIRE(cfg->method != EDG_SGMCMC_SGHMC || v, EDG_E_NULL, "SGHMC needs the velocity v");
  EDG_REQUIRE(cfg->step_size > 0.0f && cfg->friction >= 0.0f, EDG_E_VALUE,
              "step_size must be positive and friction >= 0");
  EDG_REQUIRE(C > 0 && n_iter >= 0, EDG_E_SHAPE, "C must be positive and n_iter >= 0");
  EDG_REQUIRE(!samples || T_cap > 0, EDG_E_SHAPE, "T_cap must be positive when samples is given");
  const int PP = padded_P(m.P);
  EDG_REQUIRE(PP <= 64, EDG_E_UNSUPPORTED, "tensor-core SG-MCMC supports P <= 64 (got %d)", m.P);
  if (n_iter == 0 && cache_valid) return EDG_OK;
  const int ntiles = (m.N + kNR - 1) / kNR;
  const int R = choose_R(PP, C, ntiles, 0);
  EDG_REQUIRE(R > 0, EDG_E_UNSUPPORTED, "no cluster size fits P=%d with %d row tiles", m.P,
              ntiles);
  TcArgs a = {};
  a.tiles = reinterpret_cast<const unsigned char*>(tiles);
  a.y = m.y;
  a.ntiles = ntiles;
  a.N = m.N;
  a.P = m.P;
  a.PP = PP;
  a.lik = m.lik;
  a.zscale = m.lik == EDG_LIK_BERNOULLI ? -kLog2e : 1.0f;
  a.inv_lik_var = m.inv_lik_var;
  a.lik_norm = m.lik_norm;
  a.prior_loc = m.prior_loc;
  a.prior_scale = m.prior_scale;
  a.C = C;
  a.n_iter = n_iter;
  a.n_steps = 1;  // one gradient evaluation per iteration
  a.cache_valid = cache_valid;
  a.step_size = cfg->step_size;
  a.seed = cfg->seed;
  a.z = z;
  a.grad = grad;
  a.lj = nullptr;
  a.n_accept = n_accept;
  a.state = state;
  a.samples = samples;
  a.T_cap = T_cap;
  a.sg_method = cfg->method;
  a.friction = cfg->friction;
  a.dscale = cfg->data_scale;
  a.v = cfg->method == EDG_SGMCMC_SGHMC ? v : nullptr;
  a.noise = noise_override;
  a.mh_loc = nullptr;
  a.mh_scale = nullptr;
  return launch_tc<1>(a, PP, R, stream);
}

extern "C" int edg_mh_glm_tc_run(const edg_glm_t* model, const edg_mh_t* cfg, int32_t C,
                                 int32_t n_iter, const void* tiles, float* z, float* grad,
                                 double* lj, int32_t cache_valid, int32_t* n_accept,
                                 edg_state_t* state, float* samples, int64_t T_cap,
                                 const float* e_override, const double* u_override,
                                 double* ratio_out, void* stream) {
  GLMDev m;
  int rc = make_glm(model, &m);
  if (rc) return rc;
  EDG_REQUIRE(cfg && tiles && cfg->proposal_scale, EDG_E_NULL,
              "cfg, tiles and cfg->proposal_scale must not be NULL");
  EDG_REQUIRE(z && grad && lj && state, EDG_E_NULL, "z, grad, lj and state must not be NULL");
  EDG_REQUIRE(C > 0 && n_iter >= 0, EDG_E_SHAPE, "C must be positive and n_iter >= 0");
  EDG_REQUIRE(!samples || T_cap > 0, EDG_E_SHAPE, "T_cap must be positive when samples is given");
  const int PP = padded_P(m.P);
  EDG_REQUIRE(PP <= 64, EDG_E_UNSUPPORTED, "tensor-core Metropolis-Hastings supports P <= 64 (got %d)",
              m.P);
  if (n_iter == 0 && cache_valid) return EDG_OK;
  const int ntiles = (m.N + kNR - 1) / kNR;
  const int R = choose_R(PP, C, ntiles, 0);
  EDG_REQUIRE(R > 0, EDG_E_UNSUPPORTED, "no cluster size fits P=%d with %d row tiles", m.P,
              ntiles);
  TcArgs a = {};
  a.tiles = reinterpret_cast<const unsigned char*>(tiles);
  a.y = m.y;
  a.ntiles = ntiles;
  a.N = m.N;
  a.P = m.P;
  a.PP = PP;
  a.lik = m.lik;
  a.zscale = m.lik == EDG_LIK_BERNOULLI ? -kLog2e : 1.0f;
  a.inv_lik_var = m.inv_lik_var;
  a.lik_norm = m.lik_norm;
  a.prior_loc = m.prior_loc;
  a.prior_scale = m.prior_scale;
  a.C = C;
  a.n_iter = n_iter;
  a.n_steps = 1;  // one log-joint evaluation per iteration
  a.cache_valid = cache_valid;
  a.seed = cfg->seed;
  a.z = z;
  a.grad = grad;
  a.lj = lj;
  a.n_accept = n_accept;
  a.state = state;
  a.samples = samples;
  a.T_cap = T_cap;
  a.u_ovr = u_override;
  a.ratio_out = ratio_out;
  a.sg_method = -1;
  a.dscale = 1.0f;
  a.noise = e_override;
  a.mh_loc = cfg->proposal_loc;
  a.mh_scale = cfg->proposal_scale;
  return launch_tc<2>(a, PP, R, stream);
}
