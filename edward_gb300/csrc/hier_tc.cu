// Ragged batch of hierarchical logistic regressions under HMC on the tensor
// cores.  Same model, state layout, draws and contract as hier.cu
// (edg_hmc_hier_run); every gradient evaluation is computed as tcgen05
// 3xTF32 GEMMs (hi*hi + hi*lo + lo*hi, FP32 accumulation in TMEM).
//
// One CTA per (instance, 64 chains), 512 threads, all 512 TMEM columns:
//   XF  [lanes = 128 rows of a tile, columns = features]   hi at 0, lo at 128
//   XT  [lanes = features, columns = 64 rows of a half]     hi at 256, lo at 320
//   ETA [lanes = rows, columns = 64 chains]                 at 384 (forward accumulator)
//   GT  [lanes = features, columns = 64 chains]             at 448 (backward accumulator)
// tf32 operands must be K-major (a transposed shared-memory operand reads as
// zeros), so X enters the tensor core in both orientations, and both come
// from TMEM (the A operand of the TS form).  X is read from HBM as one fp32
// plane, once per evaluation for all 64 chains.  edg_hmc_hier_tc_prepare
// re-lays each X_i once into 128-row tiles with a row pitch of Dp_i + 1
// floats (Dp_i = D_i rounded up to 8; y_i in the pad column Dp_i, zero
// elsewhere beyond D_i and beyond N_i), so that each
// 64-row half of a tile is one contiguous bulk copy (issued by one thread,
// completed on an mbarrier) into a shared staging half whose odd pitch lets
// one thread per feature (XT) and one thread per row (XF) read it without
// bank conflicts; the hi/lo split is made in registers.  The copies of the
// next tile run under the current tile's MMAs.  Shared memory holds the
// staging halves and the B operands: the
// positions W [64 chains, K = features] and the residuals R [64 chains,
// K = 128 rows], hi and lo planes in the no-swizzle K-major core-matrix layout
// with 144-byte strides (bank-conflict-free stores from either side).
//
// Per 128-row tile (staging halves A = rows 0-63, B = rows 64-127):
//   A, B -> XF (under the previous tile's last backward MMAs)
//   forward      ETA = XF W^T                      (3 x Dp/8 TS MMAs, M = 128, N = 64)
//   A -> XT (half 0), under the forward MMAs; then A takes the next tile's rows 0-63
//   epilogue     one thread per row and 16 chains: r = y - sigmoid(eta), the
//                per-row log-likelihood; R <- r (hi, lo)
//   backward     GT += XT R^T over rows 0-63 (24 TS MMAs, M = 128 features)
//   B -> XT (half 1); B takes the next tile's rows 64-127; backward over rows 64-127
// (where Dp <= 64 the second XT half is kept in XF's unused columns instead:
// both halves are written under the forward, both staging halves refill at
// once, and the backward is one run of 48 MMAs)
// After the last tile each thread reads the likelihood gradient of one
// feature for 16 chains from GT, the layout the leapfrog state is kept in
// (registers: the feature of the thread's TMEM lane, 16 chains).  The
// hierarchical prior, the softplus Jacobian, leapfrog and the FP64 Metropolis
// test follow hier.cu; per-chain sums over features and rows are warp
// reduce-scatters plus an FP64 sum over the four lane quadrants.
#include <algorithm>

#include "edg_common.cuh"
#include "tc_common.cuh"

namespace edg {
namespace htc {
using namespace ptx;

constexpr int kT = 512;      // 16 warps: four per TMEM lane quadrant
constexpr int kRows = 128;   // rows per tile (the forward M)
constexpr int kCh = 64;      // chains per CTA (the MMA N)
constexpr int kDmax = 128;   // features per instance (the backward M)
constexpr int kHW = kT / 128;    // warps per lane quadrant (the chain slices)
constexpr int kCPT = kCh / kHW;  // chains per thread: 16
constexpr int kRPH = 64 / kHW;   // rows of a 64-row half per thread (XT): 16
constexpr int kDPT = 128 / kHW;  // features per thread (XF): 32
constexpr uint32_t kStr = 144;                  // core-matrix stride along K, bytes
constexpr uint32_t kSBO = (kDmax / 4) * kStr;   // stride between 8-chain groups: 4,608 B
constexpr uint32_t kPlane = 8 * kSBO;           // one [64 chains, K <= 128] plane: 36,864 B
constexpr int kStPitch = kDmax + 1;             // largest staging row pitch (floats)
constexpr uint32_t kColXF = 0, kColXT = 256, kColEta = 384, kColGT = 448;
constexpr size_t kOffR = 2 * kPlane, kOffStage = 4 * kPlane;
constexpr size_t kStageHalf = (size_t)64 * kStPitch;  // floats per staging half
constexpr size_t kOffScal = kOffStage + 2 * kStageHalf * 4;
// scalars: 10 x 64 floats, 4 x 64 doubles, 2 x 4 x 64 floats, 4 x 64 doubles, 64 ints
constexpr size_t kSmemBytes = kOffScal + 640 * 4 + 256 * 8 + 512 * 4 + 256 * 8 + 64 * 4;

struct Args {
  const int32_t* Ns;
  const int32_t* Ds;
  const int32_t* order;
  const float* tiles;       // X re-laid by edg_hmc_hier_tc_prepare
  const int64_t* tile_off;  // [I] float offset of each instance's tiles
  int I, SP, C, tiles_per_inst;
  float mu_loc, mu_scale, tau_scale;
  int n_iter, n_steps, cache_valid;
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
  int persistent;
};

// Byte offset of element (chain c, k) in a W or R plane.
// Orders this thread's shared-memory writes before later tensor-core reads.
__device__ __forceinline__ void fence_shared_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ uint32_t bop_off(int c, int k) {
  return (uint32_t)(c >> 3) * kSBO + (uint32_t)(k >> 2) * kStr + (uint32_t)(c & 7) * 16u +
         (uint32_t)(k & 3) * 4u;
}
// High tf32 part (the 13 low mantissa bits cleared); v - hi_part(v) is exact.
__device__ __forceinline__ float hi_part(float v) {
  return __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
}
// Sum over the warp's lanes of v[0..V-1] (V = 16 or 32), scattered: lane i
// returns the total of index i % V (31 shuffles instead of V x 5).
template <int V>
__device__ __forceinline__ float reduce_scatter(float (&v)[V]) {
  const int lane = threadIdx.x & 31;
  if (V == 16) {
#pragma unroll
    for (int j = 0; j < V; ++j) v[j] += __shfl_xor_sync(0xffffffffu, v[j], 16);
  }
#pragma unroll
  for (int s = V / 2; s >= 1; s >>= 1) {
    const bool up = (lane & s) != 0;
#pragma unroll
    for (int j = 0; j < s; ++j) {
      const float send = up ? v[j] : v[j + s];
      const float keep = up ? v[j + s] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, s);
    }
  }
  return v[0];
}

// All n_iter iterations of one work item: chains [ctile*64, ctile*64 + 64)
// of instance order[item / tiles_per_inst].
__device__ void hier_tc_item(const Args& a, int item, unsigned char* smem, uint32_t tm,
                             uint32_t barF, uint32_t barB, uint32_t barX0, uint32_t (&ph)[4],
                             volatile int* err) {
  const int inst = a.order ? a.order[item / a.tiles_per_inst] : item / a.tiles_per_inst;
  const int ctile = item % a.tiles_per_inst;
  const int N = a.Ns[inst], D = a.Ds[inst];
  const int Dp = round_up(D, 8);
  const int pitch = Dp + 1;  // staging and tile row pitch (floats)
  const float* __restrict__ Xt = a.tiles + a.tile_off[inst];
  const int ntiles = (N + kRows - 1) / kRows;
  const int SP = a.SP;
  const int cbase = ctile * kCh;
  const int nc = min(kCh, a.C - cbase);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int q = warp & 3, h = warp >> 2;  // TMEM lane quadrant, chain slice
  const int d = 32 * q + lane;            // the feature this thread owns in the state
  const bool dval = d < D;
  const uint32_t lane_base = (uint32_t)(32 * q) << 16;
  unsigned char* Wb = smem;
  unsigned char* Rb = smem + kOffR;
  float* stg = reinterpret_cast<float*>(smem + kOffStage);
  float* H = reinterpret_cast<float*>(smem + kOffScal);
  float *mu0 = H, *u0 = H + 64, *gmu0 = H + 128, *gu0 = H + 192, *hmu = H + 256, *hu = H + 320;
  float *rmu = H + 384, *ru = H + 448, *gmu = H + 512, *gu = H + 576;
  double* Dd = reinterpret_cast<double*>(H + 640);
  double *lj0 = Dd, *kin0 = Dd + 64, *ljn = Dd + 128;
  float* ps1 = reinterpret_cast<float*>(Dd + 256);  // [4][64] per-quadrant partials
  float* ps2 = ps1 + 256;
  double* pd = reinterpret_cast<double*>(ps2 + 256);  // [4][64]
  int* acc = reinterpret_cast<int*>(pd + 256);
  const int64_t t0 = *(volatile int64_t*)&a.state->t;
  const float eps = a.step_size, half = 0.5f * a.step_size;
  auto gchain = [&](int c) -> size_t { return (size_t)inst * a.C + cbase + c; };

  // the accepted state: feature d of chains kCPT * h + i
  float Z[kCPT], G[kCPT], Rm[kCPT];
#pragma unroll
  for (int i = 0; i < kCPT; ++i) {
    const int c = kCPT * h + i;
    const bool ok = c < nc && dval;
    const size_t g = gchain(ok ? c : 0) * SP + (dval ? d : 0);
    Z[i] = ok ? a.z[g] : 0.0f;
    G[i] = (ok && a.cache_valid) ? a.grad[g] : 0.0f;
    Rm[i] = 0.0f;
  }
  if (tid < kCh) {
    const int c = tid;
    const bool ok = c < nc;
    const size_t g = gchain(ok ? c : 0) * SP;
    mu0[c] = ok ? a.z[g + SP - 2] : 0.0f;
    u0[c] = ok ? a.z[g + SP - 1] : 0.0f;
    gmu0[c] = (ok && a.cache_valid) ? a.grad[g + SP - 2] : 0.0f;
    gu0[c] = (ok && a.cache_valid) ? a.grad[g + SP - 1] : 0.0f;
    lj0[c] = (ok && a.cache_valid) ? a.lj[gchain(c)] : 0.0;
  }
  __syncthreads();

  // ---- X tile movement
  // rows 128 j + 64 hf .. + 63 (already zero beyond N and D) -> staging half hf
  auto prefetch = [&](int j, int hf) {
    if (tid == 0 && j < ntiles) {
      const uint32_t bytes = 64u * (uint32_t)pitch * 4u;
      const uint32_t bar = barX0 + 8u * hf;
      fence_shared_async();  // the staging half's generic reads come first
      mbar_expect_tx(bar, bytes);
      bulk_g2s(smem_u32(stg + hf * kStageHalf), Xt + ((size_t)kRows * j + 64 * hf) * pitch, bytes,
               bar);
    }
  };
  auto wait_stage = [&](int hf) {
    mbar_wait(barX0 + 8u * hf, ph[2 + hf], err);
    ph[2 + hf] ^= 1u;
  };
  // XT columns (hi at chi, lo at clo) + kRPH h + k of lane d <- staging half hf
  auto store_xt = [&](int hf, uint32_t chi, uint32_t clo) {
    const float* sh = stg + hf * kStageHalf;
#pragma unroll
    for (int s = 0; s < kRPH / 16; ++s) {
      float hv[16], lv[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const float v = sh[(kRPH * h + 16 * s + k) * pitch + d];
        hv[k] = hi_part(v);
        lv[k] = v - hv[k];
      }
      tmem_st16(tm + lane_base + chi + kRPH * h + 16 * s, hv);
      tmem_st16(tm + lane_base + clo + kRPH * h + 16 * s, lv);
    }
  };
  auto store_xf = [&]() {  // XF lane 32q + lane (tile row) <- staging
    const float* sr = stg + (q >> 1) * kStageHalf + (32 * (q & 1) + lane) * pitch;
#pragma unroll
    for (int ch = 0; ch < kDPT / 16; ++ch) {
      const int d0 = kDPT * h + 16 * ch;
      if (d0 >= Dp) break;
      float hv[16], lv[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const float v = sr[d0 + k];
        hv[k] = hi_part(v);
        lv[k] = v - hv[k];
      }
      tmem_st16(tm + lane_base + kColXF + d0, hv);
      tmem_st16(tm + lane_base + kColXF + 128 + d0, lv);
    }
  };
  auto issue_bwd = [&](int hf, bool first, uint32_t chi, uint32_t clo, bool commit) {
    if (warp == 0) {
      tc_fence_after();
      const uint32_t issue = elect_one();
      const uint32_t id = idesc_tf32(128, 64);
      const uint32_t rb = smem_u32(Rb);
#pragma unroll 1
      for (int k = 0; k < 8; ++k) {
        const uint32_t ko = (uint32_t)(16 * hf + 2 * k) * kStr;  // rows 64 hf + 8k
        const uint64_t bh = sdesc(rb + ko, kStr, kSBO), bl = sdesc(rb + kPlane + ko, kStr, kSBO);
        const uint32_t ahi = tm + chi + 8 * k, alo = tm + clo + 8 * k;
        mma_ts_if(issue, tm + kColGT, ahi, bh, id, (first && k == 0) ? 0u : 1u);
        mma_ts_if(issue, tm + kColGT, ahi, bl, id, 1u);
        mma_ts_if(issue, tm + kColGT, alo, bh, id, 1u);
      }
      if (commit) mma_commit_if(issue, barB);
      __syncwarp();
    }
  };
  // Dp <= 64: XF uses only columns [0, 64) and [128, 192), so XT's second half
  // goes to [64, 128) and [192, 256); both halves are then built under the
  // forward and the whole backward is issued at once
  const bool xt1f = Dp <= 64;

  // gradient of the log joint at Z (registers) and (msrc, usrc): likelihood
  // by the tile loop into G, then the hierarchical prior; with need_ll the
  // FP64 log joint goes to ljn
  auto eval = [&](const float* msrc, const float* usrc, bool need_ll) {
    if (d < Dp) {
#pragma unroll
      for (int i = 0; i < kCPT; ++i) {
        const float hv = hi_part(Z[i]);
        const uint32_t off = bop_off(kCPT * h + i, d);
        *reinterpret_cast<float*>(Wb + off) = hv;
        *reinterpret_cast<float*>(Wb + kPlane + off) = Z[i] - hv;
      }
    }
    fence_shared_async();
    double llacc = 0.0;  // chain kCPT h + lane % kCPT over this quadrant's rows
    prefetch(0, 0);
    prefetch(0, 1);
    for (int j = 0; j < ntiles; ++j) {
      const int row0 = j * kRows;
      wait_stage(0);  // both staging halves of tile j have landed
      wait_stage(1);
      // XF is free (the previous forward completed): built while the previous
      // tile's second backward half still runs
      store_xf();
      tmem_st_wait();
      tc_fence_before();
      __syncthreads();
      const int row = row0 + 32 * q + lane;  // this thread's row in the epilogue
      const bool rv = row < N;
      // y rides in the tile's pad column (index Dp) of the staged row
      const float yv = stg[(q >> 1) * kStageHalf + (32 * (q & 1) + lane) * pitch + Dp];
      if (warp == 0) {
        tc_fence_after();
        const uint32_t issue = elect_one();
        const uint32_t id = idesc_tf32(128, 64);
        const uint32_t wb = smem_u32(Wb);
#pragma unroll 1
        for (int k = 0; k < Dp / 8; ++k) {
          const uint64_t bh = sdesc(wb + 2u * k * kStr, kStr, kSBO);
          const uint64_t bl = sdesc(wb + kPlane + 2u * k * kStr, kStr, kSBO);
          mma_ts_if(issue, tm + kColEta, tm + kColXF + 8 * k, bh, id, k > 0 ? 1u : 0u);
          mma_ts_if(issue, tm + kColEta, tm + kColXF + 8 * k, bl, id, 1u);
          mma_ts_if(issue, tm + kColEta, tm + kColXF + 128 + 8 * k, bh, id, 1u);
        }
        mma_commit_if(issue, barF);
        __syncwarp();
      }
      if (j > 0) {  // XT and R are free once the previous tile's backward completes
        mbar_wait(barB, ph[1], err);
        ph[1] ^= 1u;
        tc_fence_after();
      }
      store_xt(0, kColXT, kColXT + 64);  // under the forward MMAs
      if (xt1f) {
        store_xt(1, kColXF + 64, kColXF + 192);
        tmem_st_wait();
        __syncthreads();     // both staging halves consumed
        prefetch(j + 1, 0);  // the next tile's copies run under this tile's MMAs
        prefetch(j + 1, 1);
      }
      mbar_wait(barF, ph[0], err);
      ph[0] ^= 1u;
      tc_fence_after();
      {
        float v[kCPT];
        tmem_ld16(tm + lane_base + kColEta + kCPT * h, v);
        // r = y - sigmoid(eta) = y - (eta >= 0 ? 1 : e) / (1 + e), e = exp(-|eta|);
        // the log-likelihood y eta - softplus(eta) only where the log joint is needed
        auto put = [&](int i, float r) {  // R <- r (hi, lo) for chain kCPT h + i, this row
          const float rh = hi_part(r);
          const uint32_t off = bop_off(kCPT * h + i, 32 * q + lane);
          *reinterpret_cast<float*>(Rb + off) = rh;
          *reinterpret_cast<float*>(Rb + kPlane + off) = r - rh;
        };
        if (need_ll) {
          // with the log-likelihood y eta - softplus(eta): e = exp(-|eta|),
          // sigmoid = (eta >= 0 ? 1 : e) / (1 + e), softplus = max(eta, 0) + log(1 + e)
          float llv[kCPT];
#pragma unroll
          for (int i = 0; i < kCPT; ++i) {
            const float eta = v[i];
            const float e = ex2_approx(-kLog2e * fabsf(eta));
            const float a1 = 1.0f + e;
            const float s = rcp_approx(a1);
            put(i, yv - (eta >= 0.0f ? s : e * s));
            llv[i] = rv ? -(fmaxf(eta, 0.0f) - eta * yv + kLn2 * lg2_approx(a1)) : 0.0f;
          }
          llacc += (double)reduce_scatter<kCPT>(llv);
        } else {
          // r = y - 1 / (1 + exp(-eta)) (exp overflows to inf for eta << 0,
          // giving 0).  Rows beyond N are not masked: their XT columns are zero.
#pragma unroll
          for (int i = 0; i < kCPT; ++i)
            put(i, yv - rcp_approx(1.0f + ex2_approx(-kLog2e * v[i])));
        }
      }
      tmem_st_wait();
      fence_shared_async();
      tc_fence_before();
      __syncthreads();
      if (xt1f) {
        issue_bwd(0, j == 0, kColXT, kColXT + 64, false);
        issue_bwd(1, false, kColXF + 64, kColXF + 192, true);
      } else {
        prefetch(j + 1, 0);  // staging half A is free
        issue_bwd(0, j == 0, kColXT, kColXT + 64, true);
        mbar_wait(barB, ph[1], err);  // XT is free once the first half's MMAs complete
        ph[1] ^= 1u;
        tc_fence_after();
        store_xt(1, kColXT, kColXT + 64);
        tmem_st_wait();
        tc_fence_before();
        __syncthreads();
        prefetch(j + 1, 1);  // staging half B is free
        issue_bwd(1, false, kColXT, kColXT + 64, true);
      }
    }
    float gl[kCPT];
    if (ntiles > 0) {
      mbar_wait(barB, ph[1], err);
      ph[1] ^= 1u;
      tc_fence_after();
      tmem_ld16(tm + lane_base + kColGT + kCPT * h, gl);
    } else {
#pragma unroll
      for (int i = 0; i < kCPT; ++i) gl[i] = 0.0f;
    }
    // hierarchical prior: d/dw = -(w - mu) / tau^2, and the per-chain sums of
    // (w - mu) and (w - mu)^2 over the features
    float s1v[kCPT], s2v[kCPT];
#pragma unroll
    for (int i = 0; i < kCPT; ++i) {
      const int c = kCPT * h + i;
      const float tau = softplusf(usrc[c]);
      const float it2 = 1.0f / (tau * tau);
      const float dev = dval ? Z[i] - msrc[c] : 0.0f;
      G[i] = dval ? gl[i] - dev * it2 : 0.0f;
      s1v[i] = dev;
      s2v[i] = dev * dev;
    }
    const float s1p = reduce_scatter<kCPT>(s1v);
    const float s2p = reduce_scatter<kCPT>(s2v);
    if (lane < kCPT) {
      ps1[q * 64 + kCPT * h + lane] = s1p;
      ps2[q * 64 + kCPT * h + lane] = s2p;
      if (need_ll) pd[q * 64 + kCPT * h + lane] = llacc;
    }
    __syncthreads();
    if (tid < kCh) {
      const int c = tid;
      const float s1 = ps1[c] + ps1[64 + c] + ps1[128 + c] + ps1[192 + c];
      const float s2 = ps2[c] + ps2[64 + c] + ps2[128 + c] + ps2[192 + c];
      const float mu = msrc[c], u = usrc[c];
      const float tau = softplusf(u);
      const float it2 = 1.0f / (tau * tau);
      gmu[c] = s1 * it2 - (mu - a.mu_loc) / (a.mu_scale * a.mu_scale);
      const float dtau = -(float)D / tau + s2 * it2 / tau - tau / (a.tau_scale * a.tau_scale);
      const float sg = sigmoidf(u);
      gu[c] = dtau * sg + (1.0f - sg);
      if (need_ll) {
        const double ll = pd[c] + pd[64 + c] + pd[128 + c] + pd[192 + c];
        const double lw = -0.5 * (double)s2 * (double)it2 - (double)D * (double)logf(tau) -
                          (double)D * kHalfLog2Pi;
        const double zm = ((double)mu - a.mu_loc) / a.mu_scale;
        const double lmu = -0.5 * zm * zm - log((double)a.mu_scale) - kHalfLog2Pi;
        const double zt = (double)tau / a.tau_scale;
        const double ltau = 0.5 * log(2.0 / 3.14159265358979323846) - log((double)a.tau_scale) -
                            0.5 * zt * zt;
        const double ldj = -(double)softplusf(-u);
        ljn[c] = ll + lw + lmu + ltau + ldj;
      }
    }
    __syncthreads();
  };

  if (!a.cache_valid) {
    eval(mu0, u0, true);
#pragma unroll
    for (int i = 0; i < kCPT; ++i) {
      const int c = kCPT * h + i;
      if (c < nc && dval) a.grad[gchain(c) * SP + d] = G[i];
    }
    if (tid < kCh) {
      gmu0[tid] = gmu[tid];
      gu0[tid] = gu[tid];
      lj0[tid] = ljn[tid];
    }
    __syncthreads();
  }

  for (int it = 0; it < a.n_iter; ++it) {
    if (*err) break;
    const int64_t t = t0 + it;
    const uint32_t iter = (uint32_t)t;
    // momenta for (w, mu, u): Philox elements 0..D-1 are w, D is mu, D + 1 is u
    float kp[kCPT];
#pragma unroll
    for (int i = 0; i < kCPT; ++i) {
      const int c = kCPT * h + i;
      float r = 0.0f;
      if (c < nc && dval)
        r = a.r_ovr ? a.r_ovr[((size_t)it * a.I * a.C + gchain(c)) * SP + d]
                    : philox_normal(a.seed, 1u, iter, (uint32_t)gchain(c), (uint32_t)d);
      Rm[i] = r;
      kp[i] = r * r;
    }
    {
      const float k0 = reduce_scatter<kCPT>(kp);
      if (lane < kCPT) pd[q * 64 + kCPT * h + lane] = (double)k0;
    }
    if (tid < kCh) {
      const int c = tid;
      float r1 = 0.0f, r2 = 0.0f;
      if (c < nc) {
        if (a.r_ovr) {
          const size_t b = ((size_t)it * a.I * a.C + gchain(c)) * SP;
          r1 = a.r_ovr[b + SP - 2];
          r2 = a.r_ovr[b + SP - 1];
        } else {
          r1 = philox_normal(a.seed, 1u, iter, (uint32_t)gchain(c), (uint32_t)D);
          r2 = philox_normal(a.seed, 1u, iter, (uint32_t)gchain(c), (uint32_t)(D + 1));
        }
      }
      rmu[c] = r1;
      ru[c] = r2;
      hmu[c] = mu0[c];
      hu[c] = u0[c];
      gmu[c] = gmu0[c];
      gu[c] = gu0[c];
    }
    __syncthreads();
    if (tid < kCh) {
      const int c = tid;
      kin0[c] = pd[c] + pd[64 + c] + pd[128 + c] + pd[192 + c] + (double)rmu[c] * rmu[c] +
                (double)ru[c] * ru[c];
    }
    __syncthreads();
    for (int l = 0; l < a.n_steps; ++l) {
#pragma unroll
      for (int i = 0; i < kCPT; ++i) {
        Rm[i] += half * G[i];
        Z[i] += eps * Rm[i];
      }
      if (tid < kCh) {
        const int c = tid;
        rmu[c] += half * gmu[c];
        ru[c] += half * gu[c];
        hmu[c] += eps * rmu[c];
        hu[c] += eps * ru[c];
      }
      __syncthreads();
      eval(hmu, hu, l == a.n_steps - 1);
#pragma unroll
      for (int i = 0; i < kCPT; ++i) Rm[i] += half * G[i];
      if (tid < kCh) {
        rmu[tid] += half * gmu[tid];
        ru[tid] += half * gu[tid];
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < kCPT; ++i) kp[i] = Rm[i] * Rm[i];
    {
      const float k1 = reduce_scatter<kCPT>(kp);
      if (lane < kCPT) pd[q * 64 + kCPT * h + lane] = (double)k1;
    }
    __syncthreads();
    if (tid < kCh) {
      const int c = tid;
      int accept = 0;
      if (c < nc) {
        const double lj_new = a.n_steps > 0 ? ljn[c] : lj0[c];
        const double k = pd[c] + pd[64 + c] + pd[128 + c] + pd[192 + c] +
                         (double)rmu[c] * rmu[c] + (double)ru[c] * ru[c];
        const double ratio = 0.5 * kin0[c] - 0.5 * k + lj_new - lj0[c];
        const double u = a.u_ovr ? a.u_ovr[(size_t)it * a.I * a.C + gchain(c)]
                                 : u01d(philox_at(a.seed, 2u, iter, (uint32_t)gchain(c), 0u).x);
        accept = log(u) < ratio ? 1 : 0;
        if (accept) {
          lj0[c] = lj_new;
          mu0[c] = hmu[c];
          u0[c] = hu[c];
          gmu0[c] = gmu[c];
          gu0[c] = gu[c];
        }
        if (a.n_accept) a.n_accept[gchain(c)] += accept;
        if (a.ratio_out) a.ratio_out[(size_t)it * a.I * a.C + gchain(c)] = ratio;
      }
      acc[c] = accept;
    }
    __syncthreads();
    // keep the proposal (written back as the accepted state) or reload the
    // accepted state; then the kept sample and the running moments
#pragma unroll
    for (int i = 0; i < kCPT; ++i) {
      const int c = kCPT * h + i;
      if (c < nc && dval) {
        const size_t g = gchain(c) * SP + d;
        if (acc[c]) {
          a.z[g] = Z[i];
          a.grad[g] = G[i];
        } else {
          Z[i] = a.z[g];
          G[i] = a.grad[g];
        }
        if (a.samples && t < a.T_cap) a.samples[(size_t)t * a.I * a.C * SP + g] = Z[i];
        if (a.moments) {
          a.moments[g] += (double)Z[i];
          a.moments[(size_t)a.I * a.C * SP + g] += (double)Z[i] * (double)Z[i];
        }
      }
    }
    if (tid < nc) {
      const int c = tid;
      const size_t g = gchain(c) * SP;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const float v = e == 0 ? mu0[c] : u0[c];
        const size_t ge = g + SP - 2 + e;
        if (a.samples && t < a.T_cap) a.samples[(size_t)t * a.I * a.C * SP + ge] = v;
        if (a.moments) {
          a.moments[ge] += (double)v;
          a.moments[(size_t)a.I * a.C * SP + ge] += (double)v * (double)v;
        }
      }
    }
    __syncthreads();
  }
  // the accepted (mu, u), their gradient and the log joint
  if (tid < nc) {
    const int c = tid;
    const size_t g = gchain(c) * SP;
    a.z[g + SP - 2] = mu0[c];
    a.z[g + SP - 1] = u0[c];
    a.grad[g + SP - 2] = gmu0[c];
    a.grad[g + SP - 1] = gu0[c];
    a.lj[gchain(c)] = lj0[c];
  }
  __syncthreads();  // the next item reuses the shared memory
}

__global__ void __launch_bounds__(kT, 1) hmc_hier_tc_kernel(const Args a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[4];  // forward, backward, staging halves A and B
  __shared__ uint32_t s_tmem;
  __shared__ int s_item, s_err;
  __shared__ bool s_last;
  __shared__ int64_t s_t0;
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_t0 = *(volatile int64_t*)&a.state->t;
    s_err = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) mbar_init(smem_u32(&bars[b]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(&s_tmem))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = s_tmem;
  const uint32_t barF = smem_u32(&bars[0]), barB = smem_u32(&bars[1]);
  const uint32_t barX0 = smem_u32(&bars[2]);  // barX0 + 8 is half B's
  uint32_t ph[4] = {0u, 0u, 0u, 0u};
  volatile int* err = &s_err;
  if (a.persistent) {
    const int total = a.I * a.tiles_per_inst;
    for (;;) {
      __syncthreads();
      if (threadIdx.x == 0) s_item = (int)atomicAdd(&a.state->reserved, 1u);
      __syncthreads();
      const int item = s_item;
      if (item >= total || *err) break;
      hier_tc_item(a, item, smem, tm, barF, barB, barX0, ph, err);
    }
  } else {
    hier_tc_item(a, blockIdx.x, smem, tm, barF, barB, barX0, ph, err);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tm) : "memory");
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    if (*err) atomicExch(&a.state->error, (uint32_t)(-EDG_E_TIMEOUT));
    const unsigned prev = atomicAdd(&a.state->done, 1u);
    s_last = (prev == gridDim.x - 1);
    if (s_last) {
      a.state->t = s_t0 + a.n_iter;
      a.state->done = 0;
      a.state->reserved = 0;
      __threadfence();
    }
  }
}

// X_i -> 128-row tiles with row pitch Dp_i + 1 at tiles + tile_off[i]:
// columns [0, D_i) hold the row of X_i, column Dp_i holds y_i, the rest and
// the rows beyond N_i are zero; blocks (instance, slice).
__global__ void __launch_bounds__(256) prep_tiles_kernel(const float* __restrict__ X,
                                                         const float* __restrict__ y,
                                                         const int64_t* __restrict__ x_off,
                                                         const int64_t* __restrict__ y_off,
                                                         const int32_t* __restrict__ Ns,
                                                         const int32_t* __restrict__ Ds,
                                                         const int64_t* __restrict__ tile_off,
                                                         float* __restrict__ tiles) {
  const int inst = blockIdx.x;
  const int N = Ns[inst], D = Ds[inst];
  const int pitch = round_up(D, 8) + 1;
  const int64_t n = (int64_t)((N + kRows - 1) / kRows) * kRows * pitch;
  const float* Xi = X + x_off[inst];
  const float* yi = y + y_off[inst];
  float* T = tiles + tile_off[inst];
  const int Dp = pitch - 1;
  for (int64_t e = threadIdx.x + (int64_t)blockIdx.y * blockDim.x; e < n;
       e += (int64_t)blockDim.x * gridDim.y) {
    const int64_t r = e / pitch;
    const int c = (int)(e - r * pitch);
    T[e] = r < N ? (c < D ? Xi[r * D + c] : (c == Dp ? yi[r] : 0.0f)) : 0.0f;
  }
}

}  // namespace htc
}  // namespace edg

using namespace edg;

extern "C" int64_t edg_hmc_hier_tc_tile_offsets(const int32_t* N, const int32_t* D, int32_t I,
                                                int64_t* tile_off) {
  if (!N || !D || I <= 0) return -1;
  int64_t off = 0;
  for (int i = 0; i < I; ++i) {
    if (N[i] < 0 || D[i] <= 0 || D[i] > htc::kDmax) return -1;
    if (tile_off) tile_off[i] = off;
    off += (int64_t)((N[i] + htc::kRows - 1) / htc::kRows) * htc::kRows * (round_up(D[i], 8) + 1);
  }
  return off;
}

extern "C" int edg_hmc_hier_tc_prepare(const edg_hier_t* model, const int64_t* tile_off,
                                       float* tiles, void* stream) {
  EDG_REQUIRE(model && tile_off && tiles, EDG_E_NULL, "model, tile_off and tiles must not be NULL");
  EDG_REQUIRE(model->X && model->y && model->x_offset && model->y_offset && model->N && model->D,
              EDG_E_NULL, "model arrays must be device pointers");
  EDG_REQUIRE(model->I > 0, EDG_E_SHAPE, "I must be positive");
  EDG_REQUIRE(((uintptr_t)tiles & 15u) == 0, EDG_E_VALUE, "tiles must be 16-byte aligned");
  htc::prep_tiles_kernel<<<dim3((unsigned)model->I, 8), 256, 0, (cudaStream_t)stream>>>(
      model->X, model->y, model->x_offset, model->y_offset, model->N, model->D, tile_off, tiles);
  return check_launch("prep_tiles_kernel");
}

extern "C" int edg_hmc_hier_tc_run(const edg_hier_t* model, const edg_hmc_t* cfg, int32_t C,
                                   int32_t n_iter, const int32_t* order, const float* tiles,
                                   const int64_t* tile_off, float* z, float* grad,
                                   double* lj, int32_t cache_valid, int32_t* n_accept,
                                   edg_state_t* state, float* samples, int64_t T_cap,
                                   double* moments, const float* r_override,
                                   const double* u_override, double* ratio_out, void* stream) {
  EDG_REQUIRE(model && cfg, EDG_E_NULL, "model and cfg must not be NULL");
  EDG_REQUIRE(model->X && model->y && model->x_offset && model->y_offset && model->N &&
                  model->D,
              EDG_E_NULL, "model arrays must be device pointers");
  EDG_REQUIRE(z && grad && lj && state, EDG_E_NULL, "z, grad, lj and state must not be NULL");
  EDG_REQUIRE(tiles && tile_off, EDG_E_NULL,
              "tiles and tile_off (edg_hmc_hier_tc_prepare) must not be NULL");
  EDG_REQUIRE(((uintptr_t)tiles & 15u) == 0, EDG_E_VALUE, "tiles must be 16-byte aligned");
  EDG_REQUIRE(model->I > 0 && C > 0 && n_iter >= 0, EDG_E_SHAPE,
              "I and C must be positive and n_iter >= 0");
  EDG_REQUIRE(model->max_D > 0 && model->max_D <= htc::kDmax, EDG_E_UNSUPPORTED,
              "the tensor-core engine supports max_D in [1, %d] (got %d)", htc::kDmax,
              model->max_D);
  EDG_REQUIRE(model->mu_scale > 0 && model->tau_scale > 0, EDG_E_VALUE,
              "mu_scale and tau_scale must be positive");
  EDG_REQUIRE(cfg->n_steps >= 0, EDG_E_VALUE, "n_steps must be >= 0");
  EDG_REQUIRE(!samples || T_cap > 0, EDG_E_SHAPE, "T_cap must be positive when samples is given");
  EDG_REQUIRE(cfg->launch == 0 || cfg->launch == 1, EDG_E_VALUE, "launch must be 0 or 1 (got %d)",
              cfg->launch);
  if (n_iter == 0 && cache_valid) return EDG_OK;
  htc::Args a;
  a.Ns = model->N;
  a.Ds = model->D;
  a.order = order;
  a.tiles = tiles;
  a.tile_off = tile_off;
  a.I = model->I;
  a.SP = model->max_D + 2;
  a.C = C;
  a.tiles_per_inst = (C + htc::kCh - 1) / htc::kCh;
  a.mu_loc = model->mu_loc;
  a.mu_scale = model->mu_scale;
  a.tau_scale = model->tau_scale;
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
  a.persistent = cfg->launch == 0 ? 1 : 0;
  const int64_t nitems = (int64_t)a.I * a.tiles_per_inst;
  EDG_REQUIRE(nitems < (1ll << 31), EDG_E_SHAPE, "too many instances x chain tiles");
  const int rc = set_max_dyn_smem(htc::hmc_hier_tc_kernel, htc::kSmemBytes, "hmc_hier_tc_kernel");
  if (rc) return rc;
  int64_t nblocks = nitems;
  if (a.persistent) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    nblocks = std::min<int64_t>(nitems, std::max(sms, 1));
  }
  htc::hmc_hier_tc_kernel<<<(unsigned)nblocks, htc::kT, htc::kSmemBytes, (cudaStream_t)stream>>>(
      a);
  return check_launch("hmc_hier_tc_kernel");
}
