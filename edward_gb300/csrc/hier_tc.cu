// Ragged batch of hierarchical logistic regressions under HMC on the tensor
// cores.  Same model, state layout, draws and contract as hier.cu
// (edg_hmc_hier_run); every gradient evaluation is computed as tcgen05
// 3xTF32 GEMMs (hi*hi + hi*lo + lo*hi, FP32 accumulation in TMEM).
//
// One CTA per (instance, 64 chains), 256 threads, all 512 TMEM columns:
//   XF  [lanes = 128 rows of a tile, columns = features]   hi at 0, lo at 128
//   XT  [lanes = features, columns = 64 rows of a half]     hi at 256, lo at 320
//   ETA [lanes = rows, columns = 64 chains]                 at 384 (forward accumulator)
//   GT  [lanes = features, columns = 64 chains]             at 448 (backward accumulator)
// tf32 operands must be K-major (a transposed shared-memory operand reads as
// zeros), so X enters the tensor core in both orientations, and both come
// from TMEM (the A operand of the TS form).  X is read from HBM as one fp32
// plane, once per evaluation for all 64 chains: coalesced warp loads (32
// consecutive features of one row) give XT directly (one lane per feature)
// and, through a padded shared staging buffer, XF (one lane per row); the
// hi/lo split is made in registers.  Shared memory holds the B operands only:
// the positions W [64 chains, K = features] and the residuals R [64 chains,
// K = 128 rows], hi and lo planes in the no-swizzle K-major core-matrix layout
// with 144-byte strides (bank-conflict-free stores from either side).
//
// Per 128-row tile:
//   rows 0-63    -> XT (half 0) and staging -> XF rows 0-63
//   rows 64-127  -> staging -> XF rows 64-127
//   forward      ETA = XF W^T                      (3 x Dp/8 TS MMAs, M = 128, N = 64)
//   epilogue     one thread per row and 32 chains: r = y - sigmoid(eta), the
//                per-row log-likelihood; R <- r (hi, lo)
//   backward     GT += XT R^T over rows 0-63 (24 TS MMAs, M = 128 features)
//   rows 64-127  -> XT (half 1); backward over rows 64-127
// After the last tile each thread reads the likelihood gradient of one
// feature for 32 chains from GT, the layout the leapfrog state is kept in
// (registers: the feature of the thread's TMEM lane, 32 chains).  The
// hierarchical prior, the softplus Jacobian, leapfrog and the FP64 Metropolis
// test follow hier.cu; per-chain sums over features and rows are warp
// reduce-scatters plus an FP64 sum over the four lane quadrants.
#include <algorithm>

#include "edg_common.cuh"
#include "tc_common.cuh"

namespace edg {
namespace htc {
using namespace ptx;

constexpr int kT = 256;
constexpr int kRows = 128;   // rows per tile (the forward M)
constexpr int kCh = 64;      // chains per CTA (the MMA N)
constexpr int kDmax = 128;   // features per instance (the backward M)
constexpr uint32_t kStr = 144;                  // core-matrix stride along K, bytes
constexpr uint32_t kSBO = (kDmax / 4) * kStr;   // stride between 8-chain groups: 4,608 B
constexpr uint32_t kPlane = 8 * kSBO;           // one [64 chains, K <= 128] plane: 36,864 B
constexpr int kStPitch = 129;                   // staging row pitch in floats (odd: no conflicts)
constexpr uint32_t kColXF = 0, kColXT = 256, kColEta = 384, kColGT = 448;
constexpr size_t kOffR = 2 * kPlane, kOffStage = 4 * kPlane;
constexpr size_t kOffScal = kOffStage + (size_t)64 * kStPitch * 4;
// scalars: 10 x 64 floats, 4 x 64 doubles, 2 x 4 x 64 floats, 4 x 64 doubles, 64 ints
constexpr size_t kSmemBytes = kOffScal + 640 * 4 + 256 * 8 + 512 * 4 + 256 * 8 + 64 * 4;

struct Args {
  const float* X;
  const float* y;
  const int64_t* x_off;
  const int64_t* y_off;
  const int32_t* Ns;
  const int32_t* Ds;
  const int32_t* order;
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
__device__ __forceinline__ uint32_t bop_off(int c, int k) {
  return (uint32_t)(c >> 3) * kSBO + (uint32_t)(k >> 2) * kStr + (uint32_t)(c & 7) * 16u +
         (uint32_t)(k & 3) * 4u;
}
// High tf32 part (the 13 low mantissa bits cleared); v - hi_part(v) is exact.
__device__ __forceinline__ float hi_part(float v) {
  return __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
}
// Sum over the warp's lanes of v[0..31], scattered: lane i returns the total
// of index i (31 shuffles instead of 32 x 5).
__device__ __forceinline__ float reduce_scatter32(float (&v)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
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
                             uint32_t barF, uint32_t barB, uint32_t (&ph)[2], volatile int* err) {
  const int inst = a.order ? a.order[item / a.tiles_per_inst] : item / a.tiles_per_inst;
  const int ctile = item % a.tiles_per_inst;
  const float* __restrict__ X = a.X + a.x_off[inst];
  const float* __restrict__ Y = a.y + a.y_off[inst];
  const int N = a.Ns[inst], D = a.Ds[inst];
  const int Dp = round_up(D, 8);
  const int ntiles = (N + kRows - 1) / kRows;
  const int SP = a.SP;
  const int cbase = ctile * kCh;
  const int nc = min(kCh, a.C - cbase);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int q = warp & 3, h = warp >> 2;  // TMEM lane quadrant, chain half
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

  // the accepted state: feature d of chains 32h + i
  float Z[32], G[32], Rm[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int c = 32 * h + i;
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
  auto load_rows = [&](int rbase, float (&x)[32]) {  // rows rbase + 32h + k, feature d
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      const int row = rbase + 32 * h + k;
      x[k] = (dval && row < N) ? __ldg(X + (size_t)row * D + d) : 0.0f;
    }
  };
  auto store_xt = [&](const float (&x)[32]) {  // XT columns 32h + k of lane d
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      float hv[16], lv[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        hv[k] = hi_part(x[16 * s + k]);
        lv[k] = x[16 * s + k] - hv[k];
      }
      tmem_st16(tm + lane_base + kColXT + 32 * h + 16 * s, hv);
      tmem_st16(tm + lane_base + kColXT + 64 + 32 * h + 16 * s, lv);
    }
  };
  auto stage = [&](const float (&x)[32]) {
#pragma unroll
    for (int k = 0; k < 32; ++k) stg[(32 * h + k) * kStPitch + d] = x[k];
  };
  auto store_xf = [&](int srow) {  // XF lane (this warp's quadrant) <- staging row srow
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      const int d0 = 64 * h + 16 * ch;
      if (d0 >= Dp) break;
      float hv[16], lv[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const float v = stg[srow * kStPitch + d0 + k];
        hv[k] = hi_part(v);
        lv[k] = v - hv[k];
      }
      tmem_st16(tm + lane_base + kColXF + d0, hv);
      tmem_st16(tm + lane_base + kColXF + 128 + d0, lv);
    }
  };
  auto issue_bwd = [&](int hf, bool first) {
    if (warp == 0) {
      tc_fence_after();
      const uint32_t issue = elect_one();
      const uint32_t id = idesc_tf32(128, 64);
      const uint32_t rb = smem_u32(Rb);
#pragma unroll 1
      for (int k = 0; k < 8; ++k) {
        const uint32_t ko = (uint32_t)(16 * hf + 2 * k) * kStr;  // rows 64 hf + 8k
        const uint64_t bh = sdesc(rb + ko, kStr, kSBO), bl = sdesc(rb + kPlane + ko, kStr, kSBO);
        const uint32_t ahi = tm + kColXT + 8 * k, alo = tm + kColXT + 64 + 8 * k;
        mma_ts_if(issue, tm + kColGT, ahi, bh, id, (first && k == 0) ? 0u : 1u);
        mma_ts_if(issue, tm + kColGT, ahi, bl, id, 1u);
        mma_ts_if(issue, tm + kColGT, alo, bh, id, 1u);
      }
      mma_commit_if(issue, barB);
      __syncwarp();
    }
  };

  // gradient of the log joint at Z (registers) and (msrc, usrc): likelihood
  // by the tile loop into G, then the hierarchical prior; with need_ll the
  // FP64 log joint goes to ljn
  auto eval = [&](const float* msrc, const float* usrc, bool need_ll) {
    if (d < Dp) {
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const float hv = hi_part(Z[i]);
        const uint32_t off = bop_off(32 * h + i, d);
        *reinterpret_cast<float*>(Wb + off) = hv;
        *reinterpret_cast<float*>(Wb + kPlane + off) = Z[i] - hv;
      }
    }
    fence_proxy_async();
    double llacc = 0.0;  // chain 32h + lane over this quadrant's rows
    float x[32];
    for (int j = 0; j < ntiles; ++j) {
      const int row0 = j * kRows;
      load_rows(row0, x);
      if (j > 0) {  // XT and R are free once the previous tile's backward completes
        mbar_wait(barB, ph[1], err);
        ph[1] ^= 1u;
        tc_fence_after();
      }
      store_xt(x);
      stage(x);
      __syncthreads();
      if (q < 2) store_xf(32 * q + lane);
      __syncthreads();
      load_rows(row0 + 64, x);
      stage(x);
      __syncthreads();
      if (q >= 2) store_xf(32 * (q - 2) + lane);
      tmem_st_wait();
      tc_fence_before();
      __syncthreads();
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
      mbar_wait(barF, ph[0], err);
      ph[0] ^= 1u;
      tc_fence_after();
      {
        float v[32];
        tmem_ld32(tm + lane_base + kColEta + 32 * h, v);
        const int row = row0 + 32 * q + lane;
        const bool rv = row < N;
        const float yv = rv ? __ldg(Y + row) : 0.0f;
        float llv[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float eta = v[i];
          const float e = ex2_approx(-kLog2e * fabsf(eta));
          const float a1 = 1.0f + e;
          const float s = rcp_approx(a1);
          const float r = rv ? yv - (eta >= 0.0f ? s : e * s) : 0.0f;
          llv[i] = rv ? -(fmaxf(eta, 0.0f) - eta * yv + kLn2 * lg2_approx(a1)) : 0.0f;
          const float rh = hi_part(r);
          const uint32_t off = bop_off(32 * h + i, 32 * q + lane);
          *reinterpret_cast<float*>(Rb + off) = rh;
          *reinterpret_cast<float*>(Rb + kPlane + off) = r - rh;
        }
        if (need_ll) llacc += (double)reduce_scatter32(llv);
      }
      fence_proxy_async();
      tc_fence_before();
      __syncthreads();
      issue_bwd(0, j == 0);
      load_rows(row0 + 64, x);
      mbar_wait(barB, ph[1], err);  // XT is free once the first half's MMAs complete
      ph[1] ^= 1u;
      tc_fence_after();
      store_xt(x);
      tmem_st_wait();
      tc_fence_before();
      __syncthreads();
      issue_bwd(1, false);
    }
    float gl[32];
    if (ntiles > 0) {
      mbar_wait(barB, ph[1], err);
      ph[1] ^= 1u;
      tc_fence_after();
      tmem_ld32(tm + lane_base + kColGT + 32 * h, gl);
    } else {
#pragma unroll
      for (int i = 0; i < 32; ++i) gl[i] = 0.0f;
    }
    // hierarchical prior: d/dw = -(w - mu) / tau^2, and the per-chain sums of
    // (w - mu) and (w - mu)^2 over the features
    float s1v[32], s2v[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const int c = 32 * h + i;
      const float tau = softplusf(usrc[c]);
      const float it2 = 1.0f / (tau * tau);
      const float dev = dval ? Z[i] - msrc[c] : 0.0f;
      G[i] = dval ? gl[i] - dev * it2 : 0.0f;
      s1v[i] = dev;
      s2v[i] = dev * dev;
    }
    const float s1p = reduce_scatter32(s1v);
    const float s2p = reduce_scatter32(s2v);
    ps1[q * 64 + 32 * h + lane] = s1p;
    ps2[q * 64 + 32 * h + lane] = s2p;
    if (need_ll) pd[q * 64 + 32 * h + lane] = llacc;
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
    for (int i = 0; i < 32; ++i) {
      const int c = 32 * h + i;
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
    float kp[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const int c = 32 * h + i;
      float r = 0.0f;
      if (c < nc && dval)
        r = a.r_ovr ? a.r_ovr[((size_t)it * a.I * a.C + gchain(c)) * SP + d]
                    : philox_normal(a.seed, 1u, iter, (uint32_t)gchain(c), (uint32_t)d);
      Rm[i] = r;
      kp[i] = r * r;
    }
    pd[q * 64 + 32 * h + lane] = (double)reduce_scatter32(kp);
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
      for (int i = 0; i < 32; ++i) {
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
      for (int i = 0; i < 32; ++i) Rm[i] += half * G[i];
      if (tid < kCh) {
        rmu[tid] += half * gmu[tid];
        ru[tid] += half * gu[tid];
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) kp[i] = Rm[i] * Rm[i];
    pd[q * 64 + 32 * h + lane] = (double)reduce_scatter32(kp);
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
    for (int i = 0; i < 32; ++i) {
      const int c = 32 * h + i;
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
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t s_tmem;
  __shared__ int s_item, s_err;
  __shared__ bool s_last;
  __shared__ int64_t s_t0;
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_t0 = *(volatile int64_t*)&a.state->t;
    s_err = 0;
    mbar_init(smem_u32(&bars[0]), 1);
    mbar_init(smem_u32(&bars[1]), 1);
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
  uint32_t ph[2] = {0u, 0u};
  volatile int* err = &s_err;
  if (a.persistent) {
    const int total = a.I * a.tiles_per_inst;
    for (;;) {
      __syncthreads();
      if (threadIdx.x == 0) s_item = (int)atomicAdd(&a.state->reserved, 1u);
      __syncthreads();
      const int item = s_item;
      if (item >= total || *err) break;
      hier_tc_item(a, item, smem, tm, barF, barB, ph, err);
    }
  } else {
    hier_tc_item(a, blockIdx.x, smem, tm, barF, barB, ph, err);
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

}  // namespace htc
}  // namespace edg

using namespace edg;

extern "C" int edg_hmc_hier_tc_run(const edg_hier_t* model, const edg_hmc_t* cfg, int32_t C,
                                   int32_t n_iter, const int32_t* order, float* z, float* grad,
                                   double* lj, int32_t cache_valid, int32_t* n_accept,
                                   edg_state_t* state, float* samples, int64_t T_cap,
                                   double* moments, const float* r_override,
                                   const double* u_override, double* ratio_out, void* stream) {
  EDG_REQUIRE(model && cfg, EDG_E_NULL, "model and cfg must not be NULL");
  EDG_REQUIRE(model->X && model->y && model->x_offset && model->y_offset && model->N &&
                  model->D,
              EDG_E_NULL, "model arrays must be device pointers");
  EDG_REQUIRE(z && grad && lj && state, EDG_E_NULL, "z, grad, lj and state must not be NULL");
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
  a.X = model->X;
  a.y = model->y;
  a.x_off = model->x_offset;
  a.y_off = model->y_offset;
  a.Ns = model->N;
  a.Ds = model->D;
  a.order = order;
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
