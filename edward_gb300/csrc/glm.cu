// GLM hot path on SIMT FP32: batched log joint + adjoint, the fused KLqp
// step and the persistent multi-chain HMC kernel.
//
// Shared building block: glm_grad_eval<CT>() runs over a row range of X for
// CT parameter vectors held in shared memory (Monte Carlo samples or HMC
// chains).  Per row tile it does
//   phase A  eta[r][c]  = X[r,:] . z_c            (2 rows x 4 vectors per thread)
//   epilogue resid[r][c] = d log p(y_r | eta) / d eta, log-lik terms (Kahan)
//   phase B  G[c][d]   += sum_r resid[r][c] X[r][d]  (4x4 register blocks)
// with X tiles streamed global -> shared by cp.async, double buffered.
// One pass over X yields the log-likelihood and its gradient for every
// vector, so X is read once per evaluation instead of 2S times
// (klqp.py:725-747 builds S separate GEMV graphs).
#include <cstdio>
#include <algorithm>
#include <mutex>

#include "edg_common.cuh"
#include "glm_tile.cuh"
#include "optim.cuh"

namespace edg {

// ============================================================ batched grad
template <int CT>
__global__ void __launch_bounds__(kThreads) glm_partial_kernel(GLMDev m, const float* __restrict__ Z,
                                                               int B, int chunk, float dscale,
                                                               float* __restrict__ ws_g,
                                                               double* __restrict__ ws_ll, int Bpad,
                                                               int need_grad) {
  extern __shared__ __align__(16) unsigned char smem[];
  GradSmem S;
  carve_grad<CT>(smem, m.PP, S);
  const int chunk_id = blockIdx.x, tile = blockIdx.y;
  const int b0 = tile * CT;
  init_x_pad<CT>(m, S);
  for (int idx = threadIdx.x; idx < CT * m.PP; idx += kThreads) {
    const int c = idx / m.PP, d = idx - c * m.PP;
    const int b = b0 + c;
    S.Zt[d * CT + c] = (b < B && d < m.P) ? Z[(size_t)b * m.P + d] : 0.0f;
  }
  __syncthreads();
  const int rb = chunk_id * chunk, re = min(m.N, rb + chunk);
  glm_grad_eval<CT>(m, rb, re, S, true, need_grad != 0, dscale);
  for (int idx = threadIdx.x; idx < CT * m.PP; idx += kThreads) {
    const int c = idx / m.PP;
    if (b0 + c < B && need_grad)
      ws_g[((size_t)chunk_id * Bpad + b0) * m.PP + idx] = S.G[idx];
  }
  if (threadIdx.x < CT && b0 + threadIdx.x < B)
    ws_ll[(size_t)chunk_id * Bpad + b0 + threadIdx.x] = S.ll[threadIdx.x];
}

__global__ void glm_reduce_kernel(GLMDev m, const float* __restrict__ Z, int B, int nchunks,
                                  const float* __restrict__ ws_g, const double* __restrict__ ws_ll,
                                  int Bpad, int include_prior, double* lp_out, float* grad_out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int P = m.P, PP = m.PP;
  if (grad_out && i < (int64_t)B * P) {
    const int b = (int)(i / P), d = (int)(i % P);
    float s = 0.0f;
    for (int k = 0; k < nchunks; ++k) s += ws_g[((size_t)k * Bpad + b) * PP + d];
    if (include_prior) {
      const float sc = m.prior_scale[d];
      s += -(Z[i] - m.prior_loc[d]) / (sc * sc);
    }
    grad_out[i] = s;
  }
  if (lp_out && i < B) {
    double s = 0.0;
    for (int k = 0; k < nchunks; ++k) s += ws_ll[(size_t)k * Bpad + i];
    if (include_prior) {
      for (int d = 0; d < P; ++d) {
        const float sc = m.prior_scale[d];
        const float zz = (Z[(size_t)i * P + d] - m.prior_loc[d]) / sc;
        s += (double)(-0.5f * zz * zz - logf(sc)) - kHalfLog2Pi;
      }
    }
    lp_out[i] = s;
  }
}

// ============================================================ KLqp step
// The fused KLqp step runs tiles of one row per thread (RT = 1024 / CT rows)
// for up to 16 samples: a 10,000-row problem then spreads over 79 blocks
// instead of 40, which halves each block's share of the latency-bound tile
// loop.  32-vector tiles keep two rows per thread (the per-sample gradients of
// the tail live in the tile buffers, 2 RT rows of them).
template <int CT>
__host__ __device__ constexpr int klqp_rpt() { return CT == 32 ? 2 : 1; }

struct KlqpArgs {
  int method, S, Spad, nblocks, chunk;
  double inv_S;  // 1 / S
  float dscale;
  const float* kl_scaling;
  const float* latent_scale;
  const int32_t* point;  // model parameters: z = mu, no prior, no q, pathwise gradient
  uint64_t seed;
  edg_opt_t opt;
  float* mu;
  float* rho;
  float* slots;
  edg_state_t* state;
  const float* eps_ovr;
  float* grad_out;
  int apply;
  float* ws_g;     // [nblocks][Spad][PP]
  double* ws_ll;   // [nblocks][Spad]
};

__device__ __forceinline__ float eps_value(const KlqpArgs& a, uint32_t iter, int s, int d, int P) {
  return a.eps_ovr ? a.eps_ovr[(size_t)s * P + d] : philox_normal(a.seed, 0u, iter, (uint32_t)s, (uint32_t)d);
}

template <int CT>
__global__ void __launch_bounds__(kThreads, 1) klqp_glm_kernel(GLMDev m, KlqpArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  GradSmem S;
  unsigned char* rest = carve_grad<CT, klqp_rpt<CT>()>(smem, m.PP, S);
  float* sig = reinterpret_cast<float*>(rest);  // [PP]
  float* epsS = sig + m.PP;                      // [Spad][PP] this step's draws
  // The step's per-coordinate inputs, loaded once by every block at the start
  // (one round trip, overlapping the X tile's copy) so that the last block's
  // serial tail reads only shared memory: mu, rho, prior loc and scale, KL and
  // latent scalings, the model-parameter flags and the four optimizer slots.
  float* s_mu = epsS + (size_t)a.Spad * m.PP;  // [PP]
  float* s_rho = s_mu + m.PP;
  float* s_pl = s_rho + m.PP;
  float* s_ps = s_pl + m.PP;
  float* s_ks = s_ps + m.PP;
  float* s_ls = s_ks + m.PP;
  float* s_sl = s_ls + m.PP;                                  // [4][PP]
  int* s_pt = reinterpret_cast<int*>(s_sl + 4 * m.PP);        // [PP]
  __shared__ bool s_last;
  const int P = m.P, PP = m.PP;
  const int rb = blockIdx.x * a.chunk, re = min(m.N, rb + a.chunk);
  // the first X tile's copy overlaps the loads and draws below
  if (re > rb) issue_tile<CT, klqp_rpt<CT>()>(m, S.Xs, S.ys, rb, re);
  cp_async_commit();
  // Launched as a programmatic dependent of the previous step: everything
  // above (the X tile's copy) may run under the previous step's tail; the
  // step's inputs are read only once that grid has completed.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int64_t t = *(volatile int64_t*)&a.state->t;
  const int64_t gstep = a.state->global_step;
  const float b1p = a.state->beta1_power, b2p = a.state->beta2_power;
  const uint32_t iter = (uint32_t)t;
  for (int d = threadIdx.x; d < PP; d += kThreads) {
    const bool ok = d < P;
    const int pt = (ok && a.point) ? a.point[d] : 0;
    const float rho = ok ? a.rho[d] : 0.0f;
    s_mu[d] = ok ? a.mu[d] : 0.0f;
    s_rho[d] = rho;
    s_pl[d] = ok ? m.prior_loc[d] : 0.0f;
    s_ps[d] = ok ? m.prior_scale[d] : 1.0f;
    s_ks[d] = (ok && a.kl_scaling) ? a.kl_scaling[d] : 1.0f;
    s_ls[d] = (ok && a.latent_scale) ? a.latent_scale[d] : 1.0f;
#pragma unroll
    for (int j = 0; j < 4; ++j) s_sl[j * PP + d] = (ok && a.slots) ? a.slots[j * P + d] : 0.0f;
    s_pt[d] = pt;
    sig[d] = (ok && !pt) ? softplusf(rho) : 0.0f;
  }
  init_x_pad<CT, klqp_rpt<CT>()>(m, S);
  __syncthreads();
  // the score method needs d log p / d z only for model parameters
  const bool need_grad = a.method != EDG_KLQP_SCORE || a.point != nullptr;
  for (int s0 = 0; s0 < a.S; s0 += CT) {
    for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
      const int c = idx / PP, d = idx - c * PP;
      const int s = s0 + c;
      float zv = 0.0f;
      if (s < a.S && d < P) {
        const float e = eps_value(a, iter, s, d, P);
        epsS[s * PP + d] = e;  // kept for the last block's gradient formula
        zv = s_mu[d] + sig[d] * e;
      }
      S.Zt[d * CT + c] = zv;
    }
    __syncthreads();
    glm_grad_eval<CT, klqp_rpt<CT>()>(m, rb, re, S, true, need_grad, a.dscale, s0 == 0);
    for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
      const int c = idx / PP;
      if (s0 + c < a.S && need_grad)
        a.ws_g[((size_t)blockIdx.x * a.Spad + s0) * PP + idx] = S.G[idx];
    }
    if (threadIdx.x < CT && s0 + threadIdx.x < a.S)
      a.ws_ll[(size_t)blockIdx.x * a.Spad + s0 + threadIdx.x] = S.ll[threadIdx.x];
    __syncthreads();
  }
  // ---- last block finishes the step; the next step's grid may start its
  // prologue once every block is here
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(&a.state->done, 1u);
    s_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // The tail: every partial load is issued first, the prior terms (KL or
  // log p(z) - log q(z), which need no partial) are computed while they are
  // in flight, then the partials are reduced in a fixed order (deterministic).
  double* llS = S.llred;                 // [S]  (reuse; 2 S + 8 fit, checked at launch)
  double* lsig = llS + a.S;              // [S] log p(z_s) - log q(z_s)
  double* red = lsig + a.S;              // [8] per-warp partial sums
  float* gS = S.Xs;                      // [S][PP] gradient per sample
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int kBatch = 96;             // partials per thread in flight at once
  // fixed-order sum of a batch: [64, 96) folded onto [0, 32), then a tree over 64
  auto batch_sum = [](float (&v)[kBatch]) {
    static_assert(kBatch == 96, "fold assumes 96 = 64 + 32");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] += v[k + 64];
#pragma unroll
    for (int w = 32; w > 0; w >>= 1) {
#pragma unroll
      for (int k = 0; k < w; ++k) v[k] += v[k + w];
    }
    return v[0];
  };
  // log-likelihood partials: one warp per sample, lanes over the blocks
  double llv[3] = {0.0, 0.0, 0.0};
  const bool ll_fast = a.nblocks <= 96 && a.S <= kThreads / 32;
  if (ll_fast && warp < a.S) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int b = lane + 32 * k;
      if (b < a.nblocks) llv[k] = __ldcg(a.ws_ll + (size_t)b * a.Spad + warp);
    }
  }
  // gradient partials: the S x P entries in use, one per thread for small
  // problems (the padding columns are never read)
  const int q0 = threadIdx.x;
  float gv[kBatch];
  const bool g_fast = need_grad && a.nblocks <= kBatch && a.S * P <= kThreads;
  if (g_fast && q0 < a.S * P) {
    const int sq = q0 / P, dq = q0 - sq * P;
    const float* src = a.ws_g + sq * PP + dq;
    const size_t st = (size_t)a.Spad * PP;
#pragma unroll
    for (int k = 0; k < kBatch; ++k) gv[k] = k < a.nblocks ? __ldcg(src + (size_t)k * st) : 0.0f;
  }
  // score / reparam: per-sample log p(z_s) - log q(z_s), one warp per sample
  if (a.method != EDG_KLQP_REPARAM_KL) {
    for (int s = warp; s < a.S; s += kThreads / 32) {
      float acc = 0.0f;  // FP32: a few terms per lane, 32 lanes
      for (int d = lane; d < P; d += 32) {
        if (s_pt[d]) continue;
        const float lsc = s_ls[d];
        const float e = epsS[s * PP + d];
        const float zv = s_mu[d] + sig[d] * e;
        const float ps = s_ps[d];
        const float zp = (zv - s_pl[d]) / ps;
        const float zq = (zv - s_mu[d]) / sig[d];
        const float lp = -0.5f * zp * zp - logf(ps);
        const float lq = -0.5f * zq * zq - logf(sig[d]);
        acc += lsc * (lp - lq);  // the 0.5 log 2pi terms cancel
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) lsig[s] = (double)acc;
    }
  }
  // analytic KL: one coordinate per thread, FP32 within a warp (FP64 runs at a
  // small fraction of the FP32 rate here), FP64 across the warps that hold
  // coordinates
  double klsum = 0.0;
  const int kl_warps = min(kThreads / 32, (P + 31) / 32);
  if (a.method == EDG_KLQP_REPARAM_KL && warp < kl_warps) {
    float kl = 0.0f;
    for (int d = threadIdx.x; d < P; d += kThreads) {
      if (s_pt[d]) continue;
      const float ks = s_ks[d];
      const float sp = s_ps[d], sq = sig[d];
      const float dm = (s_mu[d] - s_pl[d]) / sp;
      const float ratio = (sq / sp) * (sq / sp);
      kl += ks * (0.5f * dm * dm + 0.5f * ((ratio - 1.0f) - logf(ratio)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) kl += __shfl_xor_sync(0xffffffffu, kl, o);
    if (lane == 0) red[warp] = (double)kl;
  }
  // reduce the partials
  if (ll_fast) {
    if (warp < a.S) {
      double v = (llv[0] + llv[1]) + llv[2];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) llS[warp] = v;
    }
  } else {
    for (int s = warp; s < a.S; s += kThreads / 32) {
      double v = 0.0;
      for (int b = lane; b < a.nblocks; b += 32) v += __ldcg(a.ws_ll + (size_t)b * a.Spad + s);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) llS[s] = v;
    }
  }
  if (g_fast) {
    if (q0 < a.S * P) {
      const int sq = q0 / P, dq = q0 - sq * P;
      gS[sq * PP + dq] = batch_sum(gv);
    }
  } else if (need_grad) {
    for (int q = threadIdx.x; q < a.S * P; q += kThreads) {
      const int sq = q / P, dq = q - sq * P;
      const float* src = a.ws_g + sq * PP + dq;
      const size_t st = (size_t)a.Spad * PP;
      float acc = 0.0f;
      for (int b0 = 0; b0 < a.nblocks; b0 += kBatch) {
        float v[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; ++k)
          v[k] = b0 + k < a.nblocks ? __ldcg(src + (size_t)(b0 + k) * st) : 0.0f;
        acc += batch_sum(v);
      }
      gS[sq * PP + dq] = acc;
    }
  }
  __syncthreads();
  // ---- loss, on the block's last thread (the gradient loop below starts at
  // thread 0, so both run at once for P < 255)
  constexpr int kLossThread = kThreads - 1;
  if (threadIdx.x == kLossThread) {
    double mean_ll = 0.0;
    for (int s = 0; s < a.S; ++s) mean_ll += llS[s];
    mean_ll *= a.inv_S;
    double loss;
    if (a.method == EDG_KLQP_REPARAM_KL) {
      for (int w = 0; w < kl_warps; ++w) klsum += red[w];
      loss = -(mean_ll - klsum);
      a.state->aux[0] = mean_ll;
      a.state->aux[1] = klsum;
    } else {
      double ms = 0.0;
      for (int s = 0; s < a.S; ++s) ms += lsig[s];
      ms *= a.inv_S;
      loss = -(mean_ll + ms);
      a.state->aux[0] = mean_ll;
      a.state->aux[1] = ms;
    }
    a.state->loss = loss;
    if (!isfinite(loss)) atomicAdd(&a.state->nonfinite, 1u);
  }
  // ---- gradients w.r.t. (mu, rho) and the optimizer apply (they read the
  // shared-memory copies of mu, rho and the slots, so they need not wait for
  // the loss above)
  const float lr = opt_lr(a.opt, gstep);
  const float invS = 1.0f / (float)a.S;
  for (int d = threadIdx.x; d < P; d += kThreads) {
    const float mu = s_mu[d], rho = s_rho[d], sg = sig[d];
    const float ps = s_ps[d], pl = s_pl[d];
    const float lsc = s_ls[d];
    float gmu = 0.0f, gsig = 0.0f;
    const bool point = s_pt[d] != 0;
    if (point) {
      // model parameter: d loss / d theta = -mean_s d log p(x | z_s) / d theta
      float sg_mu = 0.0f;
      for (int s = 0; s < a.S; ++s) sg_mu += gS[s * PP + d];
      gmu = -sg_mu * invS;
    } else if (a.method == EDG_KLQP_REPARAM_KL) {
      float sg_mu = 0.0f, sg_sig = 0.0f;
      for (int s = 0; s < a.S; ++s) {
        const float e = epsS[s * PP + d];
        const float g = gS[s * PP + d];
        sg_mu += g;
        sg_sig += g * e;
      }
      const float ks = s_ks[d];
      gmu = -sg_mu * invS + ks * (mu - pl) / (ps * ps);
      gsig = -sg_sig * invS + ks * (sg / (ps * ps) - 1.0f / sg);
    } else if (a.method == EDG_KLQP_REPARAM) {
      float acc_mu = 0.0f, acc_sig = 0.0f;
      for (int s = 0; s < a.S; ++s) {
        const float e = epsS[s * PP + d];
        const float zv = mu + sg * e;
        const float dfdz = gS[s * PP + d] - lsc * (zv - pl) / (ps * ps) + lsc * (zv - mu) / (sg * sg);
        const float dlq_dmu = (zv - mu) / (sg * sg);
        const float dlq_dsig = -1.0f / sg + (zv - mu) * (zv - mu) / (sg * sg * sg);
        acc_mu += dfdz - lsc * dlq_dmu;
        acc_sig += dfdz * e - lsc * dlq_dsig;
      }
      gmu = -acc_mu * invS;
      gsig = -acc_sig * invS;
    } else {
      float acc_mu = 0.0f, acc_sig = 0.0f;
      for (int s = 0; s < a.S; ++s) {
        const float e = epsS[s * PP + d];
        const float zv = mu + sg * e;
        const float w = (float)(llS[s] + lsig[s]);
        acc_mu += lsc * (zv - mu) / (sg * sg) * w;
        acc_sig += lsc * (-1.0f / sg + (zv - mu) * (zv - mu) / (sg * sg * sg)) * w;
      }
      gmu = -acc_mu * invS;
      gsig = -acc_sig * invS;
    }
    const float grho = point ? 0.0f : gsig * sigmoidf(rho);
    if (!isfinite(gmu) || !isfinite(grho)) atomicAdd(&a.state->nonfinite, 1u);
    if (a.grad_out) {
      a.grad_out[d] = gmu;
      a.grad_out[P + d] = grho;
    }
    if (a.apply) {
      // slots [4][P]: mu's first, rho's first, mu's second, rho's second
      const int n = 2 * P;
      float m0 = s_sl[d], r0 = s_sl[PP + d], m1 = s_sl[2 * PP + d], r1 = s_sl[3 * PP + d];
      a.mu[d] = opt_apply(a.opt, mu, gmu, &m0, &m1, lr, b1p, b2p);
      a.slots[d] = m0;
      a.slots[n + d] = m1;
      if (!point) {
        a.rho[d] = opt_apply(a.opt, rho, grho, &r0, &r1, lr, b1p, b2p);
        a.slots[P + d] = r0;
        a.slots[n + P + d] = r1;
      }
    }
  }
  // the step counters (no other block reads them any more; the kernel's end
  // orders these writes before the next step's launch)
  if (threadIdx.x == kLossThread) {
    if (a.apply) {
      a.state->t = t + 1;
      a.state->global_step = gstep + 1;
      a.state->beta1_power = b1p * a.opt.beta1;
      a.state->beta2_power = b2p * a.opt.beta2;
    }
    a.state->done = 0;
  }
}

// ============================================================ HMC
struct HmcArgs {
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
};

// Adds the Normal prior to a likelihood gradient block and returns nothing;
// G[c][d] += -(z - loc) / scale^2 for d < P.
template <int CT>
__device__ __forceinline__ void add_prior_grad(const GLMDev& m, const float* Z, float* G) {
  for (int idx = threadIdx.x; idx < CT * m.PP; idx += kThreads) {
    const int d = idx % m.PP;
    if (d < m.P) {
      const float sc = m.prior_scale[d];
      G[idx] += -(Z[idx] - m.prior_loc[d]) / (sc * sc);
    }
  }
}

// FP64 prior log density of chain c (called by one thread per chain).
__device__ __forceinline__ double prior_lp(const GLMDev& m, const float* zc) {
  double s = 0.0;
  for (int d = 0; d < m.P; ++d) {
    const float sc = m.prior_scale[d];
    const float zz = (zc[d] - m.prior_loc[d]) / sc;
    s += (double)(-0.5f * zz * zz - logf(sc)) - kHalfLog2Pi;
  }
  return s;
}

template <int CT>
__host__ __device__ constexpr size_t hmc_smem_bytes(int PP) {
  return grad_smem_doubles<CT>() * 8 + grad_smem_floats<CT>(PP) * 4 +
         (size_t)4 * CT * PP * 4 /* Z0 G0 Z R (G is S.G) */ + (size_t)3 * CT * 8 + CT * 4;
}

template <int CT>
__global__ void __launch_bounds__(kThreads, 1) hmc_glm_kernel(GLMDev m, HmcArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  GradSmem S;
  unsigned char* rest = carve_grad<CT>(smem, m.PP, S);
  const int PP = m.PP, P = m.P;
  float* Z0 = reinterpret_cast<float*>(rest);
  float* G0 = Z0 + CT * PP;
  float* Z = G0 + CT * PP;
  float* R = Z + CT * PP;
  double* lj0 = reinterpret_cast<double*>(R + CT * PP);
  double* kin0 = lj0 + CT;
  double* ljn = kin0 + CT;
  int* acc = reinterpret_cast<int*>(ljn + CT);
  float* G = S.G;
  __shared__ bool s_last;

  const int cbase = blockIdx.x * CT;
  const int nc = min(CT, a.C - cbase);
  const int64_t t0 = *(volatile int64_t*)&a.state->t;
  const float eps = a.step_size, half = 0.5f * a.step_size;

  init_x_pad<CT>(m, S);
  for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
    const int c = idx / PP, d = idx - c * PP;
    const bool ok = c < nc && d < P;
    const size_t g = (size_t)(cbase + c) * P + d;
    Z0[idx] = ok ? a.z[g] : 0.0f;
    G0[idx] = (ok && a.cache_valid) ? a.grad[g] : 0.0f;
  }
  if (threadIdx.x < CT)
    lj0[threadIdx.x] = (a.cache_valid && threadIdx.x < nc) ? a.lj[cbase + threadIdx.x] : 0.0;
  __syncthreads();
  if (!a.cache_valid) {
    transpose_into<CT>(Z0, S.Zt, PP);
    __syncthreads();
    glm_grad_eval<CT>(m, 0, m.N, S, true, true, 1.0f);
    add_prior_grad<CT>(m, Z0, G);
    __syncthreads();
    for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) G0[idx] = G[idx];
    if (threadIdx.x < CT) lj0[threadIdx.x] = S.ll[threadIdx.x] + prior_lp(m, Z0 + threadIdx.x * PP);
    __syncthreads();
  }

  for (int it = 0; it < a.n_iter; ++it) {
    const int64_t t = t0 + it;
    const uint32_t iter = (uint32_t)t;
    // momentum draw; working copies
    for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
      const int c = idx / PP, d = idx - c * PP;
      float r = 0.0f;
      if (c < nc && d < P) {
        r = a.r_ovr ? a.r_ovr[((size_t)it * a.C + cbase + c) * P + d]
                    : philox_normal(a.seed, 1u, iter, (uint32_t)(cbase + c), (uint32_t)d);
      }
      R[idx] = r;
      Z[idx] = Z0[idx];
      G[idx] = G0[idx];
    }
    __syncthreads();
    if (threadIdx.x < CT) {
      double k = 0.0;
      const float* rc = R + threadIdx.x * PP;
      for (int d = 0; d < P; ++d) k += (double)rc[d] * (double)rc[d];
      kin0[threadIdx.x] = k;
    }
    __syncthreads();
    // leapfrog (hmc.py:195-210): r += h g; z += eps r; g = grad(z); r += h g
    for (int l = 0; l < a.n_steps; ++l) {
      for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
        const float r = R[idx] + half * G[idx];
        const float zz = Z[idx] + eps * r;
        R[idx] = r;
        Z[idx] = zz;
        const int c = idx / PP, d = idx - c * PP;
        S.Zt[d * CT + c] = zz;
      }
      __syncthreads();
      const bool last = (l == a.n_steps - 1);
      glm_grad_eval<CT>(m, 0, m.N, S, last, true, 1.0f);
      for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
        const int d = idx % PP;
        float g = G[idx];
        if (d < P) {
          const float sc = m.prior_scale[d];
          g += -(Z[idx] - m.prior_loc[d]) / (sc * sc);
        }
        G[idx] = g;
        R[idx] += half * g;
      }
      __syncthreads();
    }
    // Metropolis test in FP64 (hmc.py:100-109)
    if (threadIdx.x < CT) {
      const int c = threadIdx.x;
      int accept = 0;
      if (c < nc) {
        double lj_new;
        if (a.n_steps > 0) {
          lj_new = S.ll[c] + prior_lp(m, Z + c * PP);
        } else {
          lj_new = lj0[c];
        }
        double k = 0.0;
        const float* rc = R + c * PP;
        for (int d = 0; d < P; ++d) k += (double)rc[d] * (double)rc[d];
        const double ratio = 0.5 * kin0[c] - 0.5 * k + lj_new - lj0[c];
        const double u = a.u_ovr ? a.u_ovr[(size_t)it * a.C + cbase + c]
                                 : u01d(philox_at(a.seed, 2u, iter, (uint32_t)(cbase + c), 0u).x);
        accept = log(u) < ratio ? 1 : 0;
        if (accept) lj0[c] = lj_new;
        if (a.n_accept) a.n_accept[cbase + c] += accept;
        if (a.ratio_out) a.ratio_out[(size_t)it * a.C + cbase + c] = ratio;
      }
      acc[c] = accept;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
      const int c = idx / PP, d = idx - c * PP;
      if (acc[c]) {
        Z0[idx] = Z[idx];
        G0[idx] = G[idx];
      }
      if (c < nc && d < P) {
        const float v = acc[c] ? Z[idx] : Z0[idx];
        if (a.samples && t < a.T_cap) a.samples[((size_t)t * a.C + cbase + c) * P + d] = v;
        if (a.moments) {
          const size_t g = (size_t)(cbase + c) * P + d;
          a.moments[g] += (double)v;
          a.moments[(size_t)a.C * P + g] += (double)v * (double)v;
        }
      }
    }
    __syncthreads();
  }
  // write back state and cache
  for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
    const int c = idx / PP, d = idx - c * PP;
    if (c < nc && d < P) {
      const size_t g = (size_t)(cbase + c) * P + d;
      a.z[g] = Z0[idx];
      a.grad[g] = G0[idx];
    }
  }
  if (threadIdx.x < nc) a.lj[cbase + threadIdx.x] = lj0[threadIdx.x];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(&a.state->done, 1u);
    s_last = (prev == gridDim.x - 1);
    if (s_last) {
      a.state->t = t0 + a.n_iter;
      a.state->done = 0;
      __threadfence();
    }
  }
}

// ------------------------------------------------------------ host helpers
static int max_smem_optin() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

static int sm_count() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return v > 0 ? v : 1;
}

template <int CT>
static size_t grad_smem_bytes(int PP) {
  return grad_smem_doubles<CT>() * 8 + grad_smem_floats<CT>(PP) * 4;
}

template <int CT>
static size_t klqp_grad_smem_bytes(int PP) {
  constexpr int R = klqp_rpt<CT>();
  return grad_smem_doubles<CT, R>() * 8 + grad_smem_floats<CT, R>(PP) * 4;
}

static int pick_ct(int B) { return B <= 8 ? 8 : (B <= 16 ? 16 : 32); }

struct GradPlan {
  int CT, ntiles, nchunks, chunk, Bpad;
  size_t ws_g_bytes, ws_ll_bytes;
};

static GradPlan plan_grad(const GLMDev& m, int B) {
  GradPlan p;
  p.CT = pick_ct(B);
  p.ntiles = (B + p.CT - 1) / p.CT;
  p.Bpad = p.ntiles * p.CT;
  const int RT = 2048 / p.CT;
  const int max_chunks = (m.N + RT - 1) / RT;
  int want = std::max(1, (2 * sm_count()) / p.ntiles);
  p.nchunks = std::min(max_chunks, want);
  p.chunk = (m.N + p.nchunks - 1) / p.nchunks;
  p.chunk = round_up(p.chunk, RT);
  p.nchunks = (m.N + p.chunk - 1) / p.chunk;
  p.ws_g_bytes = (size_t)p.nchunks * p.Bpad * m.PP * sizeof(float);
  p.ws_ll_bytes = (size_t)p.nchunks * p.Bpad * sizeof(double);
  return p;
}

template <int CT>
static int launch_partial(const GLMDev& m, const float* Z, int B, const GradPlan& p, float dscale,
                          float* wg, double* wl, int need_grad, cudaStream_t st) {
  const size_t sm = grad_smem_bytes<CT>(m.PP);
  EDG_REQUIRE((int)sm <= max_smem_optin(), EDG_E_UNSUPPORTED,
              "P=%d needs %zu bytes of shared memory", m.P, sm);
  int rc = set_max_dyn_smem(glm_partial_kernel<CT>, sm, "glm_partial_kernel");
  if (rc) return rc;
  dim3 grid(p.nchunks, p.ntiles);
  glm_partial_kernel<CT><<<grid, kThreads, sm, st>>>(m, Z, B, p.chunk, dscale, wg, wl, p.Bpad,
                                                     need_grad);
  return check_launch("glm_partial_kernel");
}

}  // namespace edg

using namespace edg;

extern "C" size_t edg_glm_logjoint_grad_workspace_bytes(const edg_glm_t* model, int32_t B) {
  GLMDev m;
  if (make_glm(model, &m) != EDG_OK || B <= 0) return 0;
  const GradPlan p = plan_grad(m, B);
  return round_up_bytes(p.ws_g_bytes, 256) + p.ws_ll_bytes;
}

extern "C" int edg_glm_logjoint_grad(const edg_glm_t* model, const float* Z, int32_t B,
                                     int32_t include_prior, float data_scale, double* lp_out,
                                     float* grad_out, void* workspace, size_t workspace_bytes,
                                     void* stream) {
  GLMDev m;
  int rc = make_glm(model, &m);
  if (rc) return rc;
  EDG_REQUIRE(Z, EDG_E_NULL, "Z is NULL");
  EDG_REQUIRE(B > 0, EDG_E_SHAPE, "B must be positive (got %d)", B);
  if (!lp_out && !grad_out) return EDG_OK;
  const GradPlan p = plan_grad(m, B);
  const size_t need = round_up_bytes(p.ws_g_bytes, 256) + p.ws_ll_bytes;
  EDG_REQUIRE(workspace && workspace_bytes >= need, EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  float* wg = reinterpret_cast<float*>(workspace);
  double* wl = reinterpret_cast<double*>(reinterpret_cast<char*>(workspace) +
                                         round_up_bytes(p.ws_g_bytes, 256));
  cudaStream_t st = (cudaStream_t)stream;
  const int ng = grad_out ? 1 : 0;
  switch (p.CT) {
    case 8: rc = launch_partial<8>(m, Z, B, p, data_scale, wg, wl, ng, st); break;
    case 16: rc = launch_partial<16>(m, Z, B, p, data_scale, wg, wl, ng, st); break;
    default: rc = launch_partial<32>(m, Z, B, p, data_scale, wg, wl, ng, st); break;
  }
  if (rc) return rc;
  const int64_t n = std::max<int64_t>((int64_t)B * m.P, B);
  glm_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      m, Z, B, p.nchunks, wg, wl, p.Bpad, include_prior, lp_out, grad_out);
  return check_launch("glm_reduce_kernel");
}

// ---------------------------------------------------------------- KLqp
struct KlqpPlan {
  int CT, Spad, nblocks, chunk;
  size_t ws_g, ws_ll;
};

static KlqpPlan plan_klqp(const GLMDev& m, int S) {
  KlqpPlan p;
  p.CT = pick_ct(S);
  p.Spad = round_up(S, p.CT);
  const int RT = 1024 * (p.CT == 32 ? 2 : 1) / p.CT;
  const int ntiles = (m.N + RT - 1) / RT;
  const int sm = sm_count();
  const int tiles_per_block = std::max(1, (ntiles + sm - 1) / sm);
  p.chunk = tiles_per_block * RT;
  p.nblocks = (m.N + p.chunk - 1) / p.chunk;
  p.ws_g = (size_t)p.nblocks * p.Spad * m.PP * sizeof(float);
  p.ws_ll = (size_t)p.nblocks * p.Spad * sizeof(double);
  return p;
}

extern "C" size_t edg_klqp_glm_workspace_bytes(const edg_glm_t* model, const edg_klqp_t* cfg) {
  GLMDev m;
  if (!cfg || make_glm(model, &m) != EDG_OK || cfg->n_samples <= 0) return 0;
  const KlqpPlan p = plan_klqp(m, cfg->n_samples);
  return round_up_bytes(p.ws_g, 256) + p.ws_ll;
}

template <int CT>
static int launch_klqp(const GLMDev& m, const KlqpArgs& a, cudaStream_t st) {
  constexpr int RT = Tile<CT, klqp_rpt<CT>()>::RT;
  const size_t sm = klqp_grad_smem_bytes<CT>(m.PP) + (size_t)m.PP * 4 +
                    (size_t)a.Spad * m.PP * 4 + (size_t)11 * m.PP * 4;
  EDG_REQUIRE((int)sm <= max_smem_optin(), EDG_E_UNSUPPORTED, "P=%d too large for KLqp kernel", m.P);
  // the tail's per-sample sums and per-warp partials reuse the log-lik partials
  EDG_REQUIRE(a.S * 2 + 8 <= (RT / klqp_rpt<CT>()) * CT, EDG_E_UNSUPPORTED, "n_samples too large");
  EDG_REQUIRE((size_t)a.S * m.PP <= (size_t)2 * RT * m.PP, EDG_E_UNSUPPORTED,
              "n_samples too large");
  const int rc = set_max_dyn_smem(klqp_glm_kernel<CT>, sm, "klqp_glm_kernel");
  if (rc) return rc;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)a.nblocks);
  lc.blockDim = dim3(kThreads);
  lc.dynamicSmemBytes = sm;
  lc.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&lc, klqp_glm_kernel<CT>, m, a);
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "klqp_glm_kernel launch: %s", cudaGetErrorString(e));
  return check_launch("klqp_glm_kernel");
}

extern "C" int edg_klqp_glm_step(const edg_glm_t* model, const edg_klqp_t* cfg,
                                 const edg_opt_t* opt, float* mu, float* rho, float* opt_slots,
                                 edg_state_t* state, const float* eps_override, float* grad_out,
                                 int32_t apply, void* workspace, size_t workspace_bytes,
                                 void* stream) {
  GLMDev m;
  int rc = make_glm(model, &m);
  if (rc) return rc;
  EDG_REQUIRE(cfg && opt, EDG_E_NULL, "cfg and opt must not be NULL");
  EDG_REQUIRE(mu && rho && state, EDG_E_NULL, "mu, rho and state must not be NULL");
  EDG_REQUIRE(!apply || opt_slots, EDG_E_NULL, "opt_slots must not be NULL when apply = 1");
  EDG_REQUIRE(cfg->n_samples > 0, EDG_E_VALUE, "n_samples should be greater than zero: %d",
              cfg->n_samples);
  EDG_REQUIRE(cfg->method >= 0 && cfg->method <= 2, EDG_E_VALUE, "unknown KLqp method %d",
              cfg->method);
  EDG_REQUIRE(opt->optimizer >= 0 && opt->optimizer <= 5, EDG_E_VALUE, "unknown optimizer %d",
              opt->optimizer);
  const KlqpPlan p = plan_klqp(m, cfg->n_samples);
  const size_t need = round_up_bytes(p.ws_g, 256) + p.ws_ll;
  EDG_REQUIRE(workspace && workspace_bytes >= need, EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  KlqpArgs a;
  a.method = cfg->method;
  a.S = cfg->n_samples;
  a.inv_S = 1.0 / cfg->n_samples;
  a.Spad = p.Spad;
  a.nblocks = p.nblocks;
  a.chunk = p.chunk;
  a.dscale = cfg->data_scale;
  a.kl_scaling = cfg->kl_scaling;
  a.latent_scale = cfg->latent_scale;
  a.point = cfg->point;
  a.seed = cfg->seed;
  a.opt = *opt;
  a.mu = mu;
  a.rho = rho;
  a.slots = opt_slots;
  a.state = state;
  a.eps_ovr = eps_override;
  a.grad_out = grad_out;
  a.apply = apply;
  a.ws_g = reinterpret_cast<float*>(workspace);
  a.ws_ll = reinterpret_cast<double*>(reinterpret_cast<char*>(workspace) + round_up_bytes(p.ws_g, 256));
  cudaStream_t st = (cudaStream_t)stream;
  switch (p.CT) {
    case 8: return launch_klqp<8>(m, a, st);
    case 16: return launch_klqp<16>(m, a, st);
    default: return launch_klqp<32>(m, a, st);
  }
}

// ---------------------------------------------------------------- HMC
template <int CT>
static int launch_hmc(const GLMDev& m, const HmcArgs& a, cudaStream_t st) {
  const size_t sm = hmc_smem_bytes<CT>(m.PP);
  EDG_REQUIRE((int)sm <= max_smem_optin(), EDG_E_UNSUPPORTED,
              "P=%d needs %zu bytes of shared memory for %d chains per block", m.P, sm, CT);
  const int rc = set_max_dyn_smem(hmc_glm_kernel<CT>, sm, "hmc_glm_kernel");
  if (rc) return rc;
  const int nblocks = (a.C + CT - 1) / CT;
  hmc_glm_kernel<CT><<<nblocks, kThreads, sm, st>>>(m, a);
  return check_launch("hmc_glm_kernel");
}

extern "C" int edg_hmc_glm_run(const edg_glm_t* model, const edg_hmc_t* cfg, int32_t C,
                               int32_t n_iter, float* z, float* grad, double* lj,
                               int32_t cache_valid, int32_t* n_accept, edg_state_t* state,
                               float* samples, int64_t T_cap, double* moments,
                               const float* r_override, const double* u_override,
                               double* ratio_out, void* stream) {
  GLMDev m;
  int rc = make_glm(model, &m);
  if (rc) return rc;
  EDG_REQUIRE(cfg, EDG_E_NULL, "cfg is NULL");
  EDG_REQUIRE(z && grad && lj && state, EDG_E_NULL, "z, grad, lj and state must not be NULL");
  EDG_REQUIRE(C > 0, EDG_E_SHAPE, "C must be positive (got %d)", C);
  EDG_REQUIRE(n_iter >= 0, EDG_E_SHAPE, "n_iter must be >= 0");
  EDG_REQUIRE(cfg->n_steps >= 0, EDG_E_VALUE, "n_steps must be >= 0");
  EDG_REQUIRE(!samples || T_cap > 0, EDG_E_SHAPE, "T_cap must be positive when samples is given");
  if (n_iter == 0 && cache_valid) return EDG_OK;
  HmcArgs a;
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
  int ct = cfg->chains_per_block;
  if (ct == 0) ct = 32;
  cudaStream_t st = (cudaStream_t)stream;
  switch (ct) {
    case 8: return launch_hmc<8>(m, a, st);
    case 16: return launch_hmc<16>(m, a, st);
    case 32: return launch_hmc<32>(m, a, st);
    default: return fail(EDG_E_VALUE, "chains_per_block must be 0, 8, 16 or 32 (got %d)", ct);
  }
}

// ---------------------------------------------------------------- no-allocation variant
// Fixed device scratch for edg_glm_logjoint_grad_noalloc.  Every GPU that
// loads this library holds these bytes until the process exits.
namespace edg {
constexpr size_t kNoAllocScratchBytes = (size_t)8 << 20;  // 8 MiB
constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in, so the address is looked up once per device
// (cudaGetSymbolAddress, with that device current) and cached.
static int noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  EDG_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, EDG_E_UNSUPPORTED,
              "device %d is beyond the %d devices the fixed scratch supports", dev,
              kNoAllocMaxDevices);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(EDG_E_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return EDG_OK;
}
}  // namespace edg

extern "C" int edg_glm_logjoint_grad_noalloc(const edg_glm_t* model, const float* Z, int32_t B,
                                             int32_t include_prior, float data_scale,
                                             double* lp_out, float* grad_out, void* stream) {
  GLMDev m;
  int rc = make_glm(model, &m);
  if (rc) return rc;
  EDG_REQUIRE(Z, EDG_E_NULL, "Z is NULL");
  EDG_REQUIRE(B > 0, EDG_E_SHAPE, "B must be positive (got %d)", B);
  if (!lp_out && !grad_out) return EDG_OK;
  const GradPlan p = plan_grad(m, B);
  const size_t need = round_up_bytes(p.ws_g_bytes, 256) + p.ws_ll_bytes;
  EDG_REQUIRE(need <= kNoAllocScratchBytes, EDG_E_WORKSPACE,
              "this call needs %zu bytes of scratch but the fixed scratch holds %zu bytes; "
              "split the %d vectors into smaller batches or use edg_glm_logjoint_grad",
              need, kNoAllocScratchBytes, B);
  void* scratch = nullptr;
  rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  float* wg = reinterpret_cast<float*>(scratch);
  double* wl = reinterpret_cast<double*>(reinterpret_cast<char*>(scratch) +
                                         round_up_bytes(p.ws_g_bytes, 256));
  cudaStream_t st = (cudaStream_t)stream;
  const int ng = grad_out ? 1 : 0;
  switch (p.CT) {
    case 8: rc = launch_partial<8>(m, Z, B, p, data_scale, wg, wl, ng, st); break;
    case 16: rc = launch_partial<16>(m, Z, B, p, data_scale, wg, wl, ng, st); break;
    default: rc = launch_partial<32>(m, Z, B, p, data_scale, wg, wl, ng, st); break;
  }
  if (rc) return rc;
  const int64_t n = std::max<int64_t>((int64_t)B * m.P, B);
  glm_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      m, Z, B, p.nchunks, wg, wl, p.Bpad, include_prior, lp_out, grad_out);
  return check_launch("glm_reduce_kernel (no-alloc)");
}
