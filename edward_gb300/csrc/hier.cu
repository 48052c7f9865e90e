// Ragged batch of hierarchical logistic regressions under HMC.
//
// Instance i: X_i [N_i, D_i], y_i [N_i];  mu ~ N(mu_loc, mu_scale),
// tau ~ HalfNormal(tau_scale) sampled as u = softplus^{-1}(tau),
// w_d ~ N(mu, tau), y ~ Bernoulli(X_i w).  C chains per instance, state per
// chain stored with a fixed stride SP = max_D + 2: w in [0, D_i), zeros up to
// max_D, mu at SP - 2 and u at SP - 1.
//
// One CTA per (instance, 32 chains).  Every gradient evaluation streams the
// instance's X through shared memory with glm_grad_eval (forward + adjoint
// in one pass); the hierarchical prior, its gradient and the softplus
// Jacobian are added per chain; leapfrog and the FP64 Metropolis test run in
// the same launch for n_iter iterations.  Blocks are launched in the order
// given by `order` (heaviest instances first balances the ragged work).
#include <algorithm>

#include "edg_common.cuh"
#include "glm_tile.cuh"

namespace edg {

struct HierArgs {
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
  int persistent;  // 1: each CTA pulls (instance, chain tile) items from a work counter
};

template <int CT>
__host__ __device__ constexpr size_t hier_smem_bytes(int PPmax) {
  return grad_smem_doubles<CT>() * 8 + grad_smem_floats<CT>(PPmax) * 4 +
         (size_t)4 * CT * PPmax * 4 /* Z0 G0 Z R */ + (size_t)CT * 10 * 4 /* hyper */ +
         (size_t)4 * CT * 8 + CT * 4;
}

// Hierarchical prior terms of one chain given its w (row of Z, length D), mu, u.
// Adds d/dw to G (row), returns d/dmu, d/du and (if lp) the FP64 log density
// of (w, mu, tau) plus log sigmoid(u).  Executed by one warp per chain.
__device__ __forceinline__ void hier_prior_warp(const float* Zc, float* Gc, int D, float mu,
                                                float u, float mu_loc, float mu_scale,
                                                float tau_scale, float& gmu, float& gu,
                                                double* lp) {
  const int lane = threadIdx.x & 31;
  const float tau = softplusf(u);
  const float inv_t2 = 1.0f / (tau * tau);
  float s1 = 0.0f, s2 = 0.0f;
  for (int d = lane; d < D; d += 32) {
    const float dev = Zc[d] - mu;
    s1 += dev;
    s2 += dev * dev;
    Gc[d] += -dev * inv_t2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  gmu = s1 * inv_t2 - (mu - mu_loc) / (mu_scale * mu_scale);
  const float dtau = -(float)D / tau + s2 * inv_t2 / tau - tau / (tau_scale * tau_scale);
  const float sg = sigmoidf(u);
  gu = dtau * sg + (1.0f - sg);
  if (lp) {
    const double lw = -0.5 * (double)s2 * (double)inv_t2 - (double)D * (double)logf(tau) -
                      (double)D * kHalfLog2Pi;
    const double zm = ((double)mu - mu_loc) / mu_scale;
    const double lmu = -0.5 * zm * zm - log((double)mu_scale) - kHalfLog2Pi;
    const double zt = (double)tau / tau_scale;
    const double ltau = 0.5 * log(2.0 / 3.14159265358979323846) - log((double)tau_scale) -
                        0.5 * zt * zt;
    const double ldj = -(double)softplusf(-u);
    *lp = lw + lmu + ltau + ldj;
  }
}

// All n_iter iterations of one work item: the chains [ctile*CT, ctile*CT + CT)
// of instance order[item / tiles_per_inst].
template <int CT>
__device__ void hier_item(const HierArgs& a, int item, unsigned char* smem) {
  const int inst = a.order ? a.order[item / a.tiles_per_inst] : item / a.tiles_per_inst;
  const int ctile = item % a.tiles_per_inst;
  GLMDev m;
  m.X = a.X + a.x_off[inst];
  m.y = a.y + a.y_off[inst];
  m.prior_loc = nullptr;
  m.prior_scale = nullptr;
  m.N = a.Ns[inst];
  m.D = a.Ds[inst];
  m.P = m.D;
  m.PP = round_up(m.D, 4);
  m.bias = 0;
  m.lik = EDG_LIK_BERNOULLI;
  m.inv_lik_var = 1.0f;
  m.lik_norm = 0.0f;
  const int D = m.D, PP = m.PP, SP = a.SP;
  GradSmem S;
  // carve for this instance's PP (the allocation covers max_D)
  unsigned char* rest = carve_grad<CT>(smem, PP, S);
  float* Z0 = reinterpret_cast<float*>(rest);
  float* G0 = Z0 + CT * PP;
  float* Z = G0 + CT * PP;
  float* R = Z + CT * PP;
  float* H = R + CT * PP;   // [10][CT]: mu0 u0 gmu0 gu0 | mu u | rmu ru | gmu gu
  double* lj0 = reinterpret_cast<double*>(H + 10 * CT);
  double* kin0 = lj0 + CT;
  double* ljn = kin0 + CT;
  double* lpn = ljn + CT;
  int* acc = reinterpret_cast<int*>(lpn + CT);
  float* G = S.G;
  float *mu0 = H, *u0 = H + CT, *gmu0 = H + 2 * CT, *gu0 = H + 3 * CT;
  float *hmu = H + 4 * CT, *hu = H + 5 * CT, *rmu = H + 6 * CT, *ru = H + 7 * CT;
  float *gmu = H + 8 * CT, *gu = H + 9 * CT;

  const int cbase = ctile * CT;
  const int nc = min(CT, a.C - cbase);
  const int64_t t0 = *(volatile int64_t*)&a.state->t;
  const float eps = a.step_size, half = 0.5f * a.step_size;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto gchain = [&](int c) -> size_t { return (size_t)inst * a.C + cbase + c; };

  init_x_pad<CT>(m, S);
  for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
    const int c = idx / PP, d = idx - c * PP;
    const bool ok = c < nc && d < D;
    const size_t g = gchain(c) * SP + d;
    Z0[idx] = ok ? a.z[g] : 0.0f;
    G0[idx] = (ok && a.cache_valid) ? a.grad[g] : 0.0f;
  }
  if (threadIdx.x < CT) {
    const int c = threadIdx.x;
    const bool ok = c < nc;
    const size_t g = gchain(ok ? c : 0) * SP;
    mu0[c] = ok ? a.z[g + SP - 2] : 0.0f;
    u0[c] = ok ? a.z[g + SP - 1] : 0.0f;
    gmu0[c] = (ok && a.cache_valid) ? a.grad[g + SP - 2] : 0.0f;
    gu0[c] = (ok && a.cache_valid) ? a.grad[g + SP - 1] : 0.0f;
    lj0[c] = (ok && a.cache_valid) ? a.lj[gchain(c)] : 0.0;
  }
  __syncthreads();

  // gradient of the full log joint at Zsrc/(musrc, usrc): likelihood by
  // glm_grad_eval into G, then the hierarchical prior (one warp per chain)
  auto full_grad = [&](const float* Zsrc, const float* musrc, const float* usrc, bool need_ll) {
    transpose_into<CT>(Zsrc, S.Zt, PP);
    __syncthreads();
    glm_grad_eval<CT>(m, 0, m.N, S, need_ll, true, 1.0f);
    for (int c = warp; c < CT; c += kThreads / 32) {
      float gm, gv;
      double lp = 0.0;
      hier_prior_warp(Zsrc + c * PP, G + c * PP, D, musrc[c], usrc[c], a.mu_loc, a.mu_scale,
                      a.tau_scale, gm, gv, need_ll ? &lp : nullptr);
      if (lane == 0) {
        gmu[c] = gm;
        gu[c] = gv;
        if (need_ll) lpn[c] = lp;
      }
    }
    __syncthreads();
  };

  if (!a.cache_valid) {
    full_grad(Z0, mu0, u0, true);
    for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) G0[idx] = G[idx];
    if (threadIdx.x < CT) {
      gmu0[threadIdx.x] = gmu[threadIdx.x];
      gu0[threadIdx.x] = gu[threadIdx.x];
      lj0[threadIdx.x] = S.ll[threadIdx.x] + lpn[threadIdx.x];
    }
    __syncthreads();
  }

  for (int it = 0; it < a.n_iter; ++it) {
    const int64_t t = t0 + it;
    const uint32_t iter = (uint32_t)t;
    // momenta for (w, mu, u): Philox elements 0..D-1 are w, D is mu, D + 1 is u
    for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
      const int c = idx / PP, d = idx - c * PP;
      float r = 0.0f;
      if (c < nc && d < D)
        r = a.r_ovr ? a.r_ovr[((size_t)it * a.I * a.C + gchain(c)) * SP + d]
                    : philox_normal(a.seed, 1u, iter, (uint32_t)gchain(c), (uint32_t)d);
      R[idx] = r;
      Z[idx] = Z0[idx];
      G[idx] = G0[idx];
    }
    if (threadIdx.x < CT) {
      const int c = threadIdx.x;
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
    if (threadIdx.x < CT) {
      const int c = threadIdx.x;
      double k = (double)rmu[c] * rmu[c] + (double)ru[c] * ru[c];
      const float* rc = R + c * PP;
      for (int d = 0; d < D; ++d) k += (double)rc[d] * (double)rc[d];
      kin0[c] = k;
    }
    __syncthreads();
    for (int l = 0; l < a.n_steps; ++l) {
      for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
        const float r = R[idx] + half * G[idx];
        R[idx] = r;
        Z[idx] = Z[idx] + eps * r;
      }
      if (threadIdx.x < CT) {
        const int c = threadIdx.x;
        rmu[c] += half * gmu[c];
        ru[c] += half * gu[c];
        hmu[c] += eps * rmu[c];
        hu[c] += eps * ru[c];
      }
      __syncthreads();
      const bool last = l == a.n_steps - 1;
      full_grad(Z, hmu, hu, last);
      for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) R[idx] += half * G[idx];
      if (threadIdx.x < CT) {
        rmu[threadIdx.x] += half * gmu[threadIdx.x];
        ru[threadIdx.x] += half * gu[threadIdx.x];
        if (last) ljn[threadIdx.x] = S.ll[threadIdx.x] + lpn[threadIdx.x];
      }
      __syncthreads();
    }
    if (threadIdx.x < CT) {
      const int c = threadIdx.x;
      int accept = 0;
      if (c < nc) {
        const double lj_new = a.n_steps > 0 ? ljn[c] : lj0[c];
        double k = (double)rmu[c] * rmu[c] + (double)ru[c] * ru[c];
        const float* rc = R + c * PP;
        for (int d = 0; d < D; ++d) k += (double)rc[d] * (double)rc[d];
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
    for (int idx = threadIdx.x; idx < CT * PP; idx += kThreads) {
      if (acc[idx / PP]) {
        Z0[idx] = Z[idx];
        G0[idx] = G[idx];
      }
    }
    __syncthreads();
    // kept sample (w, mu, u) and running moments
    const int W = D + 2;
    for (int idx = threadIdx.x; idx < nc * W; idx += kThreads) {
      const int c = idx / W, d = idx - c * W;
      const float v = d < D ? Z0[c * PP + d] : (d == D ? mu0[c] : u0[c]);
      const size_t g = gchain(c) * SP + (d < D ? d : SP - 2 + (d - D));
      if (a.samples && t < a.T_cap) a.samples[(size_t)t * a.I * a.C * SP + g] = v;
      if (a.moments) {
        a.moments[g] += (double)v;
        a.moments[(size_t)a.I * a.C * SP + g] += (double)v * (double)v;
      }
    }
    __syncthreads();
  }
  // write back the state and its cache
  for (int idx = threadIdx.x; idx < nc * (D + 2); idx += kThreads) {
    const int c = idx / (D + 2), d = idx - c * (D + 2);
    const size_t g = gchain(c) * SP + (d < D ? d : SP - 2 + (d - D));
    a.z[g] = d < D ? Z0[c * PP + d] : (d == D ? mu0[c] : u0[c]);
    a.grad[g] = d < D ? G0[c * PP + d] : (d == D ? gmu0[c] : gu0[c]);
  }
  if (threadIdx.x < nc) a.lj[gchain(threadIdx.x)] = lj0[threadIdx.x];
  __syncthreads();  // the next item reuses the shared memory
}

// One launch runs every item for n_iter iterations.  Persistent form: a grid
// of resident CTAs, each taking items from the state's work counter in the
// launch order (heaviest instances first, so the ragged tail is short).
// Otherwise one CTA per item.  The last CTA to finish advances t and clears
// the counters.
template <int CT>
__global__ void __launch_bounds__(kThreads) hmc_hier_kernel(HierArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item;
  __shared__ bool s_last;
  __shared__ int64_t s_t0;
  if (threadIdx.x == 0) s_t0 = *(volatile int64_t*)&a.state->t;
  if (a.persistent) {
    const int total = a.I * a.tiles_per_inst;
    for (;;) {
      __syncthreads();
      if (threadIdx.x == 0) s_item = (int)atomicAdd(&a.state->reserved, 1u);
      __syncthreads();
      const int item = s_item;
      if (item >= total) break;
      hier_item<CT>(a, item, smem);
    }
  } else {
    hier_item<CT>(a, blockIdx.x, smem);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
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

}  // namespace edg

using namespace edg;

template <int CT>
static int launch_hier(const HierArgs& a, int64_t nitems, int PPmax, int max_D, void* stream) {
  const size_t sm = hier_smem_bytes<CT>(PPmax);
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  EDG_REQUIRE((int)sm <= optin, EDG_E_UNSUPPORTED,
              "max_D=%d needs %zu bytes of shared memory with %d chains per block", max_D, sm, CT);
  const int rc_attr = set_max_dyn_smem(hmc_hier_kernel<CT>, sm, "hmc_hier_kernel");
  if (rc_attr) return rc_attr;
  int64_t nblocks = nitems;
  if (a.persistent) {
    int per_sm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hmc_hier_kernel<CT>, kThreads, sm);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    nblocks = std::min<int64_t>(nitems, (int64_t)std::max(per_sm, 1) * std::max(sms, 1));
  }
  hmc_hier_kernel<CT><<<(unsigned)nblocks, kThreads, sm, (cudaStream_t)stream>>>(a);
  return check_launch("hmc_hier_kernel");
}

extern "C" int edg_hmc_hier_run(const edg_hier_t* model, const edg_hmc_t* cfg, int32_t C,
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
  EDG_REQUIRE(model->max_D > 0 && model->max_D <= 160, EDG_E_UNSUPPORTED,
              "max_D must be in [1, 160] (got %d)", model->max_D);
  EDG_REQUIRE(model->mu_scale > 0 && model->tau_scale > 0, EDG_E_VALUE,
              "mu_scale and tau_scale must be positive");
  EDG_REQUIRE(cfg->n_steps >= 0, EDG_E_VALUE, "n_steps must be >= 0");
  EDG_REQUIRE(!samples || T_cap > 0, EDG_E_SHAPE, "T_cap must be positive when samples is given");
  if (n_iter == 0 && cache_valid) return EDG_OK;
  // tile shape: 32 chains x 64 rows (default) or 16 chains x 128 rows
  EDG_REQUIRE(cfg->chains_per_block == 0 || cfg->chains_per_block == 16 ||
                  cfg->chains_per_block == 32,
              EDG_E_VALUE, "chains_per_block must be 0, 16 or 32 (got %d)", cfg->chains_per_block);
  const int CT = cfg->chains_per_block == 16 ? 16 : 32;
  HierArgs a;
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
  a.tiles_per_inst = (C + CT - 1) / CT;
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
  EDG_REQUIRE(cfg->launch == 0 || cfg->launch == 1, EDG_E_VALUE, "launch must be 0 or 1 (got %d)",
              cfg->launch);
  a.persistent = cfg->launch == 0 ? 1 : 0;
  const int64_t nitems = (int64_t)a.I * a.tiles_per_inst;
  EDG_REQUIRE(nitems < (1ll << 31), EDG_E_SHAPE, "too many instances x chain tiles");
  const int PPmax = round_up(model->max_D, 4);
  return CT == 16 ? launch_hier<16>(a, nitems, PPmax, model->max_D, stream)
                  : launch_hier<32>(a, nitems, PPmax, model->max_D, stream);
}
