// One constrained latent with i.i.d. observations, in the unconstrained space
// auto_transform maps it to (edward/inferences/inference.py:222-264,
// edward/util/random_variables.py:856-917):
//   Beta(a, b)       + Bernoulli(probs=z)   : z = sigmoid(u)
//   Gamma(a, rate b) + Poisson(rate=z)      : z = softplus(u)
//   Dirichlet(alpha) + Categorical(probs=z) : z = softmax([u, 0])  (SoftmaxCentered)
// The target is log p(x, z(u)) + log|det dz/du|, from the observations'
// sufficient statistics.  The chain state, the momenta and every per-term
// quantity are FP32; FP64 is used only for the sum of the log joint's terms
// and for the Hamiltonian energy difference of the Metropolis test.
//   edg_expfam_hmc_run   HMC over C chains, one thread per chain, the
//                        reference's leapfrog (hmc.py:195-210) and
//                        Metropolis test (hmc.py:98-118), n_iter iterations
//                        per launch.
//   edg_expfam_klqp_step KLqp with q(u) = N(mu, softplus(rho)): the
//                        reparameterisation gradient with Monte Carlo KL
//                        (build_reparam_loss_and_gradients, klqp.py:642-704),
//                        then the optimizer apply.
#include <algorithm>

#include "edg_common.cuh"
#include "optim.cuh"

namespace edg {
namespace ef {

constexpr int kMaxK = 32;  // unconstrained dimension (Dirichlet: categories - 1)

__device__ __forceinline__ float softplus_f(float x) {
  return fmaxf(x, 0.0f) + log1pf(expf(-fabsf(x)));
}
__device__ __forceinline__ float sigmoid_f(float x) {
  const float e = expf(-fabsf(x));
  return x >= 0.0f ? 1.0f / (1.0f + e) : e / (1.0f + e);
}

// log p(x, z(u)) + log|det dz/du| (up to the data's constant terms for
// Dirichlet-Categorical, which carries none) and its gradient g[K].  Every
// term that depends on u, and the gradient, is FP32; the terms and the
// model's constants (the priors' normalisers) are summed in FP64.
__device__ double log_joint_grad(const edg_expfam_t& m, const float* u, float* g) {
  const double* pr = m.prior;
  const double* st = m.stats;
  if (!m.transform) {
    // on the support itself (Beta: (0, 1), Gamma: (0, inf)); NaN outside it,
    // for the log density and its gradient alike
    const float z = u[0];
    const bool in = m.family == EDG_EXPFAM_BETA ? (z > 0.0f && z < 1.0f) : z > 0.0f;
    if (!in) {
      g[0] = __int_as_float(0x7fc00000);
      return __longlong_as_double(0x7ff8000000000000ll);
    }
    if (m.family == EDG_EXPFAM_BETA) {
      const float a1 = (float)pr[0] - 1.0f + (float)st[0], b1 = (float)pr[1] - 1.0f + (float)st[1];
      g[0] = a1 / z - b1 / (1.0f - z);
      return (double)(a1 * logf(z)) + (double)(b1 * log1pf(-z)) -
             (lgamma(pr[0]) + lgamma(pr[1]) - lgamma(pr[0] + pr[1]));
    }
    const float a1 = (float)pr[0] - 1.0f + (float)st[0], rn = (float)pr[1] + (float)st[1];
    g[0] = a1 / z - rn;
    return pr[0] * log(pr[1]) - lgamma(pr[0]) + (double)(a1 * logf(z)) - (double)(rn * z) - st[2];
  }
  if (m.family == EDG_EXPFAM_BETA) {
    const float a = (float)pr[0], b = (float)pr[1], n1 = (float)st[0], n0 = (float)st[1];
    const float lz = -softplus_f(-u[0]), l1z = -softplus_f(u[0]);
    const float s = sigmoid_f(u[0]);
    g[0] = (a + n1) * (1.0f - s) - (b + n0) * s;
    return (double)((a + n1) * lz) + (double)((b + n0) * l1z) -
           (lgamma(pr[0]) + lgamma(pr[1]) - lgamma(pr[0] + pr[1]));
  }
  if (m.family == EDG_EXPFAM_GAMMA) {
    const float a = (float)pr[0], rate = (float)pr[1], sx = (float)st[0], n = (float)st[1];
    const float z = softplus_f(u[0]), dz = sigmoid_f(u[0]);
    const float lz = logf(z);
    g[0] = ((a - 1.0f + sx) / z - rate - n) * dz + sigmoid_f(-u[0]);
    return pr[0] * log(pr[1]) - lgamma(pr[0]) + (double)((a - 1.0f + sx) * lz) -
           (double)((rate + n) * z) - st[2] - (double)softplus_f(-u[0]);
  }
  // Dirichlet-Categorical, SoftmaxCentered: z = softmax([u, 0])
  const int K = m.K;
  float mx = 0.0f;
  for (int j = 0; j < K; ++j) mx = fmaxf(mx, u[j]);
  float den = expf(-mx);
  for (int j = 0; j < K; ++j) den += expf(u[j] - mx);
  const float lden = mx + logf(den);
  float sw = 0.0f;
  double lj = 0.0, sa = 0.0, slga = 0.0;
  for (int k = 0; k <= K; ++k) {
    const float w = (float)pr[k] + (float)st[k];  // (alpha - 1) + counts + 1 (log-det term)
    const float lz = (k < K ? u[k] : 0.0f) - lden;
    lj += (double)(w * lz);
    sw += w;
    sa += pr[k];
    slga += lgamma(pr[k]);
  }
  for (int j = 0; j < K; ++j) g[j] = ((float)pr[j] + (float)st[j]) - expf(u[j] - lden) * sw;
  return lj + lgamma(sa) - slga;
}

struct HmcArgs {
  edg_expfam_t m;
  int C, n_iter, L, cache_valid;
  float eps;
  uint64_t seed;
  float* u;       // [C, K]
  float* grad;    // [C, K]
  double* lj;     // [C]
  int32_t* n_accept;
  edg_state_t* state;
  float* samples;  // [T_cap, C, K]
  int64_t T_cap;
  const float* r_ovr;   // [n_iter, C, K]
  const double* u_ovr;  // [n_iter, C]
};

__global__ void hmc_kernel(HmcArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int K = a.m.K;
  const int64_t t0 = a.state->t;
  if (c < a.C) {
    float z[kMaxK], g[kMaxK], z0[kMaxK], g0[kMaxK], r[kMaxK];
    for (int j = 0; j < K; ++j) z[j] = a.u[(int64_t)c * K + j];
    double lj;
    if (a.cache_valid) {
      lj = a.lj[c];
      for (int j = 0; j < K; ++j) g[j] = a.grad[(int64_t)c * K + j];
    } else {
      lj = log_joint_grad(a.m, z, g);
    }
    const float half = 0.5f * a.eps;
    for (int it = 0; it < a.n_iter; ++it) {
      const int64_t t = t0 + it;
      float k0 = 0.0f;
      for (int j = 0; j < K; ++j) {
        r[j] = a.r_ovr ? a.r_ovr[((int64_t)it * a.C + c) * K + j]
                       : philox_normal(a.seed, 1u, (uint32_t)t, (uint32_t)c, (uint32_t)j);
        k0 = fmaf(r[j], r[j], k0);
        z0[j] = z[j];
        g0[j] = g[j];
      }
      const double lj0 = lj;
      for (int l = 0; l < a.L; ++l) {
        for (int j = 0; j < K; ++j) {
          r[j] += half * g[j];
          z[j] += a.eps * r[j];
        }
        lj = log_joint_grad(a.m, z, g);
        for (int j = 0; j < K; ++j) r[j] += half * g[j];
      }
      float k1 = 0.0f;
      for (int j = 0; j < K; ++j) k1 = fmaf(r[j], r[j], k1);
      // the energy difference in FP64 (hmc.py:98-105)
      const double ratio = 0.5 * (double)k0 - 0.5 * (double)k1 + lj - lj0;
      const double uu = a.u_ovr ? a.u_ovr[(int64_t)it * a.C + c]
                                : u01d(philox_at(a.seed, 2u, (uint32_t)t, (uint32_t)c, 0u).x);
      const bool acc = isfinite(ratio) && log(uu) < ratio;
      if (acc) {
        a.n_accept[c] += 1;
      } else {
        for (int j = 0; j < K; ++j) {
          z[j] = z0[j];
          g[j] = g0[j];
        }
        lj = lj0;
      }
      if (a.samples && t < a.T_cap)
        for (int j = 0; j < K; ++j) a.samples[(t * a.C + c) * K + j] = z[j];
    }
    for (int j = 0; j < K; ++j) {
      a.u[(int64_t)c * K + j] = z[j];
      a.grad[(int64_t)c * K + j] = g[j];
    }
    a.lj[c] = lj;
  }
}

__global__ void advance_kernel(edg_state_t* state, int n) { state->t += n; }

struct KlqpArgs {
  edg_expfam_t m;
  int S;
  uint64_t seed;
  edg_opt_t opt;
  float* mu;
  float* rho;
  float* slots;  // [4K]
  edg_state_t* state;
  const float* eps_ovr;  // [S, K]
  float* grad_out;       // [2K]
  int apply;
};

// One block of 256 threads; sample s is handled by thread s (S <= 256).  The
// per-sample terms are summed in a fixed order (warp shuffles, then the warps'
// partials in order), so the step is reproducible.
__global__ void __launch_bounds__(256) klqp_kernel(KlqpArgs a) {
  __shared__ double part[8][2 * kMaxK + 1];
  const int K = a.m.K, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t iter = (uint32_t)a.state->t;
  float g[kMaxK], e[kMaxK];
  double f = 0.0;
  for (int j = 0; j < K; ++j) g[j] = e[j] = 0.0f;
  if (tid < a.S) {
    float u[kMaxK];
    double lq = 0.0;
    for (int j = 0; j < K; ++j) {
      e[j] = a.eps_ovr ? a.eps_ovr[tid * K + j]
                       : philox_normal(a.seed, 0u, iter, (uint32_t)tid, (uint32_t)j);
      const float sg = softplus_f(a.rho[j]);
      u[j] = fmaf(sg, e[j], a.mu[j]);
      lq += (double)(-0.5f * e[j] * e[j] - logf(sg)) - kHalfLog2Pi;
    }
    f = log_joint_grad(a.m, u, g) - lq;
  }
  auto wsum = [&](double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
  };
  f = wsum(f);
  if (lane == 0) part[warp][2 * kMaxK] = f;
  for (int j = 0; j < K; ++j) {
    const double a1 = wsum((double)g[j]), a2 = wsum((double)(g[j] * e[j]));
    if (lane == 0) {
      part[warp][j] = a1;
      part[warp][kMaxK + j] = a2;
    }
  }
  __syncthreads();
  if (tid != 0) return;
  const double invS = 1.0 / a.S;
  const float lr = opt_lr(a.opt, a.state->global_step);
  const float b1p = a.state->beta1_power, b2p = a.state->beta2_power;
  double loss = 0.0;
  for (int w = 0; w < 8; ++w) loss += part[w][2 * kMaxK];
  for (int j = 0; j < K; ++j) {
    double s1 = 0.0, s2 = 0.0;
    for (int w = 0; w < 8; ++w) {
      s1 += part[w][j];
      s2 += part[w][kMaxK + j];
    }
    const float sg = softplus_f(a.rho[j]);
    const float gmu = (float)(-s1 * invS);
    const float grho = ((float)(-s2 * invS) - 1.0f / sg) * sigmoid_f(a.rho[j]);
    if (a.grad_out) {
      a.grad_out[j] = gmu;
      a.grad_out[K + j] = grho;
    }
    if (!isfinite(gmu) || !isfinite(grho)) a.state->nonfinite += 1;
    if (a.apply) {
      a.mu[j] = opt_apply(a.opt, a.mu[j], gmu, a.slots + j, a.slots + 2 * K + j, lr, b1p, b2p);
      a.rho[j] = opt_apply(a.opt, a.rho[j], grho, a.slots + K + j, a.slots + 3 * K + j, lr, b1p,
                           b2p);
    }
  }
  a.state->loss = -loss * invS;
  if (!isfinite(a.state->loss)) a.state->nonfinite += 1;
  if (a.apply) {
    a.state->t += 1;
    a.state->global_step += 1;
    a.state->beta1_power = b1p * a.opt.beta1;
    a.state->beta2_power = b2p * a.opt.beta2;
  }
}

static int check_model(const edg_expfam_t* m) {
  EDG_REQUIRE(m && m->prior && m->stats, EDG_E_NULL, "model pointers must not be NULL");
  EDG_REQUIRE(m->family == EDG_EXPFAM_BETA || m->family == EDG_EXPFAM_GAMMA ||
                  m->family == EDG_EXPFAM_DIRICHLET,
              EDG_E_VALUE, "unknown family %d", m->family);
  EDG_REQUIRE(m->family == EDG_EXPFAM_DIRICHLET ? (m->K >= 1 && m->K <= kMaxK) : m->K == 1,
              EDG_E_SHAPE, "unconstrained dimension %d not supported", m->K);
  EDG_REQUIRE(m->transform == 0 || m->transform == 1, EDG_E_VALUE, "transform must be 0 or 1");
  EDG_REQUIRE(m->transform || m->family != EDG_EXPFAM_DIRICHLET, EDG_E_UNSUPPORTED,
              "the Dirichlet latent is worked in the unconstrained space only");
  return EDG_OK;
}

}  // namespace ef
}  // namespace edg

using namespace edg;

extern "C" int edg_expfam_hmc_run(const edg_expfam_t* model, const edg_hmc_t* cfg, int32_t C,
                                  int32_t n_iter, float* u, float* grad, double* lj,
                                  int32_t cache_valid, int32_t* n_accept, edg_state_t* state,
                                  float* samples, int64_t T_cap, const float* r_override,
                                  const double* u_override, void* stream) {
  int rc = ef::check_model(model);
  if (rc) return rc;
  EDG_REQUIRE(model->transform == 1, EDG_E_UNSUPPORTED,
              "HMC samples the constrained latent in its unconstrained space (transform = 1)");
  EDG_REQUIRE(cfg && u && grad && lj && n_accept && state, EDG_E_NULL,
              "pointers must not be NULL");
  EDG_REQUIRE(C > 0 && n_iter >= 0 && cfg->n_steps >= 0, EDG_E_SHAPE, "invalid sizes");
  ef::HmcArgs a;
  a.m = *model;
  a.C = C;
  a.n_iter = n_iter;
  a.L = cfg->n_steps;
  a.cache_valid = cache_valid;
  a.eps = cfg->step_size;
  a.seed = cfg->seed;
  a.u = u;
  a.grad = grad;
  a.lj = lj;
  a.n_accept = n_accept;
  a.state = state;
  a.samples = samples;
  a.T_cap = T_cap;
  a.r_ovr = r_override;
  a.u_ovr = u_override;
  cudaStream_t st = (cudaStream_t)stream;
  ef::hmc_kernel<<<(C + 127) / 128, 128, 0, st>>>(a);
  if ((rc = check_launch("expfam hmc_kernel"))) return rc;
  ef::advance_kernel<<<1, 1, 0, st>>>(state, n_iter);
  return check_launch("expfam advance_kernel");
}

extern "C" int edg_expfam_klqp_step(const edg_expfam_t* model, int32_t n_samples,
                                    uint64_t seed, const edg_opt_t* opt, float* mu, float* rho,
                                    float* opt_slots, edg_state_t* state,
                                    const float* eps_override, float* grad_out, int32_t apply,
                                    void* stream) {
  int rc = ef::check_model(model);
  if (rc) return rc;
  EDG_REQUIRE(opt && mu && rho && state && (!apply || opt_slots), EDG_E_NULL,
              "pointers must not be NULL");
  EDG_REQUIRE(n_samples > 0 && n_samples <= 256, EDG_E_VALUE,
              "n_samples must be in [1, 256] for this family");
  ef::KlqpArgs a;
  a.m = *model;
  a.S = n_samples;
  a.seed = seed;
  a.opt = *opt;
  a.mu = mu;
  a.rho = rho;
  a.slots = opt_slots;
  a.state = state;
  a.eps_ovr = eps_override;
  a.grad_out = grad_out;
  a.apply = apply;
  ef::klqp_kernel<<<1, 256, 0, (cudaStream_t)stream>>>(a);
  return check_launch("expfam klqp_kernel");
}
