// Bayesian neural network regression under KLqp (analytic KL), S weight
// samples batched: h1 = tanh(X W0 + b0), h2 = tanh(h1 W1 + b1),
// out = h2 W2 + b2, y ~ Normal(out, noise); q = N(mu, softplus(rho)) on every
// weight, prior N(0, prior_scale).
//
// One step = one minibatch ELBO gradient + optimizer apply, as a fixed
// sequence of launches on one stream (graph-capturable):
//   sample   theta_s = mu + sigma * eps_s (Philox), eps kept for the rho gradient
//   F1, F2   batched GEMMs with fused bias + tanh epilogues
//   head     out, residual, log-lik, dW2/db2 and dH2 = dout w2 (1 - h2^2) (in place of h2)
//   B1       dW1_s = h1_s^T dH2_s          (written straight into the per-sample gradient)
//   B2       dH1 = (dH2 W1^T)(1 - h1^2)    (in place of h1)
//   B3       dW0_s = X^T dH1_s
//   colsums  db1, db0
//   finalize sum over samples, KL, loss, gradients w.r.t. (mu, rho), optimizer
// Hidden activations exist only for the current minibatch (S x M), are
// recomputed every step and are overwritten by their adjoints.
#include <algorithm>

#include "edg_common.cuh"
#include "gemm_simt.cuh"
#include "optim.cuh"

namespace edg {
namespace bnn {

constexpr int kT = 256;
using simt::bgemm;
using simt::EpiBiasTanh;
using simt::EpiIdentity;
using simt::EpiTanhGrad;

// ------------------------------------------------------------ sampling
struct Layout {
  int D, H1, H2, P;
  int oW0, ob0, oW1, ob1, oW2, ob2;
};

__host__ __device__ inline Layout make_layout(int D, int H1, int H2) {
  Layout L;
  L.D = D;
  L.H1 = H1;
  L.H2 = H2;
  L.oW0 = 0;
  L.ob0 = D * H1;
  L.oW1 = L.ob0 + H1;
  L.ob1 = L.oW1 + H1 * H2;
  L.oW2 = L.ob1 + H2;
  L.ob2 = L.oW2 + H2;
  L.P = L.ob2 + 1;
  return L;
}

__global__ void sample_kernel(const float* __restrict__ mu, const float* __restrict__ rho, int P,
                              int S, uint64_t seed, const edg_state_t* state,
                              const float* __restrict__ eps_ovr, float* __restrict__ theta,
                              float* __restrict__ eps) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)S * P) return;
  const int s = (int)(i / P), p = (int)(i % P);
  const uint32_t iter = (uint32_t)state->t;
  const float e = eps_ovr ? eps_ovr[i] : philox_normal(seed, 0u, iter, (uint32_t)s, (uint32_t)p);
  eps[i] = e;
  theta[i] = mu[p] + softplusf(rho[p]) * e;
}

// ------------------------------------------------------------ output layer
// One block per sample: out, residual, FP64 log-lik, dW2, db2 and
// dH2 = dout * w2 * (1 - h2^2) written over h2.
__global__ void __launch_bounds__(kT) head_kernel(Layout L, int M, const float* __restrict__ y,
                                                  const float* __restrict__ theta, float* H2,
                                                  float* __restrict__ G, double* ll_out,
                                                  float noise, float dscale) {
  extern __shared__ __align__(16) float sm[];
  float* w2 = sm;             // [H2]
  float* dout = sm + L.H2;    // [M]
  __shared__ double red[kT / 32];
  const int s = blockIdx.x;
  const float* th = theta + (int64_t)s * L.P;
  float* Hs = H2 + (int64_t)s * M * L.H2;
  for (int k = threadIdx.x; k < L.H2; k += kT) w2[k] = th[L.oW2 + k];
  __syncthreads();
  const float b2 = th[L.ob2];
  const float inv_var = 1.0f / (noise * noise);
  const float lnorm = logf(noise) + (float)kHalfLog2Pi;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Kahan kl;
  for (int m = warp; m < M; m += kT / 32) {
    float v = 0.0f;
    for (int k = lane; k < L.H2; k += 32) v = fmaf(Hs[(int64_t)m * L.H2 + k], w2[k], v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const float res = y[m] - (v + b2);
    if (lane == 0) {
      dout[m] = dscale * res * inv_var;
      kl.add(-0.5f * res * res * inv_var - lnorm);
    }
  }
  double lls = lane == 0 ? kl.value() : 0.0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lls += __shfl_xor_sync(0xffffffffu, lls, o);
  if (lane == 0) red[warp] = lls;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; ++w) t += red[w];
    ll_out[s] = t * (double)dscale;
  }
  float* Gs = G + (int64_t)s * L.P;
  // dW2[k] = sum_m h2[m][k] dout[m]; then h2 <- dH2
  for (int k = threadIdx.x; k < L.H2; k += kT) {
    float a = 0.0f;
    for (int m = 0; m < M; ++m) a = fmaf(Hs[(int64_t)m * L.H2 + k], dout[m], a);
    Gs[L.oW2 + k] = a;
  }
  if (threadIdx.x == 0) {
    float a = 0.0f;
    for (int m = 0; m < M; ++m) a += dout[m];
    Gs[L.ob2] = a;
  }
  __syncthreads();
  for (int64_t e = threadIdx.x; e < (int64_t)M * L.H2; e += kT) {
    const int m = (int)(e / L.H2), k = (int)(e % L.H2);
    const float h = Hs[e];
    Hs[e] = dout[m] * w2[k] * (1.0f - h * h);
  }
}

// G[s][off + h] = sum_m Src[s][m][h]
__global__ void colsum_kernel(const float* __restrict__ Src, int M, int H, int P, int off,
                              float* __restrict__ G) {
  const int s = blockIdx.y;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= H) return;
  const float* p = Src + (int64_t)s * M * H + h;
  float a = 0.0f;
  for (int m = 0; m < M; ++m) a += p[(int64_t)m * H];
  G[(int64_t)s * P + off + h] = a;
}

// ------------------------------------------------------------ finalize
struct FinArgs {
  int P, S;
  float prior_scale;
  edg_opt_t opt;
  float* mu;
  float* rho;
  float* slots;
  edg_state_t* state;
  int method;  // EDG_KLQP_REPARAM_KL or EDG_KLQP_REPARAM
  const float* G;
  const float* eps;
  const float* theta;
  const double* ll;
  float* grad_out;
  int apply;
  double* kl_part;  // [gridDim.x]
};

__global__ void __launch_bounds__(kT) finalize_kernel(FinArgs a) {
  __shared__ double red[kT / 32];
  __shared__ bool s_last;
  const int p = blockIdx.x * kT + threadIdx.x;
  const float lr = opt_lr(a.opt, a.state->global_step);
  const float b1p = a.state->beta1_power, b2p = a.state->beta2_power;
  double kl = 0.0;
  if (p < a.P) {
    const float mu = a.mu[p], rho = a.rho[p];
    const float sg = softplusf(rho);
    float sg_mu = 0.0f, sg_sig = 0.0f;
    for (int s = 0; s < a.S; ++s) {
      const float g = a.G[(int64_t)s * a.P + p];
      sg_mu += g;
      sg_sig += g * a.eps[(int64_t)s * a.P + p];
    }
    const float invS = 1.0f / (float)a.S;
    const float ps = a.prior_scale;
    float gmu, gsig;
    if (a.method == EDG_KLQP_REPARAM_KL) {
      // analytic KL(N(mu, sg) || N(0, ps)) and its gradient
      gmu = -sg_mu * invS + mu / (ps * ps);
      gsig = -sg_sig * invS + (sg / (ps * ps) - 1.0f / sg);
      const float ratio = (sg / ps) * (sg / ps);
      kl = 0.5 * (double)(mu / ps) * (mu / ps) + 0.5 * ((double)ratio - 1.0 - (double)logf(ratio));
    } else {
      // Monte Carlo KL: mean_s [log q(z_s) - log p(z_s)], z_s = mu + sg eps_s, with the
      // gradient flowing through z_s and through q's own parameters
      float zz = 0.0f, zze = 0.0f;
      double lqp = 0.0;
      for (int s = 0; s < a.S; ++s) {
        const float e = a.eps[(int64_t)s * a.P + p];
        const float z = a.theta[(int64_t)s * a.P + p];
        zz += z;
        zze += z * e;
        lqp += 0.5 * ((double)(z / ps) * (z / ps) - (double)e * e);
      }
      const float ip2 = 1.0f / (ps * ps);
      gmu = -(sg_mu - zz * ip2) * invS;
      gsig = -(sg_sig - zze * ip2) * invS - 1.0f / sg;
      kl = lqp / a.S + (double)logf(ps) - (double)logf(sg);
    }
    const float grho = gsig * sigmoidf(rho);
    if (!isfinite(gmu) || !isfinite(grho)) atomicAdd(&a.state->nonfinite, 1u);
    if (a.grad_out) {
      a.grad_out[p] = gmu;
      a.grad_out[a.P + p] = grho;
    }
    if (a.apply) {
      const int n = 2 * a.P;
      a.mu[p] = opt_apply(a.opt, mu, gmu, a.slots + p, a.slots + n + p, lr, b1p, b2p);
      a.rho[p] = opt_apply(a.opt, rho, grho, a.slots + a.P + p, a.slots + n + a.P + p, lr, b1p,
                             b2p);
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) kl += __shfl_xor_sync(0xffffffffu, kl, o);
  if (lane == 0) red[warp] = kl;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; ++w) t += red[w];
    a.kl_part[blockIdx.x] = t;
    __threadfence();
    const unsigned prev = atomicAdd(&a.state->done, 1u);
    s_last = prev == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  double klsum = 0.0;
  for (int b = 0; b < (int)gridDim.x; ++b) klsum += __ldcg(a.kl_part + b);
  double llm = 0.0;
  for (int s = 0; s < a.S; ++s) llm += __ldcg(a.ll + s);
  llm /= a.S;
  const double loss = -(llm - klsum);
  a.state->loss = loss;
  a.state->aux[0] = llm;
  a.state->aux[1] = klsum;
  if (!isfinite(loss)) atomicAdd(&a.state->nonfinite, 1u);
  if (a.apply) {
    a.state->t += 1;
    a.state->global_step += 1;
    a.state->beta1_power = b1p * a.opt.beta1;
    a.state->beta2_power = b2p * a.opt.beta2;
  }
  a.state->done = 0;
  __threadfence();
}

// ------------------------------------------------------------ minibatch
__global__ void gather_kernel(const float* __restrict__ X, const float* __restrict__ y, int64_t N,
                              int D, int M, uint64_t seed, const edg_state_t* state,
                              float* __restrict__ Xb, float* __restrict__ yb) {
  const int m = blockIdx.x;
  if (m >= M) return;
  const uint32_t iter = (uint32_t)state->t;
  const uint32_t r = philox_at(seed, 4u, iter, (uint32_t)m, 0u).x;
  const int64_t row = (int64_t)(((uint64_t)r * (uint64_t)N) >> 32);  // uniform in [0, N)
  for (int d = threadIdx.x; d < D; d += blockDim.x) Xb[(int64_t)m * D + d] = X[row * D + d];
  if (threadIdx.x == 0) yb[m] = y[row];
}

struct Workspace {
  float *theta, *eps, *G, *H1, *H2;
  double *ll, *kl_part;
};

static size_t carve(const Layout& L, int S, int M, void* base, Workspace* w) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  const size_t o_theta = take((size_t)S * L.P * 4), o_eps = take((size_t)S * L.P * 4);
  const size_t o_G = take((size_t)S * L.P * 4);
  const size_t o_H1 = take((size_t)S * M * L.H1 * 4), o_H2 = take((size_t)S * M * L.H2 * 4);
  const size_t o_ll = take((size_t)S * 8), o_kl = take((size_t)((L.P + kT - 1) / kT) * 8);
  if (w && base) {
    char* b = reinterpret_cast<char*>(base);
    w->theta = reinterpret_cast<float*>(b + o_theta);
    w->eps = reinterpret_cast<float*>(b + o_eps);
    w->G = reinterpret_cast<float*>(b + o_G);
    w->H1 = reinterpret_cast<float*>(b + o_H1);
    w->H2 = reinterpret_cast<float*>(b + o_H2);
    w->ll = reinterpret_cast<double*>(b + o_ll);
    w->kl_part = reinterpret_cast<double*>(b + o_kl);
  }
  return off;
}

// Per-sample scaled log-likelihood ll[s] (FP64) and its gradient G[s] w.r.t.
// theta[s] for S weight samples over one minibatch: the batched forward pass
// and the hand-written adjoint.  H1 / H2 [S, M, H] hold the activations and
// are overwritten by their adjoints.
static int loglik_grad(const Layout& L, int S, int M, const float* X, const float* y,
                       const float* theta, float* H1, float* H2, float* G, double* ll,
                       float noise, float dscale, cudaStream_t st) {
  int rc;
  // F1: H1 = tanh(X W0 + b0)
  rc = bgemm<false, false>(X, theta + L.oW0, H1, M, L.H1, L.D, L.D, L.H1, L.H1, 0, L.P,
                           (int64_t)M * L.H1, S, EpiBiasTanh{theta + L.ob0, L.P}, st);
  if (rc) return rc;
  // F2: H2 = tanh(H1 W1 + b1)
  rc = bgemm<false, false>(H1, theta + L.oW1, H2, M, L.H2, L.H1, L.H1, L.H2, L.H2,
                           (int64_t)M * L.H1, L.P, (int64_t)M * L.H2, S,
                           EpiBiasTanh{theta + L.ob1, L.P}, st);
  if (rc) return rc;
  // head: out, ll, dW2, db2, dH2 (over H2)
  const size_t hsm = (size_t)(L.H2 + M) * 4;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  EDG_REQUIRE((int)hsm <= optin, EDG_E_UNSUPPORTED, "minibatch of %d rows too large", M);
  cudaFuncSetAttribute(head_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsm);
  head_kernel<<<S, kT, hsm, st>>>(L, M, y, theta, H2, G, ll, noise, dscale);
  if ((rc = check_launch("bnn head_kernel"))) return rc;
  // B1: dW1 = H1^T dH2  -> G[:, oW1]
  rc = bgemm<true, false>(H1, H2, G + L.oW1, L.H1, L.H2, M, L.H1, L.H2, L.H2,
                          (int64_t)M * L.H1, (int64_t)M * L.H2, L.P, S, EpiIdentity{}, st);
  if (rc) return rc;
  colsum_kernel<<<dim3((L.H2 + 127) / 128, S), 128, 0, st>>>(H2, M, L.H2, L.P, L.ob1, G);
  if ((rc = check_launch("bnn colsum"))) return rc;
  // B2: dH1 = (dH2 W1^T)(1 - h1^2), in place of H1
  rc = bgemm<false, true>(H2, theta + L.oW1, H1, M, L.H1, L.H2, L.H2, L.H2, L.H1,
                          (int64_t)M * L.H2, L.P, (int64_t)M * L.H1, S,
                          EpiTanhGrad{H1, (int64_t)M * L.H1, L.H1}, st);
  if (rc) return rc;
  // B3: dW0 = X^T dH1 -> G[:, oW0]
  rc = bgemm<true, false>(X, H1, G + L.oW0, L.D, L.H1, M, L.D, L.H1, L.H1, 0,
                          (int64_t)M * L.H1, L.P, S, EpiIdentity{}, st);
  if (rc) return rc;
  colsum_kernel<<<dim3((L.H1 + 127) / 128, S), 128, 0, st>>>(H1, M, L.H1, L.P, L.ob0, G);
  if ((rc = check_launch("bnn colsum"))) return rc;
  return EDG_OK;
}

static int check_cfg(const edg_bnn_t* c, int M) {
  EDG_REQUIRE(c, EDG_E_NULL, "cfg is NULL");
  EDG_REQUIRE(c->D > 0 && c->H1 > 0 && c->H2 > 0 && M > 0, EDG_E_SHAPE,
              "layer widths and M must be positive");
  EDG_REQUIRE(c->n_samples > 0, EDG_E_VALUE, "n_samples should be greater than zero: %d",
              c->n_samples);
  EDG_REQUIRE(c->noise > 0 && c->prior_scale > 0, EDG_E_VALUE,
              "noise and prior_scale must be positive");
  EDG_REQUIRE(c->method == EDG_KLQP_REPARAM_KL || c->method == EDG_KLQP_REPARAM, EDG_E_UNSUPPORTED,
              "method %d: the Bayesian NN step implements the reparameterisation gradient "
              "with analytic or Monte Carlo KL", c->method);
  const int64_t P = (int64_t)make_layout(c->D, c->H1, c->H2).P;
  EDG_REQUIRE(P * c->n_samples < (1ll << 31) && (int64_t)c->n_samples * M * c->H1 < (1ll << 40),
              EDG_E_SHAPE, "problem too large");
  return EDG_OK;
}

}  // namespace bnn
}  // namespace edg

using namespace edg;
using namespace edg::bnn;

extern "C" int32_t edg_bnn_num_params(int32_t D, int32_t H1, int32_t H2) {
  return make_layout(D, H1, H2).P;
}

extern "C" size_t edg_bnn_workspace_bytes(const edg_bnn_t* cfg, int32_t M) {
  if (check_cfg(cfg, M) != EDG_OK) return 0;
  const Layout L = make_layout(cfg->D, cfg->H1, cfg->H2);
  return carve(L, cfg->n_samples, M, nullptr, nullptr);
}

extern "C" int edg_minibatch_gather(const float* X, const float* y, int64_t N, int32_t D,
                                    int32_t M, uint64_t seed, const edg_state_t* state, float* Xb,
                                    float* yb, void* stream) {
  EDG_REQUIRE(X && y && state && Xb && yb, EDG_E_NULL, "pointers must not be NULL");
  EDG_REQUIRE(N > 0 && D > 0 && M > 0, EDG_E_SHAPE, "N, D and M must be positive");
  gather_kernel<<<M, 64, 0, (cudaStream_t)stream>>>(X, y, N, D, M, seed, state, Xb, yb);
  return check_launch("gather_kernel");
}

extern "C" int edg_bnn_klqp_step(const edg_bnn_t* cfg, const edg_opt_t* opt, const float* X,
                                 const float* y, int32_t M, float* mu, float* rho,
                                 float* opt_slots, edg_state_t* state, const float* eps_override,
                                 float* grad_out, int32_t apply, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  int rc = check_cfg(cfg, M);
  if (rc) return rc;
  EDG_REQUIRE(opt && X && y && mu && rho && state, EDG_E_NULL, "pointers must not be NULL");
  EDG_REQUIRE(!apply || opt_slots, EDG_E_NULL, "opt_slots must not be NULL when apply = 1");
  const Layout L = make_layout(cfg->D, cfg->H1, cfg->H2);
  const int S = cfg->n_samples;
  Workspace w;
  const size_t need = carve(L, S, M, workspace, &w);
  EDG_REQUIRE(workspace && workspace_bytes >= need, EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t SP = (int64_t)S * L.P;
  sample_kernel<<<(unsigned)((SP + 255) / 256), 256, 0, st>>>(mu, rho, L.P, S, cfg->seed, state,
                                                               eps_override, w.theta, w.eps);
  if ((rc = check_launch("bnn sample_kernel"))) return rc;
  rc = loglik_grad(L, S, M, X, y, w.theta, w.H1, w.H2, w.G, w.ll, cfg->noise, cfg->data_scale,
                   st);
  if (rc) return rc;
  FinArgs f;
  f.P = L.P;
  f.S = S;
  f.prior_scale = cfg->prior_scale;
  f.opt = *opt;
  f.mu = mu;
  f.rho = rho;
  f.slots = opt_slots;
  f.state = state;
  f.method = cfg->method;
  f.G = w.G;
  f.eps = w.eps;
  f.theta = w.theta;
  f.ll = w.ll;
  f.grad_out = grad_out;
  f.apply = apply;
  f.kl_part = w.kl_part;
  finalize_kernel<<<(L.P + kT - 1) / kT, kT, 0, st>>>(f);
  return check_launch("bnn finalize_kernel");
}

extern "C" int edg_bnn_loglik_grad(const edg_bnn_t* cfg, const float* X, const float* y,
                                   int32_t M, const float* theta, double* ll_out,
                                   float* grad_out, void* workspace, size_t workspace_bytes,
                                   void* stream) {
  int rc = check_cfg(cfg, M);
  if (rc) return rc;
  EDG_REQUIRE(X && y && theta && ll_out && grad_out, EDG_E_NULL, "pointers must not be NULL");
  const Layout L = make_layout(cfg->D, cfg->H1, cfg->H2);
  Workspace w;
  const size_t need = carve(L, cfg->n_samples, M, workspace, &w);
  EDG_REQUIRE(workspace && workspace_bytes >= need, EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  return loglik_grad(L, cfg->n_samples, M, X, y, theta, w.H1, w.H2, grad_out, ll_out, cfg->noise,
                     cfg->data_scale, (cudaStream_t)stream);
}
