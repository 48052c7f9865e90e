// Bayesian neural network regression under KLqp (analytic KL), S weight
// samples batched: h1 = tanh(X W0 + b0), h2 = tanh(h1 W1 + b1),
// out = h2 W2 + b2, y ~ Normal(out, noise); q = N(mu, softplus(rho)) on every
// weight, prior N(0, prior_scale).
//
// The flat parameter layout W0 [D,H1], b0, W1 [H1,H2], b1, W2 [H2,1], b2 puts
// every bias right after its weight matrix, i.e. each layer is one [in+1, out]
// block.  Activations carry a trailing ones column, so one GEMM gives a
// layer's pre-activation and one transposed GEMM gives its weight *and* bias
// gradient, written straight into the per-sample gradient G[s].
//
// One step = one minibatch ELBO gradient + optimizer apply, as a fixed
// sequence of launches on one stream (graph-capturable):
//   sample   theta_s = mu + sigma * eps_s (Philox), eps kept for the rho gradient;
//            Xa = [X, 1] and the ones columns of H1a / H2a
//   F1, F2   H1a = tanh(Xa W0a), H2a = tanh(H1a W1a)    (batched over samples)
//   head     one pass over h2: out, residual, FP64 log-lik partials,
//            dout = scale (y - out) / noise^2, dH2 = dout w2 (1 - h2^2) in place
//            of h2 and per-block partials of [dW2; db2] = sum_m [h2; 1] dout
//   B1       [dW1; db1] = H1a^T dH2
//   B2       dH1 = (dH2 W1^T)(1 - h1^2)                (in place of h1)
//   B3       [dW0; db0] = Xa^T dH1
//   finalize sum over samples, KL, loss, gradients w.r.t. (mu, rho), optimizer
// Hidden activations exist only for the current minibatch (S x M), are
// recomputed every step and are overwritten by their adjoints.
#include <algorithm>

#include "edg_common.cuh"
#include "gemm_simt.cuh"
#include "gemm_tc.cuh"
#include "optim.cuh"

namespace edg {
namespace bnn {

constexpr int kT = 256;
using simt::bgemm;
using simt::EpiTanh;
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

// theta[s][p] = mu[p] + softplus(rho[p]) eps[s][p]; the rows of theta / eps are
// ps >= P floats apart (16-byte aligned rows for the tensor-core loads).
__global__ void sample_kernel(const float* __restrict__ mu, const float* __restrict__ rho, int P,
                              int ps, int S, uint64_t seed, const edg_state_t* state,
                              const float* __restrict__ eps_ovr, float* __restrict__ theta,
                              float* __restrict__ eps) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)S * P) return;
  const int s = (int)(i / P), p = (int)(i % P);
  const uint32_t iter = (uint32_t)state->t;
  const float e = eps_ovr ? eps_ovr[i] : philox_normal(seed, 0u, iter, (uint32_t)s, (uint32_t)p);
  eps[(int64_t)s * ps + p] = e;
  theta[(int64_t)s * ps + p] = mu[p] + softplusf(rho[p]) * e;
}

// ------------------------------------------------------------ activations
struct Act {
  int M, ldx, ld1, ld2;
  int ps;  // floats between the parameter rows of consecutive samples (theta, G)
};

__host__ __device__ inline Act make_act(const Layout& L, int M, int ps) {
  Act a;
  a.M = M;
  a.ps = ps;
  a.ldx = round_up(L.D + 1, 4);
  a.ld1 = round_up(L.H1 + 1, 4);
  a.ld2 = round_up(L.H2 + 1, 4);
  return a;
}

// Xa = [X, 1, 0...]; the ones column (and zero padding) of every row of H1a, H2a.
__global__ void prep_kernel(Layout L, Act a, int S, const float* __restrict__ X,
                            float* __restrict__ Xa, float* __restrict__ H1a,
                            float* __restrict__ H2a) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < (int64_t)a.M * a.ldx; i += nth) {
    const int m = (int)(i / a.ldx), d = (int)(i % a.ldx);
    Xa[i] = d < L.D ? X[(int64_t)m * L.D + d] : (d == L.D ? 1.0f : 0.0f);
  }
  const int p1 = a.ld1 - L.H1, p2 = a.ld2 - L.H2;
  for (int64_t i = tid; i < (int64_t)S * a.M * (p1 + p2); i += nth) {
    const int64_t r = i / (p1 + p2);
    const int c = (int)(i % (p1 + p2));
    if (c < p1) H1a[r * a.ld1 + L.H1 + c] = c == 0 ? 1.0f : 0.0f;
    else H2a[r * a.ld2 + L.H2 + (c - p1)] = c == p1 ? 1.0f : 0.0f;
  }
}

// ------------------------------------------------------------ output layer
constexpr int kHeadRows = 32;  // rows per block (4 per warp)

// One pass over a block of kHeadRows rows of sample s (grid (M / kHeadRows, S)):
// out = h2 . w2 + b2, residual, dout = scale * res / noise^2, then
// dH2 = dout w2 (1 - h2^2) written over h2, per-block partials of
// [dW2; db2] = sum_m [h2_m; 1] dout_m (wpart[blk][s][0..H2]) and of the
// unscaled FP64 log-likelihood (ll_part[s][blk]).  Requires H2 < 1024.
__global__ void __launch_bounds__(kT) head_adj_kernel(Layout L, Act a, const float* __restrict__ y,
                                                      const float* __restrict__ theta, float* H2a,
                                                      float* __restrict__ wpart,
                                                      double* __restrict__ ll_part, float noise,
                                                      float dscale) {
  extern __shared__ float s_part[];  // [kT / 32][H2 + 1]
  __shared__ double red[kT / 32];
  const int s = blockIdx.y, nblk = gridDim.x;
  const float* w2 = theta + (int64_t)s * a.ps + L.oW2;
  const float b2 = w2[L.H2];
  const float inv_var = 1.0f / (noise * noise);
  const float lnorm = logf(noise) + (float)kHalfLog2Pi;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* my = s_part + warp * (L.H2 + 1);
  for (int k = lane; k <= L.H2; k += 32) my[k] = 0.0f;
  double acc = 0.0;
  for (int i = warp; i < kHeadRows; i += kT / 32) {
    const int m = blockIdx.x * kHeadRows + i;
    if (m >= a.M) break;
    float* h = H2a + ((int64_t)s * a.M + m) * a.ld2;
    float v = 0.0f;
    for (int k = lane; k < L.H2; k += 32) v = fmaf(h[k], __ldg(w2 + k), v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const float res = y[m] - (v + b2);
    const float d = dscale * res * inv_var;
    if (lane == 0) {
      acc += (double)(-0.5f * res * res * inv_var - lnorm);
      my[L.H2] += d;
    }
    for (int k = lane; k < L.H2; k += 32) {
      const float hk = h[k];
      my[k] = fmaf(hk, d, my[k]);
      h[k] = d * __ldg(w2 + k) * (1.0f - hk * hk);
    }
  }
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; ++w) t += red[w];
    ll_part[(int64_t)s * nblk + blockIdx.x] = t;
  }
  float* out = wpart + ((int64_t)blockIdx.x * gridDim.y + s) * (L.H2 + 1);
  for (int k = threadIdx.x; k <= L.H2; k += kT) {
    float t = 0.0f;
    for (int w = 0; w < kT / 32; ++w) t += s_part[w * (L.H2 + 1) + k];
    out[k] = t;
  }
}

// ll[s] = scale * sum of the head partials of sample s.
__global__ void __launch_bounds__(kT) ll_reduce_kernel(const double* __restrict__ ll_part,
                                                       int nparts, float dscale,
                                                       double* __restrict__ ll) {
  __shared__ double red[kT / 32];
  const int s = blockIdx.x;
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += kT) acc += ll_part[(int64_t)s * nparts + i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; ++w) t += red[w];
    ll[s] = t * (double)dscale;
  }
}

// ------------------------------------------------------------ finalize
struct FinArgs {
  int P, S, ps;
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
      const float g = a.G[(int64_t)s * a.ps + p];
      sg_mu += g;
      sg_sig += g * a.eps[(int64_t)s * a.ps + p];
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
        const float e = a.eps[(int64_t)s * a.ps + p];
        const float z = a.theta[(int64_t)s * a.ps + p];
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
  float *theta, *eps, *G, *Xa, *H1, *H2, *wpart, *part;
  double *ll, *ll_part, *kl_part;
};

static int head_blocks(int M) { return (M + kHeadRows - 1) / kHeadRows; }

constexpr int kTcChunk = 1024;  // rows per K split of the weight-gradient GEMMs

static int param_stride(const Layout& L) { return round_up(L.P, 4); }

static size_t part_floats(const Layout& L, int S, int M, int engine) {
  if (engine != EDG_GEMM_TC) return 0;
  return std::max(tcg::part_floats(L.H1 + 1, L.H2, M, S, kTcChunk),
                  tcg::part_floats(L.D + 1, L.H1, M, S, kTcChunk));
}

static size_t carve(const Layout& L, int S, int M, int engine, void* base, Workspace* w) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  const int ps = param_stride(L);
  const Act a = make_act(L, M, ps);
  const size_t o_theta = take((size_t)S * ps * 4), o_eps = take((size_t)S * ps * 4);
  const size_t o_G = take((size_t)S * ps * 4);
  const size_t o_part = take(part_floats(L, S, M, engine) * 4);
  const size_t o_Xa = take((size_t)M * a.ldx * 4);
  const size_t o_H1 = take((size_t)S * M * a.ld1 * 4), o_H2 = take((size_t)S * M * a.ld2 * 4);
  const size_t o_wpart = take((size_t)head_blocks(M) * S * (L.H2 + 1) * 4);
  const size_t o_ll = take((size_t)S * 8), o_llp = take((size_t)S * head_blocks(M) * 8);
  const size_t o_kl = take((size_t)((L.P + kT - 1) / kT) * 8);
  if (w && base) {
    char* b = reinterpret_cast<char*>(base);
    w->theta = reinterpret_cast<float*>(b + o_theta);
    w->eps = reinterpret_cast<float*>(b + o_eps);
    w->G = reinterpret_cast<float*>(b + o_G);
    w->Xa = reinterpret_cast<float*>(b + o_Xa);
    w->H1 = reinterpret_cast<float*>(b + o_H1);
    w->H2 = reinterpret_cast<float*>(b + o_H2);
    w->wpart = reinterpret_cast<float*>(b + o_wpart);
    w->part = reinterpret_cast<float*>(b + o_part);
    w->ll = reinterpret_cast<double*>(b + o_ll);
    w->ll_part = reinterpret_cast<double*>(b + o_llp);
    w->kl_part = reinterpret_cast<double*>(b + o_kl);
  }
  return off;
}

// One GEMM on the selected engine: tcgen05 (3xTF32, reductions over the
// minibatch rows split into kTcChunk-row chunks) or SIMT FP32.
template <bool TA, bool TB, class Epi>
static int gemm_on(int engine, const float* A, const float* B, float* C, int M, int N, int K,
                   int lda, int ldb, int ldc, int64_t sA, int64_t sB, int64_t sC, int batch,
                   Epi epi, float* part, unsigned* err, cudaStream_t st) {
  if (engine == EDG_GEMM_TC && N >= 16)
    return tcg::gemm<TA, TB>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch, epi,
                             TA ? kTcChunk : 0, part, err, st);
  return bgemm<TA, TB>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch, epi, st);
}

// Per-sample scaled log-likelihood ll[s] (FP64) and its gradient G[s] w.r.t.
// theta[s] for S weight samples over one minibatch: the batched forward pass
// and the hand-written adjoint.  theta / G rows are ps floats apart.
static int loglik_grad(const Layout& L, int S, int M, int ps, int engine, const float* X,
                       const float* y, const float* theta, const Workspace& w, float* G,
                       double* ll, float noise, float dscale, unsigned* err, cudaStream_t st) {
  int rc;
  const Act a = make_act(L, M, ps);
  const int64_t s1 = (int64_t)M * a.ld1, s2 = (int64_t)M * a.ld2;
  prep_kernel<<<std::min<int64_t>(((int64_t)S * M + 255) / 256, 4096), 256, 0, st>>>(
      L, a, S, X, w.Xa, w.H1, w.H2);
  if ((rc = check_launch("bnn prep_kernel"))) return rc;
  // F1: H1a = tanh(Xa W0a)
  rc = gemm_on<false, false>(engine, w.Xa, theta + L.oW0, w.H1, M, L.H1, L.D + 1, a.ldx, L.H1,
                             a.ld1, 0, ps, s1, S, EpiTanh{}, w.part, err, st);
  if (rc) return rc;
  // F2: H2a = tanh(H1a W1a)
  rc = gemm_on<false, false>(engine, w.H1, theta + L.oW1, w.H2, M, L.H2, L.H1 + 1, a.ld1, L.H2,
                             a.ld2, s1, ps, s2, S, EpiTanh{}, w.part, err, st);
  if (rc) return rc;
  const int hb = head_blocks(M);
  head_adj_kernel<<<dim3(hb, S), kT, (kT / 32) * (L.H2 + 1) * sizeof(float), st>>>(
      L, a, y, theta, w.H2, w.wpart, w.ll_part, noise, dscale);
  if ((rc = check_launch("bnn head_adj_kernel"))) return rc;
  ll_reduce_kernel<<<S, kT, 0, st>>>(w.ll_part, hb, dscale, ll);
  if ((rc = check_launch("bnn ll_reduce_kernel"))) return rc;
  // [dW2; db2] = sum of the per-block partials
  if ((rc = tcg::sum_partials(w.wpart, hb, S, 1, L.H2 + 1, G + L.oW2, L.H2 + 1, ps, st)))
    return rc;
  // B1: [dW1; db1] = H1a^T dH2
  rc = gemm_on<true, false>(engine, w.H1, w.H2, G + L.oW1, L.H1 + 1, L.H2, M, a.ld1, a.ld2, L.H2,
                            s1, s2, ps, S, EpiIdentity{}, w.part, err, st);
  if (rc) return rc;
  // B2: dH1 = (dH2 W1^T)(1 - h1^2), in place of h1
  rc = gemm_on<false, true>(engine, w.H2, theta + L.oW1, w.H1, M, L.H1, L.H2, a.ld2, L.H2, a.ld1,
                            s2, ps, s1, S, EpiTanhGrad{w.H1, s1, a.ld1}, w.part, err, st);
  if (rc) return rc;
  // B3: [dW0; db0] = Xa^T dH1
  return gemm_on<true, false>(engine, w.Xa, w.H1, G + L.oW0, L.D + 1, L.H1, M, a.ldx, a.ld1, L.H1,
                              0, s1, ps, S, EpiIdentity{}, w.part, err, st);
}

static int check_cfg(const edg_bnn_t* c, int M) {
  EDG_REQUIRE(c, EDG_E_NULL, "cfg is NULL");
  EDG_REQUIRE(c->D > 0 && c->H1 > 0 && c->H2 > 0 && M > 0, EDG_E_SHAPE,
              "layer widths and M must be positive");
  EDG_REQUIRE(c->n_samples > 0, EDG_E_VALUE, "n_samples should be greater than zero: %d",
              c->n_samples);
  EDG_REQUIRE(c->noise > 0 && c->prior_scale > 0, EDG_E_VALUE,
              "noise and prior_scale must be positive");
  EDG_REQUIRE(c->gemm_engine == EDG_GEMM_TC || c->gemm_engine == EDG_GEMM_SIMT, EDG_E_VALUE,
              "unknown gemm_engine %d", c->gemm_engine);
  EDG_REQUIRE(c->method == EDG_KLQP_REPARAM_KL || c->method == EDG_KLQP_REPARAM, EDG_E_UNSUPPORTED,
              "method %d: the Bayesian NN step implements the reparameterisation gradient "
              "with analytic or Monte Carlo KL", c->method);
  const int64_t P = (int64_t)make_layout(c->D, c->H1, c->H2).P;
  EDG_REQUIRE(c->H2 < 1024, EDG_E_SHAPE, "the second hidden layer is limited to 1023 units");
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
  return carve(L, cfg->n_samples, M, cfg->gemm_engine, nullptr, nullptr);
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
  const size_t need = carve(L, S, M, cfg->gemm_engine, workspace, &w);
  EDG_REQUIRE(workspace && workspace_bytes >= need, EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  const int ps = param_stride(L);
  const int64_t SP = (int64_t)S * L.P;
  sample_kernel<<<(unsigned)((SP + 255) / 256), 256, 0, st>>>(mu, rho, L.P, ps, S, cfg->seed,
                                                               state, eps_override, w.theta, w.eps);
  if ((rc = check_launch("bnn sample_kernel"))) return rc;
  rc = loglik_grad(L, S, M, ps, cfg->gemm_engine, X, y, w.theta, w, w.G, w.ll, cfg->noise,
                   cfg->data_scale, &state->error, st);
  if (rc) return rc;
  FinArgs f;
  f.P = L.P;
  f.ps = ps;
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
  const size_t need = carve(L, cfg->n_samples, M, cfg->gemm_engine, workspace, &w);
  EDG_REQUIRE(workspace && workspace_bytes >= need, EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  // caller layout: theta / grad_out rows are P floats apart
  return loglik_grad(L, cfg->n_samples, M, L.P, cfg->gemm_engine, X, y, theta, w, grad_out,
                     ll_out, cfg->noise, cfg->data_scale, nullptr, (cudaStream_t)stream);
}
