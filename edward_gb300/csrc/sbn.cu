// Sigmoid belief network under the score-function gradient (ScoreKLqp),
// with an optional control variate for the learning signal.
//
// Model (two stochastic layers):  z1 ~ Bern(prior_logits)          [H1]
//                                 z0 ~ Bern(z1 Wp1 + bp1)          [H0]
//                                 x  ~ Bern(z0 Wp0 + bp0)          [V]
// Recognition network:            q(z0 | x)  = Bern(x Wq0 + bq0)
//                                 q(z1 | z0) = Bern(z0 Wq1 + bq1)
// Every weight matrix is stored with its bias as one block [in + 1, out]
// (the bias is the last row) and every activation carries a trailing ones
// column, so one GEMM gives a layer's logits and one transposed GEMM gives
// its weight *and* bias gradient.
//
// One step (B rows, S samples per row, R = S B sample rows):
//   prep      Xa = [x, 1]
//   Lq0       = Xa Wq0                                        [B, H0]
//   sample0   z0 ~ Bern(sigmoid(Lq0)) per sample (Philox stream 3);
//             log q(z0|x) per row; R0 = z0 - sigmoid(Lq0)
//   Lq1       = Z0a Wq1                                       [R, H1]
//   sample1   z1, log q(z1|z0), log p(z1); Lq1 <- z1 - sigmoid(Lq1)
//   Lp1       = Z1a Wp1;  rows: log p(z0|z1), Lp1 <- z0 - sigmoid(Lp1)
//   Lp0       = Z0a Wp0;  rows: log p(x|z0),  Lp0 <- x - sigmoid(Lp0)
//   [MLP baseline forward  b(x) = c + sigma * (tanh(Xc Wb0) Wb1), Xc = [2x - 1, 1]]
//   signal    f[s,b] = log p(x, z) - log q(z | x);  F_s = sum_b f[s,b]
//   scale     learning signal A: F_s (no baseline: the reference's
//             estimator, klqp.py:894-904) or f[s,b] - b(x_b) (per row);
//             Lq1 <- A * Lq1;  R0q[b] = sum_s A R0[s,b]
//   gradients gWq0 = Xa^T R0q, gWq1 = Z0a^T Lq1, gWp1 = Z1a^T Lp1,
//             gWp0 = Z0a^T Lp0 (split-K over the R sample rows)
//   finalize  grad = -G / S, optimizer apply, loss = -mean_s F_s
//   [baseline: MLP regression of the per-row signal + running statistics]
#include <algorithm>

#include "edg_common.cuh"
#include "gemm_simt.cuh"
#include "gemm_tc.cuh"
#include "optim.cuh"

namespace edg {
namespace sbn {

constexpr int kT = 256;
constexpr int kMaxSplits = 32;

struct Dims {
  int V, H0, H1, S, B, R, BH, mode, engine, rb;
  int ldx, ld0, ld1, ldh, H0p;
  int64_t oq0, oq1, op1, op0, P;  // model parameter blocks
  int64_t ob1, PB;                // baseline: Wb0 block at 0, Wb1 block at ob1
};

static Dims make_dims(const edg_sbn_t* c, int B) {
  Dims d;
  d.V = c->V;
  d.H0 = c->H0;
  d.H1 = c->H1;
  d.S = c->n_samples;
  d.B = B;
  d.R = c->n_samples * B;
  d.BH = c->baseline_hidden;
  d.mode = c->baseline;
  d.engine = c->gemm_engine;
  d.rb = c->rao_blackwell;
  d.ldx = round_up(d.V + 1, 4);
  d.ld0 = round_up(d.H0 + 1, 4);
  d.ld1 = round_up(d.H1 + 1, 4);
  d.ldh = round_up(d.BH + 1, 4);
  d.H0p = round_up(d.H0, 4);
  d.oq0 = 0;
  d.oq1 = d.oq0 + (int64_t)(d.V + 1) * d.H0;
  d.op1 = d.oq1 + (int64_t)(d.H0 + 1) * d.H1;
  d.op0 = d.op1 + (int64_t)(d.H1 + 1) * d.H0;
  d.P = d.op0 + (int64_t)(d.H0 + 1) * d.V;
  d.ob1 = (int64_t)(d.V + 1) * d.BH;
  d.PB = d.ob1 + d.BH + 1;
  return d;
}

// Baseline statistics (float[8]): running mean c, running scale sigma, number
// of updates, the baseline optimizer's beta1/beta2 powers, last regression loss.
enum { ST_C = 0, ST_SIGMA = 1, ST_COUNT = 2, ST_B1P = 3, ST_B2P = 4, ST_MSE = 5 };

__device__ __forceinline__ float bern_u(uint64_t seed, uint32_t iter, uint32_t row, uint32_t e) {
  const uint4 r = philox_at(seed, 3u, iter, row, e >> 2);
  const uint32_t w = (e & 3u) == 0 ? r.x : (e & 3u) == 1 ? r.y : (e & 3u) == 2 ? r.z : r.w;
  return u01f(w);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Xa[b] = [x_b, 1, 0...]; Xc[b] = [2 x_b - 1, 1, 0...] (the MLP baseline's
// centred input) when Xc != NULL.
__global__ void prep_x_kernel(Dims d, const float* __restrict__ X, float* __restrict__ Xa,
                              float* __restrict__ Xc) {
  const int b = blockIdx.x;
  for (int v = threadIdx.x; v < d.ldx; v += blockDim.x) {
    const float x = v < d.V ? X[(int64_t)b * d.V + v] : 0.0f;
    Xa[(int64_t)b * d.ldx + v] = v < d.V ? x : (v == d.V ? 1.0f : 0.0f);
    if (Xc) Xc[(int64_t)b * d.ldx + v] = v < d.V ? 2.0f * x - 1.0f : (v == d.V ? 1.0f : 0.0f);
  }
}

// z0 for every (sample, row): warp per sample row r = s B + b.
__global__ void sample0_kernel(Dims d, const float* __restrict__ Lq0, float* __restrict__ Z0a,
                               float* __restrict__ R0, float* __restrict__ lq0, uint64_t seed,
                               const edg_state_t* state, const float* __restrict__ z_ovr) {
  const int r = blockIdx.x * (kT / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (r >= d.R) return;
  const int b = r % d.B;
  const uint32_t iter = (uint32_t)state->t;
  float acc = 0.0f;
  for (int j = lane; j < d.H0; j += 32) {
    const float l = Lq0[(int64_t)b * d.H0 + j];
    const float p = sigmoidf(l);
    const float z = z_ovr ? z_ovr[(int64_t)r * d.H0 + j]
                          : (bern_u(seed, iter, (uint32_t)r, (uint32_t)j) < p ? 1.0f : 0.0f);
    Z0a[(int64_t)r * d.ld0 + j] = z;
    R0[(int64_t)r * d.H0 + j] = z - p;
    acc += z * l - softplusf(l);
  }
  for (int j = d.H0 + lane; j < d.ld0; j += 32) Z0a[(int64_t)r * d.ld0 + j] = j == d.H0 ? 1.0f : 0.0f;
  acc = warp_sum(acc);
  if (lane == 0) lq0[r] = acc;
}

// z1, log q(z1 | z0), log p(z1); Lq1 <- z1 - sigmoid(Lq1).
__global__ void sample1_kernel(Dims d, float* __restrict__ Lq1, float* __restrict__ Z1a,
                               const float* __restrict__ prior_logits, float* __restrict__ lq1,
                               float* __restrict__ lp1, uint64_t seed, const edg_state_t* state,
                               const float* __restrict__ z_ovr) {
  const int r = blockIdx.x * (kT / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (r >= d.R) return;
  const uint32_t iter = (uint32_t)state->t;
  float aq = 0.0f, ap = 0.0f;
  for (int j = lane; j < d.H1; j += 32) {
    const float l = Lq1[(int64_t)r * d.H1 + j];
    const float p = sigmoidf(l);
    const float z = z_ovr ? z_ovr[(int64_t)d.R * d.H0 + (int64_t)r * d.H1 + j]
                          : (bern_u(seed, iter, (uint32_t)r, (uint32_t)(d.H0p + j)) < p ? 1.0f : 0.0f);
    Z1a[(int64_t)r * d.ld1 + j] = z;
    Lq1[(int64_t)r * d.H1 + j] = z - p;
    aq += z * l - softplusf(l);
    const float pl = prior_logits[j];
    ap += z * pl - softplusf(pl);
  }
  for (int j = d.H1 + lane; j < d.ld1; j += 32) Z1a[(int64_t)r * d.ld1 + j] = j == d.H1 ? 1.0f : 0.0f;
  aq = warp_sum(aq);
  ap = warp_sum(ap);
  if (lane == 0) {
    lq1[r] = aq;
    lp1[r] = ap;
  }
}

// Row log-likelihood of Bernoulli targets T under logits L, and L <- T - sigmoid(L).
// The target row of sample row r is r (trow_mod = 0) or r % trow_mod.
__global__ void bern_rows_kernel(int R, int n, const float* __restrict__ T, int ldt, int trow_mod,
                                 float* __restrict__ L, int ldl, float* __restrict__ out) {
  const int r = blockIdx.x * (kT / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (r >= R) return;
  const int tr = trow_mod ? r % trow_mod : r;
  float acc = 0.0f;
  for (int j = lane; j < n; j += 32) {
    const float t = T[(int64_t)tr * ldt + j];
    const float l = L[(int64_t)r * ldl + j];
    acc += t * l - softplusf(l);
    L[(int64_t)r * ldl + j] = t - sigmoidf(l);
  }
  acc = warp_sum(acc);
  if (lane == 0) out[r] = acc;
}

// MLP baseline output o_b = Hb[b] . w1 + b1 (Hb = tanh(Xc Wb0)); sets Hb's ones column.
__global__ void mlp_out_kernel(Dims d, float* __restrict__ Hb, const float* __restrict__ bp,
                               float* __restrict__ out) {
  const int b = blockIdx.x * (kT / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (b >= d.B) return;
  const float* w1 = bp + d.ob1;
  float acc = 0.0f;
  for (int k = lane; k < d.BH; k += 32) acc = fmaf(Hb[(int64_t)b * d.ldh + k], w1[k], acc);
  acc = warp_sum(acc);
  if (lane == 0) {
    out[b] = acc + w1[d.BH];
    Hb[(int64_t)b * d.ldh + d.BH] = 1.0f;
  }
}

// f[s,b] = log p(z1) + log p(z0|z1) + log p(x|z0) - log q(z0|x) - log q(z1|z0);
// Fs[s] = sum_b f[s,b] and Fs[S + s] = sum_b log p(x_b | z0_sb).
__global__ void __launch_bounds__(kT) signal_kernel(Dims d, const float* __restrict__ terms,
                                                    float* __restrict__ f, double* __restrict__ Fs) {
  __shared__ double red[kT / 32];
  const int s = blockIdx.x;
  const float* lq0 = terms;
  const float* lq1 = terms + d.R;
  const float* lp1 = terms + 2 * (int64_t)d.R;
  const float* lp0 = terms + 3 * (int64_t)d.R;
  const float* lx = terms + 4 * (int64_t)d.R;
  __shared__ double redx[kT / 32];
  double acc = 0.0, accx = 0.0;
  for (int b = threadIdx.x; b < d.B; b += kT) {
    const int r = s * d.B + b;
    const float v = (lp1[r] + lp0[r] + lx[r]) - (lq0[r] + lq1[r]);
    f[r] = v;
    acc += v;
    accx += lx[r];
  }
  acc = warp_sum_d(acc);
  accx = warp_sum_d(accx);
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5] = acc;
    redx[threadIdx.x >> 5] = accx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0, tx = 0.0;
    for (int w = 0; w < kT / 32; ++w) {
      t += red[w];
      tx += redx[w];
    }
    Fs[s] = t;
    Fs[d.S + s] = tx;
  }
}

// Learning signal of sample row r for the parameters of q(z0 | x) (layer 0) or
// q(z1 | z0) (layer 1).  Rao-Blackwellised (ScoreRBKLqp, klqp.py:1110-1139): the
// signal of a q factor keeps the log densities in the Markov blanket of its
// latent layer -- everything for q(z0 | x), everything but log p(x | z0) for
// q(z1 | z0).
__device__ __forceinline__ float signal_of(const Dims& d, int r, const float* f, const double* Fs,
                                           const float* stats, const float* mlp_out, int layer) {
  const int s = r / d.B, b = r % d.B;
  if (d.mode == EDG_BASELINE_NONE)
    return (d.rb && layer == 1) ? (float)(Fs[s] - Fs[d.S + s]) : (float)Fs[s];
  if (stats[ST_COUNT] <= 0.0f) return f[r];
  const float base = d.mode == EDG_BASELINE_MEAN ? stats[ST_C]
                                                 : stats[ST_C] + stats[ST_SIGMA] * mlp_out[b];
  return f[r] - base;
}

// Lq1[r] *= A1(r);  R0q[b][j] = sum_s A0(s B + b) R0[s B + b][j];  A_out[r] = A0(r).
__global__ void scale_kernel(Dims d, const float* __restrict__ f, const double* __restrict__ Fs,
                             const float* __restrict__ stats, const float* __restrict__ mlp_out,
                             float* __restrict__ Lq1, const float* __restrict__ R0,
                             float* __restrict__ R0q, float* __restrict__ A_out) {
  const int64_t n1 = (int64_t)d.R * d.H1, n2 = (int64_t)d.B * d.H0;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < n1 + n2;
       i += (int64_t)gridDim.x * kT) {
    if (i < n1) {
      const int r = (int)(i / d.H1);
      Lq1[i] *= signal_of(d, r, f, Fs, stats, mlp_out, 1);
      if (A_out && i % d.H1 == 0) A_out[r] = signal_of(d, r, f, Fs, stats, mlp_out, 0);
    } else {
      const int64_t e = i - n1;
      const int b = (int)(e / d.H0), j = (int)(e % d.H0);
      float acc = 0.0f;
      for (int s = 0; s < d.S; ++s) {
        const int r = s * d.B + b;
        acc = fmaf(signal_of(d, r, f, Fs, stats, mlp_out, 0), R0[(int64_t)r * d.H0 + j], acc);
      }
      R0q[e] = acc;
    }
  }
}

// C[m][n] = sum_c part[c][m][n]
__global__ void splitk_reduce_kernel(const float* __restrict__ part, int splits, int M, int N,
                                     float* __restrict__ C, int ldc) {
  const int64_t MN = (int64_t)M * N;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < MN; i += (int64_t)gridDim.x * kT) {
    float acc = 0.0f;
    for (int c = 0; c < splits; ++c) acc += part[c * MN + i];
    C[(i / N) * ldc + i % N] = acc;
  }
}

// Number of K chunks for C = A^T B with K reduction rows: enough CTAs for the
// GPU, at least 256 rows per chunk, and a divisor of K.
static int choose_splits(int M, int N, int K, int sms) {
  const int tiles = ((M + simt::BM - 1) / simt::BM) * ((N + simt::BN - 1) / simt::BN);
  int want = std::max(1, std::min(kMaxSplits, (2 * sms + tiles - 1) / tiles));
  want = std::min(want, std::max(1, K / 256));
  for (int s = want; s > 1; --s)
    if (K % s == 0) return s;
  return 1;
}

constexpr int kTcChunk = 1024;  // rows per K split on the tensor cores

static bool use_tc(int engine, int N) { return engine == EDG_GEMM_TC && N >= 16; }

// C = A^T B with A [K, M] (lda), B [K, N] (ldb), reduced over the K rows: on the
// tensor cores in kTcChunk-row chunks, on the SIMT engine split-K for parallelism.
static int gemm_tn(int engine, const float* A, int lda, const float* Bm, int ldb, float* C,
                   int ldc, int M, int N, int K, float* part, int sms, unsigned* err,
                   cudaStream_t st) {
  if (use_tc(engine, N))
    return tcg::gemm<true, false>(A, Bm, C, M, N, K, lda, ldb, ldc, 0, 0, 0, 1,
                                  simt::EpiIdentity{}, kTcChunk, part, err, st);
  const int splits = choose_splits(M, N, K, sms);
  if (splits == 1)
    return simt::bgemm<true, false>(A, Bm, C, M, N, K, lda, ldb, ldc, 0, 0, 0, 1,
                                    simt::EpiIdentity{}, st);
  const int Kc = K / splits;
  int rc = simt::bgemm<true, false>(A, Bm, part, M, N, Kc, lda, ldb, N, (int64_t)Kc * lda,
                                    (int64_t)Kc * ldb, (int64_t)M * N, splits,
                                    simt::EpiIdentity{}, st);
  if (rc) return rc;
  const int64_t MN = (int64_t)M * N;
  const int grid = (int)std::min<int64_t>((MN + kT - 1) / kT, 4 * sms);
  splitk_reduce_kernel<<<grid, kT, 0, st>>>(part, splits, M, N, C, ldc);
  return check_launch("sbn splitk_reduce_kernel");
}

static size_t gemm_tn_part_floats(int engine, int M, int N, int K, int sms) {
  if (use_tc(engine, N)) return tcg::part_floats(M, N, K, 1, kTcChunk);
  const int s = choose_splits(M, N, K, sms);
  return s == 1 ? 0 : (size_t)s * M * N;
}

static int gemm_tn_launches(int engine, int M, int N, int K, int sms) {
  if (use_tc(engine, N)) return tcg::part_floats(M, N, K, 1, kTcChunk) ? 2 : 1;
  return choose_splits(M, N, K, sms) > 1 ? 2 : 1;
}

// C = A B (+ epilogue), A [M, K] (lda), B [K, N] (ldb).
template <class Epi>
static int gemm_nn(int engine, const float* A, int lda, const float* Bm, int ldb, float* C,
                   int ldc, int M, int N, int K, Epi epi, unsigned* err, cudaStream_t st) {
  if (use_tc(engine, N))
    return tcg::gemm<false, false>(A, Bm, C, M, N, K, lda, ldb, ldc, 0, 0, 0, 1, epi, 0, nullptr,
                                   err, st);
  return simt::bgemm<false, false>(A, Bm, C, M, N, K, lda, ldb, ldc, 0, 0, 0, 1, epi, st);
}

struct FinArgs {
  Dims d;
  edg_opt_t opt;
  float* theta;
  float* slots;
  edg_state_t* state;
  const float* G;
  const double* Fs;
  float* grad_out;
  int apply;
};

__global__ void __launch_bounds__(kT) finalize_kernel(FinArgs a) {
  __shared__ bool s_last;
  const int64_t p = blockIdx.x * (int64_t)kT + threadIdx.x;
  const float lr = opt_lr(a.opt, a.state->global_step);
  const float b1p = a.state->beta1_power, b2p = a.state->beta2_power;
  const int64_t P = a.d.P;
  if (p < P) {
    const float g = -a.G[p] / (float)a.d.S;
    if (!isfinite(g)) atomicAdd(&a.state->nonfinite, 1u);
    if (a.grad_out) a.grad_out[p] = g;
    if (a.apply) a.theta[p] = opt_apply(a.opt, a.theta[p], g, a.slots + p, a.slots + P + p, lr, b1p, b2p);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&a.state->done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  double F = 0.0;
  for (int s = 0; s < a.d.S; ++s) F += __ldcg(a.Fs + s);
  const double loss = -F / a.d.S;
  a.state->loss = loss;
  a.state->aux[0] = F / a.d.S / a.d.B;  // mean per-row ELBO sample
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

// Per row b: target t_b = (mean_s f[s,b] - c) / sigma of the baseline regression;
// dout_b = 2 (o_b - t_b) / B and dHb = dout_b w1 (1 - Hb^2) (MLP mode); per-block
// partial sums of fbar, fbar^2 and (o - t)^2.
__global__ void __launch_bounds__(kT) baseline_grad_kernel(Dims d, const float* __restrict__ f,
                                                           const float* __restrict__ stats,
                                                           const float* __restrict__ mlp_out,
                                                           const float* __restrict__ Hb,
                                                           const float* __restrict__ bp,
                                                           float* __restrict__ dout,
                                                           float* __restrict__ dHb,
                                                           double* __restrict__ part) {
  __shared__ double red[3][kT / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * (kT / 32) + warp;
  const bool mlp = d.mode == EDG_BASELINE_MLP;
  double s1 = 0.0, s2 = 0.0, se = 0.0;
  if (b < d.B) {
    double fb = 0.0;
    for (int s = lane; s < d.S; s += 32) fb += f[s * d.B + b];
    fb = warp_sum_d(fb) / d.S;
    s1 = fb;
    s2 = fb * fb;
    if (mlp) {
      const bool on = stats[ST_COUNT] > 0.0f;
      const float t = on ? (float)((fb - stats[ST_C]) / stats[ST_SIGMA]) : 0.0f;
      const float o = mlp_out[b];
      const float g = on ? 2.0f * (o - t) / (float)d.B : 0.0f;
      se = on ? (double)(o - t) * (o - t) : 0.0;
      const float* w1 = bp + d.ob1;
      for (int k = lane; k < d.BH; k += 32) {
        const float h = Hb[(int64_t)b * d.ldh + k];
        dHb[(int64_t)b * d.BH + k] = g * w1[k] * (1.0f - h * h);
      }
      if (lane == 0) dout[b] = g;
    }
  }
  if (lane == 0) {
    red[0][warp] = s1;
    red[1][warp] = s2;
    red[2][warp] = se;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; ++w) t += red[threadIdx.x][w];
    part[blockIdx.x * 3 + threadIdx.x] = t;
  }
}

struct BaseArgs {
  Dims d;
  edg_opt_t opt;
  float decay;
  float* bp;
  float* bslots;
  const float* GB;
  float* stats;
  const double* part;
  int nparts;
  unsigned* done;
};

// Optimizer apply on the MLP baseline (from its second update on), then the
// running statistics (last block).
__global__ void __launch_bounds__(kT) baseline_apply_kernel(BaseArgs a) {
  __shared__ bool s_last;
  const int64_t p = blockIdx.x * (int64_t)kT + threadIdx.x;
  const bool on = a.stats[ST_COUNT] > 0.0f && a.d.mode == EDG_BASELINE_MLP;
  if (on && p < a.d.PB) {
    const float lr = opt_lr(a.opt, (int64_t)a.stats[ST_COUNT] - 1);
    a.bp[p] = opt_apply(a.opt, a.bp[p], a.GB[p], a.bslots + p, a.bslots + a.d.PB + p, lr,
                        a.stats[ST_B1P], a.stats[ST_B2P]);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(a.done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  double s1 = 0.0, s2 = 0.0, se = 0.0;
  for (int i = 0; i < a.nparts; ++i) {
    s1 += __ldcg(a.part + 3 * i);
    s2 += __ldcg(a.part + 3 * i + 1);
    se += __ldcg(a.part + 3 * i + 2);
  }
  const double m = s1 / a.d.B;
  const double var = fmax(s2 / a.d.B - m * m, 0.0);
  float* st = a.stats;
  if (st[ST_COUNT] <= 0.0f) {
    st[ST_C] = (float)m;
    st[ST_SIGMA] = (float)sqrt(fmax(var, 1e-6));
  } else {
    const double c0 = st[ST_C], dc = a.decay;
    const double s2new = dc * (double)st[ST_SIGMA] * st[ST_SIGMA] +
                         (1.0 - dc) * (var + (m - c0) * (m - c0));
    st[ST_C] = (float)(dc * c0 + (1.0 - dc) * m);
    st[ST_SIGMA] = (float)sqrt(fmax(s2new, 1e-6));
    if (a.d.mode == EDG_BASELINE_MLP) {
      st[ST_MSE] = (float)(se / a.d.B);
      st[ST_B1P] *= a.opt.beta1;
      st[ST_B2P] *= a.opt.beta2;
    }
  }
  st[ST_COUNT] += 1.0f;
  *a.done = 0;
  __threadfence();
}

struct Workspace {
  float *Xa, *Xc, *Lq0, *Z0a, *Z1a, *R0, *Lq1, *Lp1, *Lp0, *R0q, *terms, *f, *Hb, *mlp_out, *dout, *dHb,
      *G, *GB, *part;
  double *Fs, *bpart;
  unsigned* counters;
};

static size_t carve(const Dims& d, int sms, void* base, Workspace* w) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  const int64_t R = d.R, B = d.B;
  const bool mlp = d.mode == EDG_BASELINE_MLP;
  size_t part = 0;
  part = std::max(part, gemm_tn_part_floats(d.engine, d.V + 1, d.H0, d.B, sms));
  part = std::max(part, gemm_tn_part_floats(d.engine, d.H0 + 1, d.H1, d.R, sms));
  part = std::max(part, gemm_tn_part_floats(d.engine, d.H1 + 1, d.H0, d.R, sms));
  part = std::max(part, gemm_tn_part_floats(d.engine, d.H0 + 1, d.V, d.R, sms));
  if (mlp) {
    part = std::max(part, gemm_tn_part_floats(d.engine, d.V + 1, d.BH, d.B, sms));
    part = std::max(part, gemm_tn_part_floats(d.engine, d.BH + 1, 1, d.B, sms));
  }
  const int nb = (d.B + kT / 32 - 1) / (kT / 32);
  const size_t o[] = {
      take(B * d.ldx * 4),   take(mlp ? B * d.ldx * 4 : 0), take(B * d.H0 * 4),
      take(R * d.ld0 * 4),   take(R * d.ld1 * 4),
      take(R * d.H0 * 4),    take(R * d.H1 * 4), take(R * d.H0 * 4),  take(R * d.V * 4),
      take(B * d.H0 * 4),    take(5 * R * 4),    take(R * 4),
      take(mlp ? B * d.ldh * 4 : 0), take(B * 4), take(B * 4), take(mlp ? B * d.BH * 4 : 0),
      take(d.P * 4),         take(mlp ? d.PB * 4 : 0), take(part * 4),
      take(2 * d.S * 8),         take((size_t)nb * 3 * 8), take(64)};
  if (w && base) {
    char* c = reinterpret_cast<char*>(base);
    float** fp[] = {&w->Xa, &w->Xc, &w->Lq0, &w->Z0a, &w->Z1a, &w->R0, &w->Lq1, &w->Lp1,
                    &w->Lp0, &w->R0q, &w->terms, &w->f, &w->Hb, &w->mlp_out, &w->dout, &w->dHb,
                    &w->G, &w->GB, &w->part};
    constexpr int nf = sizeof(fp) / sizeof(fp[0]);
    for (int i = 0; i < nf; ++i) *fp[i] = reinterpret_cast<float*>(c + o[i]);
    w->Fs = reinterpret_cast<double*>(c + o[nf]);
    w->bpart = reinterpret_cast<double*>(c + o[nf + 1]);
    w->counters = reinterpret_cast<unsigned*>(c + o[nf + 2]);
  }
  return off;
}

static int check_cfg(const edg_sbn_t* c, int B) {
  EDG_REQUIRE(c, EDG_E_NULL, "cfg is NULL");
  EDG_REQUIRE(c->V > 0 && c->H0 > 0 && c->H1 > 0 && B > 0, EDG_E_SHAPE,
              "layer widths and the number of rows must be positive");
  EDG_REQUIRE(c->n_samples > 0, EDG_E_VALUE, "n_samples should be greater than zero: %d",
              c->n_samples);
  EDG_REQUIRE(c->baseline == EDG_BASELINE_NONE || c->baseline == EDG_BASELINE_MEAN ||
                  c->baseline == EDG_BASELINE_MLP,
              EDG_E_VALUE, "unknown baseline %d", c->baseline);
  EDG_REQUIRE(c->baseline != EDG_BASELINE_MLP || c->baseline_hidden > 0, EDG_E_SHAPE,
              "the MLP baseline needs baseline_hidden > 0");
  EDG_REQUIRE(c->baseline_decay >= 0.0f && c->baseline_decay < 1.0f, EDG_E_VALUE,
              "baseline_decay must be in [0, 1)");
  EDG_REQUIRE(c->gemm_engine == EDG_GEMM_TC || c->gemm_engine == EDG_GEMM_SIMT, EDG_E_VALUE,
              "unknown gemm_engine %d", c->gemm_engine);
  EDG_REQUIRE(!c->rao_blackwell || c->baseline == EDG_BASELINE_NONE, EDG_E_UNSUPPORTED,
              "the Rao-Blackwellised estimator takes no baseline");
  EDG_REQUIRE((int64_t)c->n_samples * B * std::max(c->V, std::max(c->H0, c->H1)) < (1ll << 31),
              EDG_E_SHAPE, "problem too large");
  return EDG_OK;
}

static int num_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

}  // namespace sbn
}  // namespace edg

using namespace edg;
using namespace edg::sbn;

extern "C" int32_t edg_sbn_num_params(int32_t V, int32_t H0, int32_t H1) {
  edg_sbn_t c{};
  c.V = V;
  c.H0 = H0;
  c.H1 = H1;
  c.n_samples = 1;
  return (int32_t)make_dims(&c, 1).P;
}

extern "C" int32_t edg_sbn_baseline_num_params(int32_t V, int32_t BH) {
  edg_sbn_t c{};
  c.V = V;
  c.H0 = c.H1 = 1;
  c.n_samples = 1;
  c.baseline_hidden = BH;
  return (int32_t)make_dims(&c, 1).PB;
}

extern "C" int32_t edg_sbn_launches_per_step(const edg_sbn_t* cfg, int32_t B, int32_t apply) {
  if (check_cfg(cfg, B) != EDG_OK) return -1;
  const Dims d = make_dims(cfg, B);
  const int sms = num_sms();
  auto tn = [&](int M, int N, int K) { return gemm_tn_launches(d.engine, M, N, K, sms); };
  int n = 9 + 2 + 1;  // prep .. bern_rows(x), signal, scale
  if (d.mode == EDG_BASELINE_MLP) n += 2;
  n += tn(d.V + 1, d.H0, d.B) + tn(d.H0 + 1, d.H1, d.R) + tn(d.H1 + 1, d.H0, d.R) +
       tn(d.H0 + 1, d.V, d.R);
  n += 1;  // finalize
  if (apply && d.mode != EDG_BASELINE_NONE) {
    n += 2;
    if (d.mode == EDG_BASELINE_MLP) n += tn(d.V + 1, d.BH, d.B) + tn(d.BH + 1, 1, d.B);
  }
  return n;
}

extern "C" size_t edg_sbn_workspace_bytes(const edg_sbn_t* cfg, int32_t B) {
  if (check_cfg(cfg, B) != EDG_OK) return 0;
  return carve(make_dims(cfg, B), num_sms(), nullptr, nullptr);
}

extern "C" int edg_sbn_score_step(const edg_sbn_t* cfg, const edg_opt_t* opt,
                                  const edg_opt_t* baseline_opt, const float* X, int32_t B,
                                  const float* prior_logits, float* theta, float* opt_slots,
                                  edg_state_t* state, float* baseline_params,
                                  float* baseline_slots, float* baseline_stats,
                                  const float* z_override, float* grad_out, float* signal_out,
                                  int32_t apply, void* workspace, size_t workspace_bytes,
                                  void* stream) {
  int rc = check_cfg(cfg, B);
  if (rc) return rc;
  EDG_REQUIRE(opt && X && prior_logits && theta && state, EDG_E_NULL,
              "pointers must not be NULL");
  EDG_REQUIRE(!apply || opt_slots, EDG_E_NULL, "opt_slots must not be NULL when apply = 1");
  const Dims d = make_dims(cfg, B);
  const bool mlp = d.mode == EDG_BASELINE_MLP;
  EDG_REQUIRE(d.mode == EDG_BASELINE_NONE || baseline_stats, EDG_E_NULL,
              "baseline_stats must not be NULL with a baseline");
  EDG_REQUIRE(!mlp || (baseline_params && baseline_opt && (!apply || baseline_slots)),
              EDG_E_NULL, "the MLP baseline needs its parameters, slots and optimizer");
  const int sms = num_sms();
  Workspace w;
  const size_t need = carve(d, sms, workspace, &w);
  EDG_REQUIRE(workspace && workspace_bytes >= need, EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  unsigned* err = &state->error;
  const int rows_grid = (d.R + kT / 32 - 1) / (kT / 32);
  const int b_grid = (d.B + kT / 32 - 1) / (kT / 32);
  float* lq0 = w.terms;
  float* lq1 = w.terms + d.R;
  float* lp1 = w.terms + 2 * (int64_t)d.R;
  float* lp0 = w.terms + 3 * (int64_t)d.R;
  float* lx = w.terms + 4 * (int64_t)d.R;
  cudaMemsetAsync(w.counters, 0, 64, st);

  prep_x_kernel<<<d.B, 256, 0, st>>>(d, X, w.Xa, mlp ? w.Xc : nullptr);
  if ((rc = check_launch("sbn prep_x_kernel"))) return rc;
  // q(z0 | x) logits, shared by all samples
  rc = gemm_nn(d.engine, w.Xa, d.ldx, theta + d.oq0, d.H0, w.Lq0, d.H0, d.B, d.H0, d.V + 1,
               simt::EpiIdentity{}, err, st);
  if (rc) return rc;
  sample0_kernel<<<rows_grid, kT, 0, st>>>(d, w.Lq0, w.Z0a, w.R0, lq0, cfg->seed, state,
                                           z_override);
  if ((rc = check_launch("sbn sample0_kernel"))) return rc;
  rc = gemm_nn(d.engine, w.Z0a, d.ld0, theta + d.oq1, d.H1, w.Lq1, d.H1, d.R, d.H1, d.H0 + 1,
               simt::EpiIdentity{}, err, st);
  if (rc) return rc;
  sample1_kernel<<<rows_grid, kT, 0, st>>>(d, w.Lq1, w.Z1a, prior_logits, lq1, lp1, cfg->seed,
                                           state, z_override);
  if ((rc = check_launch("sbn sample1_kernel"))) return rc;
  // p(z0 | z1)
  rc = gemm_nn(d.engine, w.Z1a, d.ld1, theta + d.op1, d.H0, w.Lp1, d.H0, d.R, d.H0, d.H1 + 1,
               simt::EpiIdentity{}, err, st);
  if (rc) return rc;
  bern_rows_kernel<<<rows_grid, kT, 0, st>>>(d.R, d.H0, w.Z0a, d.ld0, 0, w.Lp1, d.H0, lp0);
  if ((rc = check_launch("sbn bern_rows_kernel"))) return rc;
  // p(x | z0)
  rc = gemm_nn(d.engine, w.Z0a, d.ld0, theta + d.op0, d.V, w.Lp0, d.V, d.R, d.V, d.H0 + 1,
               simt::EpiIdentity{}, err, st);
  if (rc) return rc;
  bern_rows_kernel<<<rows_grid, kT, 0, st>>>(d.R, d.V, w.Xa, d.ldx, d.B, w.Lp0, d.V, lx);
  if ((rc = check_launch("sbn bern_rows_kernel"))) return rc;
  // MLP baseline forward (uses parameters from earlier steps only)
  if (mlp) {
    rc = gemm_nn(d.engine, w.Xc, d.ldx, baseline_params, d.BH, w.Hb, d.ldh, d.B, d.BH, d.V + 1,
                 simt::EpiTanh{}, err, st);
    if (rc) return rc;
    mlp_out_kernel<<<b_grid, kT, 0, st>>>(d, w.Hb, baseline_params, w.mlp_out);
    if ((rc = check_launch("sbn mlp_out_kernel"))) return rc;
  }
  signal_kernel<<<d.S, kT, 0, st>>>(d, w.terms, w.f, w.Fs);
  if ((rc = check_launch("sbn signal_kernel"))) return rc;
  {
    const int64_t n = (int64_t)d.R * d.H1 + (int64_t)d.B * d.H0;
    const int grid = (int)std::min<int64_t>((n + kT - 1) / kT, 8 * sms);
    scale_kernel<<<grid, kT, 0, st>>>(d, w.f, w.Fs, baseline_stats, w.mlp_out, w.Lq1, w.R0, w.R0q,
                                      signal_out ? signal_out + d.R : nullptr);
    if ((rc = check_launch("sbn scale_kernel"))) return rc;
  }
  if (signal_out) {
    cudaMemcpyAsync(signal_out, w.f, (size_t)d.R * 4, cudaMemcpyDeviceToDevice, st);
  }
  // gradients (weight and bias blocks at once)
  const int e = d.engine;
  if ((rc = gemm_tn(e, w.Xa, d.ldx, w.R0q, d.H0, w.G + d.oq0, d.H0, d.V + 1, d.H0, d.B, w.part,
                    sms, err, st)))
    return rc;
  if ((rc = gemm_tn(e, w.Z0a, d.ld0, w.Lq1, d.H1, w.G + d.oq1, d.H1, d.H0 + 1, d.H1, d.R, w.part,
                    sms, err, st)))
    return rc;
  if ((rc = gemm_tn(e, w.Z1a, d.ld1, w.Lp1, d.H0, w.G + d.op1, d.H0, d.H1 + 1, d.H0, d.R, w.part,
                    sms, err, st)))
    return rc;
  if ((rc = gemm_tn(e, w.Z0a, d.ld0, w.Lp0, d.V, w.G + d.op0, d.V, d.H0 + 1, d.V, d.R, w.part, sms,
                    err, st)))
    return rc;
  FinArgs f;
  f.d = d;
  f.opt = *opt;
  f.theta = theta;
  f.slots = opt_slots;
  f.state = state;
  f.G = w.G;
  f.Fs = w.Fs;
  f.grad_out = grad_out;
  f.apply = apply;
  finalize_kernel<<<(unsigned)((d.P + kT - 1) / kT), kT, 0, st>>>(f);
  if ((rc = check_launch("sbn finalize_kernel"))) return rc;
  if (apply && d.mode != EDG_BASELINE_NONE) {
    baseline_grad_kernel<<<b_grid, kT, 0, st>>>(d, w.f, baseline_stats, w.mlp_out, w.Hb,
                                                baseline_params, w.dout, w.dHb, w.bpart);
    if ((rc = check_launch("sbn baseline_grad_kernel"))) return rc;
    if (mlp) {
      if ((rc = gemm_tn(e, w.Xc, d.ldx, w.dHb, d.BH, w.GB, d.BH, d.V + 1, d.BH, d.B, w.part, sms,
                        err, st)))
        return rc;
      if ((rc = gemm_tn(e, w.Hb, d.ldh, w.dout, 1, w.GB + d.ob1, 1, d.BH + 1, 1, d.B, w.part, sms,
                        err, st)))
        return rc;
    }
    BaseArgs ba;
    ba.d = d;
    if (mlp) ba.opt = *baseline_opt;
    else ba.opt = *opt;
    ba.decay = cfg->baseline_decay;
    ba.bp = baseline_params;
    ba.bslots = baseline_slots;
    ba.GB = w.GB;
    ba.stats = baseline_stats;
    ba.part = w.bpart;
    ba.nparts = b_grid;
    ba.done = w.counters;
    const int grid = mlp ? (int)((d.PB + kT - 1) / kT) : 1;
    baseline_apply_kernel<<<grid, kT, 0, st>>>(ba);
    if ((rc = check_launch("sbn baseline_apply_kernel"))) return rc;
  }
  return EDG_OK;
}

namespace edg {
namespace sbn {
// Row m of the minibatch is row (u * N) >> 32 of X, u the first word of
// Philox stream 4 at counter (0, m, iteration, 4); bytes widen to floats.
__global__ void gather_u8_kernel(const uint8_t* __restrict__ X, int64_t N, int V, int B,
                                 uint64_t seed, const edg_state_t* state, float* __restrict__ Xb) {
  const int m = blockIdx.x;
  const uint32_t u = philox_at(seed, 4u, (uint32_t)state->t, (uint32_t)m, 0u).x;
  const int64_t row = (int64_t)(((uint64_t)u * (uint64_t)N) >> 32);
  for (int v = threadIdx.x; v < V; v += blockDim.x)
    Xb[(int64_t)m * V + v] = (float)X[row * V + v];
}
}  // namespace sbn
}  // namespace edg

extern "C" int edg_minibatch_gather_u8(const uint8_t* X, int64_t N, int32_t V, int32_t B,
                                       uint64_t seed, const edg_state_t* state, float* Xb,
                                       void* stream) {
  EDG_REQUIRE(X && state && Xb, EDG_E_NULL, "pointers must not be NULL");
  EDG_REQUIRE(N > 0 && V > 0 && B > 0, EDG_E_SHAPE, "N, V and B must be positive");
  gather_u8_kernel<<<B, 256, 0, (cudaStream_t)stream>>>(X, N, V, B, seed, state, Xb);
  return check_launch("gather_u8_kernel");
}
