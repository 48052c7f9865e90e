/*
 * edward_gb300 -- C ABI of the GB300 (sm_103a) inference hot path.
 *
 * The reference (blei-lab/edward 1.3.5) has no native code: its hot path is
 * Python building TensorFlow 1.x graphs.  Each entry point below replaces one
 * piece of that graph, cited as path:line inside the reference tree.
 *
 * Conventions
 *  - Every pointer argument is DEVICE memory owned by the caller, except the
 *    descriptor structs themselves (edg_glm_t, edg_klqp_t, ...), which are
 *    host structs read during the call.
 *  - `stream` is a cudaStream_t passed as void*; every call is stream-ordered
 *    and never synchronises the host.
 *  - Return value: EDG_OK (0) or a negative EDG_E_* code;
 *    edg_last_error_string() gives the detail (thread-local).
 *  - Entry points that need scratch take (workspace, workspace_bytes); the
 *    matching *_workspace_bytes() query gives the size.
 *  - State that advances between calls (iteration t, optimizer step,
 *    Adam beta powers) lives in a caller-allocated device edg_state_t so
 *    that repeated calls can be captured in a CUDA graph.
 */
#ifndef EDWARD_GB300_H_
#define EDWARD_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EDG_ABI_VERSION 1

enum {
  EDG_OK = 0,
  EDG_E_NULL = -1,        /* required pointer is NULL */
  EDG_E_SHAPE = -2,       /* bad size / dimension */
  EDG_E_VALUE = -3,       /* bad scalar argument (e.g. n_samples <= 0) */
  EDG_E_CUDA = -4,        /* CUDA launch / runtime failure */
  EDG_E_NONFINITE = -5,   /* non-finite value detected (debug mode) */
  EDG_E_TIMEOUT = -6,     /* a bounded device-side wait gave up */
  EDG_E_UNSUPPORTED = -7, /* configuration not supported by the kernels */
  EDG_E_WORKSPACE = -8    /* workspace too small */
};

/* Likelihood of the GLM family. */
enum { EDG_LIK_BERNOULLI = 0, EDG_LIK_NORMAL = 1 };

/* KLqp estimator (klqp.py builders). */
enum {
  EDG_KLQP_REPARAM_KL = 0, /* build_reparam_kl_loss_and_gradients, klqp.py:707-769 */
  EDG_KLQP_REPARAM = 1,    /* build_reparam_loss_and_gradients,    klqp.py:642-704 */
  EDG_KLQP_SCORE = 2       /* build_score_loss_and_gradients,      klqp.py:840-906 */
};

/* Optimizers accepted by VariationalInference.initialize
 * (edward/inferences/variational_inference.py:95-116). */
enum {
  EDG_OPT_ADAM = 0,
  EDG_OPT_SGD = 1,      /* 'gradientdescent' */
  EDG_OPT_MOMENTUM = 2, /* momentum 0.9 */
  EDG_OPT_ADAGRAD = 3,
  EDG_OPT_RMSPROP = 4,
  EDG_OPT_ADADELTA = 5
};

/* Generalised linear model: y_n ~ Lik(eta_n), eta = X z[:D] (+ z[D] if bias),
 * z_p ~ Normal(prior_loc[p], prior_scale[p]), P = D + bias.
 * Covers ed.dot regressions (edward/util/tensorflow.py:10-47;
 * tests/inferences/hmc_test.py:48-91) and the Normal-Normal model
 * (tests/inferences/klqp_test.py:14-44 with X = ones(N, 1)). */
typedef struct {
  const float* X;           /* [N, D] row-major */
  const float* y;           /* [N] (0/1 for Bernoulli) */
  int32_t N;
  int32_t D;
  int32_t bias;             /* 1: last coordinate of z is an intercept */
  int32_t lik;              /* EDG_LIK_* */
  float lik_scale;          /* Normal likelihood scale */
  const float* prior_loc;   /* [P] */
  const float* prior_scale; /* [P] */
} edg_glm_t;

/* Device-resident iteration state.  Zero-initialise, then set
 * beta1_power/beta2_power to beta1/beta2 (TF's Adam accumulators). */
typedef struct {
  int64_t t;             /* Inference.t (inference.py:195-197) */
  int64_t global_step;   /* optimizer global step (lr schedule) */
  float beta1_power;
  float beta2_power;
  uint32_t done;         /* internal completion counter; 0 between calls */
  uint32_t nonfinite;    /* non-finite loss/gradient values seen */
  uint32_t error;        /* EDG_E_* of a kernel that gave up a bounded wait (0 = none) */
  uint32_t reserved;      /* work counter of persistent launches; 0 between calls */
  double loss;           /* loss of the last KLqp update */
  double aux[3];         /* estimator-specific diagnostics */
} edg_state_t;

/* Optimizer + learning-rate schedule.  lr = lr0 * decay_rate^(step/decay_steps)
 * (floored if staircase) when decay_steps > 0, else lr0.  The Edward default
 * (optimizer=None) is Adam with lr0=0.1, decay_steps=100, decay_rate=0.9,
 * staircase=1 (variational_inference.py:83-97). */
typedef struct {
  int32_t optimizer;   /* EDG_OPT_* */
  float lr0;
  int64_t decay_steps;
  float decay_rate;
  int32_t staircase;
  float beta1, beta2, epsilon; /* Adam */
  float momentum;              /* momentum / rmsprop momentum */
  float rho;                   /* rmsprop decay / adadelta rho */
} edg_opt_t;

/* KLqp configuration (KLqp.initialize, klqp.py:86-113). */
typedef struct {
  int32_t method;            /* EDG_KLQP_* */
  int32_t n_samples;         /* > 0 */
  float data_scale;          /* Inference.scale[x] (inference.py:215-220) */
  const float* kl_scaling;   /* [P] or NULL (= 1) */
  const float* latent_scale; /* [P] or NULL (= 1): Inference.scale[z] */
  uint64_t seed;
  const int32_t* point;      /* [P] or NULL: 1 marks a model parameter (a trainable variable
                                of the model, not a latent: no prior and no q; z = mu and its
                                gradient is the pathwise gradient of the loss, as the
                                reference's p_vars get, klqp.py:902-904); rho is left as is */
} edg_klqp_t;

/* HMC configuration (HMC.initialize, edward/inferences/hmc.py:45-59). */
typedef struct {
  float step_size;
  int32_t n_steps;
  uint64_t seed;
  int32_t chains_per_block; /* SIMT engine: 0 = library default; else 8, 16 or 32.
                               hierarchical engine: the tile shape, 32 (or 0) = 32 chains x
                               64 rows, 16 = 16 chains x 128 rows */
  int32_t cluster_size;     /* tensor-core engine: CTAs per 128 chains (1,2,4,8); 0 = auto */
  int32_t launch;           /* hierarchical engine: 0 = persistent grid of resident CTAs taking
                               (instance, chain tile) items from a work counter, 1 = one CTA
                               per item */
} edg_hmc_t;

/* ---------------------------------------------------------------- library */
int edg_abi_version(void);
const char* edg_last_error_string(void);
/* SM count and compute capability of the current device. */
int edg_device_info(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor);

/* ---------------------------------------------------------------- RNG
 * Philox4x32-10 streams that replace tf.random_normal / tf.random_uniform
 * (hmc.py:88-91,108) and the reparameterised draw in copy(qz)
 * (klqp.py:727-731).  Counter = (element/4, row, iteration, kind). */
int edg_philox_u32(uint64_t seed, uint32_t kind, uint32_t iteration, int32_t rows,
                   int32_t n, uint32_t* out /* [rows, round_up(n,4)] */, void* stream);
int edg_philox_normal(uint64_t seed, uint32_t kind, uint32_t iteration, int32_t rows,
                      int32_t n, float* out /* [rows, n] */, void* stream);
int edg_philox_uniform64(uint64_t seed, uint32_t kind, uint32_t iteration, int32_t rows,
                         double* out /* [rows] */, void* stream);

/* ---------------------------------------------------------------- GLM log joint
 * Batched log joint and its adjoint for B parameter vectors Z [B, P]:
 *   lp[b]   = data_scale * sum_n log p(y_n | eta_nb)  (+ log prior if include_prior)
 *   grad[b] = d lp[b] / d z_b
 * Replaces the per-sample `x_copy.log_prob` + tf.gradients of
 * klqp.py:682-686,702 and hmc.py:161-192,199,206 (ed.dot:
 * edward/util/tensorflow.py:41-47). */
size_t edg_glm_logjoint_grad_workspace_bytes(const edg_glm_t* model, int32_t B);
int edg_glm_logjoint_grad(const edg_glm_t* model, const float* Z, int32_t B,
                          int32_t include_prior, float data_scale,
                          double* lp_out /* [B] or NULL */, float* grad_out /* [B,P] or NULL */,
                          void* workspace, size_t workspace_bytes, void* stream);

/* Same results as edg_glm_logjoint_grad, but this entry point allocates
 * nothing and takes no workspace.  It has no counterpart in the reference.
 * It is for callers that cannot allocate device memory at call time: host
 * frameworks that reserve all device memory in their own pool up front (an
 * extra cudaMalloc would fail or fragment it), and integrations that must
 * stay within a fixed memory budget fixed when they were loaded.
 *  - Scratch: a fixed 8 MiB array compiled into the library (a file-scope
 *    __device__ array).  Every GPU that loads the library holds it until the
 *    process exits.  Calls whose partial sums need more than 8 MiB fail with
 *    EDG_E_WORKSPACE; split B into smaller batches (e.g. 4096 vectors of
 *    P = 51 over 10,000 rows need 1.8 MB).
 *  - The first call on each device looks up the array's device address
 *    (cudaGetSymbolAddress) and caches it; make that first call before any
 *    stream capture.  The cached address belongs to the device's current
 *    primary context: after cudaDeviceReset (or anything else that destroys
 *    that context) the process must not call this entry point again.
 *  - Every call on a device uses the same array, so calls that overlap on the
 *    GPU (different streams, or threads without ordering) race and corrupt
 *    each other's results; serialise them on one stream.  Nothing needs to be
 *    cleared between calls: each call writes every scratch byte it reads. */
int edg_glm_logjoint_grad_noalloc(const edg_glm_t* model, const float* Z, int32_t B,
                                  int32_t include_prior, float data_scale,
                                  double* lp_out /* [B] or NULL */,
                                  float* grad_out /* [B,P] or NULL */, void* stream);

/* ---------------------------------------------------------------- KLqp
 * One fused ELBO-gradient step for a mean-field Normal q = N(mu, softplus(rho))
 * over a GLM: Philox eps -> z_s -> log-lik + adjoint over X for all samples
 * -> KL / log q terms -> chain rule to (mu, rho) -> optimizer apply.
 * Replaces build_*_loss_and_gradients (klqp.py:642-906) plus
 * VariationalInference.update (variational_inference.py:133-164).
 * opt_slots: [4 * P] floats (two slots of 2P: Adam m and v, etc.), zeroed at
 * start (adagrad/rmsprop initial accumulators are set by the caller).
 * eps_override: [n_samples, P] or NULL (NULL = Philox stream KIND 0 at
 * iteration state->t).  grad_out: [2P] = (dloss/dmu, dloss/drho) or NULL.
 * apply = 0 computes loss/gradients without touching mu/rho/slots/state.
 * The loss (pre-update) is written to state->loss. */
size_t edg_klqp_glm_workspace_bytes(const edg_glm_t* model, const edg_klqp_t* cfg);
int edg_klqp_glm_step(const edg_glm_t* model, const edg_klqp_t* cfg, const edg_opt_t* opt,
                      float* mu, float* rho, float* opt_slots, edg_state_t* state,
                      const float* eps_override, float* grad_out, int32_t apply,
                      void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------- batched GEMM
 * C[b] = op(A[b]) op(B[b]) in FP32, the building block of the network steps:
 * op(A)(m, k) = A[b*sA + m*lda + k] (A[b*sA + k*lda + m] when ta),
 * op(B)(k, n) = B[b*sB + k*ldb + n] (B[b*sB + n*ldb + k] when tb).
 * EDG_GEMM_TC: tcgen05 tensor cores with 3xTF32 (operands split hi/lo in
 * flight, FP32 accumulation); kchunk > 0 splits K into chunks of kchunk rows
 * summed in FP32 (workspace: edg_gemm_workspace_bytes).  EDG_GEMM_SIMT: FP32
 * CUDA cores.  The tensor-core kernel's waits are bounded: one that gives up
 * leaves C incomplete and sets the device's GEMM status word, which
 * edg_gemm_status reports. */
enum { EDG_GEMM_TC = 0, EDG_GEMM_SIMT = 1 };
size_t edg_gemm_workspace_bytes(int32_t engine, int32_t M, int32_t N, int32_t K, int32_t batch,
                                int32_t kchunk);
int edg_gemm(int32_t engine, int32_t ta, int32_t tb, int32_t M, int32_t N, int32_t K,
             const float* A, int32_t lda, int64_t sA, const float* B, int32_t ldb, int64_t sB,
             float* C, int32_t ldc, int64_t sC, int32_t batch, int32_t kchunk, void* workspace,
             size_t workspace_bytes, void* stream);
/* Status of the edg_gemm calls on the current device since the last query:
 * synchronises `stream`, stores EDG_OK or EDG_E_TIMEOUT (a bounded wait of a
 * tensor-core GEMM gave up, its C is incomplete) in *status and clears the
 * word.  Calls on several streams of one device share the word. */
int edg_gemm_status(int32_t* status, void* stream);

/* Self test of the bounded device-side wait that every tensor-core kernel
 * uses (no counterpart in the reference): one warp waits on an mbarrier that
 * nothing completes; the wait gives up after about one second.  Synchronises
 * `stream` and stores the kernel's verdict in *status: EDG_E_TIMEOUT when the
 * wait gave up and returned as designed.  The context stays usable. */
int edg_check_bounded_wait(int32_t* status, void* stream);

/* ---------------------------------------------------------------- Bayesian NN
 * KLqp for the regression network h1 = tanh(X W0 + b0), h2 = tanh(h1 W1 + b1),
 * out = h2 W2 + b2, y ~ Normal(out, noise), every weight ~ Normal(0, prior_scale),
 * q = N(mu, softplus(rho)) per weight (edward examples/bayesian_nn.py:120-162 with
 * build_reparam_kl_loss_and_gradients, klqp.py:707-769).  Parameters are
 * flattened W0 [D,H1], b0 [H1], W1 [H1,H2], b1 [H2], W2 [H2,1], b2 [1] row-major
 * (edg_bnn_num_params gives P).  One call = one minibatch step: S weight samples
 * (Philox KIND 0 at iteration state->t, or eps_override [S,P]), batched forward,
 * hand-written adjoint, KL, optimizer apply (same conventions as
 * edg_klqp_glm_step).  X [M,D] / y [M] is the minibatch; data_scale = N/M. */
typedef struct {
  int32_t D, H1, H2;     /* input width and the two hidden widths; output width 1 */
  int32_t n_samples;     /* S > 0 */
  float noise;           /* Normal likelihood scale */
  float prior_scale;     /* Normal(0, prior_scale) on every weight and bias */
  float data_scale;      /* minibatch scale N / M (Inference.scale[y]) */
  int32_t method;        /* EDG_KLQP_REPARAM_KL (analytic KL) or EDG_KLQP_REPARAM (Monte Carlo
                            KL, build_reparam_loss_and_gradients, klqp.py:642-704) */
  int32_t gemm_engine;   /* EDG_GEMM_TC (default) or EDG_GEMM_SIMT */
  uint64_t seed;
} edg_bnn_t;

int32_t edg_bnn_num_params(int32_t D, int32_t H1, int32_t H2);
size_t edg_bnn_workspace_bytes(const edg_bnn_t* cfg, int32_t M);
int edg_bnn_klqp_step(const edg_bnn_t* cfg, const edg_opt_t* opt, const float* X, const float* y,
                      int32_t M, float* mu, float* rho, float* opt_slots, edg_state_t* state,
                      const float* eps_override, float* grad_out, int32_t apply,
                      void* workspace, size_t workspace_bytes, void* stream);
/* The log-likelihood half of the step on its own: for S given weight samples
 * theta [S,P], ll_out[s] = data_scale * sum_m log N(y_m | net(X_m; theta_s), noise)
 * (FP64) and grad_out [S,P] = d ll_out[s] / d theta_s, by the batched forward
 * pass and the hand-written adjoint (what tf.gradients of the reference's
 * p_log_lik yields per sample, klqp.py:746-767).  Backs the autograd Function. */
int edg_bnn_loglik_grad(const edg_bnn_t* cfg, const float* X, const float* y, int32_t M,
                        const float* theta, double* ll_out, float* grad_out, void* workspace,
                        size_t workspace_bytes, void* stream);
/* Minibatch of M rows drawn uniformly with replacement from X [N,D] / y [N]
 * (Philox KIND 4 at iteration state->t) into Xb [M,D] / yb [M]; replaces the
 * host-side feed_dict batches of the reference examples. */
int edg_minibatch_gather(const float* X, const float* y, int64_t N, int32_t D, int32_t M,
                         uint64_t seed, const edg_state_t* state, float* Xb, float* yb,
                         void* stream);

/* ---------------------------------------------------------------- sigmoid belief network
 * ScoreKLqp for the two-layer sigmoid belief network of
 * examples/sigmoid_belief_network.py:54-86 (hidden_sizes = [H0, H1]):
 *   p: z1 ~ Bern(prior_logits), z0 ~ Bern(z1 Wp1 + bp1), x ~ Bern(z0 Wp0 + bp0)
 *   q: z0 ~ Bern(x Wq0 + bq0),  z1 ~ Bern(z0 Wq1 + bq1)
 * Parameters (edg_sbn_num_params): four blocks [in + 1, out] row-major, the
 * bias being the last row: Wq0|bq0 [V+1, H0], Wq1|bq1 [H0+1, H1],
 * Wp1|bp1 [H1+1, H0], Wp0|bp0 [H0+1, V] -- the q variables first.
 * One call = one score-function gradient of the loss -mean_s sum_b
 * [log p(x_b, z_sb) - log q(z_sb | x_b)] over B rows and S samples
 * (build_score_loss_and_gradients, klqp.py:840-906: q-gradient
 * -mean_s grad log q(z_s) * learning signal, p-gradient grad loss), then the
 * optimizer apply.  The learning signal is
 *   EDG_BASELINE_NONE: the sample's total F_s = sum_b f_sb (the reference);
 *   EDG_BASELINE_MEAN: f_sb - c per row, c a running mean of f;
 *   EDG_BASELINE_MLP:  f_sb - (c + sigma * mlp(2 x_b - 1)) per row, mlp a
 *       V -> baseline_hidden (tanh) -> 1 network trained online (one optimizer
 *       step per call, on the row targets (mean_s f_sb - c) / sigma).
 * Every variant is unbiased (the baseline depends on x and on earlier steps
 * only).  z draws: Philox stream 3 at iteration state->t, counter row
 * s*B + b, element j (z0) or round_up(H0, 4) + j (z1), z = u < sigmoid(logit)
 * (TF's Bernoulli sampler); z_override [S*B*H0 z0 | S*B*H1 z1] replaces them. */
enum { EDG_BASELINE_NONE = 0, EDG_BASELINE_MEAN = 1, EDG_BASELINE_MLP = 2 };
typedef struct {
  int32_t V, H0, H1;       /* visible width; hidden widths next to x and at the top */
  int32_t n_samples;       /* S > 0 */
  int32_t baseline;        /* EDG_BASELINE_* */
  int32_t baseline_hidden; /* hidden width of the MLP baseline */
  float baseline_decay;    /* decay of the running mean / scale, in [0, 1) */
  int32_t gemm_engine;     /* EDG_GEMM_TC (default) or EDG_GEMM_SIMT */
  uint64_t seed;
  int32_t rao_blackwell;   /* 1: ScoreRBKLqp (build_score_rb_loss_and_gradients,
                              klqp.py:1058-1152): q(z1 | z0)'s signal drops log p(x | z0),
                              the one density outside its Markov blanket; baseline must be
                              EDG_BASELINE_NONE */
  int32_t reserved;
} edg_sbn_t;

int32_t edg_sbn_num_params(int32_t V, int32_t H0, int32_t H1);
/* MLP baseline parameters: Wb0|bb0 [V+1, BH] then Wb1|bb1 [BH+1, 1]. */
int32_t edg_sbn_baseline_num_params(int32_t V, int32_t BH);
size_t edg_sbn_workspace_bytes(const edg_sbn_t* cfg, int32_t B);
/* Kernel launches one edg_sbn_score_step call makes (for throughput reports). */
int32_t edg_sbn_launches_per_step(const edg_sbn_t* cfg, int32_t B, int32_t apply);
/* X [B, V] (0/1 values as floats); prior_logits [H1]; theta [P]; opt_slots [2P];
 * baseline_params [PB] / baseline_slots [2 PB] (MLP baseline only);
 * baseline_stats float[8] (running mean, running scale, update count, the
 * baseline optimizer's beta1 / beta2 powers, last regression loss, 2 unused):
 * zero-initialise, then set [1] = 1, [3] = beta1, [4] = beta2.
 * grad_out [P] or NULL; signal_out [2, S*B] (f_sb, then the learning signal
 * used) or NULL.  apply = 0 leaves theta, slots, state and the baseline alone. */
int edg_sbn_score_step(const edg_sbn_t* cfg, const edg_opt_t* opt, const edg_opt_t* baseline_opt,
                       const float* X, int32_t B, const float* prior_logits, float* theta,
                       float* opt_slots, edg_state_t* state, float* baseline_params,
                       float* baseline_slots, float* baseline_stats, const float* z_override,
                       float* grad_out, float* signal_out, int32_t apply, void* workspace,
                       size_t workspace_bytes, void* stream);
/* uint8 rows (binary images) gathered as in edg_minibatch_gather and widened to float. */
int edg_minibatch_gather_u8(const uint8_t* X, int64_t N, int32_t V, int32_t B, uint64_t seed,
                            const edg_state_t* state, float* Xb, void* stream);

/* ---------------------------------------------------------------- SG-MCMC
 * n_iter iterations of SGLD (edward/inferences/sgld.py:52-88) or SGHMC
 * (sghmc.py:58-102) for C independent chains over a GLM: per iteration the
 * gradient of log p(z) + data_scale * log p(y | z) at every chain's state, then
 *   SGLD   lr = step_size / (t + 1)^0.55; z += lr/2 grad + sqrt(lr) e
 *   SGHMC  lr = step_size * 0.01; z += v; v = (1 - friction/2) v + lr grad + sqrt(lr friction) e
 * with t = state->t (advanced by one per iteration), e ~ N(0, 1) from Philox
 * stream 5 at iteration t, counter row c, element p (or noise_override
 * [n_iter, C, P]).  The new state goes to samples[t] ([T_cap, C, P], NULL to
 * skip) and n_accept[c] += 1 every iteration, as in the reference. */
enum { EDG_SGMCMC_SGLD = 0, EDG_SGMCMC_SGHMC = 1 };
typedef struct {
  int32_t method;   /* EDG_SGMCMC_* */
  float step_size;
  float friction;   /* SGHMC */
  float data_scale; /* Inference.scale of the observed variable */
  uint64_t seed;
} edg_sgmcmc_t;
size_t edg_sgmcmc_glm_workspace_bytes(const edg_glm_t* model, int32_t C);
int edg_sgmcmc_glm_run(const edg_glm_t* model, const edg_sgmcmc_t* cfg, int32_t C, int32_t n_iter,
                       float* z, float* v, int32_t* n_accept, edg_state_t* state, float* samples,
                       int64_t T_cap, const float* noise_override, void* workspace,
                       size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------- Metropolis-Hastings
 * n_iter iterations of MetropolisHastings (edward/inferences/metropolis_hastings.py:64-156)
 * for C chains over a GLM with Normal proposals: random walk z' = z + s e
 * (proposal_loc = NULL) or independence z' = m + s e (proposal_loc = m [P]);
 * ratio = log p(x, z') - log p(x, z) - log g(z' | z) + log g(z | z') (FP64),
 * accept if log u < ratio.  e: Philox stream 6 at iteration t = state->t,
 * counter row c, element p (or e_override [n_iter, C, P]); u: stream 7, row c
 * (or u_override [n_iter, C]).  lj [C] caches log p(x, z) (rebuilt when
 * cache_valid = 0); samples[t] and n_accept as in edg_hmc_glm_run;
 * ratio_out [n_iter, C] or NULL. */
typedef struct {
  const float* proposal_loc;   /* [P] device, or NULL for the random walk */
  const float* proposal_scale; /* [P] device */
  uint64_t seed;
} edg_mh_t;
size_t edg_mh_glm_workspace_bytes(const edg_glm_t* model, int32_t C);
int edg_mh_glm_run(const edg_glm_t* model, const edg_mh_t* cfg, int32_t C, int32_t n_iter,
                   float* z, double* lj, int32_t cache_valid, int32_t* n_accept,
                   edg_state_t* state, float* samples, int64_t T_cap, const float* e_override,
                   const double* u_override, double* ratio_out, void* workspace,
                   size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------- constrained latent
 * One latent with a constrained support and i.i.d. observations, worked in the
 * unconstrained space auto_transform maps it to (inference.py:222-264,
 * util/random_variables.py:856-917): target log p(x, z(u)) + log|det dz/du|.
 *   EDG_EXPFAM_BETA       Beta(a, b) prior, Bernoulli(probs=z) data, z = sigmoid(u)
 *   EDG_EXPFAM_GAMMA      Gamma(a, rate b) prior, Poisson(rate=z) data, z = softplus(u)
 *   EDG_EXPFAM_DIRICHLET  Dirichlet(alpha) prior, Categorical(probs=z) data,
 *                         z = softmax([u, 0]) (SoftmaxCentered), u in R^(categories - 1) */
enum { EDG_EXPFAM_BETA = 0, EDG_EXPFAM_GAMMA = 1, EDG_EXPFAM_DIRICHLET = 2 };
typedef struct {
  int32_t family;       /* EDG_EXPFAM_* */
  int32_t K;            /* unconstrained dimension: 1, or categories - 1 (<= 32) */
  const double* prior;  /* device: (a, b) | (a, rate) | alpha[K + 1] */
  const double* stats;  /* device: (n1, n0) | (sum x, N, sum log x!) | counts[K + 1] */
  int32_t transform;    /* 1: the latent is worked in the unconstrained space above;
                         * 0: on its support itself (KLqp with auto_transform=False; Beta
                         * and Gamma only): z = u, no Jacobian, and log p(x, z) and its
                         * gradient are NaN where u is outside the support */
} edg_expfam_t;
/* HMC over C chains (FP32 state u [C, K] and gradient cache, FP64 log joint
 * cache lj [C]; the reference's leapfrog and Metropolis test, with the log
 * joint's terms and the energy difference summed in FP64); Philox streams and
 * overrides (r_override FP32 [n_iter, C, K], u_override FP64 [n_iter, C]) as
 * in edg_hmc_glm_run; samples FP32 [T_cap, C, K] (unconstrained) or NULL. */
int edg_expfam_hmc_run(const edg_expfam_t* model, const edg_hmc_t* cfg, int32_t C, int32_t n_iter,
                       float* u, float* grad, double* lj, int32_t cache_valid,
                       int32_t* n_accept, edg_state_t* state, float* samples, int64_t T_cap,
                       const float* r_override, const double* u_override, void* stream);
/* One KLqp step with q(u) = N(mu, softplus(rho)) [K]: reparameterisation gradient
 * with Monte Carlo KL (klqp.py:642-704), S <= 256 draws (Philox stream 0 at
 * iteration state->t, or eps_override [S, K]), then the optimizer apply
 * (opt_slots [4K]); loss in state->loss, gradients in grad_out [2K] or NULL. */
int edg_expfam_klqp_step(const edg_expfam_t* model, int32_t n_samples, uint64_t seed,
                         const edg_opt_t* opt, float* mu, float* rho, float* opt_slots,
                         edg_state_t* state, const float* eps_override, float* grad_out,
                         int32_t apply, void* stream);

/* ---------------------------------------------------------------- criticism
 * Posterior predictive of a GLM for ed.evaluate / ed.ppc (edward/criticisms/
 * evaluate.py:20-233, ppc.py:13-104), for S parameter vectors Z [S, P] (posterior
 * draws) over the model's rows X:
 *   EDG_PREDICT_MEAN    out [N]    = mean_s E[y_n | z_s] (sigmoid(eta) or eta)
 *   EDG_PREDICT_ETA     out [S, N] = eta
 *   EDG_PREDICT_SAMPLE  out [S, N] = draws of y_n | z_s (Philox stream 8 at
 *                       `iteration`, counter row s, element n). */
enum { EDG_PREDICT_MEAN = 0, EDG_PREDICT_ETA = 1, EDG_PREDICT_SAMPLE = 2 };
int edg_glm_predict(const edg_glm_t* model, const float* Z, int32_t S, int32_t mode,
                    uint64_t seed, uint32_t iteration, float* out, void* stream);

/* ---------------------------------------------------------------- HMC
 * n_iter HMC iterations for C independent chains over a GLM in one launch.
 * Replaces HMC.build_update + leapfrog (hmc.py:61-130,195-210) and
 * MonteCarlo.update (edward/inferences/monte_carlo.py:111-150).
 * z, grad, lj: current state, its log-joint gradient and value (the cache is
 * rebuilt when cache_valid = 0).  Iteration i uses t = state->t + i for its
 * Philox counters and writes the kept sample to samples[t] (Empirical.params,
 * [T_cap, C, P]) when samples != NULL and t < T_cap.  moments (or NULL):
 * [2, C, P] FP64 running sum and sum of squares of kept samples.
 * r_override [n_iter, C, P] / u_override [n_iter, C] replace the momentum
 * and Metropolis uniform draws.  ratio_out [n_iter, C] (or NULL) receives
 * the FP64 log acceptance ratio.  state->t advances by n_iter. */
int edg_hmc_glm_run(const edg_glm_t* model, const edg_hmc_t* cfg, int32_t C, int32_t n_iter,
                    float* z, float* grad, double* lj, int32_t cache_valid,
                    int32_t* n_accept, edg_state_t* state,
                    float* samples, int64_t T_cap, double* moments,
                    const float* r_override, const double* u_override, double* ratio_out,
                    void* stream);

/* ---------------------------------------------------------------- HMC, ragged hierarchical batch
 * I independent hierarchical logistic regressions, each with C chains:
 *   mu ~ Normal(mu_loc, mu_scale), tau ~ HalfNormal(tau_scale),
 *   w_d ~ Normal(mu, tau) (d < D_i), y_n ~ Bernoulli(logits = X_i[n] . w).
 * HMC runs on (w, mu, u) with tau = softplus(u) and the log-det-Jacobian
 * log sigmoid(u) added, as auto_transform does for a 'nonnegative' latent
 * (edward/util/random_variables.py:903-904; edward/inferences/hmc.py:132-159).
 * Chain k of instance i is global chain i*C + k; its state row has stride
 * SP = max_D + 2 with w in [0, D_i) (zeros up to max_D), mu at SP-2, u at SP-1.  z / grad: [I*C, max_D+2],
 * lj / n_accept: [I*C]; samples [T_cap, I*C, max_D+2]; moments [2, I*C, max_D+2];
 * r_override [n_iter, I*C, max_D+2]; u_override / ratio_out [n_iter, I*C].
 * `order` (or NULL) is a permutation of the instances giving the launch order
 * (heaviest first balances the ragged work).  Replaces, per instance, the
 * same reference code as edg_hmc_glm_run. */
typedef struct {
  const float* X;          /* all X_i concatenated, each [N_i, D_i] row-major */
  const float* y;          /* all y_i concatenated */
  const int64_t* x_offset; /* [I] element offset of X_i in X */
  const int64_t* y_offset; /* [I] element offset of y_i in y */
  const int32_t* N;        /* [I] rows of each instance */
  const int32_t* D;        /* [I] features of each instance (<= max_D) */
  int32_t I;
  int32_t max_D;           /* <= 160 */
  float mu_loc, mu_scale, tau_scale;
} edg_hier_t;

int edg_hmc_hier_run(const edg_hier_t* model, const edg_hmc_t* cfg, int32_t C, int32_t n_iter,
                     const int32_t* order, float* z, float* grad, double* lj, int32_t cache_valid,
                     int32_t* n_accept, edg_state_t* state, float* samples, int64_t T_cap,
                     double* moments, const float* r_override, const double* u_override,
                     double* ratio_out, void* stream);

/* Same contract as edg_hmc_hier_run (same draws, state layout and results to
 * FP32 rounding), with every gradient evaluation computed as tcgen05 3xTF32
 * GEMMs: one CTA per (instance, 64 chains), X read once per evaluation for
 * all 64 chains.  Requires max_D <= 128; cfg->chains_per_block is ignored.
 * `tiles` is X and y re-laid once by edg_hmc_hier_tc_prepare: instance i at
 * float offset tile_off[i], in 128-row tiles with row pitch
 * Dp_i + 1 (Dp_i = round_up(D_i, 8)): X_i in columns [0, D_i), y_i in column
 * Dp_i, zero elsewhere and beyond N_i.  edg_hmc_hier_tc_tile_offsets fills tile_off
 * (host arrays N, D) and returns the total size in floats (-1 on bad
 * input); tile_off is then copied to the device for the two calls below. */
int64_t edg_hmc_hier_tc_tile_offsets(const int32_t* N, const int32_t* D, int32_t I,
                                     int64_t* tile_off);
int edg_hmc_hier_tc_prepare(const edg_hier_t* model, const int64_t* tile_off, float* tiles,
                            void* stream);
int edg_hmc_hier_tc_run(const edg_hier_t* model, const edg_hmc_t* cfg, int32_t C, int32_t n_iter,
                        const int32_t* order, const float* tiles, const int64_t* tile_off,
                        float* z, float* grad, double* lj, int32_t cache_valid,
                        int32_t* n_accept, edg_state_t* state, float* samples, int64_t T_cap,
                        double* moments, const float* r_override, const double* u_override,
                        double* ratio_out, void* stream);

/* ---------------------------------------------------------------- HMC, tensor cores
 * Same contract as edg_hmc_glm_run, computed with tcgen05 3xTF32 GEMMs:
 * one thread-block cluster per 128 chains, the cluster's CTAs splitting the
 * rows of X and reducing each leapfrog gradient through distributed shared
 * memory.  Requires P = D + bias <= 64 and n_steps > 0.  `tiles` is the
 * model's X re-laid into 64-row operand tiles by edg_hmc_glm_tc_prepare
 * (once per model; edg_hmc_glm_tc_tiles_bytes gives its size); y is read from
 * model->y during the run.
 * Replaces the same reference code as edg_hmc_glm_run (hmc.py:61-130,195-210;
 * monte_carlo.py:111-150). */
size_t edg_hmc_glm_tc_tiles_bytes(const edg_glm_t* model);
int edg_hmc_glm_tc_prepare(const edg_glm_t* model, void* tiles, size_t tiles_bytes, void* stream);
int edg_hmc_glm_tc_run(const edg_glm_t* model, const edg_hmc_t* cfg, int32_t C, int32_t n_iter,
                       const void* tiles, float* z, float* grad, double* lj, int32_t cache_valid,
                       int32_t* n_accept, edg_state_t* state, float* samples, int64_t T_cap,
                       double* moments, const float* r_override, const double* u_override,
                       double* ratio_out, void* stream);

/* ---------------------------------------------------------------- SG-MCMC, tensor cores
 * Same contract as edg_sgmcmc_glm_run, with the per-iteration gradient
 * computed by the tensor-core kernel above (one 3xTF32 evaluation per
 * iteration, the SGLD / SGHMC update fused into the kernel's owner phase).
 * Requires P = D + bias <= 64; `tiles` as for edg_hmc_glm_tc_run.  grad [C, P]
 * carries the gradient of the current state between calls: with
 * cache_valid = 0 it is rebuilt by one extra evaluation before the first
 * iteration; every call leaves it valid for the state it returns.  v [C, P] is
 * the SGHMC velocity (unused by SGLD).
 * Replaces the same reference code as edg_sgmcmc_glm_run (sgld.py:52-88,
 * sghmc.py:58-102). */
int edg_sgmcmc_glm_tc_run(const edg_glm_t* model, const edg_sgmcmc_t* cfg, int32_t C,
                          int32_t n_iter, const void* tiles, float* z, float* v, float* grad,
                          int32_t cache_valid, int32_t* n_accept, edg_state_t* state,
                          float* samples, int64_t T_cap, const float* noise_override,
                          void* stream);

/* ---------------------------------------------------------------- Metropolis-Hastings, tensor cores
 * Same contract as edg_mh_glm_run, with each iteration's log joint of the
 * proposals computed by the tensor-core kernel above (the proposal, the FP64
 * ratio and the accept / reject fused around it).  `grad` [C, P] is scratch
 * (the kernel writes the prior's gradient there).  Requires
 * P = D + bias <= 64; `tiles` as for edg_hmc_glm_tc_run.  Replaces the same
 * reference code as edg_mh_glm_run (metropolis_hastings.py:64-156). */
int edg_mh_glm_tc_run(const edg_glm_t* model, const edg_mh_t* cfg, int32_t C, int32_t n_iter,
                      const void* tiles, float* z, float* grad, double* lj, int32_t cache_valid,
                      int32_t* n_accept, edg_state_t* state, float* samples, int64_t T_cap,
                      const float* e_override, const double* u_override, double* ratio_out,
                      void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EDWARD_GB300_H_ */
