// Stochastic-gradient MCMC for the GLM family: SGLD and SGHMC over C
// independent chains (edward/inferences/sgld.py:52-88, sghmc.py:58-102).
//
// One iteration = the batched log-joint gradient of every chain's current
// state (prior + scale * likelihood, the same FP32 adjoint kernel as HMC) and
// an element-wise update kernel:
//   SGLD   lr = step_size / (t + 1)^0.55
//          z <- z + lr/2 * grad + sqrt(lr) * e
//   SGHMC  lr = step_size * 0.01
//          z <- z + v;   v <- (1 - friction/2) v + lr * grad + sqrt(lr * friction) * e
// with e ~ N(0, 1) from Philox stream 5 at iteration t (or an override), t the
// device-side iteration counter; the new state is written to samples[t]
// (Empirical.params) and every chain's n_accept is incremented, as the
// reference does.  The last block to finish advances t, so iterations can be
// replayed from a CUDA graph.
#include <algorithm>

#include "edg_common.cuh"

namespace edg {
namespace sg {

constexpr int kT = 256;
constexpr uint32_t kKindNoise = 5u;

struct UpdArgs {
  int method, C, P;
  float step_size, friction;
  uint64_t seed;
  float* z;
  float* v;
  const float* grad;
  int32_t* n_accept;
  edg_state_t* state;
  float* samples;
  int64_t T_cap;
  const float* noise;  // [C, P] for this iteration, or NULL
};

__global__ void __launch_bounds__(kT) update_kernel(UpdArgs a) {
  __shared__ bool s_last;
  const int64_t t = a.state->t;
  const int64_t n = (int64_t)a.C * a.P;
  const int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x;
  if (i < n) {
    const int c = (int)(i / a.P), p = (int)(i % a.P);
    const float e = a.noise ? a.noise[i]
                            : philox_normal(a.seed, kKindNoise, (uint32_t)t, (uint32_t)c,
                                            (uint32_t)p);
    const float g = a.grad[i];
    float z = a.z[i];
    if (a.method == EDG_SGMCMC_SGLD) {
      const float lr = a.step_size / powf((float)(t + 1), 0.55f);
      z = z + 0.5f * lr * g + sqrtf(lr) * e;
    } else {
      const float lr = a.step_size * 0.01f;
      const float v = a.v[i];
      z = z + v;
      a.v[i] = (1.0f - 0.5f * a.friction) * v + lr * g + sqrtf(lr * a.friction) * e;
    }
    if (!isfinite(z)) atomicAdd(&a.state->nonfinite, 1u);
    a.z[i] = z;
    if (a.samples && t < a.T_cap) a.samples[t * n + i] = z;
    if (p == 0) a.n_accept[c] += 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&a.state->done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  a.state->t = t + 1;
  a.state->done = 0;
  __threadfence();
}

}  // namespace sg
}  // namespace edg

using namespace edg;

extern "C" size_t edg_sgmcmc_glm_workspace_bytes(const edg_glm_t* model, int32_t C) {
  if (!model || C <= 0) return 0;
  const size_t g = edg_glm_logjoint_grad_workspace_bytes(model, C);
  if (!g) return 0;
  const int64_t P = (int64_t)model->D + (model->bias ? 1 : 0);
  return (g + 255) / 256 * 256 + (size_t)C * P * sizeof(float);
}

extern "C" int edg_sgmcmc_glm_run(const edg_glm_t* model, const edg_sgmcmc_t* cfg, int32_t C,
                                  int32_t n_iter, float* z, float* v, int32_t* n_accept,
                                  edg_state_t* state, float* samples, int64_t T_cap,
                                  const float* noise_override, void* workspace,
                                  size_t workspace_bytes, void* stream) {
  EDG_REQUIRE(model && cfg && z && n_accept && state, EDG_E_NULL, "pointers must not be NULL");
  EDG_REQUIRE(C > 0 && n_iter >= 0, EDG_E_SHAPE, "C must be positive and n_iter >= 0");
  EDG_REQUIRE(cfg->method == EDG_SGMCMC_SGLD || cfg->method == EDG_SGMCMC_SGHMC, EDG_E_VALUE,
              "unknown method %d", cfg->method);
  EDG_REQUIRE(cfg->method != EDG_SGMCMC_SGHMC || v, EDG_E_NULL, "SGHMC needs the velocity v");
  EDG_REQUIRE(cfg->step_size > 0.0f && cfg->friction >= 0.0f, EDG_E_VALUE,
              "step_size must be positive and friction >= 0");
  const size_t need = edg_sgmcmc_glm_workspace_bytes(model, C);
  EDG_REQUIRE(need, EDG_E_SHAPE, "invalid model");
  EDG_REQUIRE(workspace && workspace_bytes >= need, EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  const size_t gbytes = edg_glm_logjoint_grad_workspace_bytes(model, C);
  const size_t goff = (gbytes + 255) / 256 * 256;
  float* grad = reinterpret_cast<float*>(reinterpret_cast<char*>(workspace) + goff);
  const int P = model->D + (model->bias ? 1 : 0);
  sg::UpdArgs a;
  a.method = cfg->method;
  a.C = C;
  a.P = P;
  a.step_size = cfg->step_size;
  a.friction = cfg->friction;
  a.seed = cfg->seed;
  a.z = z;
  a.v = v;
  a.grad = grad;
  a.n_accept = n_accept;
  a.state = state;
  a.samples = samples;
  a.T_cap = T_cap;
  const int64_t n = (int64_t)C * P;
  for (int it = 0; it < n_iter; ++it) {
    int rc = edg_glm_logjoint_grad(model, z, C, 1, cfg->data_scale, nullptr, grad, workspace,
                                   gbytes, stream);
    if (rc) return rc;
    a.noise = noise_override ? noise_override + (int64_t)it * n : nullptr;
    sg::update_kernel<<<(unsigned)((n + sg::kT - 1) / sg::kT), sg::kT, 0, (cudaStream_t)stream>>>(
        a);
    if ((rc = check_launch("sgmcmc update_kernel"))) return rc;
  }
  return EDG_OK;
}
