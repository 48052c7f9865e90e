// Metropolis-Hastings for the GLM family over C independent chains
// (edward/inferences/metropolis_hastings.py:64-156) with Normal proposals,
// either a random walk g(z' | z) = N(z, s) or an independence proposal
// g(z') = N(m, s) (fixed location m).
//
// One iteration: propose z' (Philox stream 6 at iteration t), the batched log
// joint of z' (FP64 per chain, the same kernel as HMC's), then
//   ratio = log p(x, z') - log p(x, z) - log g(z' | z) + log g(z | z')
// (the proposal terms cancel for the random walk), accept if log u < ratio
// with u from Philox stream 7; the kept state goes to samples[t] and
// n_accept counts acceptances.  log p(x, z) of the current state is cached
// across iterations.
#include <algorithm>

#include "edg_common.cuh"

namespace edg {
namespace mh {

constexpr int kT = 256;
constexpr uint32_t kKindProposal = 6u, kKindUniform = 7u;

// z' = (random walk ? z : loc) + scale * e, and per chain
// lq[c] = log g(z | z') - log g(z' | z) (0 for the random walk).
__global__ void __launch_bounds__(kT) propose_kernel(int C, int P, uint64_t seed,
                                                     const edg_state_t* state,
                                                     const float* __restrict__ z,
                                                     const float* __restrict__ loc,
                                                     const float* __restrict__ scale,
                                                     const float* __restrict__ e_ovr,
                                                     float* __restrict__ zp,
                                                     double* __restrict__ lq) {
  const int c = blockIdx.x;
  const uint32_t t = (uint32_t)state->t;
  double acc = 0.0;
  for (int p = threadIdx.x; p < P; p += kT) {
    const int64_t i = (int64_t)c * P + p;
    const float e = e_ovr ? e_ovr[i] : philox_normal(seed, kKindProposal, t, (uint32_t)c, (uint32_t)p);
    const float s = scale[p];
    const float zn = (loc ? loc[p] : z[i]) + s * e;
    zp[i] = zn;
    if (loc) {
      // log N(z | m, s) - log N(z' | m, s)
      const double a = ((double)z[i] - loc[p]) / s, b = ((double)zn - loc[p]) / s;
      acc += -0.5 * a * a + 0.5 * b * b;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double red[kT / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < kT / 32; ++w) tot += red[w];
    lq[c] = tot;
  }
}

struct AccArgs {
  int C, P;
  uint64_t seed;
  float* z;
  const float* zp;
  double* lj;
  const double* lj_new;
  const double* lq;
  int32_t* n_accept;
  edg_state_t* state;
  float* samples;
  int64_t T_cap;
  const double* u_ovr;
  double* ratio_out;
};

// One block per chain: accept / reject, write the kept state to samples[t];
// the last block advances t.
__global__ void __launch_bounds__(kT) accept_kernel(AccArgs a) {
  __shared__ bool s_acc, s_last;
  const int c = blockIdx.x;
  const int64_t t = a.state->t;
  if (threadIdx.x == 0) {
    const double ratio = a.lj_new[c] - a.lj[c] + a.lq[c];
    const double u = a.u_ovr ? a.u_ovr[c]
                             : u01d(philox_at(a.seed, kKindUniform, (uint32_t)t, (uint32_t)c, 0u).x);
    const bool acc = log(u) < ratio;
    s_acc = acc;
    if (acc) {
      a.lj[c] = a.lj_new[c];
      a.n_accept[c] += 1;
    }
    if (a.ratio_out) a.ratio_out[c] = ratio;
  }
  __syncthreads();
  for (int p = threadIdx.x; p < a.P; p += kT) {
    const int64_t i = (int64_t)c * a.P + p;
    float zi = a.z[i];
    if (s_acc) {
      zi = a.zp[i];
      a.z[i] = zi;
    }
    if (a.samples && t < a.T_cap) a.samples[t * a.C * a.P + i] = zi;
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

}  // namespace mh
}  // namespace edg

using namespace edg;

static size_t mh_layout(const edg_glm_t* model, int C, size_t* off_zp, size_t* off_lj,
                        size_t* off_lq) {
  const size_t g = edg_glm_logjoint_grad_workspace_bytes(model, C);
  if (!g) return 0;
  const int64_t P = (int64_t)model->D + (model->bias ? 1 : 0);
  size_t off = (g + 255) / 256 * 256;
  *off_zp = off;
  off += ((size_t)C * P * 4 + 255) / 256 * 256;
  *off_lj = off;
  off += ((size_t)C * 8 + 255) / 256 * 256;
  *off_lq = off;
  off += (size_t)C * 8;
  return off;
}

extern "C" size_t edg_mh_glm_workspace_bytes(const edg_glm_t* model, int32_t C) {
  if (!model || C <= 0) return 0;
  size_t a, b, c;
  return mh_layout(model, C, &a, &b, &c);
}

extern "C" int edg_mh_glm_run(const edg_glm_t* model, const edg_mh_t* cfg, int32_t C,
                              int32_t n_iter, float* z, double* lj, int32_t cache_valid,
                              int32_t* n_accept, edg_state_t* state, float* samples,
                              int64_t T_cap, const float* e_override, const double* u_override,
                              double* ratio_out, void* workspace, size_t workspace_bytes,
                              void* stream) {
  EDG_REQUIRE(model && cfg && z && lj && n_accept && state && cfg->proposal_scale, EDG_E_NULL,
              "pointers must not be NULL");
  EDG_REQUIRE(C > 0 && n_iter >= 0, EDG_E_SHAPE, "C must be positive and n_iter >= 0");
  size_t o_zp, o_lj, o_lq;
  const size_t need = mh_layout(model, C, &o_zp, &o_lj, &o_lq);
  EDG_REQUIRE(need, EDG_E_SHAPE, "invalid model");
  EDG_REQUIRE(workspace && workspace_bytes >= need, EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  const size_t gbytes = edg_glm_logjoint_grad_workspace_bytes(model, C);
  char* w = reinterpret_cast<char*>(workspace);
  float* zp = reinterpret_cast<float*>(w + o_zp);
  double* lj_new = reinterpret_cast<double*>(w + o_lj);
  double* lq = reinterpret_cast<double*>(w + o_lq);
  const int P = model->D + (model->bias ? 1 : 0);
  cudaStream_t st = (cudaStream_t)stream;
  int rc;
  if (!cache_valid) {
    rc = edg_glm_logjoint_grad(model, z, C, 1, 1.0f, lj, nullptr, workspace, gbytes, stream);
    if (rc) return rc;
  }
  mh::AccArgs a;
  a.C = C;
  a.P = P;
  a.seed = cfg->seed;
  a.z = z;
  a.zp = zp;
  a.lj = lj;
  a.lj_new = lj_new;
  a.lq = lq;
  a.n_accept = n_accept;
  a.state = state;
  a.samples = samples;
  a.T_cap = T_cap;
  const int64_t n = (int64_t)C * P;
  for (int it = 0; it < n_iter; ++it) {
    mh::propose_kernel<<<C, mh::kT, 0, st>>>(C, P, cfg->seed, state, z, cfg->proposal_loc,
                                              cfg->proposal_scale,
                                              e_override ? e_override + it * n : nullptr, zp, lq);
    if ((rc = check_launch("mh propose_kernel"))) return rc;
    rc = edg_glm_logjoint_grad(model, zp, C, 1, 1.0f, lj_new, nullptr, workspace, gbytes, stream);
    if (rc) return rc;
    a.u_ovr = u_override ? u_override + (int64_t)it * C : nullptr;
    a.ratio_out = ratio_out ? ratio_out + (int64_t)it * C : nullptr;
    mh::accept_kernel<<<C, mh::kT, 0, st>>>(a);
    if ((rc = check_launch("mh accept_kernel"))) return rc;
  }
  return EDG_OK;
}
