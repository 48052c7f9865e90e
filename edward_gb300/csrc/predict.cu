// Posterior predictive of the GLM family for criticism (edward/criticisms/
// evaluate.py:20-233, ppc.py:13-104): for S posterior parameter vectors Z [S, P]
// and the rows of X,
//   EDG_PREDICT_MEAN    out[n]    = (1/S) sum_s E[y_n | z_s]   (sigmoid(eta) or eta)
//   EDG_PREDICT_ETA     out[s, n] = eta_sn = x_n . w_s (+ b_s)
//   EDG_PREDICT_SAMPLE  out[s, n] ~ p(y_n | z_s)  (Bernoulli or Normal draws, Philox
//                       stream 8 at `iteration`, counter row s, element n)
// One thread per row; the parameter vectors are staged through shared memory.
#include <algorithm>

#include "edg_common.cuh"

namespace edg {
namespace pred {

constexpr int kT = 128;
constexpr uint32_t kKindPredictive = 8u;

__global__ void __launch_bounds__(kT) predict_kernel(GLMDev m, const float* __restrict__ Z, int S,
                                                     int chunk, int mode, uint64_t seed,
                                                     uint32_t iteration, float* __restrict__ out) {
  extern __shared__ float zs[];  // [chunk][P]
  const int n = blockIdx.x * kT + threadIdx.x;
  const float* x = m.X + (int64_t)n * m.D;
  const float lik_scale = sqrtf(1.0f / m.inv_lik_var);
  float acc = 0.0f;
  for (int s0 = 0; s0 < S; s0 += chunk) {
    const int cs = min(chunk, S - s0);
    __syncthreads();
    for (int i = threadIdx.x; i < cs * m.P; i += kT) zs[i] = Z[(int64_t)s0 * m.P + i];
    __syncthreads();
    if (n >= m.N) continue;
    for (int k = 0; k < cs; ++k) {
      const float* z = zs + k * m.P;
      float eta = m.bias ? z[m.D] : 0.0f;
      for (int d = 0; d < m.D; ++d) eta = fmaf(x[d], z[d], eta);
      const int s = s0 + k;
      if (mode == EDG_PREDICT_MEAN) {
        acc += m.lik == EDG_LIK_BERNOULLI ? sigmoidf(eta) : eta;
      } else if (mode == EDG_PREDICT_ETA) {
        out[(int64_t)s * m.N + n] = eta;
      } else {
        const uint4 r = philox_at(seed, kKindPredictive, iteration, (uint32_t)s, (uint32_t)(n >> 2));
        const uint32_t w = (n & 3) == 0 ? r.x : (n & 3) == 1 ? r.y : (n & 3) == 2 ? r.z : r.w;
        float y;
        if (m.lik == EDG_LIK_BERNOULLI) {
          y = u01f(w) < sigmoidf(eta) ? 1.0f : 0.0f;
        } else {
          y = eta + lik_scale * philox_normal(seed, kKindPredictive, iteration, (uint32_t)s,
                                              (uint32_t)n);
        }
        out[(int64_t)s * m.N + n] = y;
      }
    }
  }
  if (mode == EDG_PREDICT_MEAN && n < m.N) out[n] = acc / (float)S;
}

}  // namespace pred
}  // namespace edg

using namespace edg;

extern "C" int edg_glm_predict(const edg_glm_t* model, const float* Z, int32_t S, int32_t mode,
                               uint64_t seed, uint32_t iteration, float* out, void* stream) {
  GLMDev m;
  int rc = make_glm(model, &m);
  if (rc) return rc;
  EDG_REQUIRE(Z && out, EDG_E_NULL, "pointers must not be NULL");
  EDG_REQUIRE(S > 0, EDG_E_SHAPE, "S must be positive");
  EDG_REQUIRE(mode == EDG_PREDICT_MEAN || mode == EDG_PREDICT_ETA || mode == EDG_PREDICT_SAMPLE,
              EDG_E_VALUE, "unknown mode %d", mode);
  EDG_REQUIRE(m.P <= 8192, EDG_E_SHAPE, "at most 8192 coordinates");
  const int chunk = std::max(1, std::min(S, 8192 / m.P));
  const size_t smem = (size_t)chunk * m.P * sizeof(float);
  pred::predict_kernel<<<(m.N + pred::kT - 1) / pred::kT, pred::kT, smem, (cudaStream_t)stream>>>(
      m, Z, S, chunk, mode, seed, iteration, out);
  return check_launch("predict_kernel");
}
