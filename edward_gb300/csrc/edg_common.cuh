// Shared device/host helpers for the edward_gb300 CUDA library: error
// reporting, the Philox4x32-10 generator, the GLM problem descriptor and small
// numeric helpers.  Target: sm_103a only.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/edward_gb300.h"

namespace edg {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int check_launch(const char* what);

#define EDG_REQUIRE(cond, code, ...)            \
  do {                                          \
    if (!(cond)) return ::edg::fail(code, __VA_ARGS__); \
  } while (0)

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon et al., SC 2011).  Counter (quad, row, iteration,
// kind), key (seed_lo, seed_hi): every draw is a pure function of its
// coordinates, so eps, momenta and uniforms need no generator state.
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    if (i) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
  }
  return c;
}

__device__ __forceinline__ uint4 philox_at(uint64_t seed, uint32_t kind, uint32_t iter,
                                           uint32_t row, uint32_t quad) {
  return philox(make_uint4(quad, row, iter, kind), (uint32_t)seed, (uint32_t)(seed >> 32));
}

// 23-bit uniform strictly inside (0,1), exact in FP32: (2 (a >> 9) + 1) 2^-24.
__device__ __forceinline__ float u01f(uint32_t a) {
  return (float)(2u * (a >> 9) + 1u) * 5.9604644775390625e-08f;
}
// 32-bit uniform strictly inside (0,1), exact in FP64: (a + 0.5) 2^-32.
__device__ __forceinline__ double u01d(uint32_t a) {
  return ((double)a + 0.5) * 2.3283064365386963e-10;
}
// Box-Muller on one pair of outputs.
__device__ __forceinline__ float2 box_muller(uint32_t a, uint32_t b) {
  const float u1 = u01f(a), u2 = u01f(b);
  const float rad = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  return make_float2(rad * c, rad * s);
}
// Normal draw for element e of (kind, iter, row).
__device__ __forceinline__ float philox_normal(uint64_t seed, uint32_t kind, uint32_t iter,
                                               uint32_t row, uint32_t e) {
  const uint4 r = philox_at(seed, kind, iter, row, e >> 2);
  const uint32_t lane = e & 3u;
  const float2 n = lane < 2 ? box_muller(r.x, r.y) : box_muller(r.z, r.w);
  return (lane & 1u) ? n.y : n.x;
}

// ---------------------------------------------------------------- math
__device__ __forceinline__ float softplusf(float x) {
  return fmaxf(x, 0.0f) + log1pf(expf(-fabsf(x)));
}
__device__ __forceinline__ float sigmoidf(float x) {
  const float e = expf(-fabsf(x));
  const float s = 1.0f / (1.0f + e);
  return x >= 0.0f ? s : e * s;
}
// The hardware approximations behind the per-row likelihood arithmetic of
// the hot loops (exp via exp2(x log2 e), log via ln 2 * log2 x).
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLn2 = 0.6931471805599453f;

// Kahan-compensated FP32 accumulation (per-thread partials of the log joint;
// the cross-thread and cross-block sums are done in FP64).
struct Kahan {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

constexpr double kHalfLog2Pi = 0.91893853320467274178;

// ---------------------------------------------------------------- GLM
// Device-side copy of edg_glm_t with derived constants.
struct GLMDev {
  const float* X;
  const float* y;
  const float* prior_loc;
  const float* prior_scale;
  int N, D, P, PP, bias, lik;
  float inv_lik_var;    // 1 / lik_scale^2
  float lik_norm;       // log(lik_scale) + 0.5 log(2 pi)
};

int make_glm(const edg_glm_t* g, GLMDev* out);

__host__ __device__ constexpr int round_up(int a, int b) { return (a + b - 1) / b * b; }
// Byte counts of workspaces: rounded in size_t (an int round-up would wrap
// once a workspace passes 2 GiB and accept an undersized buffer).
__host__ __device__ constexpr size_t round_up_bytes(size_t a, size_t b) {
  return (a + b - 1) / b * b;
}

// Raises a kernel's dynamic shared-memory limit on the CURRENT device.  The
// runtime keeps this attribute per device, so it is set on every launch
// (a host-side call of a few hundred nanoseconds) rather than cached once per
// process, which would leave a second device without it.
template <typename Kernel>
inline int set_max_dyn_smem(Kernel kernel, size_t bytes, const char* what) {
  const cudaError_t e =
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "%s: raising the shared-memory limit to %zu bytes: %s",
                                    what, bytes, cudaGetErrorString(e));
  return EDG_OK;
}

}  // namespace edg
