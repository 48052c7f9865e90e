// Library-level C ABI: error strings, device query, GLM descriptor checks and
// the Philox fill kernels used to test the in-kernel generator.
#include <cstdarg>
#include <cstdio>
#include <cmath>

#include "edg_common.cuh"

namespace edg {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return EDG_OK;
}

int make_glm(const edg_glm_t* g, GLMDev* out) {
  EDG_REQUIRE(g != nullptr, EDG_E_NULL, "model descriptor is NULL");
  EDG_REQUIRE(g->X && g->y && g->prior_loc && g->prior_scale, EDG_E_NULL,
              "model X, y, prior_loc and prior_scale must be device pointers");
  EDG_REQUIRE(g->N > 0 && g->D > 0, EDG_E_SHAPE, "model needs N > 0 and D > 0 (got N=%d D=%d)",
              g->N, g->D);
  EDG_REQUIRE(g->bias == 0 || g->bias == 1, EDG_E_VALUE, "bias must be 0 or 1");
  EDG_REQUIRE(g->lik == EDG_LIK_BERNOULLI || g->lik == EDG_LIK_NORMAL, EDG_E_UNSUPPORTED,
              "unknown likelihood %d", g->lik);
  const int P = g->D + g->bias;
  EDG_REQUIRE(P <= 256, EDG_E_UNSUPPORTED, "GLM kernels support P = D + bias <= 256 (got %d)", P);
  if (g->lik == EDG_LIK_NORMAL)
    EDG_REQUIRE(g->lik_scale > 0.0f && std::isfinite(g->lik_scale), EDG_E_VALUE,
                "Normal likelihood scale must be positive and finite");
  out->X = g->X;
  out->y = g->y;
  out->prior_loc = g->prior_loc;
  out->prior_scale = g->prior_scale;
  out->N = g->N;
  out->D = g->D;
  out->P = P;
  out->PP = round_up(P, 4);
  out->bias = g->bias;
  out->lik = g->lik;
  const float s = g->lik == EDG_LIK_NORMAL ? g->lik_scale : 1.0f;
  out->inv_lik_var = 1.0f / (s * s);
  out->lik_norm = (float)(std::log((double)s) + kHalfLog2Pi);
  return EDG_OK;
}

__global__ void philox_u32_kernel(uint64_t seed, uint32_t kind, uint32_t iter, int rows, int nq,
                                  uint32_t* out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)rows * nq) return;
  const int row = (int)(i / nq), q = (int)(i % nq);
  const uint4 r = philox_at(seed, kind, iter, row, q);
  reinterpret_cast<uint4*>(out)[i] = r;
}

__global__ void philox_normal_kernel(uint64_t seed, uint32_t kind, uint32_t iter, int rows, int n,
                                     float* out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)rows * n) return;
  const int row = (int)(i / n), e = (int)(i % n);
  out[i] = philox_normal(seed, kind, iter, row, e);
}

__global__ void philox_uniform64_kernel(uint64_t seed, uint32_t kind, uint32_t iter, int rows,
                                        double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  out[i] = u01d(philox_at(seed, kind, iter, i, 0).x);
}

}  // namespace edg

using namespace edg;

extern "C" int edg_abi_version(void) { return EDG_ABI_VERSION; }

extern "C" const char* edg_last_error_string(void) { return g_err; }

extern "C" int edg_device_info(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  int v = 0;
  if (sm_count) {
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    *sm_count = v;
  }
  if (cc_major) {
    cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMajor, dev);
    *cc_major = v;
  }
  if (cc_minor) {
    cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMinor, dev);
    *cc_minor = v;
  }
  return EDG_OK;
}

extern "C" int edg_philox_u32(uint64_t seed, uint32_t kind, uint32_t iteration, int32_t rows,
                              int32_t n, uint32_t* out, void* stream) {
  EDG_REQUIRE(out, EDG_E_NULL, "out is NULL");
  EDG_REQUIRE(rows >= 0 && n >= 0, EDG_E_SHAPE, "rows and n must be >= 0");
  const int nq = (n + 3) / 4;
  const int64_t total = (int64_t)rows * nq;
  if (total == 0) return EDG_OK;
  philox_u32_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      seed, kind, iteration, rows, nq, out);
  return check_launch("edg_philox_u32");
}

extern "C" int edg_philox_normal(uint64_t seed, uint32_t kind, uint32_t iteration, int32_t rows,
                                 int32_t n, float* out, void* stream) {
  EDG_REQUIRE(out, EDG_E_NULL, "out is NULL");
  EDG_REQUIRE(rows >= 0 && n >= 0, EDG_E_SHAPE, "rows and n must be >= 0");
  const int64_t total = (int64_t)rows * n;
  if (total == 0) return EDG_OK;
  philox_normal_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      seed, kind, iteration, rows, n, out);
  return check_launch("edg_philox_normal");
}

extern "C" int edg_philox_uniform64(uint64_t seed, uint32_t kind, uint32_t iteration,
                                    int32_t rows, double* out, void* stream) {
  EDG_REQUIRE(out, EDG_E_NULL, "out is NULL");
  EDG_REQUIRE(rows >= 0, EDG_E_SHAPE, "rows must be >= 0");
  if (rows == 0) return EDG_OK;
  philox_uniform64_kernel<<<(rows + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
      seed, kind, iteration, rows, out);
  return check_launch("edg_philox_uniform64");
}
