// Batched FP32 GEMM entry point over the two GEMM engines used by the
// network steps (tensor-core 3xTF32 and SIMT FP32), for tests and callers
// that need the building block on its own.
#define EDG_GEMM_TC_IMPL
#include "edg_common.cuh"
#include "gemm_simt.cuh"
#include "gemm_tc.cuh"

namespace edg {
namespace tcg {

// The tensor-core GEMM kernels live in this translation unit only (their
// launch attributes are set once per kernel here); the network steps call the
// instantiations below.
#define EDG_TC_GEMM(TA, TB, EPI)                                                               \
  template int gemm<TA, TB, EPI>(const float*, const float*, float*, int, int, int, int, int, \
                                 int, int64_t, int64_t, int64_t, int, EPI, int, float*,       \
                                 unsigned*, cudaStream_t);
EDG_TC_GEMM(false, false, simt::EpiIdentity)
EDG_TC_GEMM(false, false, simt::EpiTanh)
EDG_TC_GEMM(true, false, simt::EpiIdentity)
EDG_TC_GEMM(false, true, simt::EpiIdentity)
EDG_TC_GEMM(false, true, simt::EpiTanhGrad)
EDG_TC_GEMM(true, true, simt::EpiIdentity)
#undef EDG_TC_GEMM

int sum_partials(const float* part, int splits, int batch, int M, int N, float* C, int ldc,
                 int64_t sC, cudaStream_t st) {
  const int64_t total = (int64_t)M * N * batch;
  splitk_sum_kernel<<<(int)std::min<int64_t>((total + 255) / 256, 8 * sm_count()), 256, 0, st>>>(
      part, splits, batch, M, N, C, ldc, sC, simt::EpiIdentity{});
  return check_launch("splitk_sum_kernel");
}

}  // namespace tcg
}  // namespace edg

namespace edg {
// Result word of the bounded-wait self test.
__device__ int32_t g_selftest_word;
}  // namespace edg

using namespace edg;

extern "C" size_t edg_gemm_workspace_bytes(int32_t engine, int32_t M, int32_t N, int32_t K,
                                           int32_t batch, int32_t kchunk) {
  if (engine != EDG_GEMM_TC) return 0;
  return tcg::part_floats(M, N, K, batch, kchunk) * sizeof(float);
}

extern "C" int edg_gemm(int32_t engine, int32_t ta, int32_t tb, int32_t M, int32_t N, int32_t K,
                        const float* A, int32_t lda, int64_t sA, const float* B, int32_t ldb,
                        int64_t sB, float* C, int32_t ldc, int64_t sC, int32_t batch,
                        int32_t kchunk, void* workspace, size_t workspace_bytes, void* stream) {
  EDG_REQUIRE(A && B && C, EDG_E_NULL, "pointers must not be NULL");
  EDG_REQUIRE(M > 0 && N > 0 && K > 0 && batch > 0, EDG_E_SHAPE, "sizes must be positive");
  EDG_REQUIRE(engine == EDG_GEMM_TC || engine == EDG_GEMM_SIMT, EDG_E_VALUE, "unknown engine %d",
              engine);
  cudaStream_t st = (cudaStream_t)stream;
  if (engine == EDG_GEMM_SIMT) {
    if (!ta && !tb)
      return simt::bgemm<false, false>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch,
                                       simt::EpiIdentity{}, st);
    if (ta && !tb)
      return simt::bgemm<true, false>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch,
                                      simt::EpiIdentity{}, st);
    if (!ta && tb)
      return simt::bgemm<false, true>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch,
                                      simt::EpiIdentity{}, st);
    return simt::bgemm<true, true>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch,
                                   simt::EpiIdentity{}, st);
  }
  const size_t need = tcg::part_floats(M, N, K, batch, kchunk) * sizeof(float);
  EDG_REQUIRE(need == 0 || (workspace && workspace_bytes >= need), EDG_E_WORKSPACE,
              "workspace of %zu bytes needed (got %zu)", need, workspace_bytes);
  float* part = reinterpret_cast<float*>(workspace);
  if (!ta && !tb)
    return tcg::gemm<false, false>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch,
                                   simt::EpiIdentity{}, kchunk, part, nullptr, st);
  if (ta && !tb)
    return tcg::gemm<true, false>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch,
                                  simt::EpiIdentity{}, kchunk, part, nullptr, st);
  if (!ta && tb)
    return tcg::gemm<false, true>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch,
                                  simt::EpiIdentity{}, kchunk, part, nullptr, st);
  return tcg::gemm<true, true>(A, B, C, M, N, K, lda, ldb, ldc, sA, sB, sC, batch,
                               simt::EpiIdentity{}, kchunk, part, nullptr, st);
}

extern "C" int edg_gemm_status(int32_t* status, void* stream) {
  EDG_REQUIRE(status, EDG_E_NULL, "status must not be NULL");
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "edg_gemm_status: %s", cudaGetErrorString(e));
  unsigned v = 0;
  e = cudaMemcpyFromSymbol(&v, tcg::g_gemm_err, sizeof(v));
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "edg_gemm_status: %s", cudaGetErrorString(e));
  const unsigned zero = 0;
  e = cudaMemcpyToSymbol(tcg::g_gemm_err, &zero, sizeof(zero));
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "edg_gemm_status: %s", cudaGetErrorString(e));
  *status = v ? -(int32_t)v : EDG_OK;  // the kernels store -EDG_E_TIMEOUT
  return EDG_OK;
}

// ---------------------------------------------------------------- bounded-wait self test
namespace edg {
// One warp waits on an mbarrier that nothing arrives on, with the bounded
// wait every tensor-core kernel uses; the wait gives up after ~2^31 cycles
// (about one second) and the timeout is recorded in *out.
__global__ void bounded_wait_selftest_kernel(int32_t* out) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ volatile int err;
  if (threadIdx.x == 0) {
    ptx::mbar_init(ptx::smem_u32(&bar), 1);
    err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  ptx::mbar_wait(ptx::smem_u32(&bar), 0, &err);
  __syncthreads();
  if (threadIdx.x == 0) *out = err ? EDG_E_TIMEOUT : EDG_OK;
}
}  // namespace edg

extern "C" int edg_check_bounded_wait(int32_t* status, void* stream) {
  EDG_REQUIRE(status, EDG_E_NULL, "status must not be NULL");
  int32_t* d = nullptr;
  void* a = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&a, g_selftest_word);
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "edg_check_bounded_wait: %s", cudaGetErrorString(e));
  d = reinterpret_cast<int32_t*>(a);
  cudaStream_t st = (cudaStream_t)stream;
  bounded_wait_selftest_kernel<<<1, 32, 0, st>>>(d);
  int rc = check_launch("bounded_wait_selftest_kernel");
  if (rc) return rc;
  e = cudaMemcpyAsync(status, d, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(EDG_E_CUDA, "edg_check_bounded_wait: %s", cudaGetErrorString(e));
  return EDG_OK;
}
