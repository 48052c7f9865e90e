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
