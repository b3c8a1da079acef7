// BF16 tensor-core GEMM for sm_103a: tcgen05.mma with TMEM accumulators,
// operands staged by TMA.
//
//   D[m][n] = sum_k A[m][k] * B[n][k]      A: M x K, B: N x K, bf16, both
//                                          K-contiguous ("TN"); D fp32
//
// One CTA computes a 128 x BN tile with 4 warps:
//   warp 0 / lane 0  TMA producer: 128x64 A and BNx64 B tiles per K block,
//                    128-byte swizzle, STAGES-deep ring of shared buffers;
//   warp 1 / lane 0  MMA issuer: four tcgen05.mma (K = 16 each) per K
//                    block into one FP32 accumulator in TMEM, then
//                    tcgen05.commit to free the stage;
//   warp 2           allocates / frees the TMEM columns;
//   all four warps   epilogue: tcgen05.ld of their 32 accumulator lanes,
//                    passed to an epilogue functor (row, first column,
//                    32 fp32 values).
// Every mbarrier wait is bounded; on expiry the CTA records
// STATUS_GEMM_TIMEOUT in the status word, skips its epilogue, and still
// releases its TMEM.
//
// Users: the stoichiometric contraction of large mechanisms
// (wdot[k][s] = sum_r nu_kr q_sr, q split into bf16 hi + lo) and the
// surrogate network's layers.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "../../include/crs.h"
#include "crs_gemm.cuh"
#include "crs_internal.cuh"

namespace crs {

// ---- host side ------------------------------------------------------------

namespace {
using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                              const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                              const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  }
  return fn;
}
}  // namespace

bool make_tmap_bf16(CUtensorMap *map, const void *ptr, int64_t rows, int64_t cols,
                    int box_rows) {
  EncodeFn fn = encode_fn();
  if (!fn) return false;
  if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (cols * 2) % 16 || cols % gemm::BK ||
      box_rows < 1 || box_rows > 256)
    return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {(cuuint32_t)gemm::BK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides,
            box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Contraction of a chunk: wdot[n][row] += sum_k A[row][k] * B[n][k] * 2^e[row].
cudaError_t launch_gemm_wdot(const void *A, const void *B, int64_t M_pad, int64_t N_pad,
                             int64_t K, int block_n, double *out, int64_t ld, int m_valid,
                             int n_valid, const int *escale, int32_t *status,
                             cudaStream_t s) {
  CUtensorMap ta, tb;
  if (!make_tmap_bf16(&ta, A, M_pad, K, gemm::BM) || !make_tmap_bf16(&tb, B, N_pad, K, block_n))
    return cudaErrorInvalidValue;
  gemm::EpiWdot epi{out, ld, m_valid, n_valid, escale};
  switch (block_n) {
    case 64: return launch_gemm<64>(ta, tb, M_pad, N_pad, K, epi, status, s);
    case 128: return launch_gemm<128>(ta, tb, M_pad, N_pad, K, epi, status, s);
    case 192: return launch_gemm<192>(ta, tb, M_pad, N_pad, K, epi, status, s);
    case 256: return launch_gemm<256>(ta, tb, M_pad, N_pad, K, epi, status, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace crs

extern "C" int crs_gemm_bf16(const void *A, const void *B, float *D, int64_t M, int64_t N,
                             int64_t K, int64_t ldd, int block_n, int32_t *status,
                             void *stream) {
  using namespace crs;
  if (!A || !B || !D || M <= 0 || N <= 0 || K <= 0 || ldd < N) return CRS_ERR_ARG;
  if (M % gemm::BM || K % gemm::BK || N % block_n) return CRS_ERR_ARG;
  CUtensorMap ta, tb;
  if (!make_tmap_bf16(&ta, A, M, K, gemm::BM) || !make_tmap_bf16(&tb, B, N, K, block_n))
    return CRS_ERR_ARG;
  gemm::EpiStoreF32 epi{D, ldd, (int)M, (int)N};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  switch (block_n) {
    case 64: e = launch_gemm<64>(ta, tb, M, N, K, epi, status, s); break;
    case 128: e = launch_gemm<128>(ta, tb, M, N, K, epi, status, s); break;
    case 192: e = launch_gemm<192>(ta, tb, M, N, K, epi, status, s); break;
    case 256: e = launch_gemm<256>(ta, tb, M, N, K, epi, status, s); break;
    default: return CRS_ERR_ARG;
  }
  return e == cudaSuccess ? CRS_OK : CRS_ERR_CUDA;
}
