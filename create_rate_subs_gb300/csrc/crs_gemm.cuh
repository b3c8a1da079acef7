// tcgen05 BF16 GEMM kernel template and its launcher (see crs_gemm.cu for
// the design).  Included by the translation units that instantiate it with
// their own epilogues.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "crs_internal.cuh"

namespace crs {
namespace gemm {

constexpr int BM = 128, BK = 64, STAGES = 4;
constexpr int A_BYTES = BM * BK * 2;  // 16 KB per stage

__device__ __forceinline__ bool wait_bounded(uint64_t *bar, uint32_t parity) {
  const uint32_t b = smem_u32(bar);
  for (int it = 0; it < (1 << 24); ++it)
    if (mbar_try_wait(b, parity)) return true;
  return false;
}

__device__ __forceinline__ void expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void tma_2d(void *dst, const CUtensorMap *map, int x, int y,
                                       uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle,
// 8-row groups 1024 bytes apart (SBO), version 1 (sm_100 family).
__device__ __forceinline__ uint64_t sdesc(const void *p) {
  const uint64_t a = smem_u32(p);
  return ((a >> 4) & 0x3FFFull) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) |
         (1ull << 46) | (2ull << 61);
}

// Instruction descriptor of kind::f16: D fp32, A and B bf16, both K-major,
// M = 128, N = BN.
template <int BN>
__device__ __forceinline__ uint32_t idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t id,
                                    uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
        "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
        "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]),
        "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
        "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int BN>
__host__ __device__ constexpr uint32_t tmem_cols() {
  return BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : BN <= 256 ? 256 : 512;
}

template <int BN, int ST = STAGES>
constexpr size_t smem_bytes() {
  return (size_t)ST * (A_BYTES + BN * BK * 2) + 1024;
}

// One 128 x BN output tile per CTA.  Warp 0 lane 0 issues the TMA loads of
// an ST-deep ring, warp 1 lane 0 the MMAs; then all NT / 32 warps run the
// epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (the quarter its
// rank allows) and, with NT = 256, half of the columns.  ST = 2 and NT = 256
// let two CTAs share an SM (registers capped for two), so one tile's
// epilogue overlaps the next tile's loads and MMAs.
template <int BN, class Epi, int ST = STAGES, int NT = 128>
__global__ void __launch_bounds__(NT, ST <= 2 ? 2 : 1)
    k_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
           int kblocks, Epi epi, int32_t *status) {
  static_assert(NT == 128 || NT == 256, "128 or 256 threads");
  constexpr int B_BYTES = BN * BK * 2;
  constexpr uint32_t NCOL = tmem_cols<BN>();
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[ST], empty[ST], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char *sA = base;
  unsigned char *sB = base + ST * A_BYTES;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    failed = 0;
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(NCOL)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  // split-K: grid z slice z covers K blocks [z * kblocks, (z + 1) * kblocks)
  const int kb0 = blockIdx.z * kblocks;
  int issued = 0;  // K blocks whose TMA loads the producer lane started
  if (warp == 0 && lane == 0) {
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % ST;
      const uint32_t ph = (uint32_t)(kb / ST) & 1u;
      if (!wait_bounded(&empty[s], ph ^ 1u)) {
        failed = 1;
        break;
      }
      expect_tx(&full[s], A_BYTES + B_BYTES);
      tma_2d(sA + s * A_BYTES, &tmA, (kb0 + kb) * BK, m0, &full[s]);
      tma_2d(sB + s * B_BYTES, &tmB, (kb0 + kb) * BK, n0, &full[s]);
      ++issued;
    }
  } else if (warp == 1 && lane == 0) {
    const uint32_t id = idesc<BN>();
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % ST;
      const uint32_t ph = (uint32_t)(kb / ST) & 1u;
      if (!wait_bounded(&full[s], ph)) {
        failed = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int k4 = 0; k4 < BK / 16; ++k4)
        mma(tmem, sdesc(sA + s * A_BYTES + k4 * 32), sdesc(sB + s * B_BYTES + k4 * 32), id,
            (kb | k4) != 0);
      commit(&empty[s]);
    }
    commit(&done);  // arrives once every MMA issued above has completed
  }
  __syncwarp();
  const bool got = wait_bounded(&done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (got && !failed) {
    const int q = warp & 3;
    constexpr int CW = BN / (NT / 128);  // columns per warp
    const int c0 = (warp >> 2) * CW;
    const int row = m0 + q * 32 + lane;
    for (int c = c0; c < c0 + CW; c += 32) {
      uint32_t v[32];
      ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, v);
      epi(row, n0 + c, v);
    }
  } else if (threadIdx.x == 0 && status) {
    atomicOr(&status[0], STATUS_GEMM_TIMEOUT);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  const int gave_up = __syncthreads_or(failed || !got);
  // A CTA that gave up must not free its TMEM while MMAs may still write it,
  // nor leave while TMA loads may still write its shared memory: wait for
  // both once more (bounded, 4x longer).  The latest load of each stage
  // completes last, so its phase covers the stage's earlier loads.
  if (gave_up) {
    if (threadIdx.x == 0) {
      for (int r = 0; r < 4 && !wait_bounded(&done, 0); ++r) {
      }
    }
    if (warp == 0 && lane == 0) {
      for (int kb = issued > ST ? issued - ST : 0; kb < issued; ++kb)
        for (int r = 0; r < 4 && !wait_bounded(&full[kb % ST], (uint32_t)(kb / ST) & 1u); ++r) {
        }
    }
    __syncthreads();
  }
  if (warp == 2) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOL)
                 : "memory");
  }
}

// Row-major fp32 output D[m * ldd + n] (tests and the surrogate network).
struct EpiStoreF32 {
  float *D;
  int64_t ldd;
  int m_valid, n_valid;
  __device__ void operator()(int row, int col0, const uint32_t (&v)[32]) const {
    if (row >= m_valid) return;
#pragma unroll
    for (int j = 0; j < 32; ++j)
      if (col0 + j < n_valid) D[(int64_t)row * ldd + col0 + j] = __uint_as_float(v[j]);
  }
};

// wdot[col * ld + row] += acc * 2^escale[row]: the contraction's epilogue
// (column-major FP64 output: consecutive lanes write consecutive states).
struct EpiWdot {
  double *out;
  int64_t ld;
  int m_valid, n_valid;
  const int *escale;
  __device__ void operator()(int row, int col0, const uint32_t (&v)[32]) const {
    if (row >= m_valid) return;
    const double sc = __hiloint2double((escale[row] + 1023) << 20, 0);
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int col = col0 + j;
      if (col < n_valid) {
        double *o = out + (int64_t)col * ld + row;
        *o = fma((double)__uint_as_float(v[j]), sc, *o);
      }
    }
  }
};

}  // namespace gemm

// 2-D bf16 tensor map over a rows x cols row-major matrix (cols contiguous),
// box = box_rows x 64 columns, 128-byte swizzle.
bool make_tmap_bf16(CUtensorMap *map, const void *ptr, int64_t rows, int64_t cols,
                    int box_rows);

template <int BN, class Epi, int ST = gemm::STAGES, int NT = 128>
cudaError_t launch_gemm(const CUtensorMap &ta, const CUtensorMap &tb, int64_t M_pad,
                        int64_t N_pad, int64_t K, const Epi &epi, int32_t *status,
                        cudaStream_t s, int splits = 1) {
  static_assert((BN / (NT / 128)) % 32 == 0, "columns per warp must be a multiple of 32");
  if (M_pad % gemm::BM || N_pad % BN || K % gemm::BK || K <= 0 || splits < 1 ||
      (K / gemm::BK) % splits)
    return cudaErrorInvalidValue;
  auto k = gemm::k_gemm<BN, Epi, ST, NT>;
  const size_t smem = gemm::smem_bytes<BN, ST>();
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)(M_pad / gemm::BM), (unsigned)(N_pad / BN), (unsigned)splits);
  k<<<grid, NT, smem, s>>>(ta, tb, (int)(K / gemm::BK / splits), epi, status);
  return cudaGetLastError();
}

}  // namespace crs
