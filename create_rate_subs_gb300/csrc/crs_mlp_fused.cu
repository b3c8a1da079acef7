// Surrogate network inference in one kernel: every layer of the MLP for a
// tile of 128 states, with the activations kept in shared memory.
//
// The layer-by-layer path (crs_mlp.cu) writes each layer's bf16 activations
// to HBM and reads them back for the next GEMM, ~1 KB per state and layer;
// here a CTA keeps its 128 x width activation tile on chip between layers,
// so per state only the input features are read and the output written.
//
// One CTA = 128 states, 6 warps:
//   warp 4 / lane 0  TMA producer: the tile's input features into the
//                    activation buffer, then every layer's weights in
//                    blocks of <= 128 rows x 64 columns through a two-slot
//                    ring (the weights do not depend on the activations, so
//                    the next layer's first blocks load during an epilogue);
//   warp 5 / lane 0  MMA issuer: per layer, per 64-wide K block and per
//                    128-column half of the layer's outputs, four
//                    tcgen05.mma (K = 16) into the FP32 accumulator in TMEM
//                    (columns 0..255), then tcgen05.commit;
//   warps 0-3        epilogue: tcgen05.ld of their 32 accumulator lanes,
//                    + bias, SiLU, bf16, written back into the activation
//                    buffer in the 128-byte-swizzled K-major layout that the
//                    next layer's MMAs read (the layout TMA writes), or, for
//                    the last layer, + bias to the fp32 output in HBM.
// The activation buffer is both a layer's input and, after that layer's
// MMAs have completed, its output: one buffer per CTA, 64 KB for widths up
// to 256, so two CTAs share an SM and one's epilogue overlaps the other's
// MMAs.  Every mbarrier wait is bounded; on expiry the CTA records
// STATUS_GEMM_TIMEOUT, skips the rest of its work, waits (bounded) for its
// TMA loads in flight and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "../../include/crs.h"
#include "crs_gemm.cuh"
#include "crs_internal.cuh"

namespace crs {
namespace mlpf {

constexpr int MAXL = 6;           // layers
constexpr int MAXW = 256;         // widest layer input / output (padded)
constexpr int BLK = 128 * 64 * 2;  // one 128-row x 64-column bf16 block: 16 KB
constexpr int RING = 2;
constexpr int NT = 192;

struct Maps {
  CUtensorMap x;
  CUtensorMap w[MAXL];
};

struct Net {
  int L;
  int pad[MAXL + 1];  // padded widths (multiples of 64, <= 256)
  int dim[MAXL + 1];  // true widths
  const float *bias[MAXL];
  int m_valid;
  float *Y;
  int64_t ldy;
  int32_t *status;
};

__device__ __forceinline__ uint32_t idesc_n(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ float silu(float z) {
  return z * __fdividef(1.0f, 1.0f + __expf(-z));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// 32 consecutive accumulator columns of the thread's TMEM lane, without
// waiting (tcgen05.wait::ld before the registers are read)
__device__ __forceinline__ void ld32_nw(uint32_t taddr, uint32_t *v) {
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
}

// tcgen05.wait::ld, then an empty asm that rewrites v: reads of v are
// ordered after the wait (the registers of an outstanding TMEM load hold
// garbage until then)
__device__ __forceinline__ void wait_ld(uint32_t (&v)[32]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  asm volatile(""
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]),
                 "+r"(v[6]), "+r"(v[7]), "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]),
                 "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15]), "+r"(v[16]), "+r"(v[17]),
                 "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]), "+r"(v[22]), "+r"(v[23]),
                 "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]), "+r"(v[29]),
                 "+r"(v[30]), "+r"(v[31]));
}

__device__ __forceinline__ void arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__global__ void __launch_bounds__(NT, 2)
    k_mlp_infer(const __grid_constant__ Maps maps, Net net) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[RING], empty[RING], xfull, mdone, aready;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int failed, consumed;
  __shared__ __align__(16) float sbias[MAXL * MAXW];  // zero past each layer's width
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char *act = base;                          // pad/64 blocks of 16 KB
  unsigned char *ring = base + (MAXW / 64) * BLK;    // RING blocks of 16 KB
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * 128;
  const int L = net.L;

  if (threadIdx.x == 0) {
    for (int s = 0; s < RING; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&xfull)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mdone)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(smem_u32(&aready)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    failed = 0;
    consumed = 0;
  }
  for (int l = 0; l < L; ++l)
    for (int i = threadIdx.x; i < net.pad[l + 1]; i += NT)
      sbias[l * MAXW + i] = i < net.dim[l + 1] ? net.bias[l][i] : 0.0f;
  if (warp == 4) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(256u)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  int issued = 0;

  if (warp == 4 && lane == 0) {
    // ---- TMA producer ----
    const int kx = net.pad[0] / 64;
    gemm::expect_tx(&xfull, (uint32_t)(kx * BLK));
    for (int kb = 0; kb < kx; ++kb) gemm::tma_2d(act + kb * BLK, &maps.x, kb * 64, m0, &xfull);
    for (int l = 0; l < L && !failed; ++l) {
      const int nk = net.pad[l] / 64, nn = net.pad[l + 1];
      const int rows = nn < 128 ? nn : 128;
      for (int kb = 0; kb < nk && !failed; ++kb)
        for (int nh = 0; nh * 128 < nn; ++nh) {
          const int s = issued % RING;
          const uint32_t ph = (uint32_t)(issued / RING) & 1u;
          if (!gemm::wait_bounded(&empty[s], ph ^ 1u)) {
            failed = 1;
            break;
          }
          gemm::expect_tx(&full[s], (uint32_t)(rows * 128));
          gemm::tma_2d(ring + s * BLK, &maps.w[l], kb * 64, nh * 128, &full[s]);
          ++issued;
        }
    }
  } else if (warp == 5 && lane == 0) {
    // ---- MMA issuer ----
    int i = 0;
    if (!gemm::wait_bounded(&xfull, 0)) failed = 1;
    for (int l = 0; l < L && !failed; ++l) {
      if (l > 0 && !gemm::wait_bounded(&aready, (uint32_t)(l - 1) & 1u)) {
        failed = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int nk = net.pad[l] / 64, nn = net.pad[l + 1];
      for (int kb = 0; kb < nk && !failed; ++kb)
        for (int nh = 0; nh * 128 < nn; ++nh) {
          const int s = i % RING;
          const uint32_t ph = (uint32_t)(i / RING) & 1u;
          if (!gemm::wait_bounded(&full[s], ph)) {
            failed = 1;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const int n = nn - nh * 128 < 128 ? nn - nh * 128 : 128;
          const uint32_t id = idesc_n(n);
#pragma unroll
          for (int k4 = 0; k4 < 4; ++k4)
            gemm::mma(tmem + (uint32_t)(nh * 128), gemm::sdesc(act + kb * BLK + k4 * 32),
                      gemm::sdesc(ring + s * BLK + k4 * 32), id, (kb | k4) != 0);
          gemm::commit(&empty[s]);
          ++i;
          consumed = i;
        }
      if (!failed) gemm::commit(&mdone);  // arrives when this layer's MMAs are done
    }
  } else if (warp < 4) {
    // ---- epilogue ----
    const int row = warp * 32 + lane;  // the TMEM lane quarter of warp 0..3
    for (int l = 0; l < L; ++l) {
      if (!gemm::wait_bounded(&mdone, (uint32_t)l & 1u)) {
        failed = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const bool last = l == L - 1;
      const int nn = net.pad[l + 1], nv = net.dim[l + 1];
      const float4 *bias4 = reinterpret_cast<const float4 *>(sbias + l * MAXW);
      // bias, then the fp32 output (last layer) or SiLU -> bf16 into the
      // activation buffer, for accumulator columns c .. c + 31 of the row
      auto process = [&](const uint32_t(&v)[32], int c) {
        float z[32];
#pragma unroll
        for (int t = 0; t < 8; ++t) {  // padded columns: 0 + 0 (zero weights and bias)
          const float4 b = bias4[(c >> 2) + t];
          z[4 * t] = __uint_as_float(v[4 * t]) + b.x;
          z[4 * t + 1] = __uint_as_float(v[4 * t + 1]) + b.y;
          z[4 * t + 2] = __uint_as_float(v[4 * t + 2]) + b.z;
          z[4 * t + 3] = __uint_as_float(v[4 * t + 3]) + b.w;
        }
        if (last) {
          const int gr = m0 + row;
          if (gr < net.m_valid && c < nv) {
            float *y = net.Y + (int64_t)gr * net.ldy + c;
            const int w = nv - c < 32 ? nv - c : 32;  // columns to write
            const int nq = (reinterpret_cast<uintptr_t>(y) & 15) ? 0 : w >> 2;
#pragma unroll
            for (int t = 0; t < 8; ++t)
              if (t < nq)
                reinterpret_cast<float4 *>(y)[t] =
                    make_float4(z[4 * t], z[4 * t + 1], z[4 * t + 2], z[4 * t + 3]);
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (j >= 4 * nq && j < w) y[j] = z[j];
          }
        } else {
          // 32 bf16 = four of the row's 16-byte chunks of K block c / 64,
          // swizzled: chunk j of row r sits at chunk j ^ (r % 8)
          unsigned char *blk = act + (c >> 6) * BLK + row * 128;
          const int j0 = (c & 63) >> 3;
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const float *a = z + 8 * t;
            const uint4 u = make_uint4(pack_bf16(silu(a[0]), silu(a[1])),
                                       pack_bf16(silu(a[2]), silu(a[3])),
                                       pack_bf16(silu(a[4]), silu(a[5])),
                                       pack_bf16(silu(a[6]), silu(a[7])));
            *reinterpret_cast<uint4 *>(blk + (((j0 + t) ^ (row & 7)) << 4)) = u;
          }
        }
      };
      // two 32-column buffers: the TMEM load of the next columns is in
      // flight while the current ones are processed
      const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16);
      uint32_t va[32], vb[32];
      ld32_nw(ta, va);
      wait_ld(va);
      for (int c = 0; c < nn; c += 64) {  // nn is a multiple of 64
        ld32_nw(ta + (uint32_t)(c + 32), vb);
        process(va, c);
        wait_ld(vb);
        if (c + 64 < nn) ld32_nw(ta + (uint32_t)(c + 64), va);
        process(vb, c + 32);
        wait_ld(va);
      }
      if (!last) {
        // generic-proxy stores -> visible to the tensor core's async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        arrive(&aready);
      }
    }
  }
  __syncwarp();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 4 && lane == 0) {
    // a failed CTA still waits for the weight blocks it had requested
    for (int j = consumed; j < issued; ++j)
      gemm::wait_bounded(&full[j % RING], (uint32_t)(j / RING) & 1u);
    if (consumed == 0) gemm::wait_bounded(&xfull, 0);
    if (failed && net.status) atomicOr(&net.status[0], STATUS_GEMM_TIMEOUT);
  }
  if (warp == 4) {
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256u)
                 : "memory");
  }
}

}  // namespace mlpf
}  // namespace crs

namespace {
int infer_error(int code, const char *what) {
  char buf[200];
  snprintf(buf, sizeof buf, "crs_mlp_infer: %s", what);
  return crs::report(code, buf);
}
}  // namespace

extern "C" int crs_mlp_infer(const void *X, int64_t M_pad, int64_t M, int L,
                             const int64_t *dims, const int64_t *pads, const void *const *W,
                             const float *const *b, float *Y32, int64_t ldy,
                             int32_t *status, void *stream) {
  using namespace crs;
  if (!X || !dims || !pads || !W || !b || !Y32 || L < 1 || L > mlpf::MAXL || M < 0 ||
      M > M_pad || M_pad % 128)
    return infer_error(CRS_ERR_ARG, "null pointer, 1 <= L <= 6, or bad row counts "
                                    "(M_pad a multiple of 128)");
  mlpf::Net net{};
  net.L = L;
  for (int l = 0; l <= L; ++l) {
    if (pads[l] < 64 || pads[l] > mlpf::MAXW || pads[l] % 64 || dims[l] < 1 || dims[l] > pads[l])
      return infer_error(CRS_ERR_ARG, "widths must pad to multiples of 64 up to 256");
    net.pad[l] = (int)pads[l];
    net.dim[l] = (int)dims[l];
  }
  if (ldy < dims[L]) return infer_error(CRS_ERR_ARG, "ldy < output width");
  if (M == 0) return CRS_OK;
  mlpf::Maps maps;
  if (!make_tmap_bf16(&maps.x, X, M_pad, pads[0], 128))
    return infer_error(CRS_ERR_ARG, "X must be 16-byte aligned");
  for (int l = 0; l < L; ++l) {
    const int rows = pads[l + 1] < 128 ? (int)pads[l + 1] : 128;
    if (!W[l] || !b[l] || !make_tmap_bf16(&maps.w[l], W[l], pads[l + 1], pads[l], rows))
      return infer_error(CRS_ERR_ARG, "null or unaligned layer weights / bias");
    net.bias[l] = b[l];
  }
  net.m_valid = (int)M;
  net.Y = Y32;
  net.ldy = ldy;
  net.status = status;
  const size_t smem = (size_t)(mlpf::MAXW / 64 + mlpf::RING) * mlpf::BLK + 1024;
  cudaError_t e = cudaFuncSetAttribute(mlpf::k_mlp_infer,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) {
    mlpf::k_mlp_infer<<<(unsigned)(M_pad / 128), mlpf::NT, smem,
                        static_cast<cudaStream_t>(stream)>>>(maps, net);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? CRS_OK : infer_error(CRS_ERR_CUDA, cudaGetErrorString(e));
}
