// BF16 GEMM on the 5th-generation tensor cores: D[m][n] = sum_k A[m][k] * B[n][k] (both operands
// K-major, row-major in memory), FP32 accumulation in tensor memory, FP32 output.
//
// The dense layers of the learned update network are convolutions lowered to this GEMM (forward:
// columns x weights; data gradient: output gradient x transposed weights; weight gradient:
// transposed columns x transposed output gradient, split along the reduction).
//
// One CTA computes a 128 x 64 tile of D with 128 threads. Thread 0 is the producer and the MMA
// issuer: it keeps STAGES k-tiles (64 wide) in flight with TMA (one 2-D box of 64 elements = 128
// bytes x rows per operand, written with the 128-byte swizzle, the K-major SWIZZLE_128B layout of
// the tensor cores: 8-row x 128-byte atoms), waits for a stage's mbarrier, issues four tcgen05.mma
// (M 128, N 64, K 16; each K slice starts 32 bytes further into the swizzled rows) into the
// TMEM accumulator and commits them to the stage's "empty" mbarrier, which frees the stage for the
// next copy. After the last k-tile the four warps read the accumulator back with tcgen05.ld (warp w
// owns TMEM lanes 32w..32w+31 = rows of the tile) and store it. Every wait is bounded: on time-out
// the CTA records an error in the status word, waits (bounded) for its own work in flight, frees
// its tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "wave_launch.h"
#include "wgnet_gb300.h"

namespace wg {
namespace {

constexpr int BM = 128, BN = 64, BK = 64, STAGES = 4, NTHR = 128;
constexpr unsigned kStageA = BM * BK * 2, kStageB = BN * BK * 2;  // bytes
constexpr long kGemmWaitLimit = 1L << 22;

__device__ __forceinline__ unsigned su32(const void* p) { return static_cast<unsigned>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void bar_init(uint64_t* b, unsigned n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool bar_wait(uint64_t* b, unsigned parity) {
  const unsigned a = su32(b);
  for (long i = 0; i < kGemmWaitLimit; ++i) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tma2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(su32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(su32(b))
      : "memory");
}

// Shared-memory matrix descriptor, K-major with the 128-byte swizzle: rows of 128 bytes, atoms of
// 8 rows (sbo = 1024 bytes between atoms along M/N; lbo unused for this layout, encoded as 1). The
// tile base is 1024-byte aligned, so the base-offset field stays 0.
__device__ __forceinline__ uint64_t sdesc_sw128(const void* p) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((su32(p) >> 4) & 0x3FFF);
  d |= static_cast<uint64_t>(1) << 16;              // leading byte offset (unused), 16 bytes
  d |= static_cast<uint64_t>(1024 >> 4) << 32;      // stride byte offset: 8 rows x 128 bytes
  d |= static_cast<uint64_t>(1) << 46;              // descriptor version for the 5th-generation tensor cores
  d |= static_cast<uint64_t>(2) << 61;              // layout: 128-byte swizzle
  return d;
}

// Instruction descriptor of kind::f16: BF16 A and B, FP32 D, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4)                                 // D format F32
         | (1u << 7)                               // A format BF16
         | (1u << 10)                              // B format BF16
         | (static_cast<uint32_t>(n >> 3) << 17)   // N / 8
         | (static_cast<uint32_t>(m >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(b)) : "memory");
}

struct GemmArgs {
  int M, N, K;          // D is M x N; K a multiple of BK
  int k_tiles_per_split;
  float* D;             // [splits][M][N] when split, else [M][N]
  int ldd;              // row stride of D (floats)
  int* status;
};

__global__ void __launch_bounds__(NTHR, 1) gemm_bf16_kernel(const __grid_constant__ CUtensorMap mapA,
                                                            const __grid_constant__ CUtensorMap mapB,
                                                            const __grid_constant__ GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024 - (su32(smem_raw) & 1023)) & 1023);
  unsigned char* sA = smem;                              // [STAGES][BM][128 B], swizzled
  unsigned char* sB = smem + STAGES * kStageA;           // [STAGES][BN][128 B], swizzled
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + STAGES * kStageB);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  __shared__ int fail;

  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int kt0 = blockIdx.z * g.k_tiles_per_split;
  const int KT = min(g.k_tiles_per_split, g.K / BK - kt0);
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      bar_init(&full[s], 1);
      bar_init(&empty[s], 1);
    }
    bar_init(done, 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)), "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (tid == 0 && KT > 0) {
    // per stage: copies issued / consumed, MMA commits issued / waited (for the drain on failure)
    int issued[STAGES] = {}, consumed[STAGES] = {}, commits[STAGES] = {}, freed[STAGES] = {};
    auto load = [&](int kt, int s) {
      bar_expect(&full[s], kStageA + kStageB);
      const int kx = (kt0 + kt) * BK;
      tma2d(sA + s * kStageA, &mapA, kx, m0, &full[s]);
      tma2d(sB + s * kStageB, &mapB, kx, n0, &full[s]);
      ++issued[s];
    };
    const int pre = KT < STAGES ? KT : STAGES;
    for (int kt = 0; kt < pre; ++kt) load(kt, kt);
    constexpr uint32_t idesc = idesc_bf16(BM, BN);
    bool ok = true;
    for (int kt = 0; kt < KT; ++kt) {
      const int s = kt % STAGES;
      if (!bar_wait(&full[s], consumed[s] & 1)) {
        ok = false;
        break;
      }
      ++consumed[s];
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        // K slice kk: 16 elements = 32 bytes further into every (swizzled) 128-byte row
        const uint64_t a = sdesc_sw128(sA + s * kStageA + kk * 32);
        const uint64_t b = sdesc_sw128(sB + s * kStageB + kk * 32);
        mma_bf16(tmem, a, b, idesc, (kt > 0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(&empty[s]);
      ++commits[s];
      if (kt + STAGES < KT) {
        if (!bar_wait(&empty[s], freed[s] & 1)) {
          ok = false;
          break;
        }
        ++freed[s];
        load(kt + STAGES, s);
      }
    }
    if (ok) {
      mma_commit(done);
    } else {
      fail = 1;
      atomicCAS(g.status, 0, ST_CUDA);
      // drain (bounded): copies still landing and MMAs still reading shared memory / writing TMEM
      for (int s = 0; s < STAGES; ++s) {
        if (issued[s] > consumed[s]) bar_wait(&full[s], consumed[s] & 1);
        if (commits[s] > freed[s]) bar_wait(&empty[s], freed[s] & 1);
      }
    }
  }
  __syncthreads();
  bool have = !fail && KT > 0;
  if (have && !bar_wait(done, 0)) {
    have = false;
    atomicCAS(g.status, 0, ST_CUDA);
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // epilogue: warp w reads TMEM lanes 32w..32w+31 (tile rows), 64 columns, into a [BM][BN + 4]
  // staging tile in shared memory (the pipeline buffers, idle now), then the warps write whole rows
  // of the tile (coalesced 256-byte rows)
  float* stile = reinterpret_cast<float*>(smem);
  constexpr int LD = BN + 4;
  const int lrow = warp * 32 + (tid & 31);
#pragma unroll
  for (int c0 = 0; c0 < BN; c0 += 16) {
    uint32_t r[16];
    const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + c0;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j += 4)
      *reinterpret_cast<float4*>(stile + lrow * LD + c0 + j) =
          have ? make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]), __uint_as_float(r[j + 2]),
                             __uint_as_float(r[j + 3]))
               : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncthreads();
  float* dtile = g.D + static_cast<size_t>(blockIdx.z) * g.M * g.ldd + static_cast<size_t>(m0) * g.ldd + n0;
  const int ncols = min(BN, g.N - n0);
  for (int e = tid; e < BM * (BN / 4); e += NTHR) {
    const int rr = e / (BN / 4), c4 = (e % (BN / 4)) * 4;
    if (m0 + rr >= g.M) continue;
    const float4 v = *reinterpret_cast<const float4*>(stile + rr * LD + c4);
    float* dst = dtile + static_cast<size_t>(rr) * g.ldd + c4;
    if (c4 + 3 < ncols) {
      *reinterpret_cast<float4*>(dst) = v;
    } else {
      const float vv[4] = {v.x, v.y, v.z, v.w};
      for (int q = 0; q < 4; ++q)
        if (c4 + q < ncols) dst[q] = vv[q];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
}

PFN_cuTensorMapEncodeTiled_v12000 encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 2-D map over a row-major [rows][K] bf16 matrix, boxes of 64 elements (128 bytes) x box_rows,
// written to shared memory with the 128-byte swizzle.
int map_bf16(CUtensorMap* m, const void* base, long rows, long K, int box_rows) {
  auto fn = encode();
  if (!fn) return report_error(WG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(K), static_cast<cuuint64_t>(rows)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(K) * 2};
  const cuuint32_t box[2] = {BK, static_cast<cuuint32_t>(box_rows)};
  const cuuint32_t es[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return report_error(WG_ERR_CUDA, ("cuTensorMapEncodeTiled(bf16) failed: " + std::to_string(r)).c_str());
  return WG_OK;
}

constexpr size_t kGemmSmem = STAGES * (kStageA + kStageB) + (2 * STAGES + 1) * 8 + 16 + 1024;

}  // namespace

int gemm_bf16(const void* A, const void* B, float* D, int M, int N, int K, int splits, int* status, cudaStream_t st) {
  if (!A || !B || !D || M < 1 || N < 1 || K < BK || K % BK != 0 || splits < 1 || N % 4 != 0)
    return report_error(WG_ERR_ARG, "gemm: bad shape (K must be a positive multiple of 64, N of 4)");
  if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15)
    return report_error(WG_ERR_ARG, "gemm: operands must be 16-byte aligned");
  CUtensorMap ma, mb;
  int rc = map_bf16(&ma, A, M, K, BM);
  if (rc != WG_OK) return rc;
  if ((rc = map_bf16(&mb, B, N, K, BN)) != WG_OK) return rc;
  static bool attr[64] = {};  // the shared-memory attribute is set once per device
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return report_error(WG_ERR_CUDA, "no device");
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(gemm_bf16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(kGemmSmem));
    if (e != cudaSuccess) return report_error(WG_ERR_CUDA, cudaGetErrorString(e));
    attr[dev] = true;
  }
  const int KT = K / BK;
  const int per = (KT + splits - 1) / splits;
  GemmArgs g{M, N, K, per, D, N, status};
  dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN, (KT + per - 1) / per);
  note_launch();
  gemm_bf16_kernel<<<grid, NTHR, kGemmSmem, st>>>(ma, mb, g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return report_error(WG_ERR_CUDA, cudaGetErrorString(e));
  return WG_OK;
}

}  // namespace wg

extern "C" int wg_gemm_bf16_dev(const void* d_a, const void* d_b, float* d_d, int m, int n, int k, int splits,
                                int* d_status, void* stream) {
  return wg::gemm_bf16(d_a, d_b, d_d, m, n, k, splits, d_status, static_cast<cudaStream_t>(stream));
}
