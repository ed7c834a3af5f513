// BF16 Gram tiles on the 5th-generation tensor cores: TMA loads of K-major
// 128-row operand tiles (128-byte swizzle) into shared memory, tcgen05.mma
// (M = N = 128, K = 16 per instruction) accumulating in TMEM, tcgen05.ld back
// to registers. culof_bf16_gram exposes the tile product G = A B^T
// (f32 accumulation) as a stage entry point; the precision form of the k-NN
// builds on the same pieces.
#include <cudaTypedefs.h>

#include <mutex>

#include "../../include/culof_c.h"
#include "common.cuh"
#include "tc.cuh"
#include "tc_host.cuh"

namespace culof_gb300 {
namespace tc {

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    if (fn == nullptr) throw Error(kCudaError, "cuTensorMapEncodeTiled is not available from the driver");
    return fn;
}

}  // namespace

CUtensorMap make_kmajor_map(const void* base, int64_t rows, int K, bool fp16) {
    if (K % 64 != 0) throw Error(kInvalidArgument, "K must be a multiple of 64");
    if (reinterpret_cast<uintptr_t>(base) % 16 != 0) throw Error(kInvalidArgument, "operand base must be 16-byte aligned");
    CUtensorMap map;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(K), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(K) * 2};
    const cuuint32_t box[2] = {64, 128};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(&map, fp16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(kCudaError, "cuTensorMapEncodeTiled failed");
    return map;
}

namespace {

constexpr int kHalf = 128 * 128;  // one K-half of a 128-row operand tile: 128 rows x 128 bytes

struct GramSmem {
    uint8_t a[2][kHalf];
    uint8_t b[2][kHalf];
    uint64_t tma_bar;
    uint64_t mma_bar;
    uint32_t tmem_base;
};

// One 128 x 128 tile of G = A B^T for K = 128 per CTA (4 warps).
__global__ void __launch_bounds__(128)
bf16_gram_tile_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, float* G,
                      int64_t ldg, int* status) {
    extern __shared__ uint8_t raw[];
    GramSmem& sh = *reinterpret_cast<GramSmem*>((reinterpret_cast<uintptr_t>(raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * 128, col0 = blockIdx.y * 128;
    if (threadIdx.x == 0) {
        sweep::mbar_init(&sh.tma_bar, 1);
        sweep::mbar_init(&sh.mma_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(&sh.tmem_base, 128);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh.tmem_base;

    if (threadIdx.x == 0) {
        sweep::mbar_expect_tx(&sh.tma_bar, 4 * kHalf);
        tma_load_2d(sh.a[0], &ta, 0, row0, &sh.tma_bar);
        tma_load_2d(sh.a[1], &ta, 64, row0, &sh.tma_bar);
        tma_load_2d(sh.b[0], &tb, 0, col0, &sh.tma_bar);
        tma_load_2d(sh.b[1], &tb, 64, col0, &sh.tma_bar);
        if (sweep::mbar_wait(&sh.tma_bar, 0)) {
            tc_fence_after();
            constexpr uint32_t idesc = bf16_idesc(128, 128);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int half = k >> 2, sub = k & 3;
                const uint64_t ad = sw128_desc(smem_u32(sh.a[half]) + 32 * sub);
                const uint64_t bd = sw128_desc(smem_u32(sh.b[half]) + 32 * sub);
                mma_f16kind(tmem, ad, bd, idesc, k > 0);
            }
            mma_commit(&sh.mma_bar);
        }
    }
    const bool done = sweep::mbar_wait(&sh.mma_bar, 0);
    tc_fence_after();
    if (done) {
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(32 * warp) << 16);
        float* grow = G + (static_cast<int64_t>(row0) + 32 * warp + lane) * ldg + col0;
#pragma unroll
        for (int c0 = 0; c0 < 128; c0 += 32) {
            float v[32];
            tmem_ld32(lane_addr + c0, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) grow[c0 + i] = v[i];
        }
    } else if (threadIdx.x == 0) {
        atomicExch(status, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 128);
}

}  // namespace

void bf16_gram(const void* A, int64_t rows_a, const void* B, int64_t rows_b, int K, float* G, int* status,
               cudaStream_t s) {
    if (K != 128) throw Error(kInvalidArgument, "the tile kernel takes K = 128");
    if (rows_a % 128 || rows_b % 128) throw Error(kInvalidArgument, "row counts must be multiples of 128");
    const CUtensorMap ta = make_kmajor_bf16_map(A, rows_a, K);
    const CUtensorMap tb = make_kmajor_bf16_map(B, rows_b, K);
    const size_t smem = sizeof(GramSmem) + 1024;
    CG_CUDA(cudaFuncSetAttribute(bf16_gram_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem)));
    dim3 grid(static_cast<unsigned>(rows_a / 128), static_cast<unsigned>(rows_b / 128));
    bf16_gram_tile_kernel<<<grid, 128, smem, s>>>(ta, tb, G, rows_b, status);
    CG_LAUNCH_CHECK();
}

}  // namespace tc
}  // namespace culof_gb300
