// ofx_gemm.cu -- BF16 tensor-core GEMM for the surrogate network (tcgen05 + TMA).
//
// C[M, N] (+)= A[M, K] . B[N, K]^T with A and B row-major BF16 (both K-major),
// FP32 accumulation in tensor memory and FP32 output.  One CTA of 4 warps per
// 128 x 64 output tile: one thread issues the TMA loads of a 4-stage ring of
// 128x64 (A) and 64x64 (B) tiles, one thread issues tcgen05.mma (M=128, N=64,
// K=16 per instruction), and all 128 threads read the accumulator back (one TMEM
// lane per output row).  K can be split over gridDim.z; split partial sums are
// added into C with atomics.  Every wait is bounded: a timeout sets an error flag
// (optifax_tc_error) and the kernel releases its tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/optifax.h"
#include "ofx_tc.cuh"

namespace {

constexpr int BM = 128, BN = 64, BK = 64, STAGES = 4;
constexpr int A_TILE = BM * BK * 2;
constexpr int B_TILE = BN * BK * 2;
constexpr int STAGE_BYTES = A_TILE + B_TILE;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr uint32_t TMEM_COLS = 64;

__device__ int g_tc_err;

struct GemmArgs {
    float* C;
    long long ldc;
    int M, N, K;
    int k_per_split;
    int atomic;
};

__global__ void __launch_bounds__(128, 1)
    gemm_bf16_tn(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
    using namespace ofx_tc;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* tiles =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(tiles + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* accum = empty + STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
    int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
    int* consumed_s = abort_flag + 1;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * g.k_per_split;
    const int kend = min(g.K, kbeg + g.k_per_split);
    const int nk = (kend - kbeg + BK - 1) / BK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        *abort_flag = 0;
        *consumed_s = 0;
        fence_barrier_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    int issued = 0;
    if (threadIdx.x == 0) {
        // TMA producer
        for (int kb = 0; kb < nk; ++kb) {
            const int s = kb % STAGES;
            if (kb >= STAGES && !mbar_wait(&empty[s], ((kb / STAGES) - 1) & 1)) {
                atomicExch(abort_flag, 1);
                break;
            }
            if (*(volatile int*)abort_flag) break;
            unsigned char* sa = tiles + s * STAGE_BYTES;
            mbar_expect_tx(&full[s], STAGE_BYTES);
            tma_load_2d(sa, &tmA, kbeg + kb * BK, m0, &full[s]);
            tma_load_2d(sa + A_TILE, &tmB, kbeg + kb * BK, n0, &full[s]);
            ++issued;
        }
    } else if (threadIdx.x == 32) {
        // MMA issuer
        constexpr uint32_t idesc = idesc_bf16_f32(BM, BN);
        int kb = 0;
        for (; kb < nk; ++kb) {
            const int s = kb % STAGES;
            if (!mbar_wait(&full[s], (kb / STAGES) & 1)) {
                atomicExch(abort_flag, 1);
                break;
            }
            tc_fence_after();
            const uint32_t sa = smem_u32(tiles + s * STAGE_BYTES);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
                const uint64_t ad = desc_kmajor_sw128(sa + kk * 32);
                const uint64_t bd = desc_kmajor_sw128(sa + A_TILE + kk * 32);
                mma_bf16(tmem, ad, bd, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(&empty[s]);
        }
        *consumed_s = kb;
        mma_commit(accum);
    }
    __syncwarp();

    // epilogue: TMEM lane (32 warp + lane) holds output row m0 + 32 warp + lane.  The
    // tile goes through shared memory (the drained stage buffers: every TMA load was
    // consumed by an MMA before the accumulator barrier completed) so that the global
    // stores run along rows: one warp writes two 256-byte row segments per store.
    const bool ok = mbar_wait(accum, 0) && !*(volatile int*)abort_flag;
    __syncwarp();
    tc_fence_after();
    constexpr int LDT = BN + 1;                          // padded row: conflict-free column writes
    float* tile = reinterpret_cast<float*>(tiles);
    const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    const int trow = warp * 32 + lane;
#pragma unroll
    for (int c = 0; c < BN; c += 16) {
        float v[16];
        tmem_ld16(taddr + c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) tile[trow * LDT + c + j] = v[j];
    }
    __syncthreads();
    if (ok) {
        const bool vec = !g.atomic && (g.ldc % 4 == 0) && (n0 + BN <= g.N) &&
                         ((reinterpret_cast<uintptr_t>(g.C) & 15) == 0);
        for (int idx = threadIdx.x; idx < BM * (BN / 4); idx += blockDim.x) {
            const int r = idx / (BN / 4), c4 = (idx % (BN / 4)) * 4;
            const int row = m0 + r;
            if (row >= g.M) continue;
            float* dst = g.C + static_cast<long long>(row) * g.ldc + n0 + c4;
            const float* src = tile + r * LDT + c4;
            if (vec) {
                *reinterpret_cast<float4*>(dst) = make_float4(src[0], src[1], src[2], src[3]);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (n0 + c4 + j < g.N) {
                        if (g.atomic) atomicAdd(dst + j, src[j]);
                        else dst[j] = src[j];
                    }
            }
        }
    }
    if (!ok && threadIdx.x == 0) atomicOr(&g_tc_err, 1);
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && *(volatile int*)abort_flag) {
        // copies still in flight land before the shared memory is released
        for (int kb = *consumed_s; kb < issued; ++kb) mbar_wait(&full[kb % STAGES], (kb / STAGES) & 1);
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TMEM_COLS);
    }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
bool g_attr_set[64] = {};

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    std::call_once(g_encode_once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    return g_encode;
}

// rows x cols BF16 row-major with leading dimension ld (elements); box box_rows x 64
int make_map(CUtensorMap* m, const void* ptr, long long rows, long long cols, long long ld, int box_rows) {
    auto enc = encoder();
    if (!enc) return OPTIFAX_ERR_CUDA;
    cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
    cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 2};
    cuuint32_t box[2] = {static_cast<cuuint32_t>(BK), static_cast<cuuint32_t>(box_rows)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

}  // namespace

extern "C" int optifax_gemm_bf16(const void* A, int64_t lda, int64_t a_rows, const void* B, int64_t ldb,
                                 int64_t b_rows, float* C, int64_t ldc, int32_t M, int32_t N, int32_t K,
                                 int32_t splits, int32_t accumulate, void* stream) {
    if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || splits < 1) return OPTIFAX_ERR_INVALID_ARGUMENT;
    if (a_rows < BM || b_rows < BN || M > a_rows || N > b_rows || lda < K || ldb < K || ldc < N)
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    if ((lda % 8) || (ldb % 8) || (reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(B) & 15))
        return OPTIFAX_ERR_INVALID_ARGUMENT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return OPTIFAX_ERR_CUDA;
    if (!g_attr_set[dev]) {
        if (cudaFuncSetAttribute(gemm_bf16_tn, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) !=
            cudaSuccess)
            return OPTIFAX_ERR_CUDA;
        g_attr_set[dev] = true;
    }
    CUtensorMap ma, mb;
    int rc = make_map(&ma, A, a_rows, K, lda, BM);
    if (rc) return rc;
    rc = make_map(&mb, B, b_rows, K, ldb, BN);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int kps = (K + splits - 1) / splits;
    kps = (kps + BK - 1) / BK * BK;
    const int nsplit = (K + kps - 1) / kps;
    GemmArgs g{C, ldc, M, N, K, kps, (accumulate || nsplit > 1) ? 1 : 0};
    if (!accumulate && nsplit > 1 &&
        cudaMemset2DAsync(C, static_cast<size_t>(ldc) * 4, 0, static_cast<size_t>(N) * 4, M, st) != cudaSuccess)
        return OPTIFAX_ERR_CUDA;
    dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN, nsplit);
    gemm_bf16_tn<<<grid, 128, SMEM_BYTES, st>>>(ma, mb, g);
    return cudaGetLastError() == cudaSuccess ? OPTIFAX_OK : OPTIFAX_ERR_CUDA;
}

extern "C" int optifax_tc_error(int32_t* out, int32_t clear) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_err, sizeof(int)) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    if (out) *out = v;
    if (clear) {
        int z = 0;
        if (cudaMemcpyToSymbol(g_tc_err, &z, sizeof(int)) != cudaSuccess) return OPTIFAX_ERR_CUDA;
    }
    return OPTIFAX_OK;
}
