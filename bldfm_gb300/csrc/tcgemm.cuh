// tcgen05 GEMM tile: D(128 x 256) = A(128 x K) * B(256 x K)^T in BF16 with FP32
// accumulation in tensor memory, K streamed through shared memory in chunks
// of KC columns.  Operands come from global memory already in the blocked
// core-matrix layout (tc_core_offset), one contiguous block per (tile, chunk),
// so each chunk is two bulk copies.  The epilogue functor receives, per
// thread, 32 consecutive FP32 columns of one output row.
#pragma once

#include "tc.cuh"

#define TC_BLOCK_ROWS 128
#define TC_N 256

// Grid: blockIdx.x = 128-row tile of A, blockIdx.y = split of the K chunks
// (split-K: CTA y handles chunks [y * cps, (y + 1) * cps)).  The epilogue gets
// epi.row(row, col0, v[32], tile_smem) for every 32-column slice, then, after
// a barrier, epi.finish(tile, tile_smem) cooperatively; tile_smem is the
// A-operand staging area (128 x KC bf16), free once the MMAs are done.
template <class Epi>
__global__ void __launch_bounds__(128, 1) tc_gemm_kernel(const uint16_t *__restrict__ Ablk,
                                                         const uint16_t *__restrict__ Bblk, int K, int KC, Epi epi,
                                                         int *err)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    uint16_t *sA = (uint16_t *)smem;
    uint16_t *sB = (uint16_t *)(smem + (size_t)TC_BLOCK_ROWS * KC * 2);
    __shared__ uint64_t bar_load, bar_mma;
    __shared__ uint32_t tmem_slot;
    __shared__ int fail;
    const int warp = threadIdx.x >> 5;
    if (warp == 0) tc_tmem_alloc(&tmem_slot, TC_N);
    if (threadIdx.x == 0) {
        tc_mbar_init(&bar_load, 1);
        tc_mbar_init(&bar_mma, 1);
        tc_fence_init();
        fail = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const int nchunks = K / KC;
    const int cps = (nchunks + gridDim.y - 1) / gridDim.y;
    const int c0 = blockIdx.y * cps, c1 = min(nchunks, c0 + cps);
    const int tile = blockIdx.x;
    const uint32_t abytes = (uint32_t)TC_BLOCK_ROWS * KC * 2, bbytes = (uint32_t)TC_N * KC * 2;
    const uint32_t idesc = tc_idesc_bf16(TC_BLOCK_ROWS, TC_N);
    const uint32_t sbo = (uint32_t)(KC / 8) * 128;
    int issued = 0;  // MMA commits issued (for the drain on failure)
    for (int c = c0; c < c1; ++c) {
        const int it = c - c0;
        if (threadIdx.x == 0) {
            tc_expect_tx(&bar_load, abytes + bbytes);
            tc_bulk_load(sA, Ablk + ((size_t)tile * nchunks + c) * TC_BLOCK_ROWS * KC, abytes, &bar_load);
            tc_bulk_load(sB, Bblk + (size_t)c * TC_N * KC, bbytes, &bar_load);
        }
        if (!tc_mbar_wait(&bar_load, (uint32_t)(it & 1))) fail = 1;
        __syncthreads();
        if (fail) break;
        if (threadIdx.x == 0) {
            tc_fence_after();
            const uint32_t a0 = tc_smem(sA), b0 = tc_smem(sB);
            for (int s = 0; s < KC / 16; ++s)
                tc_mma(tmem, tc_desc(a0 + s * 256, 128, sbo), tc_desc(b0 + s * 256, 128, sbo), idesc,
                       (it > 0 || s > 0) ? 1u : 0u);
            tc_commit(&bar_mma);
        }
        issued = it + 1;
        if (!tc_mbar_wait(&bar_mma, (uint32_t)(it & 1))) fail = 1;
        __syncthreads();
        if (fail) break;
    }
    if (!fail && issued > 0) {
        tc_fence_after();
        const int row = warp * 32 + (threadIdx.x & 31);
#pragma unroll 1
        for (int cc = 0; cc < TC_N / 32; ++cc) {
            float v[32];
            tc_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cc * 32), v);
            epi.row(tile * TC_BLOCK_ROWS + row, cc * 32, v, sA);
        }
        __syncthreads();
        epi.finish(tile, sA);
    } else if (fail) {
        if (threadIdx.x == 0) atomicExch(err, -9);
        // let in-flight MMAs finish before the tensor memory is released
        if (issued > 0) tc_mbar_wait(&bar_mma, (uint32_t)((issued - 1) & 1));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_tmem_free(tmem, TC_N);
}

// Shared-memory bytes of one tc_gemm_kernel CTA for chunk size KC.
inline size_t tc_gemm_smem(int KC) { return (size_t)(TC_BLOCK_ROWS + TC_N) * KC * 2; }
