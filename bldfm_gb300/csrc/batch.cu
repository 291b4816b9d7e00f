// Batched FP32 solve (bldfm_solve_batch): many towers x timesteps -- each case
// with its own grid, modes, levels and profiles -- in one persistent sweep
// launch plus one launch per transform pass, optionally replayed as a CUDA
// graph.  Replaces the reference's per-case Python loop and process pool
// (src/bldfm/interface.py:141-326) for the solve itself.
#include "devattr.h"
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/bldfm_gb300.h"
#include "batch.h"
#include "common.h"
#include "devmath.cuh"
#include "fft_passes.cuh"
#include "host_exact.h"
#include "kernels.h"
#include "sweep32.cuh"

// ---------------------------------------------------------------------------
// device side
// ---------------------------------------------------------------------------

// Copies a BatchCase from global to shared memory (all threads).
__device__ __forceinline__ void load_case(BatchCase *dst, const BatchCase *src)
{
    const int nw = (int)(sizeof(BatchCase) / 4);
    const int *s = (const int *)src;
    int *d = (int *)dst;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) d[i] = s[i];
}

// Persistent sweep: CTA blockIdx.x owns tiles [cta_tiles[b], cta_tiles[b+1]);
// a tile is BATCH_MODES_PER_THREAD * blockDim.x consecutive solved modes of
// one case (two per thread, sharing the level-table loads).  The case's level
// table is brought into shared memory by one bulk copy whenever the case
// changes (the mbarrier flips phase each time; every wait is bounded).
__global__ void __launch_bounds__(256, 4) riccati32_batch_kernel(const BatchCase *__restrict__ cases,
                                                              const int *__restrict__ tile_case,
                                                              const int64_t *__restrict__ cta_tiles, int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) BatchCase sc;
    __shared__ uint64_t bar;
    __shared__ int s_fail;
    const int64_t t0 = cta_tiles[blockIdx.x], t1 = cta_tiles[blockIdx.x + 1];
    if (t0 >= t1) return;
    const uint32_t bar_a = smem_u32(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar_a), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        s_fail = 0;
    }
    __syncthreads();
    uint32_t phase = 0;
    int cur = -1;
    float *s_lv = (float *)smem_raw;
    for (int64_t t = t0; t < t1; ++t) {
        const int k = tile_case[t];
        if (k != cur) {
            __syncthreads();  // the previous case's table is no longer read
            load_case(&sc, cases + k);
            __syncthreads();
            const int L = sc.g.nz - 1;
            int *s_slot = (int *)(s_lv + (size_t)L * BLDFM_LV32);
            const uint32_t bytes = (uint32_t)((size_t)L * BLDFM_LV32 * sizeof(float));
            if (threadIdx.x == 0 && bytes > 0) {
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(bytes)
                             : "memory");
                const uint32_t chunk = 32768;
                for (uint32_t off = 0; off < bytes; off += chunk) {
                    const uint32_t nb = bytes - off < chunk ? bytes - off : chunk;
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                            "r"(smem_u32((char *)s_lv + off)),
                        "l"((const char *)sc.lv32 + off), "r"(nb), "r"(bar_a)
                        : "memory");
                }
            }
            for (int i = threadIdx.x; i < sc.g.nz; i += blockDim.x) s_slot[i] = sc.slot[i];
            if (bytes > 0) {
                uint32_t done = 0;
                for (long it = 0; it < BLDFM_WAIT_POLLS; ++it) {
                    asm volatile(
                        "{\n\t.reg .pred p;\n\t"
                        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                        "selp.u32 %0, 1, 0, p;\n\t}"
                        : "=r"(done)
                        : "r"(bar_a), "r"(phase)
                        : "memory");
                    if (done) break;
                }
                if (!done) s_fail = 1;
                phase ^= 1u;
            }
            __syncthreads();
            if (s_fail) {
                if (threadIdx.x == 0) atomicExch(err, BLDFM_ERR_TIMEOUT_DEV);
                return;
            }
            cur = k;
        }
        const int L = sc.g.nz - 1;
        const int *s_slot = (const int *)(s_lv + (size_t)L * BLDFM_LV32);
        // a tile is 2 blockDim.x modes: thread modes m0 and m0 + blockDim.x
        const int64_t m0 = (t - sc.tile0) * BATCH_MODES_PER_THREAD * (int64_t)blockDim.x + threadIdx.x;
        const int64_t m1 = m0 + blockDim.x;
        if (m0 < sc.g.nsolved && sc.g.nsnap > 0) {
            const int64_t mb = m1 < sc.g.nsolved ? m1 : -1;
            if (sc.g.nsnap == 1) {
                if (sc.g.iso)
                    ricc_mode_pair<true>(sc.g, s_lv, sc.modes, sc.q0, sc.Xp, sc.Xq, sc.ax, sc.ay, m0, mb);
                else
                    ricc_mode_pair<false>(sc.g, s_lv, sc.modes, sc.q0, sc.Xp, sc.Xq, sc.ax, sc.ay, m0, mb);
            } else {
                for (int u = 0; u < 2; ++u) {
                    const int64_t m = u == 0 ? m0 : mb;
                    if (m < 0) break;
                    if (sc.g.iso)
                        ricc_mode<true, false>(sc.g, s_lv, s_slot, sc.modes, sc.q0, sc.scratch, sc.Xp, sc.Xq, sc.ax,
                                               sc.ay, m);
                    else
                        ricc_mode<false, false>(sc.g, s_lv, s_slot, sc.modes, sc.q0, sc.scratch, sc.Xp, sc.Xq,
                                                sc.ax, sc.ay, m);
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) out_cols_batch_kernel(const BatchCase *__restrict__ cases,
                                                             const int *__restrict__ cta_case, int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) BatchCase sc;
    __shared__ uint64_t bar;
    const int k = cta_case[blockIdx.x];
    load_case(&sc, cases + k);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bar)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    const int64_t local = (int64_t)blockIdx.x - sc.col0;
    const int ncb = (sc.g.nbx + sc.cpc - 1) / sc.cpc;  // column blocks per level
    const int lvl = (int)(local / ncb), cb = (int)(local - (int64_t)lvl * ncb);
    if (!out_col_lines_staged(sc.g, sc.ply, sc.twy, sc.xband, sc.Xp, sc.Xq, sc.dc, sc.Cb, cb * sc.cpc, sc.cpc, lvl,
                              (float2 *)smem_raw, &bar) &&
        threadIdx.x == 0)
        atomicExch(err, BLDFM_ERR_TIMEOUT_DEV);
}

__global__ void __launch_bounds__(256) out_rows_batch_kernel(const BatchCase *__restrict__ cases,
                                                             const int *__restrict__ cta_case)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) BatchCase sc;
    const int k = cta_case[blockIdx.x];
    load_case(&sc, cases + k);
    __syncthreads();
    const int64_t local = (int64_t)blockIdx.x - sc.row0;
    const int nblk = (sc.g.out_ny + sc.rpc - 1) / sc.rpc;
    const int lvl = (int)(local / nblk), yb = (int)(local - (int64_t)lvl * nblk);
    out_row_lines<float>(sc.g, sc.plx, sc.twx, sc.xband, sc.Cb, sc.conc, sc.flx, yb * sc.rpc, sc.rpc, lvl,
                         (float2 *)smem_raw);
}

cudaError_t launch_batch_kernels(const BatchLaunch &bl, cudaStream_t st, int part)
{
    static uint64_t attr = 0;
    if (first_on_device(attr)) prepare_batch_attributes();
    // part 0: the sweep; part 1: the two transform passes
    if (part == 0 && bl.sweep_ctas > 0)
        riccati32_batch_kernel<<<bl.sweep_ctas, bl.threads, bl.sweep_smem, st>>>(bl.cases, bl.tile_case,
                                                                                 bl.cta_tiles, bl.err);
    if (part == 1 && bl.col_ctas > 0)
        out_cols_batch_kernel<<<bl.col_ctas, 256, bl.col_smem, st>>>(bl.cases, bl.col_case, bl.err);
    if (part == 1 && bl.row_ctas > 0)
        out_rows_batch_kernel<<<bl.row_ctas, 256, bl.row_smem, st>>>(bl.cases, bl.row_case);
    return cudaGetLastError();
}

int batch_sweep_occupancy(int threads, size_t smem)
{
    cudaFuncSetAttribute(riccati32_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, riccati32_batch_kernel, threads, smem) != cudaSuccess)
        return 1;
    return nb > 0 ? nb : 1;
}

void prepare_batch_attributes()
{
    cudaFuncSetAttribute(riccati32_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(out_cols_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(out_rows_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}
