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
#include <tuple>
#include <vector>

#include "../../include/bldfm_gb300.h"
#include "batch.h"
#include "common.h"
#include "devmath.cuh"
#include "fft_passes.cuh"
#include "host_exact.h"
#include "kernels.h"
#include "ffmath.cuh"
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
// NT = blockDim.x (128 or 256).  Register budget: 64 registers (no spills)
// for both, 32 warps per SM (256 threads x 4 CTAs, 128 threads x 8 CTAs);
// the autotuner picks the shape.
template <int NT>
__global__ void __launch_bounds__(NT, NT == 128 ? 8 : 4)
    riccati32_batch_kernel(const BatchCase *__restrict__ cases, const int *__restrict__ tile_case,
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
        // a tile is BATCH_MODES_PER_THREAD blockDim.x modes: thread modes
        // m0 + u blockDim.x, u < BATCH_MODES_PER_THREAD
        const int64_t m0 = (t - sc.tile0) * BATCH_MODES_PER_THREAD * (int64_t)blockDim.x + threadIdx.x;
        if (m0 < sc.g.nsolved && sc.g.nsnap > 0) {
            int64_t mm[BATCH_MODES_PER_THREAD];
            int nvalid = 0;
#pragma unroll
            for (int u = 0; u < BATCH_MODES_PER_THREAD; ++u) {
                mm[u] = m0 + (int64_t)u * blockDim.x;
                if (mm[u] < sc.g.nsolved) nvalid = u + 1;
            }
            if (sc.g.nsnap == 1) {
                if (sc.g.iso)
                    ricc_modes_packed<true, BATCH_MODES_PER_THREAD / 2>(sc.g, s_lv, sc.modes, sc.q0, sc.Xp, sc.Xq,
                                                                       sc.ax, sc.ay, mm, nvalid);
                else
                    ricc_modes_packed<false, BATCH_MODES_PER_THREAD / 2>(sc.g, s_lv, sc.modes, sc.q0, sc.Xp, sc.Xq,
                                                                        sc.ax, sc.ay, mm, nvalid);
            } else {
                for (int u = 0; u < nvalid; ++u) {
                    const int64_t m = mm[u];
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
                                                             const int *__restrict__ cta_case, int *err)
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
                         (float2 *)smem_raw, err);
}

// Bounded wait on phase `parity` of an mbarrier by every thread of the block;
// false (for all threads) if it ran out.
__device__ __forceinline__ bool block_wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = smem_u32(bar);
    uint32_t done = 0;
    for (long it = 0; it < BLDFM_WAIT_POLLS && !done; ++it)
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
    return !__syncthreads_or(!done);
}

// Persistent column pass, one line at a time.  CTA b takes a contiguous range
// of items (item = one band column of one level of one case, in case order)
// and, while it transforms one line, the P-side spectrum column of the next
// line of the same case arrives by bulk copy in the other of two staging
// buffers (mbarrier per buffer, bounded waits); the case and its twiddles are
// loaded when the case changes.  Cases whose arrays do not allow 16-byte
// copies take out_col_lines, one line per item.  smem: 3 maxn + 4 maxnly complex.
__global__ void __launch_bounds__(256) out_cols_persist_kernel(const BatchCase *__restrict__ cases,
                                                               const int *__restrict__ col_case, int nitems, int maxn,
                                                               int maxnly, int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) BatchCase sc;
    __shared__ uint64_t bar[2];
    const int per = (nitems + (int)gridDim.x - 1) / (int)gridDim.x;
    const int lo = (int)blockIdx.x * per, hi = min(nitems, lo + per);
    if (lo >= hi) return;
    float2 *bufA = (float2 *)smem_raw, *bufB = bufA + maxn, *stw = bufB + maxn;
    float2 *stg0 = stw + maxn, *stg1 = stg0 + 2 * (size_t)maxnly;
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bar[i])), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    uint32_t ph[2] = {0u, 0u};
    bool pend[2] = {false, false};  // thread 0: copies issued, not yet waited for
    int cur = -1, slot = 0;
    bool fast = false, ok = true;
    // item -> (level, band column) within the current case
    auto geo = [&](int it, int &lvl, int &b) {
        const int local = it - (int)sc.col0;
        lvl = local / sc.g.nbx;
        b = local - lvl * sc.g.nbx;
    };
    // thread 0: the P-side column of item `it` into staging buffer s
    auto issue = [&](int it, int s) {
        int lvl, b;
        geo(it, lvl, b);
        const int col = sc.xband[b].y;
        if (col < 0) return;
        const int nly = sc.g.nly;
        const uint32_t colb = (uint32_t)nly * 8u;
        float2 *dst = s ? stg1 : stg0;
        const uint32_t ba = smem_u32(&bar[s]);
        const size_t bp = ((size_t)lvl * sc.g.nlx + col) * nly;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ba), "r"(2u * colb) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(dst)),
                     "l"(sc.Xp + bp), "r"(colb), "r"(ba)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(dst + nly)),
                     "l"(sc.Xq + bp), "r"(colb), "r"(ba)
                     : "memory");
        pend[s] = true;
    };
    __syncthreads();
    for (int it = lo; it < hi && ok; ++it) {
        const int k = col_case[it];
        if (k != cur) {
            __syncthreads();  // the previous item is done with sc, the twiddles and the staging
            load_case(&sc, cases + k);
            __syncthreads();
            cur = k;
            const int n = sc.ply.n, nly = sc.g.nly;
            fast = !((n | nly) & 1) && n <= maxn && nly <= maxnly &&
                   !((((uintptr_t)sc.Xp) | ((uintptr_t)sc.Xq)) & 15);
            if (fast) {
                for (int i = threadIdx.x; i < n; i += blockDim.x) stw[i] = sc.twy[i];
                if (threadIdx.x == 0) issue(it, slot);
            }
            __syncthreads();
        }
        int lvl, b;
        geo(it, lvl, b);
        if (!fast) {
            out_col_lines<float>(sc.g, sc.ply, sc.twy, sc.xband, sc.Xp, sc.Xq, sc.dc, sc.Cb, b, 1, lvl, bufA);
            __syncthreads();
            continue;
        }
        const int4 bx = sc.xband[b];
        // the next line of this case into the other buffer
        if (threadIdx.x == 0 && it + 1 < hi && col_case[it + 1] == cur) issue(it + 1, slot ^ 1);
        float2 *sp = slot ? stg1 : stg0;
        if (bx.y >= 0) {
            if (!block_wait(&bar[slot], ph[slot])) {
                ok = false;
                break;
            }
            ph[slot] ^= 1u;
            if (threadIdx.x == 0) pend[slot] = false;
        }
        const int n = sc.ply.n;
        col_line_from_staged(sc.g, bx, sp, sp + sc.g.nly, sc.Xp, sc.Xq, sc.dc, n, lvl, bufA);
        float2 *res = fft_run<float2>(bufA, bufB, sc.ply, 1, stw, sc.g.out_sign);
        float2 *o = sc.Cb + (size_t)lvl * sc.g.out_ny * sc.g.nbx + b;
        for (int y = threadIdx.x; y < sc.g.out_ny; y += blockDim.x) o[(size_t)y * sc.g.nbx] = res[sc.g.py + y];
        __syncthreads();
        slot ^= 1;
    }
    if (!ok && threadIdx.x == 0) {
        atomicExch(err, BLDFM_ERR_TIMEOUT_DEV);
        // copies still in flight land before the block exits
        for (int s = 0; s < 2; ++s) {
            if (!pend[s]) continue;
            const uint32_t a = smem_u32(&bar[s]);
            uint32_t done = 0;
            for (long i = 0; i < BLDFM_WAIT_POLLS && !done; ++i)
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                    "selp.u32 %0, 1, 0, p;\n\t}"
                    : "=r"(done)
                    : "r"(a), "r"(ph[s])
                    : "memory");
        }
    }
}

// Persistent row pass, one output row at a time: CTA b takes a contiguous
// range of items (item = one output row of one level of one case) and loads
// the next row's band values into registers while it transforms the current
// one; the case and its twiddles are loaded when the case changes.
// smem: 3 maxn complex.
__global__ void __launch_bounds__(256) out_rows_persist_kernel(const BatchCase *__restrict__ cases,
                                                               const int *__restrict__ row_case, int nitems, int maxn,
                                                               int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) BatchCase sc;
    const int per = (nitems + (int)gridDim.x - 1) / (int)gridDim.x;
    const int lo = (int)blockIdx.x * per, hi = min(nitems, lo + per);
    if (lo >= hi) return;
    float2 *bufA = (float2 *)smem_raw, *bufB = bufA + maxn, *stw = bufB + maxn;
    constexpr int PF = 8;  // band values per thread held in registers (rows of up to PF x 256 band columns)
    float2 vc[PF], vn[PF];
    int cur = -1;
    bool bad = false;  // a non-finite output value seen by this thread
    for (int it = lo; it < hi; ++it) {
        const int k = row_case[it];
        if (k != cur) {
            __syncthreads();  // the previous item is done with sc and the twiddles
            load_case(&sc, cases + k);
            __syncthreads();
            cur = k;
            for (int i = threadIdx.x; i < sc.plx.n; i += blockDim.x) stw[i] = sc.twx[i];
            const float2 *row = sc.Cb + (size_t)(it - sc.row0) * sc.g.nbx;
#pragma unroll
            for (int j = 0; j < PF; ++j) {
                const int bcol = threadIdx.x + j * (int)blockDim.x;
                if (bcol < sc.g.nbx) vc[j] = row[bcol];
            }
        }
        const int nb = sc.g.nbx, n = sc.plx.n;
        const int local = it - (int)sc.row0;  // (level, row): rows of a case are consecutive in Cb
        const float2 *row = sc.Cb + (size_t)local * nb;
        // the next row of this case, in flight during this row's transform
        const bool nxt = it + 1 < hi && row_case[it + 1] == cur;
        if (nxt) {
#pragma unroll
            for (int j = 0; j < PF; ++j) {
                const int bcol = threadIdx.x + j * (int)blockDim.x;
                if (bcol < nb) vn[j] = row[nb + bcol];
            }
        }
        for (int i = threadIdx.x; i < n; i += blockDim.x) bufA[i] = make_float2(0.f, 0.f);
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PF; ++j) {
            const int bcol = threadIdx.x + j * (int)blockDim.x;
            if (bcol < nb) bufA[sc.xband[bcol].x] = vc[j];
        }
        for (int bcol = threadIdx.x + PF * (int)blockDim.x; bcol < nb; bcol += blockDim.x)
            bufA[sc.xband[bcol].x] = row[bcol];
        float2 *res = fft_run<float2>(bufA, bufB, sc.plx, 1, stw, sc.g.out_sign);
        const int lvl = local / sc.g.out_ny;
        const int y = local - lvl * sc.g.out_ny;
        const size_t o = ((size_t)lvl * sc.g.out_ny + y) * sc.g.out_nx;
        for (int x = threadIdx.x; x < sc.g.out_nx; x += blockDim.x) {
            const float2 v = res[sc.g.px + x];
            sc.conc[o + x] = (double)v.x;
            sc.flx[o + x] = (double)v.y;
            bad |= !(isfinite(v.x) && isfinite(v.y));
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PF; ++j) vc[j] = vn[j];
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicCAS(err, 0, BLDFM_ERR_NONFINITE_DEV);
}

// Accuracy guard of the surrogate's batched footprints, a stratified sample
// per case (the footprint's L2 norm sits in the low wavenumbers): local
// sample j = i - prefix[k] of case k (prefix[k] <= i < prefix[k + 1], every
// case's count padded to a multiple of SUR_GUARD_CTA, so that a CTA's samples
// belong to one case; the padding contributes nothing) is
//   j = 0              the k = 0 mode (exact from the host, error 0),
//   j = 1 .. GBOX      every solved mode with |kx|, |ky| <= 2 (weight 1),
//   j > GBOX           solved mode (j - 1 - GBOX) * stride (weight stride),
// each solved mode counted twice when its mirror is written from it.  A CTA
// stages the case's level table in shared memory and each thread takes
// samples j and j + 256 in the two lanes of packed f32x2 operations
// (ricc_rc_pair, the exact FP32 values as ricc_rc_value computes them),
// compares them with the spectra the serving kernel (and the exact low band)
// wrote and accumulates into acc[k] the weighted (sum |dXp|^2, sum |Xp|^2,
// sum |dXq|^2, sum |Xq|^2) (one atomic per warp and quantity).
__device__ __forceinline__ bool guard_sample(const BatchCase &bc, int64_t j, int stride, int &r, int &c, float &wgt)
{
    const SolveGeom &g = bc.g;
    r = c = -1;
    wgt = 1.f;
    if (j >= 1 && j <= SUR_GUARD_BOX) {
        const int t = (int)j - 1;
        int kx, ky;
        if (t < 2) {
            kx = 0;
            ky = t + 1;
        } else {
            kx = 1 + (t - 2) / 5;
            ky = (t - 2) % 5 - 2;
        }
        if (kx <= freq_max(g.nlx) && ky >= freq_min(g.nly) && ky <= freq_max(g.nly)) {
            r = index_of_freq(ky, g.nly);
            c = index_of_freq(kx, g.nlx);
        }
    } else if (j > SUR_GUARD_BOX) {
        const int64_t m = (j - 1 - SUR_GUARD_BOX) * (int64_t)stride;
        if (m < g.nsolved) {
            bool paired;
            unpack_mode(bc.modes[m], r, c, paired);
            wgt = (float)stride;
        }
    }
    return r >= 0;
}

__device__ __forceinline__ float4 guard_terms(const BatchCase &bc, int r, int c, float wgt, float2 pe, float2 qe)
{
    const SolveGeom &g = bc.g;
    const int kx = freq_of_index(c, g.nlx), ky = freq_of_index(r, g.nly);
    if (-kx >= freq_min(g.nlx) && -kx <= freq_max(g.nlx) && -ky >= freq_min(g.nly) && -ky <= freq_max(g.nly))
        wgt *= 2.f;
    const size_t o = spec_idx(g, 0, r, c);
    const float2 pn = bc.Xp[o], qn = bc.Xq[o];
    const float dpx = pn.x - pe.x, dpy = pn.y - pe.y, dqx = qn.x - qe.x, dqy = qn.y - qe.y;
    return make_float4(wgt * (dpx * dpx + dpy * dpy), wgt * (pe.x * pe.x + pe.y * pe.y),
                       wgt * (dqx * dqx + dqy * dqy), wgt * (qe.x * qe.x + qe.y * qe.y));
}

__global__ void __launch_bounds__(SUR_GUARD_THREADS) sur_guard_kernel(const BatchCase *__restrict__ cases, int n,
                                                                      const int64_t *__restrict__ prefix, int stride,
                                                                      float4 *__restrict__ acc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *s_lv = (float4 *)smem_raw;
    const int64_t i0 = (int64_t)blockIdx.x * SUR_GUARD_CTA;
    int k = 0;
    while (k + 1 < n && prefix[k + 1] <= i0) ++k;
    const BatchCase &bc = cases[k];
    const SolveGeom &g = bc.g;
    const int nrow4 = (g.nz - 1) * (BLDFM_LV32 / 4);
    const float4 *src = (const float4 *)bc.lv32;
    for (int i = threadIdx.x; i < nrow4; i += blockDim.x) s_lv[i] = src[i];
    __syncthreads();
    const int64_t j = i0 - prefix[k] + threadIdx.x;
    int r[2], c[2];
    float w[2];
    const bool v0 = guard_sample(bc, j, stride, r[0], c[0], w[0]);
    const bool v1 = guard_sample(bc, j + SUR_GUARD_THREADS, stride, r[1], c[1], w[1]);
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j == 0) {
        const double2 p = bc.dc[0], q = bc.dc[1];
        v = make_float4(0.f, (float)(p.x * p.x + p.y * p.y), 0.f, (float)(q.x * q.x + q.y * q.y));
    }
    if (v0 || v1) {
        if (!v0) {
            r[0] = r[1];
            c[0] = c[1];
        } else if (!v1) {
            r[1] = r[0];
            c[1] = c[0];
        }
        float2 pe[2], qe[2];
        if (g.iso)
            ricc_rc_pair<true>(g, (const float *)s_lv, bc.ax, bc.ay, r, c, pe, qe);
        else
            ricc_rc_pair<false>(g, (const float *)s_lv, bc.ax, bc.ay, r, c, pe, qe);
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            if (!(l ? v1 : v0)) continue;
            const float4 t = guard_terms(bc, r[l], c[l], w[l], pe[l], qe[l]);
            v.x += t.x;
            v.y += t.y;
            v.z += t.z;
            v.w += t.w;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, off);
        v.y += __shfl_down_sync(0xffffffffu, v.y, off);
        v.z += __shfl_down_sync(0xffffffffu, v.z, off);
        v.w += __shfl_down_sync(0xffffffffu, v.w, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[k].x, v.x);
        atomicAdd(&acc[k].y, v.y);
        atomicAdd(&acc[k].z, v.z);
        atomicAdd(&acc[k].w, v.w);
    }
}

cudaError_t launch_sur_guard(const BatchCase *cases, int n, const int64_t *prefix, int64_t nsamples, int stride,
                             int max_nz, float4 *acc, cudaStream_t st)
{
    if (nsamples <= 0) return cudaSuccess;
    const size_t smem = (size_t)std::max(max_nz - 1, 1) * BLDFM_LV32 * sizeof(float);
    if (smem > 48 * 1024) {
        const cudaError_t e =
            cudaFuncSetAttribute(sur_guard_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    sur_guard_kernel<<<(unsigned)((nsamples + SUR_GUARD_CTA - 1) / SUR_GUARD_CTA), SUR_GUARD_THREADS, smem, st>>>(
        cases, n, prefix, stride, acc);
    return cudaGetLastError();
}

// Exact low band of the surrogate's footprints.  A footprint's L2 norm sits
// in its lowest wavenumbers (with the network's errors: on the production
// footprint 97% of the flux error and 99.7% of the concentration error come
// from |k| z_m < 4, 1.2% of the modes), so those modes take the exact FP32
// sweep and the network serves the rest.  CTA b of case k (block0 <= b <
// block0 + its CTAs) stages the level table in shared memory and sweeps box
// positions j = 512 (b - block0) + t and j + 256 of the half box, two modes
// in the lanes of packed f32x2 operations (ricc_rc_pair, which rounds as the
// guard's ricc_rc_value does):
//   j < by            kx = 0, ky = j + 1,
//   otherwise         kx = 1 + (j - by) / (2 by + 1), ky = (j - by) % (2 by + 1) - by,
// the solved representative of each mirror pair (kx > 0, or kx = 0 and
// ky > 0; inside the mode range, so every mirror exists); then the unpaired
// Nyquist modes (no mirror in the grid) the box reaches:
//   column  kx = -nlx/2, ky in [-by, by]   (ncol = 2 by + 1 or 0),
//   row     ky = -nly/2, kx in [-bx, bx]   (nrow = 2 bx + 1 or 0),
//   corner  (-nlx/2, -nly/2)               (ncorner = 1 or 0).
__device__ __forceinline__ bool lowband_mode(const LowBandCase &lb, int j, int &r, int &c, bool &mirror)
{
    if (j >= lb.count) return false;
    int kx, ky;
    mirror = true;
    if (j < lb.nbox) {
        if (j < lb.by) {
            kx = 0;
            ky = j + 1;
        } else {
            const int t = j - lb.by, w = 2 * lb.by + 1;
            kx = 1 + t / w;
            ky = t - (kx - 1) * w - lb.by;
        }
    } else {
        mirror = false;
        j -= lb.nbox;
        if (j < lb.ncol) {
            kx = -(lb.g.nlx / 2);
            ky = j - lb.by;
        } else if ((j -= lb.ncol) < lb.nrow) {
            ky = -(lb.g.nly / 2);
            kx = j - lb.bx;
        } else {
            kx = -(lb.g.nlx / 2);
            ky = -(lb.g.nly / 2);
        }
    }
    const float lx = lb.ax * (float)kx, ly = lb.ay * (float)ky;
    if (!(fmaf(lx, lx, ly * ly) < lb.kmax2)) return false;
    r = index_of_freq(ky, lb.g.nly);
    c = index_of_freq(kx, lb.g.nlx);
    return true;
}

__global__ void __launch_bounds__(SUR_LOWBAND_THREADS) sur_lowband_kernel(const LowBandCase *__restrict__ cases,
                                                                         int n)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *s_lv = (float4 *)smem_raw;
    const int b = blockIdx.x;
    int k = 0;
    while (k + 1 < n && cases[k + 1].block0 <= b) ++k;
    const LowBandCase &lb = cases[k];
    const SolveGeom &g = lb.g;
    const int nrow4 = (g.nz - 1) * (BLDFM_LV32 / 4);
    const float4 *src = (const float4 *)lb.lv32;
    for (int i = threadIdx.x; i < nrow4; i += blockDim.x) s_lv[i] = src[i];
    __syncthreads();
    const int j = (b - lb.block0) * SUR_LOWBAND_MODES + threadIdx.x;
    int r[2] = {0, 0}, c[2] = {0, 0};
    bool mir[2] = {true, true};
    const bool v0 = lowband_mode(lb, j, r[0], c[0], mir[0]);
    const bool v1 = lowband_mode(lb, j + SUR_LOWBAND_THREADS, r[1], c[1], mir[1]);
    if (!v0 && !v1) return;
    if (!v0) {
        r[0] = r[1];
        c[0] = c[1];
    } else if (!v1) {
        r[1] = r[0];
        c[1] = c[0];
    }
    float2 p[2], q[2];
    if (g.iso)
        ricc_rc_pair<true>(g, (const float *)s_lv, lb.ax, lb.ay, r, c, p, q);
    else
        ricc_rc_pair<false>(g, (const float *)s_lv, lb.ax, lb.ay, r, c, p, q);
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        if (!(l ? v1 : v0)) continue;
        const size_t o = spec_idx(g, 0, r[l], c[l]);
        lb.Xp[o] = p[l];
        lb.Xq[o] = q[l];
        if (mir[l]) {
            const int kx = freq_of_index(c[l], g.nlx), ky = freq_of_index(r[l], g.nly);
            const size_t om = spec_idx(g, 0, index_of_freq(-ky, g.nly), index_of_freq(-kx, g.nlx));
            lb.Xp[om] = make_float2(p[l].x, -p[l].y);
            lb.Xq[om] = make_float2(q[l].x, -q[l].y);
        }
    }
}

int sur_lowband_setup(LowBandCase &c, double exact_kz, double zm)
{
    c.bx = c.by = c.nbox = c.ncol = c.nrow = c.ncorner = c.count = 0;
    c.kmax2 = 0.f;
    if (!(exact_kz > 0) || !(zm > 0) || !(c.ax > 0) || !(c.ay > 0) || c.g.nz < 2) return 0;
    const double km = exact_kz / zm;
    // the half box stays inside the mode range (freq_max), where every solved
    // mode is a mirror pair's representative; the Nyquist frequency of an
    // even mode count (-n/2, no mirror) is enumerated apart
    const double fx = floor(km / c.ax), fy = floor(km / c.ay);
    c.bx = (int)std::min<double>(fx, (double)freq_max(c.g.nlx));
    c.by = (int)std::min<double>(fy, (double)freq_max(c.g.nly));
    const bool nx = c.g.nlx % 2 == 0 && fx >= c.g.nlx / 2, ny = c.g.nly % 2 == 0 && fy >= c.g.nly / 2;
    c.nbox = c.by + c.bx * (2 * c.by + 1);
    c.ncol = nx ? 2 * c.by + 1 : 0;
    c.nrow = ny ? 2 * c.bx + 1 : 0;
    c.ncorner = nx && ny ? 1 : 0;
    c.kmax2 = (float)std::min(km * km, 1e30);
    c.count = c.nbox + c.ncol + c.nrow + c.ncorner;
    return (c.count + SUR_LOWBAND_MODES - 1) / SUR_LOWBAND_MODES;
}

cudaError_t launch_sur_lowband(const LowBandCase *cases, int n, int nblocks, int max_nz, cudaStream_t st)
{
    if (nblocks <= 0) return cudaSuccess;
    const size_t smem = (size_t)std::max(max_nz - 1, 1) * BLDFM_LV32 * sizeof(float);
    if (smem > 48 * 1024) {
        const cudaError_t e =
            cudaFuncSetAttribute(sur_lowband_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    sur_lowband_kernel<<<(unsigned)nblocks, SUR_LOWBAND_THREADS, smem, st>>>(cases, n);
    return cudaGetLastError();
}

// Accuracy check of a batched FP32 solve (no reference counterpart: the
// statement of each result's error).  The exact values of a sampled mode at
// every output level come from the invariant-imbedding recursion in
// float-float arithmetic (~48-bit significand, ffmath.cuh) on the case's
// float-pair level table (the FP64 rows split into hi + lo, generic layout),
// with the top radiation condition, flux product and source spectrum of the
// FP32 sweep, times the FP32 sweep's own phase factor; it is compared with the
// FP32 spectra.  The footprint's L2 norm sits in the low wavenumbers, where
// the relative FP32 error is smallest, so the sample is stratified
// (CHECK_NS = 32 samples per case):
//   sample 0      the k = 0 mode (exact FP64 values from the host, error 0),
//   samples 1-12  every solved mode with |kx|, |ky| <= 2 (weight 1),
//   samples 13-31 equal slices of the mode list (weight (nsolved - 12) / 19),
// each solved mode counted twice when its mirror is written from it; acc[k]
// accumulates the weighted (sum |dXp|^2, sum |Xp|^2, sum |dXq|^2, sum |Xq|^2).
// Not included: the FP32 rounding of the phase factor and, off footprint
// mode, of the forward transform of the source at k != 0 (both enter as
// given; the k = 0 source value is an FP64 sum, dc_partial_kernel).
//
// One warp per sample, the levels split over its lanes: each step
// R_i = (a R_{i+1} - b) / (a - c R_{i+1}) is the Moebius map of the matrix
// A_i = [[a, -b], [-c, a]], so lane l composes its run of levels
// [lo_l, hi_l) into M_l = A_lo ... A_{hi-1}; a suffix scan over the lanes
// gives S_l = M_l ... M_31, from which lane l takes the ratio at the top of
// its run, R_{hi_l} = S_{l+1}(R_L); the lane's flux factors below the
// highest output level follow from the halves of its map without a division
// per level (check_mode), and the flux product at an output level is the
// product of the lower lanes' factors and this lane's below it.  A serial
// float-float sweep took 0.32 ms per 16-footprint batch (206 dependent steps
// per sample); the split one with a ratio-and-flux pass per lane (a complex
// float-float division per level) 0.08 ms.
#define CHECK_NS 32
#define CHECK_BOX 2
__device__ __forceinline__ ff ffrow(const float2 *row, int j) { return {row[j].x, row[j].y}; }

// a, b, c of level row i (generic layout {-Kx, -Ky, -u, -v, A, B0, B1, H, C1,
// -2 C1}) for wavenumbers (lx, ly), lx2 = lx^2, ly2 = ly^2: T = Tr + i Ti,
// a = 1 - A T, b = B0 - B1 T, c = H T - C1 T^2
__device__ __noinline__ void coef_ff(const float2 *row, const ff lx, const ff ly, const ff lx2, const ff ly2, cff &a,
                                     cff &b, cff &c)
{
    const ff one = ff_from(1.f);
    const ff Tr = ff_add(ff_mul(ffrow(row, 0), lx2), ff_mul(ffrow(row, 1), ly2));
    const ff Ti = ff_add(ff_mul(ffrow(row, 2), lx), ff_mul(ffrow(row, 3), ly));
    const ff A = ffrow(row, 4), B1 = ffrow(row, 6), H = ffrow(row, 7), C1 = ffrow(row, 8);
    a = {ff_sub(one, ff_mul(A, Tr)), ff_neg(ff_mul(A, Ti))};
    b = {ff_sub(ffrow(row, 5), ff_mul(B1, Tr)), ff_neg(ff_mul(B1, Ti))};
    const cff T = {Tr, Ti};
    const cff T2 = cff_mul(T, T);
    c = {ff_sub(ff_mul(H, Tr), ff_mul(C1, T2.re)), ff_sub(ff_mul(H, Ti), ff_mul(C1, T2.im))};
}

// 2 x 2 complex float-float matrix (a Moebius map, defined up to scale)
struct mff {
    cff m11, m12, m21, m22;
};
__device__ __noinline__ mff mff_mul(const mff &x, const mff &y)
{
    return {cff_add(cff_mul(x.m11, y.m11), cff_mul(x.m12, y.m21)), cff_add(cff_mul(x.m11, y.m12), cff_mul(x.m12, y.m22)),
            cff_add(cff_mul(x.m21, y.m11), cff_mul(x.m22, y.m21)), cff_add(cff_mul(x.m21, y.m12), cff_mul(x.m22, y.m22))};
}
__device__ __forceinline__ cff cff_scale(cff a, float s)
{
    return {{a.re.hi * s, a.re.lo * s}, {a.im.hi * s, a.im.lo * s}};
}
__device__ __forceinline__ float cff_maxabs(cff a) { return fmaxf(fabsf(a.re.hi), fabsf(a.im.hi)); }
// exact power-of-two rescaling (the map is unchanged); E receives the
// exponent taken out (the matrix equals x * 2^E)
__device__ __forceinline__ void mff_norm(mff &x, int &E)
{
    const float m = fmaxf(fmaxf(cff_maxabs(x.m11), cff_maxabs(x.m12)), fmaxf(cff_maxabs(x.m21), cff_maxabs(x.m22)));
    if (m > 0.f && isfinite(m)) {
        const int e = ilogbf(m);
        const float s = ldexpf(1.f, -e);
        x = {cff_scale(x.m11, s), cff_scale(x.m12, s), cff_scale(x.m21, s), cff_scale(x.m22, s)};
        E += e;
    }
}
__device__ __forceinline__ void mff_norm(mff &x)
{
    int e = 0;
    mff_norm(x, e);
}
__device__ __forceinline__ cff cff_shfl_down(cff a, int d)
{
    return {{__shfl_down_sync(0xffffffffu, a.re.hi, d), __shfl_down_sync(0xffffffffu, a.re.lo, d)},
            {__shfl_down_sync(0xffffffffu, a.im.hi, d), __shfl_down_sync(0xffffffffu, a.im.lo, d)}};
}
__device__ __forceinline__ cff cff_shfl_xor(cff a, int d)
{
    return {{__shfl_xor_sync(0xffffffffu, a.re.hi, d), __shfl_xor_sync(0xffffffffu, a.re.lo, d)},
            {__shfl_xor_sync(0xffffffffu, a.im.hi, d), __shfl_xor_sync(0xffffffffu, a.im.lo, d)}};
}
__device__ __forceinline__ cff cff_shfl(cff a, int src)
{
    return {{__shfl_sync(0xffffffffu, a.re.hi, src), __shfl_sync(0xffffffffu, a.re.lo, src)},
            {__shfl_sync(0xffffffffu, a.im.hi, src), __shfl_sync(0xffffffffu, a.im.lo, src)}};
}
__device__ __forceinline__ mff mff_shfl_down(const mff &x, int d)
{
    return {cff_shfl_down(x.m11, d), cff_shfl_down(x.m12, d), cff_shfl_down(x.m21, d), cff_shfl_down(x.m22, d)};
}
// keep |Q| near 1 with the power of two in E
__device__ __forceinline__ void cff_renorm(cff &Q, int &E)
{
    const float m = cff_maxabs(Q);
    if (m > 0.f && isfinite(m)) {
        const int e = ilogbf(m);
        Q = cff_scale(Q, ldexpf(1.f, -e));
        E += e;
    }
}

// the same for a homogeneous pair (N, D) with one exponent
__device__ __forceinline__ void cff_renorm2(cff &N, cff &D, int &E)
{
    const float m = fmaxf(cff_maxabs(N), cff_maxabs(D));
    if (m > 0.f && isfinite(m)) {
        const int e = ilogbf(m);
        const float s = ldexpf(1.f, -e);
        N = cff_scale(N, s);
        D = cff_scale(D, s);
        E += e;
    }
}

__device__ __forceinline__ cff cff_shfl_up(cff a, int d)
{
    return {{__shfl_up_sync(0xffffffffu, a.re.hi, d), __shfl_up_sync(0xffffffffu, a.re.lo, d)},
            {__shfl_up_sync(0xffffffffu, a.im.hi, d), __shfl_up_sync(0xffffffffu, a.im.lo, d)}};
}

// exact (p, q) of mode (r, c) at every output level vs the FP32 spectra, the
// whole warp together; every lane returns its part of
// v = (sum |dXp|^2, sum |Xp|^2, sum |dXq|^2, sum |Xq|^2) over the output levels
// in its run of levels.
//
// Homogeneous form: with v_i = A_i v_{i+1}, v = (N, D), the ratio is
// R_i = N_i / D_i and the flux factor telescopes,
//   f_i = c_i R_i + a_i = (c_i N_i + a_i D_i) / D_i = det A_i D_{i+1} / D_i,
// det A_i = a_i^2 - b_i c_i, so a lane's factors below the highest output
// level jm, over [lo, s) with s = clamp(jm, lo, hi), multiply to
//   F = (prod det A_i) D_s / D_lo,  v_s = M_high (R_top, 1), v_lo = M_low v_s,
// from the two halves M_low = A_lo ... A_{s-1}, M_high = A_s ... A_{hi-1} of
// the lane's map: no division per level.  The flux product at an output
// level j of the lane is Q(j) = P F_j, P the lower lanes' product (an
// exclusive prefix product over the lanes) and F_j the factors of [lo, j):
// F for j = s, else (det product over [lo, j)) D_j / D_lo from a second
// pass down from s to the lane's lowest output level.
__device__ __forceinline__ void check_mode(const BatchCase &bc, int r, int c, int lane, float4 &v)
{
    const SolveGeom &g = bc.g;
    const int kx = freq_of_index(c, g.nlx), ky = freq_of_index(r, g.nly);
    const ff lx = ff_mul(ff_from((float)kx), ff_from_double(g.lx_scale * g.valx));
    const ff ly = ff_mul(ff_from((float)ky), ff_from_double(g.ly_scale * g.valy));
    const ff lx2 = ff_mul(lx, lx), ly2 = ff_mul(ly, ly);
    // top radiation ratio R_L = 1 / (Kz_top lam), lam the principal root
    const cff w = {ff_add(ff_mul(ff_from_double(g.kxk_top), lx2), ff_mul(ff_from_double(g.kyk_top), ly2)),
                   ff_add(ff_mul(ff_from_double(g.uk_top), lx), ff_mul(ff_from_double(g.vk_top), ly))};
    const cff lam = cff_sqrt(w);
    const ff kz = ff_from_double(g.kz_top);
    const cff one = {ff_from(1.f), ff_from(0.f)}, zero = {ff_from(0.f), ff_from(0.f)};
    const cff RL = cff_div(one, cff{ff_mul(kz, lam.re), ff_mul(kz, lam.im)});
    const int L = g.nz - 1, jm = g.jmax;
    const int lo = (int)(((int64_t)lane * L) / 32), hi = (int)(((int64_t)(lane + 1) * L) / 32);
    const int sp = jm < lo ? lo : (jm > hi ? hi : jm);  // split level s
    // the lane's map in two halves (each times 2^E) and the det product of
    // the lower half
    mff Ml = {one, zero, zero, one}, Mh = {one, zero, zero, one};
    int EMl = 0, EMh = 0, EDet = 0;
    cff Det = one;
    for (int i = lo; i < hi; ++i) {
        cff a, b, cc;
        coef_ff(bc.lvff + (size_t)i * BLDFM_LV32, lx, ly, lx2, ly2, a, b, cc);
        const mff Ai = {a, cff{ff_neg(b.re), ff_neg(b.im)}, cff{ff_neg(cc.re), ff_neg(cc.im)}, a};
        if (i < sp) {
            Ml = mff_mul(Ml, Ai);
            mff_norm(Ml, EMl);
            Det = cff_mul(Det, cff_sub(cff_mul(a, a), cff_mul(b, cc)));
            cff_renorm(Det, EDet);
        } else {
            Mh = mff_mul(Mh, Ai);
            mff_norm(Mh, EMh);
        }
    }
    mff M = mff_mul(Ml, Mh);
    mff_norm(M);
    // suffix scan: S = M_lane ... M_31
    mff S = M;
#pragma unroll 1
    for (int d = 1; d < 32; d <<= 1) {
        const mff T = mff_shfl_down(S, d);
        if (lane + d < 32) {
            S = mff_mul(S, T);
            mff_norm(S);
        }
    }
    // ratio at the top of this lane's run: S_{lane+1}(R_L), or R_L for lane 31
    const mff Sn = mff_shfl_down(S, 1);
    cff Rtop = RL;
    if (lane < 31)
        Rtop = cff_div(cff_add(cff_mul(Sn.m11, RL), Sn.m12), cff_add(cff_mul(Sn.m21, RL), Sn.m22));
    // v_s = M_high (R_top, 1) (times 2^EMh), v_lo = M_low v_s (times 2^(EMl + EMh))
    const cff Ns = cff_add(cff_mul(Mh.m11, Rtop), Mh.m12), Ds = cff_add(cff_mul(Mh.m21, Rtop), Mh.m22);
    const cff Dlo = cff_add(cff_mul(Ml.m21, Ns), cff_mul(Ml.m22, Ds));
    // the lane's flux factors: F = Det Ds / Dlo (times 2^(EDet - EMl))
    cff F = one;
    int EF = 0;
    if (sp > lo) {
        F = cff_div(cff_mul(Det, Ds), Dlo);
        EF = EDet - EMl;
        cff_renorm(F, EF);
    }
    // exclusive prefix product over the lanes: P = F_0 ... F_{lane-1}
    cff P = F;
    int EP = EF;
#pragma unroll 1
    for (int d = 1; d < 32; d <<= 1) {
        const cff Po = cff_shfl_up(P, d);
        const int Eo = __shfl_up_sync(0xffffffffu, EP, d);
        if (lane >= d) {
            P = cff_mul(P, Po);
            EP += Eo;
            cff_renorm(P, EP);
        }
    }
    P = cff_shfl_up(P, 1);
    EP = __shfl_up_sync(0xffffffffu, EP, 1);
    if (lane == 0) {
        P = one;
        EP = 0;
    }
    const cff PF = cff_mul(P, F);  // the flux product up to level s of this lane
    const int EPF = EP + EF;
    // source spectrum and the FP32 sweep's phase factor (taken as exact)
    cff q0 = {ff_from_double(g.q0dc_fp), ff_from(0.f)};
    if (bc.q0) {
        const float2 f = bc.q0[(size_t)c * g.nly + r];
        q0 = {ff_from(f.x), ff_from(f.y)};
    }
    float2 sh = make_float2(1.f, 0.f);
    if (g.do_shift) {
        const uint32_t turns = (uint32_t)kx * g.turn_x + (uint32_t)ky * g.turn_y;
        float sn, cs;
        sincospif((float)(int32_t)turns * 4.656612873077393e-10f, &sn, &cs);
        sh = make_float2(cs, sn);
    }
    const cff qsh = cff_mul(q0, cff{ff_from(sh.x), ff_from(sh.y)});
    v = make_float4(0.f, 0.f, 0.f, 0.f);
    // exact values of output level j (flux product Qj * 2^E, ratio Rj) against
    // the spectra of its slot
    auto emit = [&](int j, cff Qj, int E, cff Rj) {
        const cff q = cff_mul(qsh, Qj);
        const cff p = cff_mul(Rj, q);
        const size_t o = spec_idx(g, bc.slot[j], r, c);
        const float2 pn = bc.Xp[o], qn = bc.Xq[o];
        const float pe0 = ldexpf(p.re.hi, E) + ldexpf(p.re.lo, E), pe1 = ldexpf(p.im.hi, E) + ldexpf(p.im.lo, E);
        const float qe0 = ldexpf(q.re.hi, E) + ldexpf(q.re.lo, E), qe1 = ldexpf(q.im.hi, E) + ldexpf(q.im.lo, E);
        // differences formed in float-float, so they keep their digits
        const float dpx = ldexpf(ff_sub(p.re, ff_from(ldexpf(pn.x, -E))).hi, E);
        const float dpy = ldexpf(ff_sub(p.im, ff_from(ldexpf(pn.y, -E))).hi, E);
        const float dqx = ldexpf(ff_sub(q.re, ff_from(ldexpf(qn.x, -E))).hi, E);
        const float dqy = ldexpf(ff_sub(q.im, ff_from(ldexpf(qn.y, -E))).hi, E);
        v.x += dpx * dpx + dpy * dpy;
        v.y += pe0 * pe0 + pe1 * pe1;
        v.z += dqx * dqx + dqy * dqy;
        v.w += qe0 * qe0 + qe1 * qe1;
    };
    // the top level as an output level (no run contains it)
    if (lane == 31 && jm == L && bc.slot[L] >= 0) emit(L, PF, EPF, RL);
    // the highest output level in this lane's run (s = jm)
    if (jm >= lo && jm < hi && bc.slot[jm] >= 0) emit(jm, PF, EPF, cff_div(Ns, Ds));
    // output levels below s in this lane's run: down from s, v_i and the det
    // product G over [i, s) (a footprint has none: its only level is jm)
    int jlo = sp;
    for (int i = lo; i < sp; ++i)
        if (bc.slot[i] >= 0) {
            jlo = i;
            break;
        }
    cff N = Ns, D = Ds, G = one;
    int ED = EMh, EG = 0;
    for (int i = sp - 1; i >= jlo; --i) {
        cff a, b, cc;
        coef_ff(bc.lvff + (size_t)i * BLDFM_LV32, lx, ly, lx2, ly2, a, b, cc);
        const cff Nn = cff_sub(cff_mul(a, N), cff_mul(b, D));
        const cff Dn = cff_sub(cff_mul(a, D), cff_mul(cc, N));
        N = Nn;
        D = Dn;
        cff_renorm2(N, D, ED);
        G = cff_mul(G, cff_sub(cff_mul(a, a), cff_mul(b, cc)));
        cff_renorm(G, EG);
        if (bc.slot[i] >= 0) {
            // Q(i) = P (Det / G) (D_i / D_lo)
            cff Qj = cff_mul(P, cff_div(cff_mul(Det, D), cff_mul(G, Dlo)));
            int E = EP + EDet - EG + ED - EMl - EMh;
            cff_renorm(Qj, E);
            emit(i, Qj, E, cff_div(N, D));
        }
    }
}

// true when -k of (kx, ky) lies in the mode range, so the sweep writes the
// mirror from this mode
__device__ __forceinline__ bool mirrored(const SolveGeom &g, int kx, int ky)
{
    return -kx >= freq_min(g.nlx) && -kx <= freq_max(g.nlx) && -ky >= freq_min(g.nly) && -ky <= freq_max(g.nly);
}

// one warp per sample, four samples per CTA
__global__ void __launch_bounds__(128) fp32_check_kernel(const BatchCase *__restrict__ cases, int n,
                                                         float4 *__restrict__ acc)
{
    const int wg = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (wg >= n * CHECK_NS) return;  // whole warps
    const int k = wg / CHECK_NS, j = wg - k * CHECK_NS;
    const BatchCase &bc = cases[k];
    const SolveGeom &g = bc.g;
    if (g.nsolved <= 0 || g.jmax < 0 || !bc.lvff) return;
    constexpr int NBOX = 2 * CHECK_BOX * CHECK_BOX + 2 * CHECK_BOX;  // solved modes with |kx|, |ky| <= CHECK_BOX
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    float wgt = 1.f;
    int kx = 0, ky = 0;
    bool have = false;
    if (j == 0) {
        // k = 0: the host's exact values at every output level, no error
        if (lane == 0)
            for (int i = 0; i <= g.jmax; ++i) {
                const int sl = bc.slot[i];
                if (sl < 0) continue;
                const double2 p = bc.dc[2 * sl], q = bc.dc[2 * sl + 1];
                v.y += (float)(p.x * p.x + p.y * p.y);
                v.w += (float)(q.x * q.x + q.y * q.y);
            }
    } else if (j <= NBOX) {
        const int t = j - 1;
        if (t < CHECK_BOX) {
            kx = 0;
            ky = t + 1;
        } else {
            kx = 1 + (t - CHECK_BOX) / (2 * CHECK_BOX + 1);
            ky = (t - CHECK_BOX) % (2 * CHECK_BOX + 1) - CHECK_BOX;
        }
        have = kx <= freq_max(g.nlx) && ky >= freq_min(g.nly) && ky <= freq_max(g.nly);
    } else {
        const int nb = CHECK_NS - 1 - NBOX, i = j - 1 - NBOX;
        const int64_t m = ((2 * (int64_t)i + 1) * g.nsolved) / (2 * (int64_t)nb);
        int r, c;
        bool paired;
        unpack_mode(bc.modes[m], r, c, paired);
        kx = freq_of_index(c, g.nlx);
        ky = freq_of_index(r, g.nly);
        have = true;
        wgt = (float)((double)(g.nsolved > NBOX ? g.nsolved - NBOX : 0) / nb);
    }
    if (have) {
        check_mode(bc, index_of_freq(ky, g.nly), index_of_freq(kx, g.nlx), lane, v);
        if (mirrored(g, kx, ky)) wgt *= 2.f;
        v = make_float4(wgt * v.x, wgt * v.y, wgt * v.z, wgt * v.w);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            v.x += __shfl_down_sync(0xffffffffu, v.x, off);
            v.y += __shfl_down_sync(0xffffffffu, v.y, off);
            v.z += __shfl_down_sync(0xffffffffu, v.z, off);
            v.w += __shfl_down_sync(0xffffffffu, v.w, off);
        }
    }
    if (lane == 0) {
        atomicAdd(&acc[k].x, v.x);
        atomicAdd(&acc[k].y, v.y);
        atomicAdd(&acc[k].z, v.z);
        atomicAdd(&acc[k].w, v.w);
    }
}

cudaError_t launch_fp32_check(const BatchCase *cases, int n, float4 *acc, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int64_t nthreads = (int64_t)n * CHECK_NS * 32;
    fp32_check_kernel<<<(unsigned)((nthreads + 127) / 128), 128, 0, st>>>(cases, n, acc);
    return cudaGetLastError();
}

void prepare_batch_attributes();

cudaError_t launch_batch_kernels(const BatchLaunch &bl, cudaStream_t st, int part)
{
    static uint64_t attr = 0;
    if (first_on_device(attr)) prepare_batch_attributes();
    // part 0: the sweep; part 1: the two transform passes
    if (part == 0 && bl.sweep_ctas > 0) {
        if (bl.threads == 128)
            riccati32_batch_kernel<128><<<bl.sweep_ctas, 128, bl.sweep_smem, st>>>(bl.cases, bl.tile_case,
                                                                                  bl.cta_tiles, bl.err);
        else
            riccati32_batch_kernel<256><<<bl.sweep_ctas, 256, bl.sweep_smem, st>>>(bl.cases, bl.tile_case,
                                                                                  bl.cta_tiles, bl.err);
    }
    if (part == 1 && bl.rx_col >= 0) {
        // every group's column pass, then every group's row pass
        for (int pass = 0; pass < 2; ++pass)
            for (int i = 0; i < bl.nxg; ++i) {
                const XGroup &x = bl.xg[i];
                BatchLaunch gl = bl;
                gl.col_case = bl.col_case + x.col_start;
                gl.row_case = bl.row_case + x.row_start;
                const cudaError_t e = pass == 0 ? launch_rx_pass(x.rx_col, true, gl, x.col_ctas, st)
                                                : launch_rx_pass(x.rx_row, false, gl, x.row_ctas, st);
                if (e != cudaSuccess) return e;
            }
        return cudaGetLastError();
    }
    if (part == 1 && bl.persist) {
        if (bl.col_ctas > 0)
            out_cols_persist_kernel<<<bl.col_grid, 256, bl.col_smem, st>>>(bl.cases, bl.col_case, bl.col_ctas,
                                                                           bl.maxn_col, bl.maxnly, bl.err);
        if (bl.row_ctas > 0)
            out_rows_persist_kernel<<<bl.row_grid, 256, bl.row_smem, st>>>(bl.cases, bl.row_case, bl.row_ctas,
                                                                           bl.maxn_row, bl.err);
    } else {
        if (part == 1 && bl.col_ctas > 0)
            out_cols_batch_kernel<<<bl.col_ctas, 256, bl.col_smem, st>>>(bl.cases, bl.col_case, bl.err);
        if (part == 1 && bl.row_ctas > 0)
            out_rows_batch_kernel<<<bl.row_ctas, 256, bl.row_smem, st>>>(bl.cases, bl.row_case, bl.err);
    }
    return cudaGetLastError();
}

// resident CTAs per SM of the persistent sweep, memoised per (device, shape,
// shared memory): the first query sets every batch kernel's attributes
int batch_sweep_occupancy(int threads, size_t smem)
{
    static std::mutex m;
    static std::map<std::tuple<int, int, size_t>, int> memo;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    const auto key = std::make_tuple(dev, threads, smem);
    {
        std::lock_guard<std::mutex> lk(m);
        const auto it = memo.find(key);
        if (it != memo.end()) return it->second;
    }
    prepare_batch_attributes();
    int nb = 0;
    const cudaError_t e =
        threads == 128 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, riccati32_batch_kernel<128>, 128, smem)
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, riccati32_batch_kernel<256>, 256, smem);
    const int r = e == cudaSuccess && nb > 0 ? nb : 1;
    if (e == cudaSuccess) {
        std::lock_guard<std::mutex> lk(m);
        memo[key] = r;
    }
    return r;
}

// resident CTAs per SM of the persistent column (col != 0) or row transform
int batch_xform_occupancy(int col, size_t smem)
{
    prepare_batch_attributes();
    int nb = 0;
    const cudaError_t e =
        col ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, out_cols_persist_kernel, 256, smem)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, out_rows_persist_kernel, 256, smem);
    return e == cudaSuccess && nb > 0 ? nb : 1;
}

void prepare_batch_attributes()
{
    prepare_rx_attributes();
    cudaFuncSetAttribute(riccati32_batch_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(riccati32_batch_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(out_cols_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(out_rows_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(out_cols_persist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(out_rows_persist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}
