// Output transform (solver.py:264-290), one line at a time, shared by the
// single-solve and batched kernels.
#pragma once

#include <limits.h>

#include "devmath.cuh"
#include "fft_core.cuh"

// Band columns b0 .. b0 + ncols - 1 of level lvl (those < nbx): builds
// Z = Hp + i Hq with H(P) = (X(P) + conj X(-P)) / 2 (the k = 0 entry from dc),
// transforms along y and keeps rows [py, py + out_ny).  Output row-major,
// Cout[(lvl * out_ny + y') * nbx + b], so that ncols adjacent columns fill
// whole 32-byte sectors here and the row pass reads contiguous rows.  ncols
// is a power of two.  smem: (2 ncols + 1) n complex (two ping-pong buffers of
// ncols lines, twiddles).
template <typename R>
__device__ __forceinline__ void out_col_lines(const SolveGeom &g, const FftPlan &pl,
                                              const typename cvec<R>::T *__restrict__ tw,
                                              const int4 *__restrict__ xband,
                                              const typename cvec<R>::T *__restrict__ Xp,
                                              const typename cvec<R>::T *__restrict__ Xq,
                                              const double2 *__restrict__ dc, typename cvec<R>::T *__restrict__ Cout,
                                              int b0, int ncols, int lvl, typename cvec<R>::T *smem)
{
    typedef typename cvec<R>::T C;
    const int n = pl.n;
    C *bufA = smem;
    C *bufB = bufA + (size_t)ncols * n;
    C *stw = bufB + (size_t)ncols * n;
    const int nc = min(ncols, g.nbx - b0);
    if (nc <= 0) return;
    const R h = (R)0.5;
    const double2 dp = dc[2 * lvl], dq = dc[2 * lvl + 1];
    for (int i = threadIdx.x; i < n; i += blockDim.x) stw[i] = tw[i];
    // one gather per line position: the position holds X(ky) of column bx.y
    // for the mode ky = pos or pos - n, and conj X(ky) of column bx.z for the
    // mode ky = -pos or n - pos (whichever lies in [fmin, fmax]; at most one
    // of each pair does); every other position is zero
    const int fmin = freq_min(g.nly), fmax = freq_max(g.nly);
    for (int c = 0; c < nc; ++c) {
        const int4 bx = xband[b0 + c];  // x = position, y = column of X at P, z = column of X at -P
        C *line = bufA + (size_t)c * n;
        const size_t bp = ((size_t)lvl * g.nlx + max(bx.y, 0)) * g.nly;
        const size_t bm = ((size_t)lvl * g.nlx + max(bx.z, 0)) * g.nly;
#pragma unroll 4
        for (int pos = threadIdx.x; pos < n; pos += blockDim.x) {
            const int kp = pos <= fmax ? pos : (pos - n >= fmin ? pos - n : INT_MIN);
            const int km = -pos >= fmin ? -pos : (n - pos <= fmax ? n - pos : INT_MIN);
            R re = (R)0, im = (R)0;
            if (bx.y >= 0 && kp != INT_MIN) {
                const int r = index_of_freq(kp, g.nly);
                C p = Xp[bp + r], q = Xq[bp + r];
                if (bx.y == 0 && r == 0) {
                    p = cx_make<C>(dp.x, dp.y);
                    q = cx_make<C>(dq.x, dq.y);
                }
                re = h * (p.x - q.y);
                im = h * (p.y + q.x);
            }
            if (bx.z >= 0 && km != INT_MIN) {
                const int r = index_of_freq(km, g.nly);
                C p = Xp[bm + r], q = Xq[bm + r];
                if (bx.z == 0 && r == 0) {
                    p = cx_make<C>(dp.x, dp.y);
                    q = cx_make<C>(dq.x, dq.y);
                }
                re += h * (p.x + q.y);
                im += h * (q.x - p.y);
            }
            line[pos] = cx_make<C>(re, im);
        }
    }
    C *res = fft_run<C>(bufA, bufB, pl, nc, stw, g.out_sign);
    const int lc = 31 - __clz(ncols);  // log2 ncols
    C *o = Cout + (size_t)lvl * g.out_ny * g.nbx + b0;
    for (int i = threadIdx.x; i < (g.out_ny << lc); i += blockDim.x) {
        const int y = i >> lc, c = i & (ncols - 1);
        if (c < nc) o[(size_t)y * g.nbx + c] = res[(size_t)c * n + g.py + y];
    }
}

// Line of band column bx = (position, column of X at P, column of X at -P)
// of level lvl, for a Hermitian-complete FP32 spectrum, from the P-side
// column staged in shared memory (sp: Xp, sq: Xq, nly each); positions with
// one side out of range and the zero mode read the -P side from global
// memory.  The thread block writes the n entries of line.
__device__ __forceinline__ void col_line_from_staged(const SolveGeom &g, const int4 bx, const float2 *sp,
                                                     const float2 *sq, const float2 *__restrict__ Xp,
                                                     const float2 *__restrict__ Xq, const double2 *__restrict__ dc,
                                                     int n, int lvl, float2 *line)
{
    const int nly = g.nly;
    const float h = 0.5f;
    const int fmin = freq_min(nly), fmax = freq_max(nly);
    {
        if (bx.y > 0 && bx.z > 0) {
            // both columns present and not the zero column: positions
            // [0, fmax] and [n + fmin, n) hold mode kp = pos or pos - n (row
            // pos or pos - n + nly); the mirror -kp is in range except at
            // kp = fmin; position -fmin holds only the conjugate half of
            // X(-P) at ky = fmin; every other position is zero
            const int nlo = fmax + 1, nhi = -fmin;  // counts of the two runs
            for (int i = threadIdx.x; i < nlo + nhi; i += blockDim.x) {
                const int pos = i < nlo ? i : n - nhi + (i - nlo);
                const int r = i < nlo ? i : nly - nhi + (i - nlo);
                const float2 p = sp[r], q = sq[r];
                float re = p.x - q.y, im = p.y + q.x;
                if (pos == n + fmin && -fmin > fmax) {  // kp = fmin: the mirror -fmin is out of range
                    re = h * re;
                    im = h * im;
                }
                line[pos] = make_float2(re, im);
            }
            for (int i = nlo + 1 + threadIdx.x; i < n - nhi; i += blockDim.x) line[i] = make_float2(0.f, 0.f);
            if (threadIdx.x == 0) {
                const size_t bm = ((size_t)lvl * g.nlx + bx.z) * nly + index_of_freq(fmin, nly);
                const float2 p = Xp[bm], q = Xq[bm];
                line[nlo] = make_float2(h * (p.x + q.y), h * (q.x - p.y));
            }
            return;
        }
#pragma unroll 4
        for (int pos = threadIdx.x; pos < n; pos += blockDim.x) {
            const int kp = pos <= fmax ? pos : (pos - n >= fmin ? pos - n : INT_MIN);
            const int km = -pos >= fmin ? -pos : (n - pos <= fmax ? n - pos : INT_MIN);
            const bool pin = bx.y >= 0 && kp != INT_MIN, min_ = bx.z >= 0 && km != INT_MIN;
            float re = 0.f, im = 0.f;
            if (pin && min_ && !(bx.y == 0 && kp == 0)) {
                // mirror pair: H(P) = X(P)
                const int r = index_of_freq(kp, nly);
                const float2 p = sp[r], q = sq[r];
                re = p.x - q.y;
                im = p.y + q.x;
            } else {
                if (pin) {
                    const int r = index_of_freq(kp, nly);
                    float2 p = sp[r], q = sq[r];
                    if (bx.y == 0 && r == 0) {
                        const double2 dp = dc[2 * lvl], dq = dc[2 * lvl + 1];
                        p = make_float2((float)dp.x, (float)dp.y);
                        q = make_float2((float)dq.x, (float)dq.y);
                    }
                    re = h * (p.x - q.y);
                    im = h * (p.y + q.x);
                }
                if (min_) {
                    const int r = index_of_freq(km, nly);
                    float2 p, q;
                    if (bx.z == 0 && r == 0) {
                        const double2 dp = dc[2 * lvl], dq = dc[2 * lvl + 1];
                        p = make_float2((float)dp.x, (float)dp.y);
                        q = make_float2((float)dq.x, (float)dq.y);
                    } else {
                        const size_t bm = ((size_t)lvl * g.nlx + bx.z) * nly;
                        p = Xp[bm + r];
                        q = Xq[bm + r];
                    }
                    re += h * (p.x + q.y);
                    im += h * (q.x - p.y);
                }
            }
            line[pos] = make_float2(re, im);
        }
    }
}

// out_col_lines (FP32) with its inputs staged by bulk copies.  The spectrum
// of every solve is Hermitian-complete: each in-range mode P with -P also in
// range holds X(-P) = conj X(P) exactly (the sweep writes the mirror), so
// where both lie in range H(P) = (X(P) + conj X(-P)) / 2 is X(P) to the bit,
// and the line needs only the column at P.  Thread 0 brings that column of
// Xp and Xq (nly complex each, into the second line buffer, which the FFT
// overwrites only later) and the twiddles in with bulk copies completing on
// one mbarrier: the gather costs one memory round trip.  The few positions
// with one side out of range, and the zero mode, take the general formula
// (the -P side from global memory).  Needs n and nly even, 2 nly <= n and
// 16-byte aligned arrays; otherwise it runs out_col_lines.  bar: an
// initialised mbarrier in phase 0.  smem: (2 ncols + 1) n complex.  Returns
// false if the bounded wait for the copies ran out.
__device__ __forceinline__ bool out_col_lines_staged(const SolveGeom &g, const FftPlan &pl,
                                                     const float2 *__restrict__ tw, const int4 *__restrict__ xband,
                                                     const float2 *__restrict__ Xp, const float2 *__restrict__ Xq,
                                                     const double2 *__restrict__ dc, float2 *__restrict__ Cout,
                                                     int b0, int ncols, int lvl, float2 *smem, uint64_t *bar)
{
    const int n = pl.n, nly = g.nly;
    float2 *bufA = smem;
    float2 *bufB = bufA + (size_t)ncols * n;
    float2 *stw = bufB + (size_t)ncols * n;
    const int nc = min(ncols, g.nbx - b0);
    if (nc <= 0) return true;
    if (((n | nly) & 1) || 2 * nly > n ||
        ((((uintptr_t)Xp) | ((uintptr_t)Xq) | ((uintptr_t)tw) | ((uintptr_t)smem)) & 15)) {
        out_col_lines<float>(g, pl, tw, xband, Xp, Xq, dc, Cout, b0, ncols, lvl, smem);
        return true;
    }
    const uint32_t colb = (uint32_t)nly * 8u;
    if (threadIdx.x == 0) {
        uint32_t bytes = (uint32_t)n * 8u;
        for (int c = 0; c < nc; ++c) bytes += xband[b0 + c].y >= 0 ? 2u * colb : 0u;
        const uint32_t ba = (uint32_t)__cvta_generic_to_shared(bar);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ba), "r"(bytes) : "memory");
        auto bulk = [&](float2 *dst, const float2 *src, uint32_t nb) {
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                             (uint32_t)__cvta_generic_to_shared(dst)),
                         "l"(src), "r"(nb), "r"(ba)
                         : "memory");
        };
        bulk(stw, tw, (uint32_t)n * 8u);
        for (int c = 0; c < nc; ++c) {
            const int col = xband[b0 + c].y;
            if (col >= 0) {
                const size_t bp = ((size_t)lvl * g.nlx + col) * nly;
                bulk(bufB + (size_t)c * n, Xp + bp, colb);
                bulk(bufB + (size_t)c * n + nly, Xq + bp, colb);
            }
        }
    }
    bool done = false;
    {
        const uint32_t ba = (uint32_t)__cvta_generic_to_shared(bar);
        for (long it = 0; it < BLDFM_WAIT_POLLS && !done; ++it) {
            uint32_t d;
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(d)
                : "r"(ba), "r"(0u)
                : "memory");
            done = d != 0;
        }
    }
    if (__syncthreads_or(!done)) return false;
    for (int c = 0; c < nc; ++c) {
        const float2 *sp = bufB + (size_t)c * n;
        col_line_from_staged(g, xband[b0 + c], sp, sp + nly, Xp, Xq, dc, n, lvl, bufA + (size_t)c * n);
    }
    float2 *res = fft_run<float2>(bufA, bufB, pl, nc, stw, g.out_sign);
    const int lc = 31 - __clz(ncols);  // log2 ncols
    float2 *o = Cout + (size_t)lvl * g.out_ny * g.nbx + b0;
    for (int i = threadIdx.x; i < (g.out_ny << lc); i += blockDim.x) {
        const int y = i >> lc, c = i & (ncols - 1);
        if (c < nc) o[(size_t)y * g.nbx + c] = res[(size_t)c * n + g.py + y];
    }
    return true;
}

// rpc output rows starting at y0 of level lvl: places the band columns,
// transforms along x, writes the cropped window: conc = Re, flx = Im.  A
// non-finite output value sets *err to BLDFM_ERR_NONFINITE_DEV (if err is not
// null and no earlier error is recorded).  Every thread of the block calls it.
// smem: (2 rpc + 1) n complex.
template <typename R>
__device__ __forceinline__ void out_row_lines(const SolveGeom &g, const FftPlan &pl,
                                              const typename cvec<R>::T *__restrict__ tw,
                                              const int4 *__restrict__ xband,
                                              const typename cvec<R>::T *__restrict__ Cin, double *__restrict__ conc,
                                              double *__restrict__ flx, int y0, int rows_per_cta, int lvl,
                                              typename cvec<R>::T *smem, int *err)
{
    typedef typename cvec<R>::T C;
    const int n = pl.n;
    C *bufA = smem;
    C *bufB = bufA + (size_t)rows_per_cta * n;
    C *stw = bufB + (size_t)rows_per_cta * n;
    const int nl = min(rows_per_cta, g.out_ny - y0);
    // the rows' band values (contiguous: nl x nbx from row y0) go into
    // registers first, so that their loads overlap the zero fill and the
    // twiddle loads; entries past the first PF x blockDim are placed after
    constexpr int PF = 8;
    const int nb = g.nbx, tot = nl * nb;
    const C *rows = Cin + ((size_t)lvl * g.out_ny + y0) * nb;
    C pre[PF];
#pragma unroll
    for (int k = 0; k < PF; ++k) {
        const int i = threadIdx.x + k * (int)blockDim.x;
        if (i < tot) pre[k] = rows[i];
    }
    for (int i = threadIdx.x; i < nl * n; i += blockDim.x) bufA[i] = cx_make<C>(0.0, 0.0);
    for (int i = threadIdx.x; i < n; i += blockDim.x) stw[i] = tw[i];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < PF; ++k) {
        const int i = threadIdx.x + k * (int)blockDim.x;
        if (i < tot) {
            const int l = i / nb, b = i - l * nb;
            bufA[(size_t)l * n + xband[b].x] = pre[k];
        }
    }
    for (int i = threadIdx.x + PF * (int)blockDim.x; i < tot; i += blockDim.x) {
        const int l = i / nb, b = i - l * nb;
        bufA[(size_t)l * n + xband[b].x] = rows[i];
    }
    C *res = fft_run<C>(bufA, bufB, pl, nl, stw, g.out_sign);
    bool bad = false;
    for (int i = threadIdx.x; i < nl * g.out_nx; i += blockDim.x) {
        const int l = i / g.out_nx, x = i - l * g.out_nx;
        const C v = res[(size_t)l * n + g.px + x];
        const size_t o = ((size_t)lvl * g.out_ny + y0 + l) * g.out_nx + x;
        conc[o] = (double)v.x;
        flx[o] = (double)v.y;
        bad |= !(isfinite(v.x) && isfinite(v.y));
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0 && err) atomicCAS(err, 0, BLDFM_ERR_NONFINITE_DEV);
}
