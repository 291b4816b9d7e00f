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

// rpc output rows starting at y0 of level lvl: places the band columns,
// transforms along x, writes the cropped window: conc = Re, flx = Im.
// smem: (2 rpc + 1) n complex.
template <typename R>
__device__ __forceinline__ void out_row_lines(const SolveGeom &g, const FftPlan &pl,
                                              const typename cvec<R>::T *__restrict__ tw,
                                              const int4 *__restrict__ xband,
                                              const typename cvec<R>::T *__restrict__ Cin, double *__restrict__ conc,
                                              double *__restrict__ flx, int y0, int rows_per_cta, int lvl,
                                              typename cvec<R>::T *smem)
{
    typedef typename cvec<R>::T C;
    const int n = pl.n;
    C *bufA = smem;
    C *bufB = bufA + (size_t)rows_per_cta * n;
    C *stw = bufB + (size_t)rows_per_cta * n;
    const int nl = min(rows_per_cta, g.out_ny - y0);
    for (int i = threadIdx.x; i < nl * n; i += blockDim.x) bufA[i] = cx_make<C>(0.0, 0.0);
    for (int i = threadIdx.x; i < n; i += blockDim.x) stw[i] = tw[i];
    __syncthreads();
    for (int l = 0; l < nl; ++l) {
        const C *row = Cin + ((size_t)lvl * g.out_ny + y0 + l) * g.nbx;
        C *dst = bufA + (size_t)l * n;
        for (int b = threadIdx.x; b < g.nbx; b += blockDim.x) dst[xband[b].x] = row[b];
    }
    C *res = fft_run<C>(bufA, bufB, pl, nl, stw, g.out_sign);
    for (int i = threadIdx.x; i < nl * g.out_nx; i += blockDim.x) {
        const int l = i / g.out_nx, x = i - l * g.out_nx;
        const C v = res[(size_t)l * n + g.px + x];
        const size_t o = ((size_t)lvl * g.out_ny + y0 + l) * g.out_nx + x;
        conc[o] = (double)v.x;
        flx[o] = (double)v.y;
    }
}
