// Output transform (solver.py:264-290), one line at a time, shared by the
// single-solve and batched kernels.
#pragma once

#include "devmath.cuh"
#include "fft_core.cuh"

// One band column b of level lvl: builds Z = Hp + i Hq with
// H(P) = (X(P) + conj X(-P)) / 2 (the k = 0 entry from dc), transforms along y
// and keeps rows [py, py + out_ny).  Output Cout[(lvl * nbx + b) * out_ny + y'].
// smem: 3 n complex (two ping-pong buffers, twiddles).
template <typename R>
__device__ __forceinline__ void out_col_line(const SolveGeom &g, const FftPlan &pl,
                                             const typename cvec<R>::T *__restrict__ tw,
                                             const int4 *__restrict__ xband,
                                             const typename cvec<R>::T *__restrict__ Xp,
                                             const typename cvec<R>::T *__restrict__ Xq,
                                             const double2 *__restrict__ dc, typename cvec<R>::T *__restrict__ Cout,
                                             int b, int lvl, typename cvec<R>::T *smem)
{
    typedef typename cvec<R>::T C;
    const int n = pl.n;
    C *bufA = smem;
    C *bufB = bufA + n;
    C *stw = bufB + n;
    const int4 bx = xband[b];  // x = position, y = column of X at P, z = column of X at -P
    // issue every global load of this line before the first barrier
    const R h = (R)0.5;
    const double2 dp = dc[2 * lvl], dq = dc[2 * lvl + 1];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        bufA[i] = cx_make<C>(0.0, 0.0);
        stw[i] = tw[i];
    }
    __syncthreads();
    if (bx.y >= 0) {
        const size_t base = ((size_t)lvl * g.nlx + bx.y) * g.nly;
        for (int r = threadIdx.x; r < g.nly; r += blockDim.x) {
            const int ky = freq_of_index(r, g.nly);
            const int pos = ky >= 0 ? ky : ky + n;
            C p = Xp[base + r], q = Xq[base + r];
            if (bx.y == 0 && r == 0) {
                p = cx_make<C>(dp.x, dp.y);
                q = cx_make<C>(dq.x, dq.y);
            }
            bufA[pos] = cx_make<C>(h * (p.x - q.y), h * (p.y + q.x));
        }
    }
    __syncthreads();
    if (bx.z >= 0) {
        const size_t base = ((size_t)lvl * g.nlx + bx.z) * g.nly;
        for (int r = threadIdx.x; r < g.nly; r += blockDim.x) {
            const int ky = freq_of_index(r, g.nly);
            const int pm = ky > 0 ? n - ky : -ky;  // position of -ky
            C p = Xp[base + r], q = Xq[base + r];
            if (bx.z == 0 && r == 0) {
                p = cx_make<C>(dp.x, dp.y);
                q = cx_make<C>(dq.x, dq.y);
            }
            C cur = bufA[pm];
            cur.x += h * (p.x + q.y);
            cur.y += h * (q.x - p.y);
            bufA[pm] = cur;
        }
    }
    C *res = fft_run<C>(bufA, bufB, pl, 1, stw, g.out_sign);
    C *o = Cout + ((size_t)lvl * g.nbx + b) * g.out_ny;
    for (int y = threadIdx.x; y < g.out_ny; y += blockDim.x) o[y] = res[g.py + y];
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
    for (int i = threadIdx.x; i < nl * g.nbx; i += blockDim.x) {
        const int b = i / nl, l = i - b * nl;
        bufA[(size_t)l * n + xband[b].x] = Cin[((size_t)lvl * g.nbx + b) * g.out_ny + y0 + l];
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
