// Batched output transform (solver.py:264-290) with register-resident lines:
// the column pass (spectrum columns -> band-column lines along y, crop) and
// the row pass (band rows -> lines along x, crop, conc = Re, flx = Im) of
// bldfm_solve_batch for line lengths 64 * E.  One CTA = 256 threads = G
// groups of P threads, one line per group (xform_reg.cuh); the row pass
// runs two lines per group in the two lanes of packed FP32x2 arithmetic for
// E <= 24.  Inputs are read
// straight from global memory into registers (consecutive threads read
// consecutive positions of a line); the column pass stages its G lines'
// kept rows through shared memory so that every row of the intermediate
// gets whole 32-byte sectors; the row pass writes its outputs directly.
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include "batch.h"
#include "common.h"
#include "devmath.cuh"
#include "xform_reg.cuh"
#include "xform_zoom.cuh"

namespace {

using S768 = rx::Shape<24, 4, 8>;
using S512 = rx::Shape<8, 8, 8>;
using S1024 = rx::Shape<16, 8, 8>;
using S1536 = rx::Shape<24, 8, 8>;
using S2048 = rx::Shape<32, 8, 8>;
using S3072 = rx::Shape<48, 8, 8>;

constexpr int kThreads = 256;

// CTAs per SM the register budget is sized for: 3 (24 warps) up to E = 24,
// else whatever fits
template <class S>
constexpr int min_ctas()
{
    return S::E <= 24 ? 3 : 1;
}

__device__ __forceinline__ void load_case_rx(BatchCase *dst, const BatchCase *src)
{
    const int nw = (int)(sizeof(BatchCase) / 4);
    const int *s = (const int *)src;
    int *d = (int *)dst;
    for (int i = threadIdx.x; i < nw; i += blockDim.x) d[i] = s[i];
}

// Value at position pos of band column bx of level lvl: Z = Hp + i Hq,
// H(P) = (X(P) + conj X(-P)) / 2 with -P taken on the periodic grid (the
// k = 0 entry from dc).  The FP32 spectra are Hermitian-complete: the sweep
// writes every paired mode's mirror as its exact conjugate, so where -P is
// the signed mirror of P inside the mode range, H(P) = X(P).  That excludes
// the Nyquist row and column of an untruncated spectrum, whose periodic
// mirror (-N/2 -> -N/2) is a separately solved mode.  xpair: the column at -P
// (bx.z) holds the signed mirror -kx of the column at P (bx.y).  Out of line:
// the passes call it only for the few positions the staged one-sided path
// does not cover, and inlining it at every unrolled position made the column
// pass wait on instruction fetches.
__device__ __noinline__ float2 col_value(const SolveGeom &g, const int4 bx, bool xpair,
                                            const float2 *__restrict__ Xp, const float2 *__restrict__ Xq,
                                            const double2 *__restrict__ dc, int lvl, int n, int pos)
{
    const int nly = g.nly, fmin = freq_min(nly), fmax = freq_max(nly);
    const int kp = pos <= fmax ? pos : (pos - n >= fmin ? pos - n : INT_MIN);
    const int km = -pos >= fmin ? -pos : (n - pos <= fmax ? n - pos : INT_MIN);
    const bool pin = bx.y >= 0 && kp != INT_MIN, mn = bx.z >= 0 && km != INT_MIN;
    if (!pin && !mn) return make_float2(0.f, 0.f);
    if (pin && mn && xpair && km == -kp && !(bx.y == 0 && kp == 0)) {
        const size_t o = ((size_t)lvl * g.nlx + bx.y) * nly + index_of_freq(kp, nly);
        const float2 p = __ldg(Xp + o), q = __ldg(Xq + o);
        return make_float2(p.x - q.y, p.y + q.x);
    }
    float re = 0.f, im = 0.f;
    if (pin) {
        const int r = index_of_freq(kp, nly);
        float2 p, q;
        if (bx.y == 0 && r == 0) {
            const double2 dp = dc[2 * lvl], dq = dc[2 * lvl + 1];
            p = make_float2((float)dp.x, (float)dp.y);
            q = make_float2((float)dq.x, (float)dq.y);
        } else {
            const size_t o = ((size_t)lvl * g.nlx + bx.y) * nly + r;
            p = __ldg(Xp + o);
            q = __ldg(Xq + o);
        }
        re = 0.5f * (p.x - q.y);
        im = 0.5f * (p.y + q.x);
    }
    if (mn) {
        const int r = index_of_freq(km, nly);
        float2 p, q;
        if (bx.z == 0 && r == 0) {
            const double2 dp = dc[2 * lvl], dq = dc[2 * lvl + 1];
            p = make_float2((float)dp.x, (float)dp.y);
            q = make_float2((float)dq.x, (float)dq.y);
        } else {
            const size_t o = ((size_t)lvl * g.nlx + bx.z) * nly + r;
            p = __ldg(Xp + o);
            q = __ldg(Xq + o);
        }
        re += 0.5f * (p.x + q.y);
        im += 0.5f * (q.x - p.y);
    }
    return make_float2(re, im);
}

// Band column of a line position along x: the band holds the frequencies
// f in [-h, h] (h = max(-fmin, fmax) of nlx) at positions f mod nfx, in the
// order of f; when 2 h = nfx the position of -h and h coincide and -h is
// kept.  Returns -1 for positions outside the band.
__device__ __forceinline__ int band_of(int pos, int h, int nfx)
{
    if (pos >= nfx - h) return pos - nfx + h;
    if (pos <= h) return pos + h;
    return -1;
}

// Column pass.  When a line's two spectrum columns (Xp and Xq at P, nly
// complex each) fit in the group's exchange buffer, one thread of the group
// brings them in with two bulk copies completing on the group's mbarrier
// (every load of the line in flight at once, none in registers); the few
// positions that need the column at -P read it from global memory.
template <class S>
__global__ void __launch_bounds__(kThreads, min_ctas<S>()) rx_cols_batch_kernel(const BatchCase *__restrict__ cases,
                                                                                const int *__restrict__ cta_case,
                                                                                int *err)
{
    constexpr int P = S::P, E = S::E, G = kThreads / P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *sbuf = (float2 *)smem_raw;
    __shared__ __align__(16) BatchCase sc;
    __shared__ uint64_t gbar[G];
    load_case_rx(&sc, cases + cta_case[blockIdx.x]);
    const int grp = threadIdx.x / P, t = threadIdx.x - grp * P;
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&gbar[grp])), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    const SolveGeom &g = sc.g;
    // 32-bit index arithmetic: a pass launches fewer than 2^31 CTAs
    const int local = (int)((int64_t)blockIdx.x - sc.col0);
    const int ncb = (g.nbx + G - 1) / G;
    const int lvl = local / ncb, cb = local - lvl * ncb;
    const int b = cb * G + grp;
    const bool active = b < g.nbx;
    const float cj = g.out_sign > 0 ? -1.f : 1.f;  // inverse transform: conjugate in and out
    float2 *buf = sbuf + grp * S::BUF;
    float2 x[E];
    bool timed_out = false;
    if (active) {
        const int4 bx = sc.xband[b];
        const bool xpair =
            bx.y >= 0 && bx.z >= 0 && freq_of_index(bx.z, g.nlx) == -freq_of_index(bx.y, g.nlx);
        const int nly = g.nly;
        const size_t colp = ((size_t)lvl * g.nlx + (bx.y > 0 ? bx.y : 0)) * nly;
        const bool stage = bx.y >= 0 && 2 * nly <= S::BUF && (nly & 1) == 0 &&
                           ((((uintptr_t)sc.Xp) | ((uintptr_t)sc.Xq)) & 15) == 0;
        if (stage) {
            const uint32_t ba = smem_u32(&gbar[grp]);
            if (t == 0) {
                const uint32_t nb = (uint32_t)nly * 8u;
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ba), "r"(2u * nb)
                             : "memory");
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        smem_u32(buf)),
                    "l"(sc.Xp + colp), "r"(nb), "r"(ba)
                    : "memory");
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        smem_u32(buf + nly)),
                    "l"(sc.Xq + colp), "r"(nb), "r"(ba)
                    : "memory");
            }
            uint32_t done = 0;
            for (long it = 0; it < BLDFM_WAIT_POLLS && !done; ++it)
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                    "selp.u32 %0, 1, 0, p;\n\t}"
                    : "=r"(done)
                    : "r"(ba), "r"(0u)
                    : "memory");
            timed_out = !done;
            const int fmin = freq_min(nly), fmax = freq_max(nly), n = S::N;
#pragma unroll
            for (int m = 0; m < E; ++m) {
                const int pos = t + P * m;
                const int kp = pos <= fmax ? pos : (pos - n >= fmin ? pos - n : INT_MIN);
                const int km = -pos >= fmin ? -pos : (n - pos <= fmax ? n - pos : INT_MIN);
                const bool mn = bx.z >= 0 && km != INT_MIN;
                float2 v = make_float2(0.f, 0.f);
                if (kp != INT_MIN && mn && xpair && km == -kp && !(bx.y == 0 && kp == 0)) {
                    const int r = index_of_freq(kp, nly);
                    const float2 p = buf[r], q = buf[nly + r];
                    v = make_float2(p.x - q.y, p.y + q.x);
                } else if (kp != INT_MIN || mn) {
                    v = col_value(g, bx, xpair, sc.Xp, sc.Xq, sc.dc, lvl, n, pos);
                }
                x[m] = make_float2(v.x, cj * v.y);
            }
            rx::group_bar(grp + 1, P);  // the staged columns are read before the buffer is reused
        } else {
#pragma unroll
            for (int m = 0; m < E; ++m) {
                const float2 v = col_value(g, bx, xpair, sc.Xp, sc.Xq, sc.dc, lvl, S::N, t + P * m);
                x[m] = make_float2(v.x, cj * v.y);
            }
        }
        rx::line_fft<S>(x, t, buf, sc.twy, grp + 1);
    }
    if (__syncthreads_or(timed_out) && threadIdx.x == 0) atomicExch(err, BLDFM_ERR_TIMEOUT_DEV);
    // kept rows [py, py + out_ny) of the G lines staged line-major, [G][ys]
    // with ys = out_ny rounded up to 4 mod 16 words: conflict-free writes
    // along y here and reads across the G lines below
    const int ony = g.out_ny, py = g.py;
    const int ys = ((ony + 11) & ~15) + 4;
    if (active) {
#pragma unroll
        for (int m = 0; m < E; ++m) {
            const int y = t + P * m - py;
            if (y >= 0 && y < ony) sbuf[(size_t)grp * ys + y] = make_float2(x[m].x, cj * x[m].y);
        }
    }
    __syncthreads();
    const int ng = min(G, g.nbx - cb * G);
    float2 *o = sc.Cb + (size_t)lvl * ony * g.nbx + cb * G;
    for (int i = threadIdx.x; i < ony * G; i += kThreads) {
        const int y = i / G, gg = i - y * G;
        if (gg < ng) o[(size_t)y * g.nbx + gg] = sbuf[(size_t)gg * ys + y];
    }
}

template <class S>
__global__ void __launch_bounds__(kThreads, min_ctas<S>()) rx_rows_batch_kernel(const BatchCase *__restrict__ cases,
                                                                const int *__restrict__ cta_case, int *err)
{
    constexpr int P = S::P, E = S::E, G = kThreads / P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *sbuf = (float2 *)smem_raw;
    __shared__ __align__(16) BatchCase sc;
    load_case_rx(&sc, cases + cta_case[blockIdx.x]);
    __syncthreads();
    const SolveGeom &g = sc.g;
    const int local = (int)((int64_t)blockIdx.x - sc.row0);  // fewer than 2^31 CTAs
    const int nblk = (g.out_ny + G - 1) / G;
    const int lvl = local / nblk, yb = local - lvl * nblk;
    const int grp = threadIdx.x / P, t = threadIdx.x - grp * P;
    const int y = yb * G + grp;
    bool bad = false;
    if (y < g.out_ny) {
        const float cj = g.out_sign > 0 ? -1.f : 1.f;
        const int f0 = freq_min(g.nlx), f1 = freq_max(g.nlx);
        const int h = -f0 > f1 ? -f0 : f1;
        const float2 *row = sc.Cb + ((size_t)lvl * g.out_ny + y) * g.nbx;
        float2 x[E];
#pragma unroll
        for (int m = 0; m < E; ++m) {
            const int bcol = band_of(t + P * m, h, S::N);
            float2 v = make_float2(0.f, 0.f);
            if (bcol >= 0) v = __ldg(row + bcol);
            x[m] = make_float2(v.x, cj * v.y);
        }
        rx::line_fft<S>(x, t, sbuf + grp * S::BUF, sc.twx, grp + 1);
        const int onx = g.out_nx, px = g.px;
        const size_t ob = ((size_t)lvl * g.out_ny + y) * onx;
#pragma unroll
        for (int m = 0; m < E; ++m) {
            const int xo = t + P * m - px;
            if (xo >= 0 && xo < onx) {
                const float re = x[m].x, im = cj * x[m].y;
                rx::store_f64(sc.conc + ob + xo, re);
                rx::store_f64(sc.flx + ob + xo, im);
                bad |= !(isfinite(re) && isfinite(im));
            }
        }
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicCAS(err, 0, BLDFM_ERR_NONFINITE_DEV);
}

// Paired row pass: each group transforms output rows 2 grp and 2 grp + 1 of
// the CTA's block together.  Its inputs are read from global memory (the
// column pass's output, in L2): staging the pair's two adjacent rows by one
// bulk copy, as the column pass stages its spectrum columns, measured no
// faster (0.0963 against 0.0955 ms for both passes per 16 footprints).
template <class S>
__global__ void __launch_bounds__(kThreads, 2) rx2_rows_batch_kernel(const BatchCase *__restrict__ cases,
                                                                    const int *__restrict__ cta_case, int *err)
{
    constexpr int P = S::P, E = S::E, G = kThreads / P, L = 2 * G;
    using Q = rx::Pair<S>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    rx::C2 *sbuf = (rx::C2 *)smem_raw;
    __shared__ __align__(16) BatchCase sc;
    load_case_rx(&sc, cases + cta_case[blockIdx.x]);
    __syncthreads();
    const SolveGeom &g = sc.g;
    const int local = (int)((int64_t)blockIdx.x - sc.row0);  // fewer than 2^31 CTAs
    const int nblk = (g.out_ny + L - 1) / L;
    const int lvl = local / nblk, yb = local - lvl * nblk;
    const int grp = threadIdx.x / P, t = threadIdx.x - grp * P;
    const int yA = yb * L + 2 * grp;
    bool bad = false;
    if (yA < g.out_ny) {
        const bool actB = yA + 1 < g.out_ny;
        const float cj = g.out_sign > 0 ? -1.f : 1.f;
        const int f0 = freq_min(g.nlx), f1 = freq_max(g.nlx);
        const int h = -f0 > f1 ? -f0 : f1;
        const float2 *rowA = sc.Cb + ((size_t)lvl * g.out_ny + yA) * g.nbx;
        const float2 *rowB = rowA + (actB ? g.nbx : 0);
        rx::C2 x[E];
#pragma unroll
        for (int m = 0; m < E; ++m) {
            const int bcol = band_of(t + P * m, h, S::N);
            float2 va = make_float2(0.f, 0.f), vb = make_float2(0.f, 0.f);
            if (bcol >= 0) {
                va = __ldg(rowA + bcol);
                vb = __ldg(rowB + bcol);
            }
            x[m].re = make_float2(va.x, vb.x);
            x[m].im = make_float2(cj * va.y, cj * vb.y);
        }
        rx::line_fft2<S>(x, t, sbuf + grp * Q::BUF, sc.twx, grp + 1);
        const int onx = g.out_nx, px = g.px;
        const size_t oA = ((size_t)lvl * g.out_ny + yA) * onx, oB = oA + onx;
#pragma unroll
        for (int m = 0; m < E; ++m) {
            const int xo = t + P * m - px;
            if (xo >= 0 && xo < onx) {
                const float ra = x[m].re.x, ia = cj * x[m].im.x;
                rx::store_f64(sc.conc + oA + xo, ra);
                rx::store_f64(sc.flx + oA + xo, ia);
                bad |= !(isfinite(ra) && isfinite(ia));
                if (actB) {
                    const float rb = x[m].re.y, ib = cj * x[m].im.y;
                    rx::store_f64(sc.conc + oB + xo, rb);
                    rx::store_f64(sc.flx + oB + xo, ib);
                    bad |= !(isfinite(rb) && isfinite(ib));
                }
            }
        }
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicCAS(err, 0, BLDFM_ERR_NONFINITE_DEV);
}

// ---------------------------------------------------------------------------
// Zoomed passes (xform_zoom.cuh): line length N = 3 M, band of at most M + 1
// frequencies, at most M kept positions.  S is the M-point shape.
// ---------------------------------------------------------------------------

// Fill the CTA's twist table from the case record in global memory (threads
// 0 .. 3 E + 2), so that it is ready after the block's first barrier.
template <class S>
__device__ __forceinline__ void zoom_twists_of(rx::ZoomTw<S> &z, const BatchCase *gc, bool col)
{
    if (threadIdx.x < 3 * S::E + 3) rx::zoom_twists<S>(z, col ? gc->twy : gc->twx, col ? gc->g.py : gc->g.px);
}

// Value Z = Hp + i Hq of frequency n (|n| <= M/2) of band column bx, from the
// staged columns (sp: Xp at P, sp + nly: Xq at P) where -P is the signed
// mirror inside the mode range, else from global memory (col_value).
__device__ __forceinline__ float2 zoom_col_value(const SolveGeom &g, const int4 bx, bool xpair, const float2 *sp,
                                                 bool staged, const BatchCase &sc, int lvl, int n_line, int n)
{
    const int nly = g.nly, fmin = freq_min(nly), fmax = freq_max(nly);
    const bool pin = n >= fmin && n <= fmax, min_ = -n >= fmin && -n <= fmax && bx.z >= 0;
    if (staged && pin && min_ && xpair && !(bx.y == 0 && n == 0)) {
        const int r = index_of_freq(n, nly);
        const float2 p = sp[r], q = sp[nly + r];
        return make_float2(p.x - q.y, p.y + q.x);
    }
    if (!pin && !min_) return make_float2(0.f, 0.f);
    return col_value(g, bx, xpair, sc.Xp, sc.Xq, sc.dc, lvl, n_line, n >= 0 ? n : n + n_line);
}

// Zoomed column pass: one band column per group of P threads; the kept rows
// [py, py + out_ny) staged line-major as in rx_cols_batch_kernel.
template <class S>
__global__ void __launch_bounds__(kThreads, 3) rz_cols_batch_kernel(const BatchCase *__restrict__ cases,
                                                                   const int *__restrict__ cta_case, int *err)
{
    constexpr int P = S::P, E = S::E, G = kThreads / P, M = S::N, N = 3 * M, MK = (E + 2) / 3;
    using B = rx::ZoomBuf<S, float2>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *sbuf = (float2 *)smem_raw;
    __shared__ __align__(16) BatchCase sc;
    __shared__ __align__(16) rx::ZoomTw<S> zt;
    __shared__ uint64_t gbar[G];
    const BatchCase *gc = cases + cta_case[blockIdx.x];
    load_case_rx(&sc, gc);
    zoom_twists_of<S>(zt, gc, true);
    const int grp = threadIdx.x / P, t = threadIdx.x - grp * P;
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&gbar[grp])), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    const SolveGeom &g = sc.g;
    // 32-bit index arithmetic: a pass launches fewer than 2^31 CTAs
    const int local = (int)((int64_t)blockIdx.x - sc.col0);
    const int ncb = (g.nbx + G - 1) / G;
    const int lvl = local / ncb, cb = local - lvl * ncb;
    const int b = cb * G + grp;
    const bool active = b < g.nbx;
    const float cj = g.out_sign > 0 ? -1.f : 1.f;  // inverse transform: conjugate in and out
    float2 *buf = sbuf + grp * B::BUF;
    float2 y[3 * E];
    bool timed_out = false;
    if (active) {
        const int4 bx = sc.xband[b];
        const bool xpair =
            bx.y >= 0 && bx.z >= 0 && freq_of_index(bx.z, g.nlx) == -freq_of_index(bx.y, g.nlx);
        const int nly = g.nly;
        const size_t colp = ((size_t)lvl * g.nlx + (bx.y > 0 ? bx.y : 0)) * nly;
        const bool stage = bx.y >= 0 && 2 * nly <= B::BUF && (nly & 1) == 0 &&
                           ((((uintptr_t)sc.Xp) | ((uintptr_t)sc.Xq)) & 15) == 0;
        if (stage) {
            const uint32_t ba = smem_u32(&gbar[grp]);
            if (t == 0) {
                const uint32_t nb = (uint32_t)nly * 8u;
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ba), "r"(2u * nb)
                             : "memory");
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        smem_u32(buf)),
                    "l"(sc.Xp + colp), "r"(nb), "r"(ba)
                    : "memory");
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        smem_u32(buf + nly)),
                    "l"(sc.Xq + colp), "r"(nb), "r"(ba)
                    : "memory");
            }
            uint32_t done = 0;
            for (long it = 0; it < BLDFM_WAIT_POLLS && !done; ++it)
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                    "selp.u32 %0, 1, 0, p;\n\t}"
                    : "=r"(done)
                    : "r"(ba), "r"(0u)
                    : "memory");
            timed_out = !done;
        }
        float2 v[E];
#pragma unroll
        for (int m = 0; m < E; ++m) {
            const int n = t + P * m - (m >= E / 2 ? M : 0);
            const float2 z = zoom_col_value(g, bx, xpair, buf, stage, sc, lvl, N, n);
            v[m] = make_float2(z.x, cj * z.y);
        }
        float2 vp = make_float2(0.f, 0.f);
        if (t == 0) {
            const float2 z = zoom_col_value(g, bx, xpair, buf, stage, sc, lvl, N, M / 2);
            vp = make_float2(z.x, cj * z.y);
        }
        if (stage) rx::group_bar(grp + 1, P);  // the staged columns are read before the buffer is reused
        rx::zoom_line<S, float2>(y, v, vp, t, buf, sc.twy, zt, g.py, grp + 1);
    }
    if (__syncthreads_or(timed_out) && threadIdx.x == 0) atomicExch(err, BLDFM_ERR_TIMEOUT_DEV);
    // kept rows j = 3 (t + P m) + r < out_ny of the G lines staged line-major,
    // [G][ys], ys = out_ny rounded up to 4 mod 16 words
    const int ony = g.out_ny;
    const int ys = ((ony + 11) & ~15) + 4;
    if (active) {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int m = 0; m < MK; ++m) {
                const int j = 3 * (t + P * m) + r;
                if (j < ony) sbuf[(size_t)grp * ys + j] = make_float2(y[r * E + m].x, cj * y[r * E + m].y);
            }
    }
    __syncthreads();
    const int ng = min(G, g.nbx - cb * G);
    float2 *o = sc.Cb + (size_t)lvl * ony * g.nbx + cb * G;
    for (int i = threadIdx.x; i < ony * G; i += kThreads) {
        const int yy = i / G, gg = i - yy * G;
        if (gg < ng) o[(size_t)yy * g.nbx + gg] = sbuf[(size_t)gg * ys + yy];
    }
}

using Z256 = rx::Shape<8, 4, 8>;
using Z512 = rx::Shape<8, 8, 8>;

// The zoomed form exists for the column pass only: a zoomed row pass (two
// rows per group in FP32x2 lanes, outputs staged through shared memory for
// contiguous stores) issued 13% fewer instructions than rx2_rows_batch_kernel
// but ran 7% slower (43.3 against 40.6 us per 16 footprints, ncu): its
// staging round trip added shared-memory and barrier waits at the same two
// CTAs per SM.  The column pass stays one line per group: the same pass with
// two band columns per group in FP32x2 lanes (zoom_line<S, C2>, four staged
// columns per group, 128 registers, 2 CTAs per SM instead of 3) made both
// passes 0.0978 against 0.0951 ms per 16 footprints (CUDA events).  The three
// twisted transforms run side by side: one after another through a third of
// the exchange buffer (64 registers, 4 CTAs per SM, three times the named
// barriers, kept rows written as they form) measured 5.94 against 5.98 us per
// footprint for both passes, within noise.
template <class S>
size_t rz_smem_of()
{
    return (size_t)(kThreads / S::P) * rx::ZoomBuf<S, float2>::BUF * sizeof(float2);
}

template <class S>
void rz_set_attr()
{
    cudaFuncSetAttribute(rz_cols_batch_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rz_smem_of<S>());
}

template <class S>
cudaError_t rz_launch(bool col, const BatchLaunch &bl, int nctas, cudaStream_t st)
{
    if (!col) return cudaErrorInvalidValue;
    rz_cols_batch_kernel<S><<<nctas, kThreads, rz_smem_of<S>(), st>>>(bl.cases, bl.col_case, bl.err);
    return cudaGetLastError();
}

template <class S>
constexpr int rz_lines_of(bool col)
{
    return col ? kThreads / S::P : 0;
}

// paired passes for line shapes up to E = 24 (registers: two lines' values
// per thread), single-line passes beyond
// Measured on the 16-footprint 512^2 batch (ncu, per launch): the paired row
// pass ran in 41.3 us against 44.5 us single-line (29% fewer instructions at
// half the resident warps); the paired column pass ran in 82.9 us against
// 61.6 us (its doubled gather code stalls on instruction fetch).  So rows are
// paired for line shapes up to E = 24 (two lines' values fit in 128
// registers) and columns are not.
template <class S>
constexpr bool paired(bool col)
{
    return !col && S::E <= 24;
}

template <class S>
size_t rx_smem_of(bool col)
{
    if (paired<S>(col))
        return (size_t)(kThreads / S::P) * rx::Pair<S>::BUF * sizeof(rx::C2);
    return (size_t)(kThreads / S::P) * S::BUF * sizeof(float2);
}

// the kernel a pass launches, its shared memory and its lines per CTA all
// follow paired<S>(col), so the three can never disagree
template <class S>
void rx_set_attr()
{
    static_assert(!paired<S>(true), "the column pass has no paired kernel");
    if constexpr (paired<S>(false))
        cudaFuncSetAttribute(rx2_rows_batch_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)rx_smem_of<S>(false));
    else
        cudaFuncSetAttribute(rx_rows_batch_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)rx_smem_of<S>(false));
    cudaFuncSetAttribute(rx_cols_batch_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)rx_smem_of<S>(true));
}

template <class S>
cudaError_t rx_launch(bool col, const BatchLaunch &bl, int nctas, cudaStream_t st)
{
    const size_t b = rx_smem_of<S>(col);
    if (col)
        rx_cols_batch_kernel<S><<<nctas, kThreads, b, st>>>(bl.cases, bl.col_case, bl.err);
    else if constexpr (paired<S>(false))
        rx2_rows_batch_kernel<S><<<nctas, kThreads, b, st>>>(bl.cases, bl.row_case, bl.err);
    else
        rx_rows_batch_kernel<S><<<nctas, kThreads, b, st>>>(bl.cases, bl.row_case, bl.err);
    return cudaGetLastError();
}

template <class S>
constexpr int rx_lines_of(bool col)
{
    return (paired<S>(col) ? 2 : 1) * (kThreads / S::P);
}

}  // namespace

int rx_zoom_config(int n, int band_half, int nout)
{
    int m = 0;
    if (n == 768) m = 256;
    else if (n == 1536) m = 512;
    else return -1;
    if (2 * band_half > m || nout > m || nout < 1) return -1;
    return m == 256 ? RX_ZOOM_BASE : RX_ZOOM_BASE + 1;
}

int rx_config(int n)
{
    switch (n) {
    case 512: return 0;
    case 768: return 1;
    case 1024: return 2;
    case 1536: return 3;
    case 2048: return 4;
    case 3072: return 5;
    default: return -1;
    }
}

int rx_lines_per_cta(int cfg, bool col)
{
    switch (cfg) {
    case RX_ZOOM_BASE: return rz_lines_of<Z256>(col);
    case RX_ZOOM_BASE + 1: return rz_lines_of<Z512>(col);
    case 0: return rx_lines_of<S512>(col);
    case 1: return rx_lines_of<S768>(col);
    case 2: return rx_lines_of<S1024>(col);
    case 3: return rx_lines_of<S1536>(col);
    case 4: return rx_lines_of<S2048>(col);
    case 5: return rx_lines_of<S3072>(col);
    default: return 0;
    }
}

size_t rx_smem(int cfg, bool col)
{
    switch (cfg) {
    case RX_ZOOM_BASE: return col ? rz_smem_of<Z256>() : 0;
    case RX_ZOOM_BASE + 1: return col ? rz_smem_of<Z512>() : 0;
    case 0: return rx_smem_of<S512>(col);
    case 1: return rx_smem_of<S768>(col);
    case 2: return rx_smem_of<S1024>(col);
    case 3: return rx_smem_of<S1536>(col);
    case 4: return rx_smem_of<S2048>(col);
    case 5: return rx_smem_of<S3072>(col);
    default: return 0;
    }
}

void prepare_rx_attributes()
{
    rx_set_attr<S512>();
    rx_set_attr<S768>();
    rx_set_attr<S1024>();
    rx_set_attr<S1536>();
    rx_set_attr<S2048>();
    rx_set_attr<S3072>();
    rz_set_attr<Z256>();
    rz_set_attr<Z512>();
}

cudaError_t launch_rx_pass(int cfg, bool col, const BatchLaunch &bl, int nctas, cudaStream_t st)
{
    if (nctas <= 0) return cudaSuccess;
    switch (cfg) {
    case RX_ZOOM_BASE: return rz_launch<Z256>(col, bl, nctas, st);
    case RX_ZOOM_BASE + 1: return rz_launch<Z512>(col, bl, nctas, st);
    case 0: return rx_launch<S512>(col, bl, nctas, st);
    case 1: return rx_launch<S768>(col, bl, nctas, st);
    case 2: return rx_launch<S1024>(col, bl, nctas, st);
    case 3: return rx_launch<S1536>(col, bl, nctas, st);
    case 4: return rx_launch<S2048>(col, bl, nctas, st);
    case 5: return rx_launch<S3072>(col, bl, nctas, st);
    default: return cudaErrorInvalidValue;
    }
}
