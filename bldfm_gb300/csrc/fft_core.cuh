// Mixed-radix Stockham autosort FFT on lines held in shared memory.
//
// State after stage q (radix p, L_q = L_{q-1} * p, r_q = N / L_q):
//   y_q[j, k] = sum_{n < L_q} x[n r_q + k] w_{L_q}^{j n},  stored at j*r_q + k.
// One butterfly per (j1 < L_{q-1}, k < r_q):
//   y_q[j1 + L_{q-1} j2, k] = sum_t (w_N^{j1 t r_q} y_{q-1}[j1, t r_q + k]) w_p^{j2 t}.
// Input and output are in natural order (autosort), ping-ponging between two
// buffers.  Twiddles come from a table tw[m] = exp(-2 pi i m / N); the
// inverse sign conjugates them.
#pragma once

#include "common.h"


template <typename C>
__device__ __forceinline__ C cx_make(double a, double b)
{
    C o;
    o.x = a;
    o.y = b;
    return o;
}

template <typename C>
__device__ __forceinline__ C cx_mul(C a, C b)
{
    C o;
    o.x = a.x * b.x - a.y * b.y;
    o.y = a.x * b.y + a.y * b.x;
    return o;
}

template <typename C>
__device__ __forceinline__ C cx_add(C a, C b)
{
    C o;
    o.x = a.x + b.x;
    o.y = a.y + b.y;
    return o;
}

template <typename C>
__device__ __forceinline__ C cx_sub(C a, C b)
{
    C o;
    o.x = a.x - b.x;
    o.y = a.y - b.y;
    return o;
}

// multiply by -i*sign... helper: rotate by +/- 90 degrees: (x + iy) * (i*s) = (-s y, s x)
template <typename C>
__device__ __forceinline__ C cx_rot(C a, float s)
{
    C o;
    o.x = -s * a.y;
    o.y = s * a.x;
    return o;
}

template <typename C, int SIGN>
__device__ __forceinline__ C tw_get(const C *tw, int m)
{
    C w = tw[m];
    if (SIGN > 0) w.y = -w.y;
    return w;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t x, const FDiv &f)
{
    return f.s < 0 ? x : (__umulhi(x, f.m) >> f.s);
}

// Radix-p butterfly body for one (j1, k).  u[] already twiddled.
template <typename C, int P, int SIGN>
__device__ __forceinline__ void dft_small(C *u, const C *tw, int n)
{
    constexpr int sign = SIGN;
    typedef decltype(u[0].x) RR;
    if (P == 2) {
        C a = u[0], b = u[1];
        u[0] = cx_add(a, b);
        u[1] = cx_sub(a, b);
    } else if (P == 4) {
        C a0 = cx_add(u[0], u[2]), a1 = cx_sub(u[0], u[2]);
        C b0 = cx_add(u[1], u[3]), b1 = cx_sub(u[1], u[3]);
        // w_4 = exp(sign * 2 pi i / 4) = sign*i  (forward sign = -1 -> -i)
        C b1r = cx_rot(b1, (float)sign);
        u[0] = cx_add(a0, b0);
        u[2] = cx_sub(a0, b0);
        u[1] = cx_add(a1, b1r);
        u[3] = cx_sub(a1, b1r);
    } else if (P == 3) {
        // w_3 = -1/2 + sign * i sqrt(3)/2
        const RR c1 = (RR)-0.5;
        const RR s1 = (RR)(sign * 0.86602540378443864676372317075294);
        C s = cx_add(u[1], u[2]);
        C d = cx_sub(u[1], u[2]);
        C a = u[0];
        u[0] = cx_add(a, s);
        C m;
        m.x = a.x + c1 * s.x;
        m.y = a.y + c1 * s.y;
        C r;  // i * s1 * d
        r.x = -s1 * d.y;
        r.y = s1 * d.x;
        u[1] = cx_add(m, r);
        u[2] = cx_sub(m, r);
    } else if (P == 8) {
        // two radix-4 layers with internal twiddles w_8^{k}
        C a[4], b[4];
        for (int t = 0; t < 4; ++t) {
            a[t] = u[2 * t];
            b[t] = u[2 * t + 1];
        }
        // radix-4 on even and odd halves
        {
            C x0 = cx_add(a[0], a[2]), x1 = cx_sub(a[0], a[2]);
            C y0 = cx_add(a[1], a[3]), y1 = cx_rot(cx_sub(a[1], a[3]), (float)sign);
            a[0] = cx_add(x0, y0);
            a[2] = cx_sub(x0, y0);
            a[1] = cx_add(x1, y1);
            a[3] = cx_sub(x1, y1);
        }
        {
            C x0 = cx_add(b[0], b[2]), x1 = cx_sub(b[0], b[2]);
            C y0 = cx_add(b[1], b[3]), y1 = cx_rot(cx_sub(b[1], b[3]), (float)sign);
            b[0] = cx_add(x0, y0);
            b[2] = cx_sub(x0, y0);
            b[1] = cx_add(x1, y1);
            b[3] = cx_sub(x1, y1);
        }
        const RR h = (RR)0.70710678118654752440084436210485;
        // b[k] *= w_8^k, w_8 = (1 + sign*i)/sqrt2
        C t1;
        t1.x = h * (b[1].x - sign * b[1].y);
        t1.y = h * (b[1].y + sign * b[1].x);
        b[1] = t1;
        b[2] = cx_rot(b[2], (float)sign);
        C t3;  // w_8^3 = (-1 + sign*i)/sqrt2
        t3.x = h * (-b[3].x - sign * b[3].y);
        t3.y = h * (-b[3].y + sign * b[3].x);
        b[3] = t3;
        for (int t = 0; t < 4; ++t) {
            u[t] = cx_add(a[t], b[t]);
            u[t + 4] = cx_sub(a[t], b[t]);
        }
    } else if (P == 5) {
        C o[5];
        for (int j = 0; j < 5; ++j) {
            C acc = u[0];
            for (int t = 1; t < 5; ++t) {
                int m = ((j * t) % 5) * (n / 5);
                acc = cx_add(acc, cx_mul(u[t], tw_get<C, SIGN>(tw, m)));
            }
            o[j] = acc;
        }
        for (int j = 0; j < 5; ++j) u[j] = o[j];
    }
}

// One Stockham stage of specialised radix P over nlines lines of length n;
// stage constants from the plan (rq, divisions by rq and by n / P).
template <typename C, int P, int SIGN>
__device__ void stage_p(const C *__restrict__ src, C *__restrict__ dst, int n, int nlines, int L1, int rq,
                        const FDiv drq, const FDiv dnb, const C *__restrict__ tw)
{
    const int nb = n / P;  // butterflies per line
    const int total = nb * nlines;
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        const int line = (int)fdiv((uint32_t)b, dnb);
        const int loc = b - line * nb;
        const int j1 = (int)fdiv((uint32_t)loc, drq);
        const int k = loc - j1 * rq;
        const C *s = src + (size_t)line * n;
        C *d = dst + (size_t)line * n;
        C u[P];
        const int base = j1 * rq * P + k;
#pragma unroll
        for (int t = 0; t < P; ++t) {
            C v = s[base + t * rq];
            if (t > 0 && j1 > 0) v = cx_mul(v, tw_get<C, SIGN>(tw, j1 * t * rq));
            u[t] = v;
        }
        dft_small<C, P, SIGN>(u, tw, n);
#pragma unroll
        for (int t = 0; t < P; ++t) d[(j1 + L1 * t) * rq + k] = u[t];
    }
}

// Generic radix (direct size-p DFT per butterfly, O(p^2)).
template <typename C, int SIGN>
__device__ void stage_generic(const C *__restrict__ src, C *__restrict__ dst, int n, int nlines, int L1, int p,
                              int rq, const FDiv drq, const FDiv dnb, const C *__restrict__ tw)
{
    const int nb = n / p;
    const int total = nb * nlines;
    const int np_ = n / p;
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        const int line = (int)fdiv((uint32_t)b, dnb);
        const int loc = b - line * nb;
        const int j1 = (int)fdiv((uint32_t)loc, drq);
        const int k = loc - j1 * rq;
        const C *s = src + (size_t)line * n;
        C *d = dst + (size_t)line * n;
        const int base = j1 * rq * p + k;
        for (int j2 = 0; j2 < p; ++j2) {
            C acc = s[base];
            for (int t = 1; t < p; ++t) {
                C v = s[base + t * rq];
                if (j1 > 0) v = cx_mul(v, tw_get<C, SIGN>(tw, j1 * t * rq));
                int m = ((j2 * t) % p) * np_;
                acc = cx_add(acc, cx_mul(v, tw_get<C, SIGN>(tw, m)));
            }
            d[(j1 + L1 * j2) * rq + k] = acc;
        }
    }
}

// Run all stages with a compile-time transform sign; returns the buffer
// holding the result (a or b).
template <typename C, int SIGN>
__device__ C *fft_run_s(C *a, C *b, const FftPlan &pl, int nlines, const C *__restrict__ tw)
{
    int L1 = 1;
    C *src = a, *dst = b;
    for (int q = 0; q < pl.nstages; ++q) {
        const int p = pl.radix[q];
        const int rq = pl.rq[q];
        const FDiv drq = pl.drq[q], dnb = pl.dnb[q];
        __syncthreads();
        switch (p) {
        case 2: stage_p<C, 2, SIGN>(src, dst, pl.n, nlines, L1, rq, drq, dnb, tw); break;
        case 3: stage_p<C, 3, SIGN>(src, dst, pl.n, nlines, L1, rq, drq, dnb, tw); break;
        case 4: stage_p<C, 4, SIGN>(src, dst, pl.n, nlines, L1, rq, drq, dnb, tw); break;
        case 5: stage_p<C, 5, SIGN>(src, dst, pl.n, nlines, L1, rq, drq, dnb, tw); break;
        case 8: stage_p<C, 8, SIGN>(src, dst, pl.n, nlines, L1, rq, drq, dnb, tw); break;
        default: stage_generic<C, SIGN>(src, dst, pl.n, nlines, L1, p, rq, drq, dnb, tw); break;
        }
        L1 *= p;
        C *t = src;
        src = dst;
        dst = t;
    }
    __syncthreads();
    return src;
}

template <typename C>
__device__ C *fft_run(C *a, C *b, const FftPlan &pl, int nlines, const C *__restrict__ tw, int sign)
{
    return sign > 0 ? fft_run_s<C, 1>(a, b, pl, nlines, tw) : fft_run_s<C, -1>(a, b, pl, nlines, tw);
}
