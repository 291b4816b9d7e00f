// Register-resident output transform lines (solver.py:264-290), FP32.
//
// A line of length N = E * P is owned by P = R2 * R3 threads ("a group");
// thread t holds the E values at positions t + P m (m < E) in registers.
// The transform is the Cooley-Tukey split N = E x R2 x R3:
//   X[k1 + E (c + R2 d)] = sum_u w_R3^{u d} w_P^{u c}
//                           sum_v w_R2^{v c} w_N^{t k1} Y_t[k1],  t = u + R3 v,
// with Y_t the E-point DFT of thread t's values.  Three in-register DFT
// phases (E, R2, R3 points) and two exchanges through the group's shared
// memory; the groups of a CTA synchronise with their own named barriers, not
// with the block.  The output lands in the same pattern as the input: thread
// t ends with X[t + P m], m < E.  All transforms use the forward sign
// w = exp(-2 pi i / N); the inverse sign is the conjugate transform of the
// conjugated input (the callers conjugate on load and on store).
//
// Shared-memory layouts (float2 words, padded so that a half-warp's accesses
// fall on 16 distinct 8-byte bank pairs):
//   phase-1 -> phase-2 exchange  S1[k1][t]      row stride P + 8
//   phase-2 -> phase-3 exchange  S2[c][u][k1]   u stride E + 2, c stride
//                                               R3 (E + 2) + 8
#pragma once

#include <type_traits>

#include "fft_core.cuh"

namespace rx {

// cos / sin of 2 pi m / n at compile time: the angle reduced to [-pi, pi],
// then the Taylor series (30 terms; the truncation error is far below FP32
// resolution).
constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double taylor_cos(double x)
{
    double t = 1.0, s = 1.0;
    for (int k = 1; k < 30; ++k) {
        t *= -x * x / ((2.0 * k - 1.0) * (2.0 * k));
        s += t;
    }
    return s;
}
constexpr double taylor_sin(double x)
{
    double t = x, s = x;
    for (int k = 1; k < 30; ++k) {
        t *= -x * x / ((2.0 * k) * (2.0 * k + 1.0));
        s += t;
    }
    return s;
}
constexpr double angle(int m, int n)
{
    const int r = ((m % n) + n) % n;
    const double a = 2.0 * kPi * (double)r / (double)n;
    return a > kPi ? a - 2.0 * kPi : a;
}
template <int M, int N>
struct Tw {
    static constexpr float c = (float)taylor_cos(angle(M, N));
    static constexpr float s = (float)taylor_sin(angle(M, N));
};

template <int I, int N, class F>
__device__ __forceinline__ void sfor(F &&f)
{
    if constexpr (I < N) {
        f(std::integral_constant<int, I>());
        sfor<I + 1, N>(f);
    }
}

// u * exp(-2 pi i M / N)
template <int M, int N>
__device__ __forceinline__ float2 mul_w(float2 u)
{
    constexpr float c = Tw<M, N>::c, s = -Tw<M, N>::s;
    return make_float2(u.x * c - u.y * s, u.x * s + u.y * c);
}

// In-register DFT of length N, forward sign, in place: natural order in, and
// X[k] left in x[Dft<N>::slot(k)] (a compile-time permutation, so that the
// transform needs no second array of N values).  N = A F with A = 8, 4, 2
// or 3:  X[k1 + A k2] = sum_s1 w_F^{s1 k2} w_N^{s1 k1} sum_s2 w_A^{s2 k1}
// x[s1 + F s2]; the inner DFTs overwrite x[s1 + F k1], then each block
// x[F k1 .. F k1 + F) is transformed in place.
template <int N>
struct Dft {
    static constexpr bool direct = N == 1 || N == 2 || N == 3 || N == 4 || N == 8;
    static constexpr int A = direct ? N : ((N % 8 == 0) ? 8 : ((N % 4 == 0) ? 4 : ((N % 2 == 0) ? 2 : 3)));
    static constexpr int F = N / A;
    static constexpr int slot(int k)
    {
        if constexpr (direct)
            return k;
        else
            return F * (k % A) + Dft<F>::slot(k / A);
    }
    __device__ __forceinline__ static void run(float2 *x)
    {
        if constexpr (direct) {
            if constexpr (N > 1) dft_small<float2, N, -1>(x, nullptr, 0);
        } else {
            sfor<0, F>([&](auto S1) {
                constexpr int s1 = decltype(S1)::value;
                float2 u[A];
#pragma unroll
                for (int s2 = 0; s2 < A; ++s2) u[s2] = x[s1 + F * s2];
                dft_small<float2, A, -1>(u, nullptr, 0);
                sfor<0, A>([&](auto K1) {
                    constexpr int k1 = decltype(K1)::value;
                    constexpr int m = (s1 * k1) % N;
                    if constexpr (m == 0)
                        x[s1 + F * k1] = u[k1];
                    else
                        x[s1 + F * k1] = mul_w<m, N>(u[k1]);
                });
            });
#pragma unroll
            for (int k1 = 0; k1 < A; ++k1) Dft<F>::run(x + F * k1);
        }
    }
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ void group_bar(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <int E_, int R2_, int R3_>
struct Shape {
    static constexpr int E = E_, R2 = R2_, R3 = R3_;
    static constexpr int P = R2 * R3;  // threads per line
    static constexpr int N = E * P;    // line length
    static constexpr int S1 = P + 8;
    static constexpr int EU = E + 2;
    static constexpr int CS = R3 * EU + 8;
    static constexpr int BUF = (E * S1 > R2 * CS) ? E * S1 : R2 * CS;  // float2 per line
    static_assert(E % R2 == 0 && E % R3 == 0, "E must be a multiple of R2 and R3");
};

// The line transform.  x: the thread's E values (positions t + P m) in,
// X at the same positions out.  buf: the group's BUF-word exchange buffer.
// tw: exp(-2 pi i m / N), m < N (global, read through the read-only path).
// bar: the group's named barrier id.  The group's threads call it together;
// the buffer is free again when it returns.
//
// Twiddles: phase 1 needs w_N^{t k1}, k1 < E.  Per block of 8 consecutive
// k1 one value is loaded and the rest follow by multiplying with w_N^t
// (at most 7 products in a chain: relative error a few 1e-7, well inside the
// FP32 path's error); phase 2 loads its R2 - 1 twiddles w_P^{u c} once.
template <class S>
__device__ __forceinline__ void line_fft(float2 *x, int t, float2 *buf, const float2 *__restrict__ tw, int bar)
{
    constexpr int E = S::E, R2 = S::R2, R3 = S::R3, P = S::P;
    using D = Dft<E>;
    // loads that only depend on t go out before the first DFT
    float2 wb[(E + 7) / 8];
#pragma unroll
    for (int b = 0; b < (E + 7) / 8; ++b) wb[b] = __ldg(tw + 8 * b * t);  // 8 b t < 8 (E / 8) P <= N
    const float2 w1 = __ldg(tw + t);
    const int u = t % R3, k1b = t / R3;
    float2 w2[R2];
#pragma unroll
    for (int c = 1; c < R2; ++c) w2[c] = __ldg(tw + u * c * E);
    // phase 1: E-point DFT of the thread's values, twiddle w_N^{t k1}
    D::run(x);
#pragma unroll
    for (int b = 0; b < (E + 7) / 8; ++b) {
        float2 w = wb[b];
#pragma unroll
        for (int j = 0; j < 8 && 8 * b + j < E; ++j) {
            const int k1 = 8 * b + j;
            const float2 y = k1 == 0 ? x[D::slot(0)] : cmul(x[D::slot(k1)], w);
            buf[k1 * S::S1 + t] = y;
            w = cmul(w, w1);
        }
    }
    group_bar(bar, P);
    // phase 2: for (k1, u) = (t / R3 + R2 i, t % R3), R2-point DFT over v of
    // S1[k1][u + R3 v], twiddle w_P^{u c} = w_N^{u c E}
#pragma unroll
    for (int i = 0; i < E / R2; ++i) {
        float2 *v = x + i * R2;
        const int k1 = k1b + R2 * i;
#pragma unroll
        for (int vv = 0; vv < R2; ++vv) v[vv] = buf[k1 * S::S1 + u + R3 * vv];
        Dft<R2>::run(v);  // R2 <= 8: natural order
#pragma unroll
        for (int c = 1; c < R2; ++c) v[c] = cmul(v[c], w2[c]);
    }
    group_bar(bar, P);
#pragma unroll
    for (int i = 0; i < E / R2; ++i) {
        const int k1 = k1b + R2 * i;
#pragma unroll
        for (int c = 0; c < R2; ++c) buf[c * S::CS + u * S::EU + k1] = x[i * R2 + c];
    }
    group_bar(bar, P);
    // phase 3: for h = t + P i (k1 = h % E, c = h / E), R3-point DFT over u of
    // S2[c][u][k1]; output d lands at position k1 + E (c + R2 d) = t + P (i + (E / R3) d)
#pragma unroll
    for (int i = 0; i < E / R3; ++i) {
        const int h = t + P * i;
        const int k1 = h % E, c = h / E;
        float2 w[R3];
#pragma unroll
        for (int uu = 0; uu < R3; ++uu) w[uu] = buf[c * S::CS + uu * S::EU + k1];
        Dft<R3>::run(w);
#pragma unroll
        for (int d = 0; d < R3; ++d) x[i + (E / R3) * d] = w[d];
    }
    group_bar(bar, P);  // the buffer may be rewritten after this
}

}  // namespace rx

// ---------------------------------------------------------------------------
// Paired lines: two lines of the same length transformed together by one
// group, line A in lane 0 and line B in lane 1 of packed FP32x2 arithmetic
// (__fadd2_rn / __fmul2_rn / __ffma2_rn).  Every operation of the transform
// is the same for both lines, so the arithmetic, the index arithmetic and the
// shared-memory instructions are shared: one 16-byte exchange word carries
// both lines' values.  Same rounding per lane as the single-line transform.
// ---------------------------------------------------------------------------
namespace rx {

struct __align__(16) C2 {
    float2 re, im;  // (A.re, B.re), (A.im, B.im)
};

__device__ __forceinline__ float2 bc(float v) { return make_float2(v, v); }
__device__ __forceinline__ C2 c2add(C2 a, C2 b) { return {__fadd2_rn(a.re, b.re), __fadd2_rn(a.im, b.im)}; }
__device__ __forceinline__ C2 c2sub(C2 a, C2 b)
{
    return {__ffma2_rn(b.re, bc(-1.f), a.re), __ffma2_rn(b.im, bc(-1.f), a.im)};
}
// a * (c + i s), the same scalar in both lanes
__device__ __forceinline__ C2 c2mul(C2 a, float c, float s)
{
    return {__ffma2_rn(a.im, bc(-s), __fmul2_rn(a.re, bc(c))), __ffma2_rn(a.im, bc(c), __fmul2_rn(a.re, bc(s)))};
}
// a * (-i)
__device__ __forceinline__ C2 c2rot_m(C2 a) { return {a.im, __fmul2_rn(a.re, bc(-1.f))}; }

// forward DFTs of length 2, 3, 4, 8 on paired values, natural order (the
// formulas of dft_small with sign -1)
template <int N>
__device__ __forceinline__ void dft2_small(C2 *u)
{
    if constexpr (N == 2) {
        const C2 a = u[0], b = u[1];
        u[0] = c2add(a, b);
        u[1] = c2sub(a, b);
    } else if constexpr (N == 4) {
        const C2 a0 = c2add(u[0], u[2]), a1 = c2sub(u[0], u[2]);
        const C2 b0 = c2add(u[1], u[3]), b1 = c2rot_m(c2sub(u[1], u[3]));
        u[0] = c2add(a0, b0);
        u[2] = c2sub(a0, b0);
        u[1] = c2add(a1, b1);
        u[3] = c2sub(a1, b1);
    } else if constexpr (N == 3) {
        const float s1 = -0.86602540378443864676f;
        const C2 s = c2add(u[1], u[2]), d = c2sub(u[1], u[2]), a = u[0];
        u[0] = c2add(a, s);
        const C2 m = {__ffma2_rn(s.re, bc(-0.5f), a.re), __ffma2_rn(s.im, bc(-0.5f), a.im)};
        const C2 r = {__fmul2_rn(d.im, bc(-s1)), __fmul2_rn(d.re, bc(s1))};  // i s1 d
        u[1] = c2add(m, r);
        u[2] = c2sub(m, r);
    } else if constexpr (N == 8) {
        C2 a[4], b[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            a[t] = u[2 * t];
            b[t] = u[2 * t + 1];
        }
        dft2_small<4>(a);
        dft2_small<4>(b);
        const float h = 0.70710678118654752440f;
        // b[k] *= w_8^k, w_8 = (1 - i) / sqrt2
        b[1] = {__fmul2_rn(__fadd2_rn(b[1].re, b[1].im), bc(h)),
                __fmul2_rn(__ffma2_rn(b[1].re, bc(-1.f), b[1].im), bc(h))};
        b[2] = c2rot_m(b[2]);
        b[3] = {__fmul2_rn(__ffma2_rn(b[3].re, bc(-1.f), b[3].im), bc(h)),
                __fmul2_rn(__ffma2_rn(b[3].im, bc(-1.f), __fmul2_rn(b[3].re, bc(-1.f))), bc(h))};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            u[t] = c2add(a[t], b[t]);
            u[t + 4] = c2sub(a[t], b[t]);
        }
    }
}

// In-place paired DFT, output permutation Dft<N>::slot.
template <int N>
__device__ __forceinline__ void dft2(C2 *x)
{
    using D = Dft<N>;
    if constexpr (D::direct) {
        if constexpr (N > 1) dft2_small<N>(x);
    } else {
        constexpr int A = D::A, F = D::F;
        sfor<0, F>([&](auto S1) {
            constexpr int s1 = decltype(S1)::value;
            C2 u[A];
#pragma unroll
            for (int s2 = 0; s2 < A; ++s2) u[s2] = x[s1 + F * s2];
            dft2_small<A>(u);
            sfor<0, A>([&](auto K1) {
                constexpr int k1 = decltype(K1)::value;
                constexpr int m = (s1 * k1) % N;
                if constexpr (m == 0)
                    x[s1 + F * k1] = u[k1];
                else
                    x[s1 + F * k1] = c2mul(u[k1], Tw<m, N>::c, -Tw<m, N>::s);
            });
        });
#pragma unroll
        for (int k1 = 0; k1 < A; ++k1) dft2<F>(x + F * k1);
    }
}

// Exchange layouts for 16-byte words (a quarter-warp per wavefront):
// S1[k1][t] row stride P; S2[c][u][k1] u stride E + 1 (odd), c stride R3 (E + 1).
template <class S>
struct Pair {
    static constexpr int S1 = S::P;
    static constexpr int EU = S::E + 1;
    static constexpr int CS = S::R3 * EU;
    static constexpr int BUF = (S::E * S1 > S::R2 * CS) ? S::E * S1 : S::R2 * CS;  // C2 words per group
};

// The paired line transform: x holds the E paired values at positions
// t + P m of lines A and B in, the paired outputs at the same positions out.
// buf: the group's Pair<S>::BUF words.  Twiddles as in line_fft.
template <class S>
__device__ __forceinline__ void line_fft2(C2 *x, int t, C2 *buf, const float2 *__restrict__ tw, int bar)
{
    constexpr int E = S::E, R2 = S::R2, R3 = S::R3, P = S::P;
    using D = Dft<E>;
    using Q = Pair<S>;
    float2 wb[(E + 7) / 8];
#pragma unroll
    for (int b = 0; b < (E + 7) / 8; ++b) wb[b] = __ldg(tw + 8 * b * t);
    const float2 w1 = __ldg(tw + t);
    const int u = t % R3, k1b = t / R3;
    float2 w2[R2];
#pragma unroll
    for (int c = 1; c < R2; ++c) w2[c] = __ldg(tw + u * c * E);
    dft2<E>(x);
#pragma unroll
    for (int b = 0; b < (E + 7) / 8; ++b) {
        float2 w = wb[b];
#pragma unroll
        for (int j = 0; j < 8 && 8 * b + j < E; ++j) {
            const int k1 = 8 * b + j;
            buf[k1 * Q::S1 + t] = k1 == 0 ? x[D::slot(0)] : c2mul(x[D::slot(k1)], w.x, w.y);
            w = cmul(w, w1);
        }
    }
    group_bar(bar, P);
#pragma unroll
    for (int i = 0; i < E / R2; ++i) {
        C2 *v = x + i * R2;
        const int k1 = k1b + R2 * i;
#pragma unroll
        for (int vv = 0; vv < R2; ++vv) v[vv] = buf[k1 * Q::S1 + u + R3 * vv];
        dft2<R2>(v);
#pragma unroll
        for (int c = 1; c < R2; ++c) v[c] = c2mul(v[c], w2[c].x, w2[c].y);
    }
    group_bar(bar, P);
#pragma unroll
    for (int i = 0; i < E / R2; ++i) {
        const int k1 = k1b + R2 * i;
#pragma unroll
        for (int c = 0; c < R2; ++c) buf[c * Q::CS + u * Q::EU + k1] = x[i * R2 + c];
    }
    group_bar(bar, P);
#pragma unroll
    for (int i = 0; i < E / R3; ++i) {
        const int h = t + P * i;
        const int k1 = h % E, c = h / E;
        C2 w[R3];
#pragma unroll
        for (int uu = 0; uu < R3; ++uu) w[uu] = buf[c * Q::CS + uu * Q::EU + k1];
        dft2<R3>(w);
#pragma unroll
        for (int d = 0; d < R3; ++d) x[i + (E / R3) * d] = w[d];
    }
    group_bar(bar, P);
}

// Exact FP32 -> FP64 store without the FP64 pipe for normal numbers and zero
// (sign, exponent rebiased by 1023 - 127, mantissa shifted by 29); subnormal,
// infinite and NaN values take the conversion instruction.
__device__ __forceinline__ void store_f64(double *p, float v)
{
    const uint32_t b = __float_as_uint(v), a = b & 0x7fffffffu;
    if (a - 0x00800000u < 0x7f000000u) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(b << 29, (b & 0x80000000u) | ((a >> 3) + 0x38000000u));
    } else if (a == 0) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(0u, b);
    } else {
        *p = (double)v;
    }
}

}  // namespace rx
