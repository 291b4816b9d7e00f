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
