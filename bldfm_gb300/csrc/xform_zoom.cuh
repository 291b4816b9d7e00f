// Zoomed output-transform lines (solver.py:264-290), FP32: a line of length
// N = 3 M whose input is zero outside a band of at most M + 1 frequencies
// centred on 0 and whose output is kept only on a window of at most M
// consecutive positions [k0, k0 + J).  With the default halo of the
// reference (halo = max(xmax, ymax), solver.py:108-120) and modes no finer
// than the grid, both passes of every square footprint have this shape:
// 1536 = 3 x 512 at 512^2.
//
// For a band position n (the frequency, -M/2 <= n <= M/2) write m = n mod M.
// With j = 3 j1 + r (r < 3):
//   X[k0 + j] = sum_n x[n] w_N^{n (k0 + j)} = sum_m y_r[m] w_M^{m j1},
//   y_r[m]   = sum_{n = m mod M} x[n] w_N^{n (k0 + r)},
// because w_N^{3 n j1} = w_M^{n j1} depends on n only through m.  So the line
// is three M-point transforms of twisted copies of the same M values
// ("zoom"), each needed only at j1 < ceil(J / 3): a third of the outputs.
// Only the frequencies +-M/2 share a wrapped position (m = M/2, when the band
// has M + 1 entries).
//
// Layout: the M-point transforms have the register-resident shape S
// (xform_reg.cuh: M = E P, P threads per line, E values per thread); thread
// t holds the wrapped positions m = t + P m' (m' < E), so m < M/2 exactly for
// m' < E/2 (frequency n = m) and m >= M/2 for m' >= E/2 (n = m - M).  The
// twist w_N^{n (k0 + r)} splits into a per-thread factor w_N^{t (k0 + r)},
// which commutes with the first in-register DFT over m' and is folded into
// its twiddles, and a factor of (r, m') alone, the same for every line of a
// case (a table in shared memory, ZoomTw).  The three transforms run side by
// side through the same phases as line_fft: 3 E values per thread, two
// exchanges, one named barrier per exchange.
#pragma once

#include "xform_reg.cuh"

namespace rx {

// operations of the zoom line on one line (float2) or two lines in the lanes
// of FP32x2 arithmetic (C2)
__device__ __forceinline__ float2 twist(float2 v, float2 w) { return cmul(v, w); }
__device__ __forceinline__ C2 twist(C2 v, float2 w) { return c2mul(v, w.x, w.y); }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ C2 vadd(C2 a, C2 b) { return c2add(a, b); }
template <int N>
__device__ __forceinline__ void dft_in_place(float2 *x)
{
    Dft<N>::run(x);
}
template <int N>
__device__ __forceinline__ void dft_in_place(C2 *x)
{
    dft2<N>(x);
}

// Exchange layouts of the zoom line, per value type: S1[r E + k1][t] with
// row stride P + pad; S2 blocks per r of R2 rows c, each of R3 runs u of the
// E values k1 (u stride E + pad2, c stride R3 (E + pad2) + pad3).
template <class S, class V>
struct ZoomBuf {
    static constexpr bool two = sizeof(V) == 16;
    static constexpr int S1 = two ? S::P : S::P + 8;
    static constexpr int EU = two ? S::E + 1 : S::E + 2;
    static constexpr int CS = two ? S::R3 * EU : S::R3 * EU + 8;
    static constexpr int RB = S::R2 * CS;  // one r block of the second exchange
    static constexpr int W1 = 3 * S::E * S1, W2 = 3 * RB;
    static constexpr int BUF = W1 > W2 ? W1 : W2;  // words of V per line (group)
};

// Per-case twists of a line family: U[r E + m'] = w_N^{e} with
// e = P m' (k0 + r) - [m' >= E/2] M (k0 + r) (mod N), and Up[r] =
// w_N^{(M/2)(k0 + r)} for the frequency +M/2 folded onto m = M/2.
template <class S>
struct ZoomTw {
    float2 U[3 * S::E];
    float2 Up[3];
};

// Fill the twist table (threads 0 .. 3 E + 2 of the block).  tw: w_N^i, i < N.
template <class S>
__device__ __forceinline__ void zoom_twists(ZoomTw<S> &z, const float2 *__restrict__ tw, int k0)
{
    constexpr int E = S::E, P = S::P, M = S::N, N = 3 * M;
    const int i = threadIdx.x;
    if (i < 3 * E) {
        const int r = i / E, mp = i - r * E;
        const int kr = k0 + r;
        // |exponent| < M (N + 2) < 2^31 for the supported lengths: 32-bit
        int e = P * mp * kr - (mp >= E / 2 ? M * kr : 0);
        e %= N;
        if (e < 0) e += N;
        z.U[i] = __ldg(tw + e);
    } else if (i < 3 * E + 3) {
        const int r = i - 3 * E;
        z.Up[r] = __ldg(tw + ((M / 2) * (k0 + r)) % N);
    }
}

// The zoom line.  In: v[m'] (m' < E) the thread's wrapped values x~[t + P m']
// (for m' >= E/2 the frequency t + P m' - M), vp the value of frequency
// +M/2 (used by thread 0 only; zero when the band has no such entry).
// Out: y[r E + m''] = X[k0 + 3 (t + P m'') + r] for m'' < ceil(E / 3) (the
// only outputs a window of at most M positions can need); the other entries
// of y are left undefined.  buf: the group's ZoomBuf<S, V>::BUF words; the
// group's threads call this together and the buffer is free on return.
template <class S, class V>
__device__ __forceinline__ void zoom_line(V (&y)[3 * S::E], const V (&v)[S::E], V vp, int t, V *buf,
                                          const float2 *__restrict__ tw, const ZoomTw<S> &z, int k0, int bar)
{
    constexpr int E = S::E, R2 = S::R2, R3 = S::R3, P = S::P, M = S::N, N = 3 * M;
    using D = Dft<E>;
    using B = ZoomBuf<S, V>;
    const int u = t % R3, k1b = t / R3;
    // phase-1 twiddle starts w_N^{t (k0 + r) + 24 b t} per block b of 8 k1,
    // steps w_M^t = w_N^{3 t}; phase-2 twiddles w_P^{u c} = w_N^{3 u c E}
    float2 wb[3][(E + 7) / 8];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int b = 0; b < (E + 7) / 8; ++b)
            wb[r][b] = __ldg(tw + (t * (k0 + r) + 24 * b * t) % N);  // < P (N + 24 E) < 2^31
    const float2 w1 = __ldg(tw + 3 * t);
    float2 w2[R2];
#pragma unroll
    for (int c = 1; c < R2; ++c) w2[c] = __ldg(tw + (3 * u * c * E) % N);
    // twists of (r, m') and phase 1 of each r: E-point DFT, twiddles
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        V *x = y + r * E;
#pragma unroll
        for (int m = 0; m < E; ++m) x[m] = twist(v[m], z.U[r * E + m]);
        if (t == 0) x[E / 2] = vadd(x[E / 2], twist(vp, z.Up[r]));
        dft_in_place<E>(x);
#pragma unroll
        for (int b = 0; b < (E + 7) / 8; ++b) {
            float2 w = wb[r][b];
#pragma unroll
            for (int j = 0; j < 8 && 8 * b + j < E; ++j) {
                const int k1 = 8 * b + j;
                buf[(r * E + k1) * B::S1 + t] = twist(x[D::slot(k1)], w);
                w = cmul(w, w1);
            }
        }
    }
    group_bar(bar, P);
    // phase 2: per r, for k1 = t / R3 + R2 i, R2-point DFT over v of
    // S1[r E + k1][u + R3 v], twiddle w_P^{u c}
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int i = 0; i < E / R2; ++i) {
            V *x = y + r * E + i * R2;
            const int k1 = k1b + R2 * i;
#pragma unroll
            for (int vv = 0; vv < R2; ++vv) x[vv] = buf[(r * E + k1) * B::S1 + u + R3 * vv];
            dft_in_place<R2>(x);
#pragma unroll
            for (int c = 1; c < R2; ++c) x[c] = twist(x[c], w2[c]);
        }
    group_bar(bar, P);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int i = 0; i < E / R2; ++i) {
            const int k1 = k1b + R2 * i;
#pragma unroll
            for (int c = 0; c < R2; ++c) buf[r * B::RB + c * B::CS + u * B::EU + k1] = y[r * E + i * R2 + c];
        }
    group_bar(bar, P);
    // phase 3: per r, for h = t + P i (k1 = h % E, c = h / E), R3-point DFT
    // over u; output d is X_r[t + P (i + (E / R3) d)], kept for m'' < ceil(E / 3)
    constexpr int MK = (E + 2) / 3;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int i = 0; i < E / R3; ++i) {
            const int h = t + P * i;
            const int k1 = h % E, c = h / E;
            V w[R3];
#pragma unroll
            for (int uu = 0; uu < R3; ++uu) w[uu] = buf[r * B::RB + c * B::CS + uu * B::EU + k1];
            dft_in_place<R3>(w);
#pragma unroll
            for (int d = 0; d < R3; ++d) {
                const int mm = i + (E / R3) * d;
                if (mm < MK) y[r * E + mm] = w[d];
            }
        }
    group_bar(bar, P);  // the buffer may be rewritten after this
}

}  // namespace rx
