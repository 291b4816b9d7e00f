// FP32 invariant-imbedding (Riccati) sweep: per-step device functions and the
// per-mode body shared by the single-solve and batched kernels.
#pragma once

#include "devmath.cuh"

// ---------------------------------------------------------------------------
// FP32 invariant-imbedding (Riccati) sweep
// ---------------------------------------------------------------------------
// Same discrete boundary-value problem as the shooting method: with
// s_{i+1} = M_i s_i, M_i = [[a, b], [c, a]] and the radiation condition at the
// top, the ratio R_i = p_i / q_i obeys R_i = (a R_{i+1} - b) / (a - c R_{i+1})
// from R_L = 1 / (Kz_top * eig), and q_{i+1} = (c R_i + a) q_i.  The backward
// recursion is contractive (it follows the decaying solution), so FP32 loses
// nothing to the cancellation that forces FP64 in the forward shooting form.
// The running product Q_i = prod_{k>=i} (c_k R_k + a_k) is kept as an FP32
// mantissa with an integer power-of-two exponent, renormalised every 8 steps.
__device__ __forceinline__ float2 csqrt_f(float2 w)
{
    // principal branch, Kahan's formulation
    float x = w.x, y = w.y;
    float t = sqrtf(0.5f * (fabsf(x) + hypotf(x, y)));
    if (t == 0.f) return make_float2(0.f, 0.f);
    if (x >= 0.f) return make_float2(t, y / (2.f * t));
    return make_float2(fabsf(y) / (2.f * t), copysignf(t, y));
}

__device__ __forceinline__ float2 fc_mul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Coefficients a, b, c of step i for one mode.
//   ISO: Kx == Ky and (u, v) = U (ex, ey) at every level, so
//        T = -K k2 - i U kw with per-mode k2 = lx^2 + ly^2, kw = ex lx + ey ly;
//        row = {AK, AU, B0, B1K, B1U, -HK, -C1K2, C1U2, -HU, -2 C1 K U}
//   generic: row = {-Kx, -Ky, -u, -v, A, B0, B1, H, C1, -2 C1}
template <bool ISO>
struct StepCoef;

template <>
struct StepCoef<true> {
    float k2, kw, k4, kw2, k2kw;
    __device__ __forceinline__ void init(float lx, float ly, float ex, float ey)
    {
        k2 = fmaf(lx, lx, ly * ly);
        kw = fmaf(ex, lx, ey * ly);
        k4 = k2 * k2;
        kw2 = kw * kw;
        k2kw = k2 * kw;
    }
    __device__ __forceinline__ void eval(const float *lv, float2 &a, float2 &b, float2 &c) const
    {
        const float4 r0 = *(const float4 *)lv, r1 = *(const float4 *)(lv + 4), r2 = *(const float4 *)(lv + 8);
        eval_row(r0, r1, r2, a, b, c);
    }
    __device__ __forceinline__ void eval_row(const float4 r0, const float4 r1, const float4 r2, float2 &a, float2 &b,
                                             float2 &c) const
    {
        a = make_float2(fmaf(r0.x, k2, 1.f), r0.y * kw);
        b = make_float2(fmaf(r0.w, k2, r0.z), r1.x * kw);
        c = make_float2(fmaf(r1.z, k4, fmaf(r1.w, kw2, r1.y * k2)), fmaf(r2.y, k2kw, r2.x * kw));
    }
};

template <>
struct StepCoef<false> {
    float lx, ly, lx2, ly2;
    __device__ __forceinline__ void init(float lx_, float ly_, float, float)
    {
        lx = lx_;
        ly = ly_;
        lx2 = lx * lx;
        ly2 = ly * ly;
    }
    __device__ __forceinline__ void eval(const float *lv, float2 &a, float2 &b, float2 &c) const
    {
        const float4 r0 = *(const float4 *)lv, r1 = *(const float4 *)(lv + 4), r2 = *(const float4 *)(lv + 8);
        eval_row(r0, r1, r2, a, b, c);
    }
    __device__ __forceinline__ void eval_row(const float4 r0, const float4 r1, const float4 r2, float2 &a, float2 &b,
                                             float2 &c) const
    {
        const float Tr = fmaf(r0.x, lx2, r0.y * ly2);
        const float Ti = fmaf(r0.z, lx, r0.w * ly);
        a = make_float2(fmaf(-r1.x, Tr, 1.f), -r1.x * Ti);
        b = make_float2(fmaf(-r1.z, Tr, r1.y), -r1.z * Ti);
        const float t2r = fmaf(Tr, Tr, -Ti * Ti);
        c = make_float2(fmaf(-r2.x, t2r, r1.w * Tr), Ti * fmaf(r2.y, Tr, r1.w));
    }
};

// One backward step: R <- (a R - b) / (a - c R).
__device__ __forceinline__ void ricc_step(float2 &R, const float2 a, const float2 b, const float2 c)
{
    // D = a - c R with the product folded into the subtraction
    const float Dr = fmaf(-c.x, R.x, fmaf(c.y, R.y, a.x)), Di = fmaf(-c.x, R.y, fmaf(-c.y, R.x, a.y));
    const float Nr = fmaf(a.x, R.x, fmaf(-a.y, R.y, -b.x));
    const float Ni = fmaf(a.x, R.y, fmaf(a.y, R.x, -b.y));
    const float inv = rcp_approx(fmaf(Dr, Dr, Di * Di));
    R.x = fmaf(Nr, Dr, Ni * Di) * inv;
    R.y = fmaf(Ni, Dr, -Nr * Di) * inv;
}

// flux factor of step i with the updated ratio: Q *= c R + a
__device__ __forceinline__ void flux_step(float2 &Q, const float2 R, const float2 a, const float2 c)
{
    const float fr = fmaf(c.x, R.x, fmaf(-c.y, R.y, a.x));
    const float fi = fmaf(c.x, R.y, fmaf(c.y, R.x, a.y));
    const float qr = fmaf(Q.x, fr, -Q.y * fi);
    Q.y = fmaf(Q.x, fi, Q.y * fr);
    Q.x = qr;
}

__device__ __forceinline__ void renorm(float2 &Q, int &E)
{
    const float mx = fmaxf(fabsf(Q.x), fabsf(Q.y));
    const int e = ((__float_as_int(mx) >> 23) & 0xff) - 127;
    if (mx > 0.f && e > -126 && e < 127) {
        const float sc = __int_as_float((127 - e) << 23);
        Q.x *= sc;
        Q.y *= sc;
        E += e;
    }
}

// One solved mode m of a solve: backward Riccati sweep over the level table
// in shared memory (s_lv, s_slot), then the level values, phase shift and
// mirror write.  SINGLE: exactly one output slot (no per-step slot test).
template <bool ISO, bool SINGLE>
__device__ __forceinline__ void ricc_mode(const SolveGeom &g, const float *__restrict__ s_lv,
                                          const int *__restrict__ s_slot, const uint32_t *__restrict__ modes,
                                          const float2 *__restrict__ q0spec, float *__restrict__ scratch,
                                          float2 *__restrict__ Xp, float2 *__restrict__ Xq, float ax, float ay,
                                          int64_t m)
{
    const int L = g.nz - 1;
    const int jmax = g.jmax;
    const int64_t ns = g.nsolved;
    int r, c;
    bool paired;
    unpack_mode(modes[m], r, c, paired);
    const int kx = freq_of_index(c, g.nlx), ky = freq_of_index(r, g.nly);
    const float lx = ax * (float)kx, ly = ay * (float)ky;
    StepCoef<ISO> sc;
    sc.init(lx, ly, g.ex, g.ey);
    // top eigenvalue and radiation ratio R_L = 1 / (Kz_top eig)
    const float2 w = make_float2(fmaf(g.kxk_top_f, lx * lx, g.kyk_top_f * ly * ly),
                                 fmaf(g.uk_top_f, lx, g.vk_top_f * ly));
    const float2 eg = csqrt_f(w);
    const float2 ke = make_float2(g.kz_top_f * eg.x, g.kz_top_f * eg.y);
    const float inv = 1.0f / fmaf(ke.x, ke.x, ke.y * ke.y);
    float2 R = make_float2(ke.x * inv, -ke.y * inv);
    // above the highest output level: only the ratio
    int i = L - 1;
    for (; i >= jmax; --i) {
        float2 a, b, cc;
        sc.eval(s_lv + (size_t)i * BLDFM_LV32, a, b, cc);
        ricc_step(R, a, b, cc);
    }
    float2 Rj = R;
    float2 Q = make_float2(1.f, 0.f);
    int E = 0;
    if (!SINGLE) {
        const int s = s_slot[jmax];
        float *o = scratch + (size_t)s * 5 * ns + m;
        o[0] = R.x;
        o[ns] = R.y;
        o[2 * ns] = 1.f;
        o[3 * ns] = 0.f;
        o[4 * ns] = __int_as_float(0);
    }
    // below it: ratio and flux product, renormalised every 8 steps
    int cnt = 0;
    for (; i >= 0; --i) {
        float2 a, b, cc;
        sc.eval(s_lv + (size_t)i * BLDFM_LV32, a, b, cc);
        ricc_step(R, a, b, cc);
        flux_step(Q, R, a, cc);
        if (++cnt == 8) {
            cnt = 0;
            renorm(Q, E);
        }
        if (!SINGLE) {
            const int s = s_slot[i];
            if (s >= 0) {
                float *o = scratch + (size_t)s * 5 * ns + m;
                o[0] = R.x;
                o[ns] = R.y;
                o[2 * ns] = Q.x;
                o[3 * ns] = Q.y;
                o[4 * ns] = __int_as_float(E);
            }
        }
    }
    const float2 q0 = q0spec ? q0spec[(size_t)c * g.nly + r] : make_float2(g.q0dc_f, 0.f);
    float2 sh = make_float2(1.f, 0.f);
    if (g.do_shift) {
        const uint32_t turns = (uint32_t)kx * g.turn_x + (uint32_t)ky * g.turn_y;
        float sn, cs;
        sincospif((float)(int32_t)turns * 4.656612873077393e-10f, &sn, &cs);
        sh = make_float2(cs, sn);
    }
    const int rm = paired ? index_of_freq(-ky, g.nly) : 0;
    const int cm = paired ? index_of_freq(-kx, g.nlx) : 0;
    for (int s = 0; s < (SINGLE ? 1 : g.nsnap); ++s) {
        float2 ratio;
        if (SINGLE) {
            ratio = make_float2(ldexpf(Q.x, E), ldexpf(Q.y, E));
        } else {
            const float *o = scratch + (size_t)s * 5 * ns + m;
            Rj = make_float2(o[0], o[ns]);
            const float2 Qj = make_float2(o[2 * ns], o[3 * ns]);
            const int Ej = __float_as_int(o[4 * ns]);
            const float qn = fmaf(Qj.x, Qj.x, Qj.y * Qj.y);
            ratio = make_float2(0.f, 0.f);
            if (qn > 0.f) {
                const float2 t = make_float2(fmaf(Q.x, Qj.x, Q.y * Qj.y), fmaf(Q.y, Qj.x, -Q.x * Qj.y));
                const float scl = ldexpf(1.0f / qn, E - Ej);
                ratio = make_float2(t.x * scl, t.y * scl);
            }
        }
        float2 q = fc_mul(q0, ratio);
        float2 p = fc_mul(Rj, q);
        p = fc_mul(p, sh);
        q = fc_mul(q, sh);
        Xp[spec_idx(g, s, r, c)] = p;
        Xq[spec_idx(g, s, r, c)] = q;
        if (paired) {
            Xp[spec_idx(g, s, rm, cm)] = make_float2(p.x, -p.y);
            Xq[spec_idx(g, s, rm, cm)] = make_float2(q.x, -q.y);
        }
    }
}

// ---------------------------------------------------------------------------
// Packed form for two modes: lane x of every f32x2 value belongs to the first
// mode, lane y to the second, and each f32x2 instruction (fma/mul/add .rn)
// does both modes' operation in one issue slot.  Every operation is the one
// of the scalar functions above with the same operands, so each lane rounds
// exactly as the scalar recursion does.
// ---------------------------------------------------------------------------
struct PCplx {
    float2 re, im;
};

__device__ __forceinline__ float2 pbc(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 pneg(float2 a) { return make_float2(-a.x, -a.y); }

template <bool ISO>
struct PStep;

template <>
struct PStep<true> {
    float2 k2, kw, k4, kw2, k2kw;
    __device__ __forceinline__ void init(const StepCoef<true> &a, const StepCoef<true> &b)
    {
        k2 = make_float2(a.k2, b.k2);
        kw = make_float2(a.kw, b.kw);
        k4 = make_float2(a.k4, b.k4);
        kw2 = make_float2(a.kw2, b.kw2);
        k2kw = make_float2(a.k2kw, b.k2kw);
    }
    // StepCoef<true>::eval_row in both lanes
    __device__ __forceinline__ void eval_row(const float4 r0, const float4 r1, const float4 r2, PCplx &a, PCplx &b,
                                             PCplx &c) const
    {
        a.re = pfma(pbc(r0.x), k2, pbc(1.f));
        a.im = pmul(pbc(r0.y), kw);
        b.re = pfma(pbc(r0.w), k2, pbc(r0.z));
        b.im = pmul(pbc(r1.x), kw);
        c.re = pfma(pbc(r1.z), k4, pfma(pbc(r1.w), kw2, pmul(pbc(r1.y), k2)));
        c.im = pfma(pbc(r2.y), k2kw, pmul(pbc(r2.x), kw));
    }
};

template <>
struct PStep<false> {
    float2 lx, ly, lx2, ly2;
    __device__ __forceinline__ void init(const StepCoef<false> &a, const StepCoef<false> &b)
    {
        lx = make_float2(a.lx, b.lx);
        ly = make_float2(a.ly, b.ly);
        lx2 = make_float2(a.lx2, b.lx2);
        ly2 = make_float2(a.ly2, b.ly2);
    }
    // StepCoef<false>::eval_row in both lanes
    __device__ __forceinline__ void eval_row(const float4 r0, const float4 r1, const float4 r2, PCplx &a, PCplx &b,
                                             PCplx &c) const
    {
        const float2 Tr = pfma(pbc(r0.x), lx2, pmul(pbc(r0.y), ly2));
        const float2 Ti = pfma(pbc(r0.z), lx, pmul(pbc(r0.w), ly));
        a.re = pfma(pbc(-r1.x), Tr, pbc(1.f));
        a.im = pmul(pbc(-r1.x), Ti);
        b.re = pfma(pbc(-r1.z), Tr, pbc(r1.y));
        b.im = pmul(pbc(-r1.z), Ti);
        const float2 t2r = pfma(Tr, Tr, pneg(pmul(Ti, Ti)));
        c.re = pfma(pbc(-r2.x), t2r, pmul(pbc(r1.w), Tr));
        c.im = pmul(Ti, pfma(pbc(r2.y), Tr, pbc(r1.w)));
    }
};

// ricc_step in both lanes
__device__ __forceinline__ void pricc_step(PCplx &R, const PCplx a, const PCplx b, const PCplx c)
{
    const float2 Dr = pfma(pneg(c.re), R.re, pfma(c.im, R.im, a.re));
    const float2 Di = pfma(pneg(c.re), R.im, pfma(pneg(c.im), R.re, a.im));
    const float2 Nr = pfma(a.re, R.re, pfma(pneg(a.im), R.im, pneg(b.re)));
    const float2 Ni = pfma(a.re, R.im, pfma(a.im, R.re, pneg(b.im)));
    const float2 den = pfma(Dr, Dr, pmul(Di, Di));
    const float2 inv = make_float2(rcp_approx(den.x), rcp_approx(den.y));
    R.re = pmul(pfma(Nr, Dr, pmul(Ni, Di)), inv);
    R.im = pmul(pfma(Ni, Dr, pneg(pmul(Nr, Di))), inv);
}

// flux_step in both lanes
__device__ __forceinline__ void pflux_step(PCplx &Q, const PCplx R, const PCplx a, const PCplx c)
{
    const float2 fr = pfma(c.re, R.re, pfma(pneg(c.im), R.im, a.re));
    const float2 fi = pfma(c.re, R.im, pfma(c.im, R.re, a.im));
    const float2 qr = pfma(Q.re, fr, pneg(pmul(Q.im, fi)));
    Q.im = pfma(Q.re, fi, pmul(Q.im, fr));
    Q.re = qr;
}

// 2 NP solved modes per thread with one output level (SINGLE): the same
// arithmetic per mode as ricc_mode<ISO, true>, with the level-table row and
// the loop control shared by the recursions, which run in the two lanes of
// NP independent chains of packed f32x2 operations.  Slots u >= nvalid
// repeat mode m[0] and write nothing.  The mode's indices are unpacked again
// for the final writes rather than held in registers through the sweep.
template <bool ISO, int NP>
__device__ __forceinline__ void ricc_modes_packed(const SolveGeom &g, const float *__restrict__ s_lv,
                                                  const uint32_t *__restrict__ modes,
                                                  const float2 *__restrict__ q0spec, float2 *__restrict__ Xp,
                                                  float2 *__restrict__ Xq, float ax, float ay, const int64_t *m,
                                                  int nvalid)
{
    constexpr int NM = 2 * NP;
    const int L = g.nz - 1;
    const int jmax = g.jmax;
    PStep<ISO> ps[NP];
    PCplx PR[NP];
#pragma unroll
    for (int h = 0; h < NP; ++h) {
        StepCoef<ISO> sc[2];
        float2 R[2];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const int u = 2 * h + l;
            int r, c;
            bool paired;
            unpack_mode(modes[u < nvalid ? m[u] : m[0]], r, c, paired);
            const float lx = ax * (float)freq_of_index(c, g.nlx), ly = ay * (float)freq_of_index(r, g.nly);
            sc[l].init(lx, ly, g.ex, g.ey);
            const float2 w = make_float2(fmaf(g.kxk_top_f, lx * lx, g.kyk_top_f * ly * ly),
                                         fmaf(g.uk_top_f, lx, g.vk_top_f * ly));
            const float2 eg = csqrt_f(w);
            const float2 ke = make_float2(g.kz_top_f * eg.x, g.kz_top_f * eg.y);
            const float inv = 1.0f / fmaf(ke.x, ke.x, ke.y * ke.y);
            R[l] = make_float2(ke.x * inv, -ke.y * inv);
        }
        ps[h].init(sc[0], sc[1]);
        PR[h] = {make_float2(R[0].x, R[1].x), make_float2(R[0].y, R[1].y)};
    }
    // one step of the ratio recursion (above the highest output level) and
    // one of ratio and flux product (below it), at level row i
    auto ratio_step = [&](int i) {
        const float *lv = s_lv + (size_t)i * BLDFM_LV32;
        const float4 r0 = *(const float4 *)lv, r1 = *(const float4 *)(lv + 4), r2 = *(const float4 *)(lv + 8);
#pragma unroll
        for (int h = 0; h < NP; ++h) {
            PCplx a, b, cc;
            ps[h].eval_row(r0, r1, r2, a, b, cc);
            pricc_step(PR[h], a, b, cc);
        }
    };
    PCplx Rj[NP], PQ[NP];
    int E[NM];
    auto flux_step = [&](int i) {
        const float *lv = s_lv + (size_t)i * BLDFM_LV32;
        const float4 r0 = *(const float4 *)lv, r1 = *(const float4 *)(lv + 4), r2 = *(const float4 *)(lv + 8);
#pragma unroll
        for (int h = 0; h < NP; ++h) {
            PCplx a, b, cc;
            ps[h].eval_row(r0, r1, r2, a, b, cc);
            pricc_step(PR[h], a, b, cc);
            pflux_step(PQ[h], PR[h], a, cc);
        }
    };
    // loops unrolled by 4 and 8 (no per-step loop control)
    int i = L - 1;
    for (; i - 3 >= jmax; i -= 4) {
#pragma unroll
        for (int s = 0; s < 4; ++s) ratio_step(i - s);
    }
    for (; i >= jmax; --i) ratio_step(i);
#pragma unroll
    for (int h = 0; h < NP; ++h) {
        Rj[h] = PR[h];
        PQ[h] = {make_float2(1.f, 1.f), make_float2(0.f, 0.f)};
        E[2 * h] = E[2 * h + 1] = 0;
    }
    // below it: groups of 8 steps, each followed by the renormalisation of
    // the flux product; then the remaining steps (fewer than 8)
    for (; i >= 7; i -= 8) {
#pragma unroll
        for (int s = 0; s < 8; ++s) flux_step(i - s);
#pragma unroll
        for (int h = 0; h < NP; ++h) {
            float2 q0 = make_float2(PQ[h].re.x, PQ[h].im.x), q1 = make_float2(PQ[h].re.y, PQ[h].im.y);
            renorm(q0, E[2 * h]);
            renorm(q1, E[2 * h + 1]);
            PQ[h].re = make_float2(q0.x, q1.x);
            PQ[h].im = make_float2(q0.y, q1.y);
        }
    }
    for (; i >= 0; --i) flux_step(i);
#pragma unroll
    for (int u = 0; u < NM; ++u) {
        if (u >= nvalid) break;
        const int h = u >> 1;
        const float2 Q = (u & 1) ? make_float2(PQ[h].re.y, PQ[h].im.y) : make_float2(PQ[h].re.x, PQ[h].im.x);
        const float2 Rju = (u & 1) ? make_float2(Rj[h].re.y, Rj[h].im.y) : make_float2(Rj[h].re.x, Rj[h].im.x);
        int r, c;
        bool paired;
        unpack_mode(modes[m[u]], r, c, paired);
        const int kx = freq_of_index(c, g.nlx), ky = freq_of_index(r, g.nly);
        const float2 q0 = q0spec ? q0spec[(size_t)c * g.nly + r] : make_float2(g.q0dc_f, 0.f);
        float2 sh = make_float2(1.f, 0.f);
        if (g.do_shift) {
            const uint32_t turns = (uint32_t)kx * g.turn_x + (uint32_t)ky * g.turn_y;
            float sn, cs;
            sincospif((float)(int32_t)turns * 4.656612873077393e-10f, &sn, &cs);
            sh = make_float2(cs, sn);
        }
        const float2 ratio = make_float2(ldexpf(Q.x, E[u]), ldexpf(Q.y, E[u]));
        float2 q = fc_mul(q0, ratio);
        float2 p = fc_mul(Rju, q);
        p = fc_mul(p, sh);
        q = fc_mul(q, sh);
        Xp[spec_idx(g, 0, r, c)] = p;
        Xq[spec_idx(g, 0, r, c)] = q;
        if (paired) {
            const int rm = index_of_freq(-ky, g.nly);
            const int cm = index_of_freq(-kx, g.nlx);
            Xp[spec_idx(g, 0, rm, cm)] = make_float2(p.x, -p.y);
            Xq[spec_idx(g, 0, rm, cm)] = make_float2(q.x, -q.y);
        }
    }
}

// Two solved modes per thread (ma and, if mb >= 0, mb) in one packed chain.
template <bool ISO>
__device__ __forceinline__ void ricc_mode_pair(const SolveGeom &g, const float *__restrict__ s_lv,
                                               const uint32_t *__restrict__ modes,
                                               const float2 *__restrict__ q0spec, float2 *__restrict__ Xp,
                                               float2 *__restrict__ Xq, float ax, float ay, int64_t ma, int64_t mb)
{
    const int64_t m[2] = {ma, mb};
    ricc_modes_packed<ISO, 1>(g, s_lv, modes, q0spec, Xp, Xq, ax, ay, m, mb >= 0 ? 2 : 1);
}

// Exact FP32 values (p, q) of one solved mode m at the single output level,
// phase-shifted like the solve's spectra, with the level table read from
// global memory (rows of BLDFM_LV32 floats): the sweep of ricc_mode (ratio
// above the output level, ratio and flux product below it) for a footprint
// (unit source spectrum q0dc_fp).  (r, c) receive the mode's row and column.
// Used by the surrogate's accuracy guard on a sample of modes.
template <bool ISO>
__device__ __forceinline__ void ricc_rc_value(const SolveGeom &g, const float *__restrict__ lv, float ax, float ay,
                                              int r, int c, float2 &p, float2 &q)
{
    const int L = g.nz - 1;
    const int jmax = g.jmax;
    const int kx = freq_of_index(c, g.nlx), ky = freq_of_index(r, g.nly);
    const float lx = ax * (float)kx, ly = ay * (float)ky;
    StepCoef<ISO> sc;
    sc.init(lx, ly, g.ex, g.ey);
    const float2 w = make_float2(fmaf(g.kxk_top_f, lx * lx, g.kyk_top_f * ly * ly),
                                 fmaf(g.uk_top_f, lx, g.vk_top_f * ly));
    const float2 eg = csqrt_f(w);
    const float2 ke = make_float2(g.kz_top_f * eg.x, g.kz_top_f * eg.y);
    const float inv = 1.0f / fmaf(ke.x, ke.x, ke.y * ke.y);
    float2 R = make_float2(ke.x * inv, -ke.y * inv);
    int i = L - 1;
    for (; i >= jmax; --i) {
        float2 a, b, cc;
        sc.eval(lv + (size_t)i * BLDFM_LV32, a, b, cc);
        ricc_step(R, a, b, cc);
    }
    const float2 Rj = R;
    float2 Q = make_float2(1.f, 0.f);
    int E = 0, cnt = 0;
    for (; i >= 0; --i) {
        float2 a, b, cc;
        sc.eval(lv + (size_t)i * BLDFM_LV32, a, b, cc);
        ricc_step(R, a, b, cc);
        flux_step(Q, R, a, cc);
        if (++cnt == 8) {
            cnt = 0;
            renorm(Q, E);
        }
    }
    float2 sh = make_float2(1.f, 0.f);
    if (g.do_shift) {
        const uint32_t turns = (uint32_t)kx * g.turn_x + (uint32_t)ky * g.turn_y;
        float sn, cs;
        sincospif((float)(int32_t)turns * 4.656612873077393e-10f, &sn, &cs);
        sh = make_float2(cs, sn);
    }
    const float2 q0 = make_float2(g.q0dc_f, 0.f);
    q = fc_mul(q0, make_float2(ldexpf(Q.x, E), ldexpf(Q.y, E)));
    p = fc_mul(fc_mul(Rj, q), sh);
    q = fc_mul(q, sh);
}

// ricc_rc_value for two modes (r[l], c[l]), l = 0, 1, in the two lanes of
// packed f32x2 operations (each lane rounds exactly as ricc_rc_value does),
// the level table in shared or global memory.
template <bool ISO>
__device__ __forceinline__ void ricc_rc_pair(const SolveGeom &g, const float *__restrict__ lv, float ax, float ay,
                                             const int (&r)[2], const int (&c)[2], float2 (&p)[2], float2 (&q)[2])
{
    const int L = g.nz - 1;
    const int jmax = g.jmax;
    StepCoef<ISO> sc[2];
    float2 R0[2];
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        const float lx = ax * (float)freq_of_index(c[l], g.nlx), ly = ay * (float)freq_of_index(r[l], g.nly);
        sc[l].init(lx, ly, g.ex, g.ey);
        const float2 w = make_float2(fmaf(g.kxk_top_f, lx * lx, g.kyk_top_f * ly * ly),
                                     fmaf(g.uk_top_f, lx, g.vk_top_f * ly));
        const float2 eg = csqrt_f(w);
        const float2 ke = make_float2(g.kz_top_f * eg.x, g.kz_top_f * eg.y);
        const float inv = 1.0f / fmaf(ke.x, ke.x, ke.y * ke.y);
        R0[l] = make_float2(ke.x * inv, -ke.y * inv);
    }
    PStep<ISO> ps;
    ps.init(sc[0], sc[1]);
    PCplx R = {make_float2(R0[0].x, R0[1].x), make_float2(R0[0].y, R0[1].y)};
    int i = L - 1;
    for (; i >= jmax; --i) {
        const float *row = lv + (size_t)i * BLDFM_LV32;
        const float4 r0 = *(const float4 *)row, r1 = *(const float4 *)(row + 4), r2 = *(const float4 *)(row + 8);
        PCplx a, b, cc;
        ps.eval_row(r0, r1, r2, a, b, cc);
        pricc_step(R, a, b, cc);
    }
    const PCplx Rj = R;
    PCplx Q = {make_float2(1.f, 1.f), make_float2(0.f, 0.f)};
    int E[2] = {0, 0};
    int cnt = 0;
    for (; i >= 0; --i) {
        const float *row = lv + (size_t)i * BLDFM_LV32;
        const float4 r0 = *(const float4 *)row, r1 = *(const float4 *)(row + 4), r2 = *(const float4 *)(row + 8);
        PCplx a, b, cc;
        ps.eval_row(r0, r1, r2, a, b, cc);
        pricc_step(R, a, b, cc);
        pflux_step(Q, R, a, cc);
        if (++cnt == 8) {
            cnt = 0;
            float2 q0 = make_float2(Q.re.x, Q.im.x), q1 = make_float2(Q.re.y, Q.im.y);
            renorm(q0, E[0]);
            renorm(q1, E[1]);
            Q.re = make_float2(q0.x, q1.x);
            Q.im = make_float2(q0.y, q1.y);
        }
    }
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        const float2 Ql = l ? make_float2(Q.re.y, Q.im.y) : make_float2(Q.re.x, Q.im.x);
        const float2 Rjl = l ? make_float2(Rj.re.y, Rj.im.y) : make_float2(Rj.re.x, Rj.im.x);
        const int kx = freq_of_index(c[l], g.nlx), ky = freq_of_index(r[l], g.nly);
        float2 sh = make_float2(1.f, 0.f);
        if (g.do_shift) {
            const uint32_t turns = (uint32_t)kx * g.turn_x + (uint32_t)ky * g.turn_y;
            float sn, cs;
            sincospif((float)(int32_t)turns * 4.656612873077393e-10f, &sn, &cs);
            sh = make_float2(cs, sn);
        }
        const float2 q0 = make_float2(g.q0dc_f, 0.f);
        q[l] = fc_mul(q0, make_float2(ldexpf(Ql.x, E[l]), ldexpf(Ql.y, E[l])));
        p[l] = fc_mul(fc_mul(Rjl, q[l]), sh);
        q[l] = fc_mul(q[l], sh);
    }
}

// the same for solved mode m of the mode list; (r, c) receive its row and column
template <bool ISO>
__device__ __forceinline__ void ricc_mode_value(const SolveGeom &g, const float *__restrict__ lv,
                                                const uint32_t *__restrict__ modes, float ax, float ay, int64_t m,
                                                float2 &p, float2 &q, int &r, int &c)
{
    bool paired;
    unpack_mode(modes[m], r, c, paired);
    ricc_rc_value<ISO>(g, lv, ax, ay, r, c, p, q);
}
