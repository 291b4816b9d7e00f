// Nondimensional per-mode transfer functions for the learned surrogate.
//
// With MOST profiles (u = u*/kappa (ln z/z0 + psi(z/L)), K = kappa u* z /
// phi(z/L), Kx = Ky = Kz, src/bldfm/pbl_model.py:8-204) the wind keeps one
// direction, so per mode the solver's operator is T = -K k^2 - i U(z) k_par
// (solver.py:307-374).  Scaling heights by z_m, velocities by the wind speed U
// at z_m and diffusivities by U z_m leaves a discrete problem that depends on
// (k_par z_m, |k_perp| z_m, z_m / L, ln(z_m / z0)) and on the grid in units of
// z_m (fixed by ln(z_m / z0) and the level count for the default stretch and
// top).  The quantities learned are the flux transfer Tq = q(z_m) / q(0) and
// the ratio R~ = U p(z_m) / q(z_m), as the targets
//   t0 = log|Tq| / (1 + k), t1 = arg Tq / (1 + k),
//   t2 = log|R~ / R~top|, t3 = arg(R~ / R~top),
// with k = |k~|, arg Tq unwrapped as the sum of the per-step factor arguments
// and R~top = 1 / (K~top lam) the top radiation ratio (singular as k -> 0,
// where R~ / R~top -> 1).  Negative k_par gives the complex conjugates.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

struct TransferCase {  // one nondimensional met case
    int nz, jm;        // levels, index of z_m
    float ktop, utop;  // K~ and U~ at the top level
    float s1, s2, s3;  // z_m / L, ln(z_m / z0), u* / U
    int pad;
};

__device__ __forceinline__ float2 sp_cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// Invariant-imbedding sweep of one mode (k_par >= 0) in nondimensional
// variables; st[i] = (h~, K~, U~, 0) of step i.  out: the four targets.
__device__ __forceinline__ void transfer_one(const TransferCase &tc, const float4 *__restrict__ st, float kpar,
                                             float kperp, float *out)
{
    const float k2 = fmaf(kpar, kpar, kperp * kperp);
    // top radiation condition: R~ = 1 / (K~ lam), lam^2 = k^2 + i U~ k_par / K~
    const float l2i = tc.utop * kpar / tc.ktop;
    const float t = sqrtf(0.5f * (k2 + hypotf(k2, l2i)));
    const float2 lam = t > 0.f ? make_float2(t, l2i / (2.f * t)) : make_float2(0.f, 0.f);
    const float2 ke = make_float2(tc.ktop * lam.x, tc.ktop * lam.y);
    const float inv = 1.f / fmaf(ke.x, ke.x, ke.y * ke.y);
    float2 R = make_float2(ke.x * inv, -ke.y * inv);
    float2 Rj = R;
    float la = 0.f, ph = 0.f;
    for (int i = tc.nz - 2; i >= 0; --i) {
        const float4 s = st[i];
        const float h = s.x, K = s.y, U = s.z;
        const float kap = 1.f / K;
        const float2 T = make_float2(-K * k2, -U * kpar);
        const float A = 0.5f * kap * h * h, B1 = kap * kap * h * h * h * (1.f / 6.f), C1 = kap * h * h * h * (1.f / 6.f);
        const float2 a = make_float2(fmaf(-A, T.x, 1.f), -A * T.y);
        const float2 b = make_float2(fmaf(-B1, T.x, -kap * h), -B1 * T.y);
        const float2 T2 = sp_cmul(T, T);
        const float2 c = make_float2(fmaf(-C1, T2.x, h * T.x), fmaf(-C1, T2.y, h * T.y));
        const float2 cR = sp_cmul(c, R);
        const float2 D = make_float2(a.x - cR.x, a.y - cR.y);
        const float2 N = make_float2(fmaf(a.x, R.x, fmaf(-a.y, R.y, -b.x)), fmaf(a.x, R.y, fmaf(a.y, R.x, -b.y)));
        const float dinv = 1.f / fmaf(D.x, D.x, D.y * D.y);
        R = make_float2(fmaf(N.x, D.x, N.y * D.y) * dinv, fmaf(N.y, D.x, -N.x * D.y) * dinv);
        if (i == tc.jm) Rj = R;
        if (i < tc.jm) {
            const float2 f = make_float2(fmaf(c.x, R.x, fmaf(-c.y, R.y, a.x)), fmaf(c.x, R.y, fmaf(c.y, R.x, a.y)));
            la += 0.5f * logf(fmaf(f.x, f.x, f.y * f.y));
            ph += atan2f(f.y, f.x);
        }
    }
    const float kk = 1.f + sqrtf(k2);
    out[0] = la / kk;
    out[1] = ph / kk;
    // R~ / R~top = R~ K~top lam
    const float2 rr = sp_cmul(Rj, ke);
    out[2] = 0.5f * logf(fmaf(rr.x, rr.x, rr.y * rr.y));
    out[3] = atan2f(rr.y, rr.x);
}

// top radiation ratio R~top = 1 / (K~top lam) of a mode (k_par >= 0)
__device__ __forceinline__ float2 top_ratio(float ktop, float utop, float kpar, float kperp)
{
    const float k2 = fmaf(kpar, kpar, kperp * kperp);
    const float l2i = utop * kpar / ktop;
    const float t = sqrtf(0.5f * (k2 + hypotf(k2, l2i)));
    const float2 ke = make_float2(ktop * t, ktop * (t > 0.f ? l2i / (2.f * t) : 0.f));
    const float inv = 1.f / fmaf(ke.x, ke.x, ke.y * ke.y);
    return make_float2(ke.x * inv, -ke.y * inv);
}

// MLP input row of a mode (k_par >= 0, k > 0): 8 features of order one
__device__ __forceinline__ void feature_row(float *x, float kpar, float kperp, float s1, float s2, float s3)
{
    const float k = sqrtf(fmaf(kpar, kpar, kperp * kperp));
    x[0] = kpar * 0.1f;
    x[1] = kperp * 0.1f;
    x[2] = (s1 + 0.5f) * 2.f;
    x[3] = (s2 - 6.f) * (2.f / 3.f);
    x[4] = (s3 - 0.085f) * 30.f;
    x[5] = logf(k) * (1.f / 3.f);
    x[6] = kpar / k;
    x[7] = fmaxf(s1, 0.f) * 4.f;  // the stability functions change form at s1 = 0
}

// targets -> (Tq, R~ / R~top) for k_par >= 0; magnitudes clamped to finite values
__device__ __forceinline__ void decode_transfer(const float *y, float k, float2 &Tq, float2 &Rt)
{
    const float kk = 1.f + k;
    const float la = fminf(y[0] * kk, 2.f), ph = y[1] * kk;
    const float lr = fminf(y[2], 60.f);
    float sn, cs;
    sincosf(ph, &sn, &cs);
    const float mq = expf(la);
    Tq = make_float2(mq * cs, mq * sn);
    sincosf(y[3], &sn, &cs);
    const float mr = expf(lr);
    Rt = make_float2(mr * cs, mr * sn);
}
