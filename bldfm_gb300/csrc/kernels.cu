// Device kernels of the steady-state transport solve.
//
//   sweep64_kernel     ivp_solver (src/bldfm/solver.py:307-374), both shooting IVPs
//   combine64_kernel   alpha + level combination + shift (solver.py:228-235, 253-262)
//   trapezoid_kernel   k = 0 mode (solver.py:237-251)
//   analytic64_kernel  constant-profile closed form (solver.py:193-202)
//   riccati32_kernel   FP32 invariant-imbedding sweep of the same discrete BVP
//   fwd_rows / fwd_cols   truncated forward FFT of the source (solver.py:136-145)
//   out_cols / out_rows   un-truncate + output FFT + crop (solver.py:264-290)
//
// FP64 kernels reproduce the reference's numpy rounding: every operation is an
// explicit round-to-nearest intrinsic (no contraction), and complex products use
// numpy's x86-64 pattern re = fma(ar, br, -(ai*bi)), im = fma(ar, bi, ai*br).
#include "devattr.h"
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.h"
#include "devmath.cuh"
#include "fft_core.cuh"
#include "kernels.h"
#include "sweep32.cuh"
#include "fft_passes.cuh"

#define LAUNCH_CHECK() (cudaGetLastError())

// ---------------------------------------------------------------------------
// FP64 shooting sweep
// ---------------------------------------------------------------------------
// One thread per solved mode.  Writes per mode: top states (p1,q1,p2,q2) and
// the same four states at every snapshot slot.
//   snap layout: [(slot * 4 + j) * nsolved + m],  top layout: [j * nsolved + m]
__global__ void __launch_bounds__(128) sweep64_kernel(SolveGeom g, const double *__restrict__ lvtab,
                                                      const int *__restrict__ slot_of_step,
                                                      const uint32_t *__restrict__ modes,
                                                      const double2 *__restrict__ q0spec,
                                                      double2 *__restrict__ snap, double2 *__restrict__ top,
                                                      int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    double *s_lv = (double *)smem_raw;
    const int L = g.nz - 1;
    int *s_slot = (int *)(s_lv + (size_t)L * BLDFM_LV64);
    if (L > 0) {
        if (!bulk_load_to_smem(s_lv, lvtab, (uint32_t)((size_t)L * BLDFM_LV64 * sizeof(double)), &bar, err))
            return;
    }
    for (int i = threadIdx.x; i < g.nz; i += blockDim.x) s_slot[i] = slot_of_step[i];
    __syncthreads();

    const int64_t ns = g.nsolved;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < ns; m += (int64_t)gridDim.x * blockDim.x) {
        int r, c;
        bool paired;
        unpack_mode(modes[m], r, c, paired);
        const double lx = wavenumber(freq_of_index(c, g.nlx), g.valx, g.lx_scale);
        const double ly = wavenumber(freq_of_index(r, g.nly), g.valy, g.ly_scale);
        const double lx2 = __dmul_rn(lx, lx), ly2 = __dmul_rn(ly, ly);
        double2 p1 = make_double2(1.0, 0.0), q1 = make_double2(0.0, 0.0);
        double2 p2 = make_double2(0.0, 0.0);
        double2 q2 = q0spec ? q0spec[(size_t)c * g.nly + r] : make_double2(g.q0dc_fp, 0.0);
        for (int i = 0; i < L; ++i) {
            const int s = s_slot[i];
            if (s >= 0) {
                double2 *o = snap + (size_t)s * 4 * ns + m;
                o[0] = p1;
                o[ns] = q1;
                o[2 * ns] = p2;
                o[3 * ns] = q2;
            }
            const double *lv = s_lv + (size_t)i * BLDFM_LV64;
            // T = -(Kx Lx^2 + Ky Ly^2) - 1j u Lx - 1j v Ly
            double2 T;
            T.x = -__dadd_rn(__dmul_rn(lv[LV_KX], lx2), __dmul_rn(lv[LV_KY], ly2));
            T.y = __dsub_rn(-__dmul_rn(lv[LV_U], lx), __dmul_rn(lv[LV_V], ly));
            // a = d = 1 - 0.5 Kzinv T dz^2
            double2 a;
            a.x = __dsub_rn(1.0, __dmul_rn(__dmul_rn(lv[LV_S1], T.x), lv[LV_H2]));
            a.y = __dsub_rn(0.0, __dmul_rn(__dmul_rn(lv[LV_S1], T.y), lv[LV_H2]));
            // b = -Kzinv dz - 1/6 Kzinv^2 T dz^3
            double2 b;
            b.x = __dsub_rn(lv[LV_S3], __dmul_rn(__dmul_rn(lv[LV_S2], T.x), lv[LV_H3]));
            b.y = __dsub_rn(0.0, __dmul_rn(__dmul_rn(lv[LV_S2], T.y), lv[LV_H3]));
            // c = T dz - 1/6 Kzinv T^2 dz^3
            const double2 T2 = np_cmul(T, T);
            double2 cc;
            cc.x = __dsub_rn(__dmul_rn(T.x, lv[LV_H]), __dmul_rn(__dmul_rn(lv[LV_S4], T2.x), lv[LV_H3]));
            cc.y = __dsub_rn(__dmul_rn(T.y, lv[LV_H]), __dmul_rn(__dmul_rn(lv[LV_S4], T2.y), lv[LV_H3]));
            const double2 np1 = np_cadd(np_cmul(a, p1), np_cmul(b, q1));
            const double2 nq1 = np_cadd(np_cmul(cc, p1), np_cmul(a, q1));
            const double2 np2 = np_cadd(np_cmul(a, p2), np_cmul(b, q2));
            const double2 nq2 = np_cadd(np_cmul(cc, p2), np_cmul(a, q2));
            p1 = np1;
            q1 = nq1;
            p2 = np2;
            q2 = nq2;
        }
        {
            const int s = s_slot[g.nz - 1];
            if (s >= 0) {
                double2 *o = snap + (size_t)s * 4 * ns + m;
                o[0] = p1;
                o[ns] = q1;
                o[2 * ns] = p2;
                o[3 * ns] = q2;
            }
        }
        top[m] = p1;
        top[ns + m] = q1;
        top[2 * ns + m] = p2;
        top[3 * ns + m] = q2;
    }
}

// ---------------------------------------------------------------------------
// FP64 combination: alpha, levels, complex64 rounding, phase shift, mirror
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) combine64_kernel(SolveGeom g, const uint32_t *__restrict__ modes,
                                                        const double2 *__restrict__ eig,
                                                        const double2 *__restrict__ snap,
                                                        const double2 *__restrict__ top, double2 *__restrict__ Xp,
                                                        double2 *__restrict__ Xq)
{
    const int64_t ns = g.nsolved;
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= ns) return;
    int r, c;
    bool paired;
    unpack_mode(modes[m], r, c, paired);
    const int kx = freq_of_index(c, g.nlx), ky = freq_of_index(r, g.nly);
    // alpha = -(q2 - Kz eig p2) / (q1 - Kz eig p1)
    const double2 e = eig[m];
    const double2 keig = make_double2(__dmul_rn(g.kz_top, e.x), __dmul_rn(g.kz_top, e.y));
    double2 num = np_csub(top[3 * ns + m], np_cmul(keig, top[2 * ns + m]));
    const double2 den = np_csub(top[ns + m], np_cmul(keig, top[m]));
    num.x = -num.x;
    num.y = -num.y;
    const double2 alpha = np_cdiv(num, den);

    double2 shift = make_double2(1.0, 0.0);
    if (g.do_shift) {
        const double lx = wavenumber(kx, g.valx, g.lx_scale);
        const double ly = wavenumber(ky, g.valy, g.ly_scale);
        const double th = __dadd_rn(__dmul_rn(lx, g.sx), __dmul_rn(ly, g.sy));
        double sn, cs;
        sincos(th, &sn, &cs);
        shift = make_double2(cs, sn);
    }
    const int rm = paired ? index_of_freq(-ky, g.nly) : 0;
    const int cm = paired ? index_of_freq(-kx, g.nlx) : 0;
    for (int s = 0; s < g.nsnap; ++s) {
        const double2 *sp = snap + (size_t)s * 4 * ns + m;
        double2 p = np_cadd(np_cmul(alpha, sp[0]), sp[2 * ns]);
        double2 q = np_cadd(np_cmul(alpha, sp[ns]), sp[3 * ns]);
        if (g.precision == 0) {
            p = round_c64(p);
            q = round_c64(q);
        }
        if (g.do_shift) {
            p = np_cmul(p, shift);
            q = np_cmul(q, shift);
        }
        Xp[spec_idx(g, s, r, c)] = p;
        Xq[spec_idx(g, s, r, c)] = q;
        if (paired) {
            Xp[spec_idx(g, s, rm, cm)] = make_double2(p.x, -p.y);
            Xq[spec_idx(g, s, rm, cm)] = make_double2(q.x, -q.y);
        }
    }
}

// ---------------------------------------------------------------------------
// k = 0 mode: trapezoid rule, one thread.  lvtab column LV_PAD holds
// w_i = 0.5/Kz[i] + 0.5/Kz[i+1], column LV_H holds dz[i].
// ---------------------------------------------------------------------------
// k = 0 mode when q0 lives on the device (dispersion mode): writes the
// reference's trapezoid values (solver.py:237-251) into dc[2 s] (p), dc[2 s + 1]
// (q).  The terms (q0 dz_i) w_i are independent and computed in parallel; the
// running difference keeps the reference's order on one thread.
// dcp (may be NULL): DC_PARTS partial FP64 sums of the source field
// (dc_partial_kernel); the k = 0 source value is then their sum / (nxe nye)
// in FP64 instead of the transform's k = 0 output.
template <typename C>
__global__ void __launch_bounds__(256) trapezoid_kernel(SolveGeom g, const double *__restrict__ lvtab,
                                                        const int *__restrict__ slot_of_step,
                                                        const C *__restrict__ q0spec, double p000,
                                                        double2 *__restrict__ dc, const double *__restrict__ dcp)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *term = (double2 *)smem_raw;
    int *sl = (int *)(term + (g.nz > 1 ? g.nz - 1 : 1));
    double2 q0 = make_double2((double)q0spec[0].x, (double)q0spec[0].y);
    if (dcp) {
        double sum = 0.0;
        for (int b = 0; b < DC_PARTS; ++b) sum += dcp[b];
        q0 = make_double2(sum * g.inv_nxe * g.inv_nye, 0.0);
    }
    const bool single = g.precision == 0;
    const double2 qs = single ? round_c64(q0) : q0;
    for (int s = threadIdx.x; s < g.nlvls; s += blockDim.x) {
        dc[2 * s + 1] = qs;
        if (s > 0) dc[2 * s] = make_double2(0.0, 0.0);
    }
    for (int i = threadIdx.x; i < g.nz - 1; i += blockDim.x) {
        const double dz = lvtab[(size_t)i * BLDFM_LV64 + LV_H];
        const double w = lvtab[(size_t)i * BLDFM_LV64 + LV_PAD];
        term[i] = make_double2(__dmul_rn(__dmul_rn(q0.x, dz), w), __dmul_rn(__dmul_rn(q0.y, dz), w));
    }
    for (int i = threadIdx.x; i < g.nz; i += blockDim.x) sl[i] = slot_of_step[i];
    __syncthreads();
    if (threadIdx.x != 0) return;
    dc[0] = make_double2(single ? (double)__double2float_rn(p000) : p000, 0.0);
    if (g.analytic) return;
    double2 p00 = make_double2(p000, 0.0);
    for (int i = 0; i < g.nz - 1; ++i) {
        const int s = sl[i];
        if (s >= 0) dc[2 * s] = single ? round_c64(p00) : p00;
        p00.x = __dsub_rn(p00.x, term[i].x);
        p00.y = __dsub_rn(p00.y, term[i].y);
    }
    const int s = sl[g.nz - 1];
    if (s >= 0) dc[2 * s] = single ? round_c64(p00) : p00;
}

// ---------------------------------------------------------------------------
// analytic branch (constant profiles, one output level)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) analytic64_kernel(SolveGeom g, const uint32_t *__restrict__ modes,
                                                         const double2 *__restrict__ eig,
                                                         const double2 *__restrict__ q0spec, double kzinv,
                                                         double hlev, double2 *__restrict__ Xp,
                                                         double2 *__restrict__ Xq)
{
    const int64_t ns = g.nsolved;
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= ns) return;
    int r, c;
    bool paired;
    unpack_mode(modes[m], r, c, paired);
    const int kx = freq_of_index(c, g.nlx), ky = freq_of_index(r, g.nly);
    const double2 e = eig[m];
    const double2 q0 = q0spec ? q0spec[(size_t)c * g.nly + r] : make_double2(g.q0dc_fp, 0.0);
    // tfftq = q0 * exp(-eig * h)
    const double er = __dmul_rn(-e.x, hlev), ei = __dmul_rn(-e.y, hlev);
    double sn, cs;
    sincos(ei, &sn, &cs);
    const double ex = exp(er);
    double2 q = np_cmul(q0, make_double2(ex * cs, ex * sn));
    if (g.precision == 0) q = round_c64(q);
    // tfftp = tfftq * Kzinv / eig
    double2 p = np_cdiv(make_double2(__dmul_rn(q.x, kzinv), __dmul_rn(q.y, kzinv)), e);
    if (g.precision == 0) p = round_c64(p);
    if (g.do_shift) {
        const double lx = wavenumber(kx, g.valx, g.lx_scale);
        const double ly = wavenumber(ky, g.valy, g.ly_scale);
        const double th = __dadd_rn(__dmul_rn(lx, g.sx), __dmul_rn(ly, g.sy));
        double s2, c2;
        sincos(th, &s2, &c2);
        const double2 sh = make_double2(c2, s2);
        p = np_cmul(p, sh);
        q = np_cmul(q, sh);
    }
    Xp[spec_idx(g, 0, r, c)] = p;
    Xq[spec_idx(g, 0, r, c)] = q;
    if (paired) {
        const int rm = index_of_freq(-ky, g.nly), cm = index_of_freq(-kx, g.nlx);
        Xp[spec_idx(g, 0, rm, cm)] = make_double2(p.x, -p.y);
        Xq[spec_idx(g, 0, rm, cm)] = make_double2(q.x, -q.y);
    }
}

// analytic k = 0 (dispersion mode, q0 on the device): p = p000 - q0 Kzinv h, q = q0
__global__ void analytic_dc_kernel(SolveGeom g, const double2 *__restrict__ q0spec, double p000, double kzinv,
                                   double hlev, double2 *__restrict__ dc)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double2 q0 = q0spec[0];
    double2 p = make_double2(__dsub_rn(p000, __dmul_rn(__dmul_rn(q0.x, kzinv), hlev)),
                             __dsub_rn(0.0, __dmul_rn(__dmul_rn(q0.y, kzinv), hlev)));
    double2 q = q0;
    if (g.precision == 0) {
        p = round_c64(p);
        q = round_c64(q);
    }
    dc[0] = p;
    dc[1] = q;
}

// One thread per solved mode, grid-stride.
template <bool ISO, bool SINGLE>
__global__ void __launch_bounds__(256) riccati32_kernel(SolveGeom g, const float *__restrict__ lv32,
                                                        const int *__restrict__ slot_of_step,
                                                        const uint32_t *__restrict__ modes,
                                                        const float2 *__restrict__ q0spec,
                                                        float *__restrict__ scratch, float2 *__restrict__ Xp,
                                                        float2 *__restrict__ Xq, float ax, float ay, int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    float *s_lv = (float *)smem_raw;
    const int L = g.nz - 1;
    int *s_slot = (int *)(s_lv + (size_t)L * BLDFM_LV32);
    if (L > 0) {
        if (!bulk_load_to_smem(s_lv, lv32, (uint32_t)((size_t)L * BLDFM_LV32 * sizeof(float)), &bar, err)) return;
    }
    for (int i = threadIdx.x; i < g.nz; i += blockDim.x) s_slot[i] = slot_of_step[i];
    __syncthreads();
    const int64_t ns = g.nsolved;
    if (SINGLE) {
        // two modes per thread (m and m + blockDim.x) in the lanes of packed f32x2 operations
        const int64_t step = 2 * (int64_t)gridDim.x * blockDim.x;
        for (int64_t m = 2 * (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < ns; m += step) {
            const int64_t mb = m + blockDim.x < ns ? m + blockDim.x : -1;
            ricc_mode_pair<ISO>(g, s_lv, modes, q0spec, Xp, Xq, ax, ay, m, mb);
        }
    } else {
        for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < ns; m += (int64_t)gridDim.x * blockDim.x)
            ricc_mode<ISO, SINGLE>(g, s_lv, s_slot, modes, q0spec, scratch, Xp, Xq, ax, ay, m);
    }
}

// ---------------------------------------------------------------------------
// FP64 invariant-imbedding sweep (accurate mode)
// ---------------------------------------------------------------------------
// The FP32 kernel's recursion in FP64 with exact division: the solution of the
// reference's discrete problem without the shooting method's cancellation.
__device__ __forceinline__ double2 csqrt_d(double2 w)
{
    const double x = w.x, y = w.y;
    const double t = sqrt(0.5 * (fabs(x) + hypot(x, y)));
    if (t == 0.0) return make_double2(0.0, 0.0);
    if (x >= 0.0) return make_double2(t, y / (2.0 * t));
    return make_double2(fabs(y) / (2.0 * t), copysign(t, y));
}

__device__ __forceinline__ double2 dc_mul(double2 a, double2 b)
{
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// 1/x for a positive normal x: the approximate hardware reciprocal refined by
// two Newton-Raphson steps for f(y) = 1/y - x (y <- y + y (1 - x y)), each of
// which doubles the number of correct bits, to within an ulp or two of the
// rounded quotient.  Faster than the IEEE division, whose exact rounding the
// accurate FP64 mode does not need.
__device__ __forceinline__ double rcp_newton(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

// Per-level products of the accurate FP64 sweep's step coefficients
// (A = S1 H2, B1 = S2 H3, C1 = S4 H3), formed once per CTA in shared memory
#define RICC64_K 3
#define RICC64_SMEM (200 * 1024)  // dynamic shared memory the kernel is set up for

template <bool SINGLE>
__global__ void __launch_bounds__(128) riccati64_kernel(SolveGeom g, const double *__restrict__ lvtab,
                                                        const int *__restrict__ slot_of_step,
                                                        const uint32_t *__restrict__ modes,
                                                        const double2 *__restrict__ q0spec,
                                                        double *__restrict__ scratch, double2 *__restrict__ Xp,
                                                        double2 *__restrict__ Xq, int *err, bool kprod)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    double *s_lv = (double *)smem_raw;
    const int L = g.nz - 1;
    int *s_slot = (int *)(s_lv + (size_t)L * BLDFM_LV64);
    if (L > 0) {
        if (!bulk_load_to_smem(s_lv, lvtab, (uint32_t)((size_t)L * BLDFM_LV64 * sizeof(double)), &bar, err))
            return;
    }
    for (int i = threadIdx.x; i < g.nz; i += blockDim.x) s_slot[i] = slot_of_step[i];
    // after the slot map, 8-byte aligned
    double *s_k = (double *)(smem_raw + ((((size_t)L * BLDFM_LV64 * sizeof(double) + (size_t)g.nz * sizeof(int)) + 7) &
                                         ~(size_t)7));
    __syncthreads();
    for (int i = threadIdx.x; kprod && i < L; i += blockDim.x) {
        const double *lv = s_lv + (size_t)i * BLDFM_LV64;
        s_k[RICC64_K * i] = lv[LV_S1] * lv[LV_H2];
        s_k[RICC64_K * i + 1] = lv[LV_S2] * lv[LV_H3];
        s_k[RICC64_K * i + 2] = lv[LV_S4] * lv[LV_H3];
    }
    __syncthreads();
    const int jmax = g.jmax;
    const int64_t ns = g.nsolved;
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < ns; m += (int64_t)gridDim.x * blockDim.x) {
        int r, c;
        bool paired;
        unpack_mode(modes[m], r, c, paired);
        const int kx = freq_of_index(c, g.nlx), ky = freq_of_index(r, g.nly);
        const double lx = wavenumber(kx, g.valx, g.lx_scale), ly = wavenumber(ky, g.valy, g.ly_scale);
        const double lx2 = lx * lx, ly2 = ly * ly;
        const double2 eg = csqrt_d(make_double2(fma(g.kxk_top, lx2, g.kyk_top * ly2), fma(g.uk_top, lx, g.vk_top * ly)));
        const double2 ke = make_double2(g.kz_top * eg.x, g.kz_top * eg.y);
        const double kn = 1.0 / fma(ke.x, ke.x, ke.y * ke.y);
        double2 R = make_double2(ke.x * kn, -ke.y * kn);
        double2 Q = make_double2(1.0, 0.0), Rj = R;
        int E = 0;
        auto coef = [&](int i, double2 &a, double2 &b, double2 &cc) {
            const double *lv = s_lv + (size_t)i * BLDFM_LV64;
            const double Tr = -fma(lv[LV_KX], lx2, lv[LV_KY] * ly2);
            const double Ti = -fma(lv[LV_U], lx, lv[LV_V] * ly);
            double A, B1, C1;
            if (kprod) {  // the same for every thread of the launch
                const double *k = s_k + RICC64_K * i;
                A = k[0];
                B1 = k[1];
                C1 = k[2];
            } else {
                A = lv[LV_S1] * lv[LV_H2];
                B1 = lv[LV_S2] * lv[LV_H3];
                C1 = lv[LV_S4] * lv[LV_H3];
            }
            a = make_double2(fma(-A, Tr, 1.0), -A * Ti);
            b = make_double2(fma(-B1, Tr, lv[LV_S3]), -B1 * Ti);
            const double t2r = fma(Tr, Tr, -Ti * Ti), t2i = 2.0 * Tr * Ti;
            cc = make_double2(fma(-C1, t2r, lv[LV_H] * Tr), fma(-C1, t2i, lv[LV_H] * Ti));
        };
        auto step = [&](const double2 a, const double2 b, const double2 cc) {
            const double2 cR = dc_mul(cc, R);
            const double2 D = make_double2(a.x - cR.x, a.y - cR.y);
            const double2 N = make_double2(fma(a.x, R.x, fma(-a.y, R.y, -b.x)), fma(a.x, R.y, fma(a.y, R.x, -b.y)));
            const double dinv = rcp_newton(fma(D.x, D.x, D.y * D.y));
            R = make_double2(fma(N.x, D.x, N.y * D.y) * dinv, fma(N.y, D.x, -N.x * D.y) * dinv);
        };
        int i = L - 1;
        for (; i >= jmax; --i) {
            double2 a, b, cc;
            coef(i, a, b, cc);
            step(a, b, cc);
        }
        Rj = R;
        if (!SINGLE) {
            const int s = s_slot[jmax];
            double *o = scratch + (size_t)s * 5 * ns + m;
            o[0] = R.x;
            o[ns] = R.y;
            o[2 * ns] = 1.0;
            o[3 * ns] = 0.0;
            o[4 * ns] = 0.0;
        }
        for (; i >= 0; --i) {
            double2 a, b, cc;
            coef(i, a, b, cc);
            step(a, b, cc);
            Q = dc_mul(Q, make_double2(fma(cc.x, R.x, fma(-cc.y, R.y, a.x)), fma(cc.x, R.y, fma(cc.y, R.x, a.y))));
            if ((i & 15) == 0) {
                int e;
                frexp(fmax(fabs(Q.x), fabs(Q.y)), &e);
                Q.x = ldexp(Q.x, -e);
                Q.y = ldexp(Q.y, -e);
                E += e;
            }
            if (!SINGLE) {
                const int s = s_slot[i];
                if (s >= 0) {
                    double *o = scratch + (size_t)s * 5 * ns + m;
                    o[0] = R.x;
                    o[ns] = R.y;
                    o[2 * ns] = Q.x;
                    o[3 * ns] = Q.y;
                    o[4 * ns] = (double)E;
                }
            }
        }
        const double2 q0 = q0spec ? q0spec[(size_t)c * g.nly + r] : make_double2(g.q0dc_fp, 0.0);
        double2 sh = make_double2(1.0, 0.0);
        if (g.do_shift) {
            const double th = lx * g.sx + ly * g.sy;
            double sn, cs;
            sincos(th, &sn, &cs);
            sh = make_double2(cs, sn);
        }
        const int rm = paired ? index_of_freq(-ky, g.nly) : 0;
        const int cm = paired ? index_of_freq(-kx, g.nlx) : 0;
        for (int s = 0; s < (SINGLE ? 1 : g.nsnap); ++s) {
            double2 ratio;
            if (SINGLE) {
                ratio = make_double2(ldexp(Q.x, E), ldexp(Q.y, E));
            } else {
                const double *o = scratch + (size_t)s * 5 * ns + m;
                Rj = make_double2(o[0], o[ns]);
                const double2 Qj = make_double2(o[2 * ns], o[3 * ns]);
                const int Ej = (int)o[4 * ns];
                const double qn = fma(Qj.x, Qj.x, Qj.y * Qj.y);
                ratio = make_double2(0.0, 0.0);
                if (qn > 0.0) {
                    const double scl = ldexp(1.0 / qn, E - Ej);
                    ratio = make_double2(fma(Q.x, Qj.x, Q.y * Qj.y) * scl, fma(Q.y, Qj.x, -Q.x * Qj.y) * scl);
                }
            }
            double2 q = dc_mul(q0, ratio);
            double2 p = dc_mul(Rj, q);
            if (g.precision == 0) {
                p = round_c64(p);
                q = round_c64(q);
            }
            if (g.do_shift) {
                p = dc_mul(p, sh);
                q = dc_mul(q, sh);
            }
            Xp[spec_idx(g, s, r, c)] = p;
            Xq[spec_idx(g, s, r, c)] = q;
            if (paired) {
                Xp[spec_idx(g, s, rm, cm)] = make_double2(p.x, -p.y);
                Xq[spec_idx(g, s, rm, cm)] = make_double2(q.x, -q.y);
            }
        }
    }
}

cudaError_t launch_riccati64(const SolveGeom &g, const double *lvtab, const int *slot, const uint32_t *modes,
                             const double2 *q0spec, double *scratch, double2 *Xp, double2 *Xq, int *err, int nsm,
                             cudaStream_t st)
{
    if (g.nsnap < 1 || g.nsolved == 0) return cudaSuccess;
    // level table, slot map, then (8-byte aligned) the per-level products
    // when they fit in the shared memory the kernel is set up for
    const size_t base = (((size_t)(g.nz - 1) * BLDFM_LV64 * sizeof(double) + (size_t)g.nz * sizeof(int) + 7) &
                         ~(size_t)7) +
                        16;
    const size_t withk = base + (size_t)(g.nz - 1) * RICC64_K * sizeof(double);
    const bool kprod = withk <= RICC64_SMEM;
    const size_t smem = kprod ? withk : base;
    const int threads = 128;
    int64_t blocks = (g.nsolved + threads - 1) / threads;
    if (blocks > 64LL * nsm) blocks = 64LL * nsm;
    if (g.nsnap == 1)
        riccati64_kernel<true><<<(unsigned)blocks, threads, smem, st>>>(g, lvtab, slot, modes, q0spec, scratch, Xp,
                                                                        Xq, err, kprod);
    else
        riccati64_kernel<false><<<(unsigned)blocks, threads, smem, st>>>(g, lvtab, slot, modes, q0spec, scratch, Xp,
                                                                         Xq, err, kprod);
    return LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// FFT passes
// ---------------------------------------------------------------------------
// fwd_rows: lines are source rows y < ny, length nxe, input at offset px.
// Output A[c][y] (c < nlx truncated columns) scaled by 1/nxe.
template <typename R>
__global__ void __launch_bounds__(256) fwd_rows_kernel(SolveGeom g, FftPlan pl, const typename cvec<R>::T *__restrict__ tw,
                                                       const double *__restrict__ src, typename cvec<R>::T *__restrict__ A,
                                                       int rows_per_cta)
{
    typedef typename cvec<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = pl.n;
    C *bufA = (C *)smem_raw;
    C *bufB = bufA + (size_t)rows_per_cta * n;
    const int y0 = blockIdx.x * rows_per_cta;
    const int nl = min(rows_per_cta, g.ny - y0);
    for (int i = threadIdx.x; i < nl * n; i += blockDim.x) {
        const int l = i / n, x = i - l * n;
        const int xs = x - g.px;
        R v = (xs >= 0 && xs < g.nx) ? (R)src[(size_t)(y0 + l) * g.nx + xs] : (R)0;
        bufA[i] = cx_make<C>(v, 0.0);
    }
    C *res = fft_run<C>(bufA, bufB, pl, nl, tw, -1);
    const R sc = (R)g.inv_nxe;
    for (int i = threadIdx.x; i < nl * g.nlx; i += blockDim.x) {
        const int c = i / nl, l = i - c * nl;
        const int kx = freq_of_index(c, g.nlx);
        const int pos = kx >= 0 ? kx : kx + n;
        C v = res[(size_t)l * n + pos];
        v.x *= sc;
        v.y *= sc;
        A[(size_t)c * g.ny + y0 + l] = v;
    }
}

// fwd_cols: lines are truncated columns c < nlx, length nye, input A[c][y] at
// offset py.  Output Q0[c][r] (r < nly) scaled by 1/nye.
template <typename R>
__global__ void __launch_bounds__(256) fwd_cols_kernel(SolveGeom g, FftPlan pl, const typename cvec<R>::T *__restrict__ tw,
                                                       const typename cvec<R>::T *__restrict__ A,
                                                       typename cvec<R>::T *__restrict__ Q0, int cols_per_cta)
{
    typedef typename cvec<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = pl.n;
    C *bufA = (C *)smem_raw;
    C *bufB = bufA + (size_t)cols_per_cta * n;
    const int c0 = blockIdx.x * cols_per_cta;
    const int nl = min(cols_per_cta, g.nlx - c0);
    for (int i = threadIdx.x; i < nl * n; i += blockDim.x) {
        const int l = i / n, y = i - l * n;
        const int ys = y - g.py;
        bufA[i] = (ys >= 0 && ys < g.ny) ? A[(size_t)(c0 + l) * g.ny + ys] : cx_make<C>(0.0, 0.0);
    }
    C *res = fft_run<C>(bufA, bufB, pl, nl, tw, -1);
    const R sc = (R)g.inv_nye;
    for (int i = threadIdx.x; i < nl * g.nly; i += blockDim.x) {
        const int l = i / g.nly, r = i - l * g.nly;
        const int ky = freq_of_index(r, g.nly);
        const int pos = ky >= 0 ? ky : ky + n;
        C v = res[(size_t)l * n + pos];
        v.x *= sc;
        v.y *= sc;
        Q0[(size_t)(c0 + l) * g.nly + r] = v;
    }
}

// out_cols: cols_per_cta band columns per CTA (blockIdx.x), one level (blockIdx.y).
template <typename R>
__global__ void __launch_bounds__(256) out_cols_kernel(SolveGeom g, FftPlan pl, const typename cvec<R>::T *__restrict__ tw,
                                                       const int4 *__restrict__ xband,
                                                       const typename cvec<R>::T *__restrict__ Xp,
                                                       const typename cvec<R>::T *__restrict__ Xq,
                                                       const double2 *__restrict__ dc,
                                                       typename cvec<R>::T *__restrict__ Cout, int cols_per_cta,
                                                       int *err)
{
    typedef typename cvec<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if constexpr (sizeof(R) == 4) {
        // FP32 spectra are Hermitian-complete: the staged gather
        __shared__ uint64_t bar;
        if (threadIdx.x == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(&bar)),
                         "r"(1)
                         : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncthreads();
        if (!out_col_lines_staged(g, pl, tw, xband, Xp, Xq, dc, Cout, blockIdx.x * cols_per_cta, cols_per_cta,
                                  blockIdx.y, (C *)smem_raw, &bar) &&
            threadIdx.x == 0 && err)
            atomicExch(err, BLDFM_ERR_TIMEOUT_DEV);
    } else {
        out_col_lines<R>(g, pl, tw, xband, Xp, Xq, dc, Cout, blockIdx.x * cols_per_cta, cols_per_cta, blockIdx.y,
                         (C *)smem_raw);
    }
}

// out_rows: rows_per_cta output rows per CTA, one level (blockIdx.y).
template <typename R>
__global__ void __launch_bounds__(256) out_rows_kernel(SolveGeom g, FftPlan pl, const typename cvec<R>::T *__restrict__ tw,
                                                       const int4 *__restrict__ xband,
                                                       const typename cvec<R>::T *__restrict__ Cin,
                                                       double *__restrict__ conc, double *__restrict__ flx,
                                                       int rows_per_cta, int *err)
{
    typedef typename cvec<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    out_row_lines<R>(g, pl, tw, xband, Cin, conc, flx, blockIdx.x * rows_per_cta, rows_per_cta, blockIdx.y,
                     (C *)smem_raw, err);
}

// ---------------------------------------------------------------------------
// small utility kernels
// ---------------------------------------------------------------------------
// twiddle table tw[m] = exp(-2 pi i m / n) converted from the FP64 table
__global__ void tw_to_float_kernel(const double2 *__restrict__ src, float2 *__restrict__ dst, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_float2((float)src[i].x, (float)src[i].y);
}

__global__ void spec_to_float_kernel(const double2 *__restrict__ src, float2 *__restrict__ dst, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_float2((float)src[i].x, (float)src[i].y);
}

// non-finite detector over the outputs
__global__ void nonfinite_kernel(const double *__restrict__ a, const double *__restrict__ b, int64_t n, int *flag)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!isfinite(a[i]) || !isfinite(b[i])) {
            atomicExch(flag, 1);
            return;
        }
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------


cudaError_t launch_sweep64(const SolveGeom &g, const double *lvtab, const int *slot, const uint32_t *modes,
                           const double2 *q0spec, double2 *snap, double2 *top, int *err, int nsm, cudaStream_t st)
{
    const int L = g.nz - 1;
    const size_t smem = (size_t)L * BLDFM_LV64 * sizeof(double) + (size_t)g.nz * sizeof(int) + 16;
    static uint64_t attr = 0;
    if (first_on_device(attr))
        cudaFuncSetAttribute(sweep64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    const int threads = 128;
    int64_t blocks = (g.nsolved + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
    if (blocks > 64LL * nsm) blocks = 64LL * nsm;
    sweep64_kernel<<<(unsigned)blocks, threads, smem, st>>>(g, lvtab, slot, modes, q0spec, snap, top, err);
    return LAUNCH_CHECK();
}

cudaError_t launch_combine64(const SolveGeom &g, const uint32_t *modes, const double2 *eig, const double2 *snap,
                             const double2 *top, double2 *Xp, double2 *Xq, cudaStream_t st)
{
    if (g.nsolved == 0) return cudaSuccess;
    const int threads = 256;
    const unsigned blocks = (unsigned)((g.nsolved + threads - 1) / threads);
    combine64_kernel<<<blocks, threads, 0, st>>>(g, modes, eig, snap, top, Xp, Xq);
    return LAUNCH_CHECK();
}

cudaError_t launch_trapezoid64(const SolveGeom &g, const double *lvtab, const int *slot, const double2 *q0spec,
                               double p000, double2 *dc, cudaStream_t st)
{
    const size_t smem = (size_t)(g.nz > 1 ? g.nz - 1 : 1) * sizeof(double2) + (size_t)g.nz * sizeof(int);
    trapezoid_kernel<double2><<<1, 256, smem, st>>>(g, lvtab, slot, q0spec, p000, dc, nullptr);
    return LAUNCH_CHECK();
}

// FP64 partial sums of the source field: CTA b of DC_PARTS sums its slice in a
// fixed order (deterministic), thread sums then a shared-memory tree
__global__ void __launch_bounds__(256) dc_partial_kernel(const double *__restrict__ src, int64_t n,
                                                         double *__restrict__ dcp)
{
    __shared__ double red[256];
    const int64_t chunk = (n + DC_PARTS - 1) / DC_PARTS;
    const int64_t b0 = (int64_t)blockIdx.x * chunk, b1 = b0 + chunk < n ? b0 + chunk : n;
    double acc = 0.0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) acc += src[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) dcp[blockIdx.x] = red[0];
}

cudaError_t launch_trapezoid32(const SolveGeom &g, const double *lvtab, const int *slot, const float2 *q0spec,
                               double p000, double2 *dc, cudaStream_t st, const double *src, double *dcp)
{
    const size_t smem = (size_t)(g.nz > 1 ? g.nz - 1 : 1) * sizeof(double2) + (size_t)g.nz * sizeof(int);
    const bool exact = src && dcp;
    if (exact) dc_partial_kernel<<<DC_PARTS, 256, 0, st>>>(src, (int64_t)g.nx * g.ny, dcp);
    trapezoid_kernel<float2><<<1, 256, smem, st>>>(g, lvtab, slot, q0spec, p000, dc, exact ? dcp : nullptr);
    return LAUNCH_CHECK();
}

cudaError_t launch_analytic64(const SolveGeom &g, const uint32_t *modes, const double2 *eig, const double2 *q0spec,
                              double p000, double kzinv, double hlev, double2 *Xp, double2 *Xq, double2 *dc,
                              cudaStream_t st)
{
    if (g.nsolved > 0) {
        const int threads = 256;
        const unsigned blocks = (unsigned)((g.nsolved + threads - 1) / threads);
        analytic64_kernel<<<blocks, threads, 0, st>>>(g, modes, eig, q0spec, kzinv, hlev, Xp, Xq);
    }
    if (q0spec) analytic_dc_kernel<<<1, 32, 0, st>>>(g, q0spec, p000, kzinv, hlev, dc);
    return LAUNCH_CHECK();
}

cudaError_t launch_riccati32(const SolveGeom &g, const float *lv32, const int *slot, const uint32_t *modes,
                             const float2 *q0spec, float *scratch, float2 *Xp, float2 *Xq, float ax, float ay,
                             int *err, int nsm, int threads, cudaStream_t st)
{
    const int L = g.nz - 1;
    const size_t smem = (size_t)L * BLDFM_LV32 * sizeof(float) + (size_t)g.nz * sizeof(int) + 16;
    static uint64_t attr = 0;
    if (first_on_device(attr)) {
        cudaFuncSetAttribute(riccati32_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(riccati32_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(riccati32_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(riccati32_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    }
    if (threads <= 0) threads = 256;
    const int64_t per_thread = g.nsnap == 1 ? 2 : 1;  // modes per thread
    int64_t blocks = (g.nsolved + per_thread * threads - 1) / (per_thread * threads);
    if (blocks < 1) blocks = 1;
    if (blocks > 64LL * nsm) blocks = 64LL * nsm;
    const bool single = g.nsnap == 1;
    if (g.nsnap < 1) return cudaSuccess;  // no output level inside the grid: spectra stay zero
    if (g.iso) {
        if (single)
            riccati32_kernel<true, true><<<(unsigned)blocks, threads, smem, st>>>(g, lv32, slot, modes, q0spec, scratch,
                                                                                Xp, Xq, ax, ay, err);
        else
            riccati32_kernel<true, false><<<(unsigned)blocks, threads, smem, st>>>(g, lv32, slot, modes, q0spec,
                                                                                 scratch, Xp, Xq, ax, ay, err);
    } else {
        if (single)
            riccati32_kernel<false, true><<<(unsigned)blocks, threads, smem, st>>>(g, lv32, slot, modes, q0spec,
                                                                                 scratch, Xp, Xq, ax, ay, err);
        else
            riccati32_kernel<false, false><<<(unsigned)blocks, threads, smem, st>>>(g, lv32, slot, modes, q0spec,
                                                                                  scratch, Xp, Xq, ax, ay, err);
    }
    return LAUNCH_CHECK();
}

static int lines_per_cta(int n, size_t elem, size_t budget)
{
    int l = (int)(budget / (2 * (size_t)n * elem));
    if (l < 1) l = 1;
    if (l > 8) l = 8;
    return l;
}

template <typename R>
static void set_fft_smem_attr()
{
    static uint64_t done = 0;
    if (!first_on_device(done)) return;
    cudaFuncSetAttribute(fwd_rows_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(fwd_cols_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(out_cols_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(out_rows_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

template <typename R>
cudaError_t launch_forward_fft(const SolveGeom &g, const FftPlan &plx, const FftPlan &ply,
                               const typename cvec<R>::T *twx, const typename cvec<R>::T *twy, const double *src,
                               typename cvec<R>::T *A, typename cvec<R>::T *Q0, cudaStream_t st)
{
    typedef typename cvec<R>::T C;
    set_fft_smem_attr<R>();
    if (g.ny <= 0 || g.nlx <= 0) return cudaSuccess;
    const size_t budget = 96 * 1024;
    int rpc = lines_per_cta(plx.n, sizeof(C), budget);
    fwd_rows_kernel<R><<<(g.ny + rpc - 1) / rpc, 256, 2 * (size_t)rpc * plx.n * sizeof(C), st>>>(g, plx, twx, src, A,
                                                                                                  rpc);
    int cpc = lines_per_cta(ply.n, sizeof(C), budget);
    fwd_cols_kernel<R><<<(g.nlx + cpc - 1) / cpc, 256, 2 * (size_t)cpc * ply.n * sizeof(C), st>>>(g, ply, twy, A, Q0,
                                                                                                   cpc);
    return LAUNCH_CHECK();
}

template <typename R>
cudaError_t launch_output_fft(const SolveGeom &g, const FftPlan &plx, const FftPlan &ply,
                              const typename cvec<R>::T *twx, const typename cvec<R>::T *twy, const int4 *xband,
                              const typename cvec<R>::T *Xp, const typename cvec<R>::T *Xq, const double2 *dc,
                              typename cvec<R>::T *Cbuf, double *conc, double *flx, int *err, cudaStream_t st)
{
    typedef typename cvec<R>::T C;
    set_fft_smem_attr<R>();
    if (g.nbx <= 0 || g.out_ny <= 0 || g.out_nx <= 0 || g.nlvls <= 0) return cudaSuccess;
    // lines per CTA: as many as shared memory allows, but at least two CTAs
    // per SM over the launch (a single footprint has few lines)
    int dev = 0, nsm = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int cpc = out_cols_per_cta(ply.n, sizeof(C));
    while (cpc > 1 && (int64_t)((g.nbx + cpc - 1) / cpc) * g.nlvls < 2 * (int64_t)nsm) cpc >>= 1;
    dim3 gc((g.nbx + cpc - 1) / cpc, g.nlvls);
    out_cols_kernel<R><<<gc, 256, (2 * (size_t)cpc + 1) * ply.n * sizeof(C), st>>>(g, ply, twy, xband, Xp, Xq, dc,
                                                                                   Cbuf, cpc, err);
    // two rows per CTA in FP32, one in FP64, bounded by shared memory and by
    // the same two CTAs per SM
    int rpc = sizeof(C) == 8 ? 2 : 1;
    while (rpc > 1 && (2 * (size_t)rpc + 1) * plx.n * sizeof(C) > 190 * 1024) --rpc;
    while (rpc > 1 && (int64_t)((g.out_ny + rpc - 1) / rpc) * g.nlvls < 2 * (int64_t)nsm) --rpc;
    dim3 gr((g.out_ny + rpc - 1) / rpc, g.nlvls);
    out_rows_kernel<R><<<gr, 256, (2 * (size_t)rpc + 1) * plx.n * sizeof(C), st>>>(g, plx, twx, xband, Cbuf, conc,
                                                                                   flx, rpc, err);
    return LAUNCH_CHECK();
}

template cudaError_t launch_forward_fft<double>(const SolveGeom &, const FftPlan &, const FftPlan &, const double2 *,
                                                const double2 *, const double *, double2 *, double2 *, cudaStream_t);
template cudaError_t launch_forward_fft<float>(const SolveGeom &, const FftPlan &, const FftPlan &, const float2 *,
                                               const float2 *, const double *, float2 *, float2 *, cudaStream_t);
template cudaError_t launch_output_fft<double>(const SolveGeom &, const FftPlan &, const FftPlan &, const double2 *,
                                               const double2 *, const int4 *, const double2 *, const double2 *,
                                               const double2 *, double2 *, double *, double *, int *, cudaStream_t);
template cudaError_t launch_output_fft<float>(const SolveGeom &, const FftPlan &, const FftPlan &, const float2 *,
                                              const float2 *, const int4 *, const float2 *, const float2 *,
                                              const double2 *, float2 *, double *, double *, int *, cudaStream_t);

cudaError_t launch_tw_to_float(const double2 *src, float2 *dst, int n, cudaStream_t st)
{
    tw_to_float_kernel<<<(n + 255) / 256, 256, 0, st>>>(src, dst, n);
    return LAUNCH_CHECK();
}

cudaError_t launch_spec_to_float(const double2 *src, float2 *dst, int64_t n, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    spec_to_float_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst, n);
    return LAUNCH_CHECK();
}

cudaError_t launch_nonfinite(const double *a, const double *b, int64_t n, int *flag, int nsm, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 4LL * nsm) blocks = 4LL * nsm;
    nonfinite_kernel<<<(unsigned)blocks, 256, 0, st>>>(a, b, n, flag);
    return LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// FMA throughput probe: independent FMA chains per thread, CUDA-event timed.
// Measures the FP32 / FP64 pipe peaks that bound the sweep kernels.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) fma_peak_kernel(T *out, int iters, T b, T c)
{
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = (T)(threadIdx.x + k) * (T)1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == (T)-12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Packed FP32: eight independent f32x2 FMA chains per thread.
__global__ void __launch_bounds__(256) fma2_peak_kernel(float *out, int iters, float b, float c)
{
    float2 a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = make_float2((float)(threadIdx.x + k) * 1e-3f, (float)(threadIdx.x + 2 * k) * 1e-3f);
    const float2 b2 = make_float2(b, b), c2 = make_float2(c, c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = __ffma2_rn(a[k], b2, c2);
    }
    float s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k].x + a[k].y;
    if (s == -12345.678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t run_fma_peak(int kind, int nsm, cudaStream_t st, double *flops_per_s)
{
    const bool fp64 = kind == 1;
    const int threads = 256, blocks = nsm * 8;
    const int iters = fp64 ? 2048 : (kind == 2 ? 32768 : 65536);
    void *out = nullptr;
    cudaError_t e = cudaMalloc(&out, (size_t)threads * blocks * 8);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(a, st);
        if (fp64)
            fma_peak_kernel<double><<<blocks, threads, 0, st>>>((double *)out, iters, 0.999999, 1e-7);
        else if (kind == 2)
            fma2_peak_kernel<<<blocks, threads, 0, st>>>((float *)out, iters, 0.999999f, 1e-7f);
        else
            fma_peak_kernel<float><<<blocks, threads, 0, st>>>((float *)out, iters, 0.999999f, 1e-7f);
        cudaEventRecord(b, st);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best) best = ms;
    }
    e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    *flops_per_s = 2.0 * 8.0 * (kind == 2 ? 2 : 1) * iters * (double)threads * blocks / (best * 1e-3);
    return e;
}

// Shared-memory limits of every kernel, set once per device before any launch
// (and so before any stream capture).
void prepare_kernel_attributes()
{
    set_fft_smem_attr<double>();
    set_fft_smem_attr<float>();
    cudaFuncSetAttribute(sweep64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(riccati64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, RICC64_SMEM);
    cudaFuncSetAttribute(riccati64_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, RICC64_SMEM);
    cudaFuncSetAttribute(riccati32_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(riccati32_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(riccati32_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(riccati32_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}
