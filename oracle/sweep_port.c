/*
 * CPU oracle -- test infrastructure, not product code.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and
 * its --impl reference arm) load this file's library, and only as the test
 * oracle or as the timed CPU baseline.  The GPU product path never calls it.
 *
 * C restatement of the reference's linear-shooting sweep and the shooting
 * combination:
 *   - ivp_solver                      src/bldfm/solver.py:307-374
 *   - the two IVP calls               src/bldfm/solver.py:220-226
 *   - alpha and the level combination src/bldfm/solver.py:228-235
 *
 * Rounding model.  Every floating-point operation below is the one numpy
 * performs for the reference's array expressions, in the same order, so the
 * results are bit-identical to the reference's numpy evaluation:
 *   - complex128 multiply:  re = fma(ar, br, -(ai*bi)),  im = fma(ar, bi, ai*br)
 *     (numpy's SIMD complex multiply on x86-64; verified bitwise on 1e6
 *     random pairs);
 *   - complex128 divide:    Smith's method with a reciprocal scale;
 *   - real scalar x complex array is exact componentwise rounding;
 *   - scalar powers (dz**2, dz**3, (1/Kz)**2) come from libm pow() via the
 *     caller's level table, as numpy's scalar ** does;
 *   - eigval (complex sqrt) comes from the caller, computed by libm csqrt.
 * The file must be compiled with -ffp-contract=off so that the compiler does
 * not fuse any other multiply-add pair.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    double r, i;
} cplx;

static inline cplx cmul(cplx a, cplx b)
{
    cplx o;
    o.r = fma(a.r, b.r, -(a.i * b.i));
    o.i = fma(a.r, b.i, a.i * b.r);
    return o;
}

static inline cplx cadd(cplx a, cplx b)
{
    cplx o = {a.r + b.r, a.i + b.i};
    return o;
}

static inline cplx csub(cplx a, cplx b)
{
    cplx o = {a.r - b.r, a.i - b.i};
    return o;
}

/* Smith's algorithm (R. L. Smith, CACM 5(8), 1962), reciprocal-scale form. */
static inline cplx cdiv(cplx a, cplx b)
{
    cplx o;
    if (fabs(b.r) >= fabs(b.i)) {
        double rat = b.i / b.r;
        double scl = 1.0 / (b.r + b.i * rat);
        o.r = (a.r + a.i * rat) * scl;
        o.i = (a.i - a.r * rat) * scl;
    } else {
        double rat = b.r / b.i;
        double scl = 1.0 / (b.i + b.r * rat);
        o.r = (a.r * rat + a.i) * scl;
        o.i = (a.i * rat - a.r) * scl;
    }
    return o;
}

/* Level table row layout (12 doubles per sweep step i = 0..nz-2). */
enum {
    LV_KX = 0,   /* Kx[i]                          */
    LV_KY,       /* Ky[i]                          */
    LV_U,        /* u[i]                           */
    LV_V,        /* v[i]                           */
    LV_S1,       /* 0.5 * (1/Kz[i])                */
    LV_H2,       /* pow(dz[i], 2)                  */
    LV_S2,       /* (1/6) * pow(1/Kz[i], 2)        */
    LV_H3,       /* pow(dz[i], 3)                  */
    LV_S3,       /* (-(1/Kz[i])) * dz[i]           */
    LV_S4,       /* (1/6) * (1/Kz[i])              */
    LV_H,        /* dz[i]                          */
    LV_PAD,
    LV_STRIDE
};

/*
 * One mode, both IVPs, snapshots at the snapshot steps, then the combination.
 *   snap_of_step[i] = slot index (0..nsnap-1) when step i is snapshotted
 *                     before stepping, else -1; i ranges over 0..nz-1 and
 *                     slot of step nz-1 is taken after the loop.
 * Writes p_out[s], q_out[s] for s < nsnap.
 */
static void sweep_mode(double lx, double ly, cplx q0, cplx eig, double kz_top,
                       int nz, const double *lv, const int *snap_of_step,
                       int nsnap, cplx *p_out, cplx *q_out, cplx *sp1,
                       cplx *sq1, cplx *sp2, cplx *sq2)
{
    const double lx2 = lx * lx, ly2 = ly * ly;
    cplx p1 = {1.0, 0.0}, q1 = {0.0, 0.0};
    cplx p2 = {0.0, 0.0}, q2 = q0;
    for (int i = 0; i < nz - 1; ++i) {
        int s = snap_of_step[i];
        if (s >= 0) {
            sp1[s] = p1; sq1[s] = q1; sp2[s] = p2; sq2[s] = q2;
        }
        const double *L = lv + (size_t)i * LV_STRIDE;
        /* T = -(Kx*Lx^2 + Ky*Ly^2) - 1j*u*Lx - 1j*v*Ly   (solver.py:357) */
        cplx T;
        T.r = -(L[LV_KX] * lx2 + L[LV_KY] * ly2);
        T.i = -(L[LV_U] * lx) - L[LV_V] * ly;
        /* a = d = 1 - 0.5*Kzinv*T*dz**2                   (solver.py:361,364) */
        cplx a;
        a.r = 1.0 - (L[LV_S1] * T.r) * L[LV_H2];
        a.i = 0.0 - (L[LV_S1] * T.i) * L[LV_H2];
        /* b = -Kzinv*dz - 1/6*Kzinv**2*T*dz**3             (solver.py:362) */
        cplx b;
        b.r = L[LV_S3] - (L[LV_S2] * T.r) * L[LV_H3];
        b.i = 0.0 - (L[LV_S2] * T.i) * L[LV_H3];
        /* c = T*dz - 1/6*Kzinv*T**2*dz**3                  (solver.py:363) */
        cplx T2 = cmul(T, T);
        cplx c;
        c.r = T.r * L[LV_H] - (L[LV_S4] * T2.r) * L[LV_H3];
        c.i = T.i * L[LV_H] - (L[LV_S4] * T2.i) * L[LV_H3];
        /* (p, q) <- (a p + b q, c p + d q)                  (solver.py:366-368) */
        cplx np1 = cadd(cmul(a, p1), cmul(b, q1));
        cplx nq1 = cadd(cmul(c, p1), cmul(a, q1));
        cplx np2 = cadd(cmul(a, p2), cmul(b, q2));
        cplx nq2 = cadd(cmul(c, p2), cmul(a, q2));
        p1 = np1; q1 = nq1; p2 = np2; q2 = nq2;
    }
    {
        int s = snap_of_step[nz - 1];
        if (s >= 0) {
            sp1[s] = p1; sq1[s] = q1; sp2[s] = p2; sq2[s] = q2;
        }
    }
    /* alpha = -(q2 - Kz*eig*p2) / (q1 - Kz*eig*p1)      (solver.py:228-230) */
    cplx keig = {kz_top * eig.r, kz_top * eig.i};
    cplx num = csub(q2, cmul(keig, p2));
    cplx den = csub(q1, cmul(keig, p1));
    num.r = -num.r;
    num.i = -num.i;
    cplx alpha = cdiv(num, den);
    /* p = alpha*p1 + p2, q = alpha*q1 + q2 at each level (solver.py:233-235) */
    for (int s = 0; s < nsnap; ++s) {
        p_out[s] = cadd(cmul(alpha, sp1[s]), sp2[s]);
        q_out[s] = cadd(cmul(alpha, sq1[s]), sq2[s]);
    }
}

/*
 * Solve all modes.
 *   lx, ly:   (nmodes,) wavenumbers of the masked modes (reference Lx[msk])
 *   q0:       (nmodes,) complex IVP-2 initial flux (reference tfftq0[msk])
 *   eig:      (nmodes,) complex top eigenvalue (reference eigval)
 *   lv:       (nz-1, 12) level table
 *   snap_of_step: (nz,) slot per step or -1
 *   p_out, q_out: (nsnap, nmodes) complex128, slot-major
 * Returns 0, or -1 if nsnap exceeds the supported maximum.
 */
int oracle_sweep(int64_t nmodes, const double *lx, const double *ly,
                 const double *q0, const double *eig, double kz_top, int nz,
                 const double *lv, const int *snap_of_step, int nsnap,
                 double *p_out, double *q_out, int nthreads)
{
    enum { MAXSNAP = 1024 };
    if (nsnap > MAXSNAP || nsnap < 0 || nz < 1)
        return -1;
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        cplx sp1[MAXSNAP], sq1[MAXSNAP], sp2[MAXSNAP], sq2[MAXSNAP];
        cplx po[MAXSNAP], qo[MAXSNAP];
#pragma omp for schedule(static)
        for (int64_t m = 0; m < nmodes; ++m) {
            cplx qq = {q0[2 * m], q0[2 * m + 1]};
            cplx ee = {eig[2 * m], eig[2 * m + 1]};
            sweep_mode(lx[m], ly[m], qq, ee, kz_top, nz, lv, snap_of_step, nsnap,
                       po, qo, sp1, sq1, sp2, sq2);
            for (int s = 0; s < nsnap; ++s) {
                size_t o = ((size_t)s * (size_t)nmodes + (size_t)m) * 2;
                p_out[o] = po[s].r;
                p_out[o + 1] = po[s].i;
                q_out[o] = qo[s].r;
                q_out[o + 1] = qo[s].i;
            }
        }
    }
    return 0;
}

/* Top eigenvalue by libm csqrt of the caller's eigval**2 (reference
 * solver.py:164-174 uses numpy's sqrt, which calls libm csqrt). */
#include <complex.h>
void oracle_csqrt(int64_t n, const double *w, double *out)
{
    for (int64_t k = 0; k < n; ++k) {
        double complex z = CMPLX(w[2 * k], w[2 * k + 1]);
        double complex r = csqrt(z);
        out[2 * k] = creal(r);
        out[2 * k + 1] = cimag(r);
    }
}
