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

/* ------------------------------------------------------------------------
 * Extended-precision shooting: the reference's own algorithm (two IVPs
 * bottom-up, then the alpha combination; src/bldfm/solver.py:220-235 and
 * :307-374) carried out in double-double arithmetic (about 106 significant
 * bits).  The shooting method loses up to log10(e^{2G}) digits to
 * cancellation between the growing IVP states; with about 32 digits instead
 * of 16 its result is the solution of the reference's discrete problem to
 * well below 1e-10 wherever the reference's own FP64 evaluation keeps any
 * digit at all.  This is the "exact" yardstick the accurate and fast paths
 * are checked against.
 *
 * Double-double building blocks: error-free transformations TwoSum
 * (Knuth, TAOCP vol. 2, 4.2.2) and TwoProduct by fused multiply-add, with the
 * accurate pairwise sum of Hida, Li and Bailey ("Library for double-double
 * and quad-double arithmetic", 2000).  They need every + and * rounded as
 * written: the file is compiled with -ffp-contract=off.
 *
 * Inputs are the reference's FP64 values (the z grid, the five profiles,
 * the masked wavenumbers, the top eigenvalue); everything computed from them
 * is carried in double-double: dz, 1/Kz, dz^2, dz^3, the Taylor coefficients,
 * both IVPs, alpha and the level values.  The initial flux of IVP 2 is 1, so
 * the output is the per-mode transfer (p, q at each level per unit source
 * flux); the caller multiplies by the source spectrum.
 * ---------------------------------------------------------------------- */
typedef struct {
    double hi, lo;
} dd;

static inline dd dd_two_sum(double a, double b)
{
    double s = a + b;
    double bb = s - a;
    dd r = {s, (a - (s - bb)) + (b - bb)};
    return r;
}

static inline dd dd_fast_sum(double a, double b) /* |a| >= |b| */
{
    double s = a + b;
    dd r = {s, b - (s - a)};
    return r;
}

static inline dd dd_d(double a)
{
    dd r = {a, 0.0};
    return r;
}

static inline dd dd_add(dd x, dd y)
{
    dd s = dd_two_sum(x.hi, y.hi);
    dd t = dd_two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = dd_fast_sum(s.hi, s.lo);
    s.lo += t.lo;
    return dd_fast_sum(s.hi, s.lo);
}

static inline dd dd_neg(dd x)
{
    dd r = {-x.hi, -x.lo};
    return r;
}

static inline dd dd_sub(dd x, dd y) { return dd_add(x, dd_neg(y)); }

static inline dd dd_mul(dd x, dd y)
{
    double p = x.hi * y.hi;
    double e = fma(x.hi, y.hi, -p);
    e += x.hi * y.lo + x.lo * y.hi;
    return dd_fast_sum(p, e);
}

static inline dd dd_mul_d(dd x, double b)
{
    double p = x.hi * b;
    double e = fma(x.hi, b, -p);
    e += x.lo * b;
    return dd_fast_sum(p, e);
}

static inline dd dd_div(dd x, dd y)
{
    /* three quotient digits: x/y = q1 + q2 + q3 to double-double accuracy */
    double q1 = x.hi / y.hi;
    dd r = dd_sub(x, dd_mul_d(y, q1));
    double q2 = r.hi / y.hi;
    r = dd_sub(r, dd_mul_d(y, q2));
    double q3 = r.hi / y.hi;
    dd q = dd_fast_sum(q1, q2);
    return dd_add(q, dd_d(q3));
}

typedef struct {
    dd r, i;
} cdd;

static inline cdd cdd_mul(cdd a, cdd b)
{
    cdd o = {dd_sub(dd_mul(a.r, b.r), dd_mul(a.i, b.i)), dd_add(dd_mul(a.r, b.i), dd_mul(a.i, b.r))};
    return o;
}

static inline cdd cdd_add(cdd a, cdd b)
{
    cdd o = {dd_add(a.r, b.r), dd_add(a.i, b.i)};
    return o;
}

static inline cdd cdd_sub(cdd a, cdd b)
{
    cdd o = {dd_sub(a.r, b.r), dd_sub(a.i, b.i)};
    return o;
}

static inline cdd cdd_scale(cdd a, dd s)
{
    cdd o = {dd_mul(a.r, s), dd_mul(a.i, s)};
    return o;
}

/* a / b: both operands scaled by a power of two near 1/max(|b.r|, |b.i|)
 * (exact), then a * conj(b) / |b|^2 */
static inline cdd cdd_div(cdd a, cdd b)
{
    double m = fmax(fabs(b.r.hi), fabs(b.i.hi));
    int ex = 0;
    frexp(m, &ex);
    double s = ldexp(1.0, -ex);
    cdd bs = {dd_mul_d(b.r, s), dd_mul_d(b.i, s)};
    cdd as = {dd_mul_d(a.r, s), dd_mul_d(a.i, s)};
    dd den = dd_add(dd_mul(bs.r, bs.r), dd_mul(bs.i, bs.i));
    dd nr = dd_add(dd_mul(as.r, bs.r), dd_mul(as.i, bs.i));
    dd ni = dd_sub(dd_mul(as.i, bs.r), dd_mul(as.r, bs.i));
    cdd o = {dd_div(nr, den), dd_div(ni, den)};
    return o;
}

/* per-step coefficients of the reference's Taylor propagator, in double-double */
typedef struct {
    double kx, ky, u, v;
    dd h;        /* dz = z[i+1] - z[i]         */
    dd s1h2;     /* 0.5 * Kzinv * dz^2         */
    dd s2h3;     /* 1/6 * Kzinv^2 * dz^3       */
    dd s3;       /* -Kzinv * dz                */
    dd s4h3;     /* 1/6 * Kzinv * dz^3         */
} dd_level;

static void dd_levels(int nz, const double *z, const double *prof, dd_level *lv)
{
    const double *u = prof, *v = prof + nz, *Kx = prof + 2 * nz, *Ky = prof + 3 * nz, *Kz = prof + 4 * nz;
    const dd sixth = dd_div(dd_d(1.0), dd_d(6.0));
    for (int i = 0; i < nz - 1; ++i) {
        dd h = dd_two_sum(z[i + 1], -z[i]);
        dd kinv = dd_div(dd_d(1.0), dd_d(Kz[i]));
        dd h2 = dd_mul(h, h), h3 = dd_mul(h2, h);
        lv[i].kx = Kx[i];
        lv[i].ky = Ky[i];
        lv[i].u = u[i];
        lv[i].v = v[i];
        lv[i].h = h;
        lv[i].s1h2 = dd_mul_d(dd_mul(kinv, h2), 0.5);
        lv[i].s2h3 = dd_mul(dd_mul(sixth, dd_mul(kinv, kinv)), h3);
        lv[i].s3 = dd_neg(dd_mul(kinv, h));
        lv[i].s4h3 = dd_mul(dd_mul(sixth, kinv), h3);
    }
}

static void sweep_mode_dd(double lx, double ly, cdd keig, int nz, const dd_level *lv, const int *snap_of_step,
                          int nsnap, cdd *sp1, cdd *sq1, cdd *sp2, cdd *sq2, double *po, double *qo)
{
    const dd zero = {0.0, 0.0}, one = {1.0, 0.0};
    const dd lx2 = dd_mul(dd_d(lx), dd_d(lx)), ly2 = dd_mul(dd_d(ly), dd_d(ly));
    cdd p1 = {one, zero}, q1 = {zero, zero}, p2 = {zero, zero}, q2 = {one, zero};
    for (int i = 0; i < nz - 1; ++i) {
        int s = snap_of_step[i];
        if (s >= 0) {
            sp1[s] = p1; sq1[s] = q1; sp2[s] = p2; sq2[s] = q2;
        }
        const dd_level *L = lv + i;
        /* T = -(Kx lx^2 + Ky ly^2) - i (u lx + v ly)   (solver.py:357) */
        cdd T;
        T.r = dd_neg(dd_add(dd_mul_d(lx2, L->kx), dd_mul_d(ly2, L->ky)));
        T.i = dd_neg(dd_add(dd_mul(dd_d(L->u), dd_d(lx)), dd_mul(dd_d(L->v), dd_d(ly))));
        /* a = 1 - 0.5 Kzinv T dz^2; b = -Kzinv dz - 1/6 Kzinv^2 T dz^3;
         * c = T dz - 1/6 Kzinv T^2 dz^3                (solver.py:361-364) */
        cdd a = {dd_sub(one, dd_mul(L->s1h2, T.r)), dd_neg(dd_mul(L->s1h2, T.i))};
        cdd b = {dd_sub(L->s3, dd_mul(L->s2h3, T.r)), dd_neg(dd_mul(L->s2h3, T.i))};
        cdd T2 = cdd_mul(T, T);
        cdd c = cdd_sub(cdd_scale(T, L->h), cdd_scale(T2, L->s4h3));
        /* (p, q) <- (a p + b q, c p + a q)              (solver.py:366-368) */
        cdd np1 = cdd_add(cdd_mul(a, p1), cdd_mul(b, q1));
        cdd nq1 = cdd_add(cdd_mul(c, p1), cdd_mul(a, q1));
        cdd np2 = cdd_add(cdd_mul(a, p2), cdd_mul(b, q2));
        cdd nq2 = cdd_add(cdd_mul(c, p2), cdd_mul(a, q2));
        p1 = np1; q1 = nq1; p2 = np2; q2 = nq2;
    }
    {
        int s = snap_of_step[nz - 1];
        if (s >= 0) {
            sp1[s] = p1; sq1[s] = q1; sp2[s] = p2; sq2[s] = q2;
        }
    }
    /* alpha = -(q2 - Kz eig p2) / (q1 - Kz eig p1)     (solver.py:228-230) */
    cdd num = cdd_sub(q2, cdd_mul(keig, p2));
    cdd den = cdd_sub(q1, cdd_mul(keig, p1));
    num.r = dd_neg(num.r);
    num.i = dd_neg(num.i);
    cdd alpha = cdd_div(num, den);
    /* p = alpha p1 + p2, q = alpha q1 + q2            (solver.py:233-235) */
    for (int s = 0; s < nsnap; ++s) {
        cdd p = cdd_add(cdd_mul(alpha, sp1[s]), sp2[s]);
        cdd q = cdd_add(cdd_mul(alpha, sq1[s]), sq2[s]);
        po[2 * s] = p.r.hi + p.r.lo;
        po[2 * s + 1] = p.i.hi + p.i.lo;
        qo[2 * s] = q.r.hi + q.r.lo;
        qo[2 * s + 1] = q.i.hi + q.i.lo;
    }
}

/*
 * Per-mode transfer functions of the shooting method in double-double.
 *   lx, ly, eig: (nmodes,) as oracle_sweep (eig complex interleaved)
 *   z, prof:     (nz,) and (5, nz) -- the reference's z grid and profiles
 *   p_out, q_out: (nsnap, nmodes) complex128, slot-major, per unit source flux
 * Returns 0, or -1 on bad sizes.
 */
int oracle_sweep_dd(int64_t nmodes, const double *lx, const double *ly, const double *eig, int nz,
                    const double *z, const double *prof, const int *snap_of_step, int nsnap, double *p_out,
                    double *q_out, int nthreads)
{
    enum { MAXSNAP = 1024, MAXNZ = 8192 };
    if (nsnap > MAXSNAP || nsnap < 0 || nz < 1 || nz > MAXNZ)
        return -1;
    static dd_level lv[MAXNZ];
    dd_levels(nz, z, prof, lv);
    const dd kz_top = dd_d(prof[4 * nz + nz - 1]);
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        cdd sp1[MAXSNAP], sq1[MAXSNAP], sp2[MAXSNAP], sq2[MAXSNAP];
        double po[2 * MAXSNAP], qo[2 * MAXSNAP];
#pragma omp for schedule(dynamic, 256)
        for (int64_t m = 0; m < nmodes; ++m) {
            cdd keig = {dd_mul(kz_top, dd_d(eig[2 * m])), dd_mul(kz_top, dd_d(eig[2 * m + 1]))};
            sweep_mode_dd(lx[m], ly[m], keig, nz, lv, snap_of_step, nsnap, sp1, sq1, sp2, sq2, po, qo);
            for (int s = 0; s < nsnap; ++s) {
                size_t o = ((size_t)s * (size_t)nmodes + (size_t)m) * 2;
                p_out[o] = po[2 * s];
                p_out[o + 1] = po[2 * s + 1];
                q_out[o] = qo[2 * s];
                q_out[o + 1] = qo[2 * s + 1];
            }
        }
    }
    return 0;
}
