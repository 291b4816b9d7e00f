/*
 * Host-side arithmetic that must round exactly as the reference's numpy code.
 * Compiled with -ffp-contract=off: every + - * / below is one IEEE operation,
 * pow() and csqrt() are the process's libm (numpy's scalar ** and complex
 * sqrt call the same libm).  Also compiled with -fno-builtin, so that the
 * compiler does not replace pow(x, 2.0) by x * x: libm's pow is not always
 * correctly rounded, and the reference's dz**2 and Kzinv**2 are libm's.
 */
#include <complex.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "host_exact.h"

/* Level table of the sweep (src/bldfm/solver.py:357-364) plus the trapezoid
 * weight w_i = 0.5/Kz[i] + 0.5/Kz[i+1] (solver.py:249) in the last column. */
void hx_level_table(int nz, const double *z, const double *prof, double *lv)
{
    const double *u = prof, *v = prof + nz, *Kx = prof + 2 * nz, *Ky = prof + 3 * nz, *Kz = prof + 4 * nz;
    for (int i = 0; i < nz - 1; ++i) {
        double Kzinv = 1.0 / Kz[i];
        double dzi = z[i + 1] - z[i];
        double *row = lv + (size_t)i * 12;
        row[0] = Kx[i];
        row[1] = Ky[i];
        row[2] = u[i];
        row[3] = v[i];
        row[4] = 0.5 * Kzinv;
        row[5] = pow(dzi, 2.0);
        row[6] = (1.0 / 6.0) * pow(Kzinv, 2.0);
        row[7] = pow(dzi, 3.0);
        row[8] = (-Kzinv) * dzi;
        row[9] = (1.0 / 6.0) * Kzinv;
        row[10] = dzi;
        row[11] = 0.5 / Kz[i] + 0.5 / Kz[i + 1];
    }
}

/* The two columns of hx_level_table that hx_dc_values reads (dz, column 10,
   and the averaged 1/Kz weight, column 11), with the same arithmetic; the
   other columns are left untouched. */
void hx_level_dz_w(int nz, const double *z, const double *prof, double *lv)
{
    const double *Kz = prof + 4 * nz;
    for (int i = 0; i < nz - 1; ++i) {
        double *row = lv + (size_t)i * 12;
        row[10] = z[i + 1] - z[i];
        row[11] = 0.5 / Kz[i] + 0.5 / Kz[i + 1];
    }
}

/* FP32 level table of the Riccati sweep, from the same per-step scalars
 * (lv may be NULL); lvff (may be NULL) receives the same rows unrounded as
 * float pairs (hi, lo), hi + lo the FP64 value to about 2^-48. */
void hx_level_table32(int nz, const double *z, const double *prof, float *lv, float *lvff)
{
    const double *u = prof, *v = prof + nz, *Kx = prof + 2 * nz, *Ky = prof + 3 * nz, *Kz = prof + 4 * nz;
    for (int i = 0; i < nz - 1; ++i) {
        double k = 1.0 / Kz[i];
        double h = z[i + 1] - z[i];
        double c1 = k * h * h * h / 6.0;
        double r[12];
        r[0] = -Kx[i];
        r[1] = -Ky[i];
        r[2] = -u[i];
        r[3] = -v[i];
        r[4] = 0.5 * k * h * h;
        r[5] = -k * h;
        r[6] = k * k * h * h * h / 6.0;
        r[7] = h;
        r[8] = c1;
        r[9] = -2.0 * c1;
        r[10] = 0.0;
        r[11] = 0.0;
        if (lv)
            for (int j = 0; j < 12; ++j) lv[(size_t)i * 12 + j] = (float)r[j];
        if (lvff)
            for (int j = 0; j < 12; ++j) {
                const float h = (float)r[j];
                lvff[((size_t)i * 12 + j) * 2] = h;
                lvff[((size_t)i * 12 + j) * 2 + 1] = (float)(r[j] - (double)h);
            }
    }
}

/* fftfreq(n, d=1/n) scale: results * (1 / (n * (1/n))) */
double hx_fftfreq_val(int n)
{
    double d = 1.0 / (double)n;
    return 1.0 / ((double)n * d);
}

/* Top eigenvalue of the solved modes (solver.py:164-174):
 *   eig = sqrt(KxKzinv Lx^2 + KyKzinv Ly^2 + 1j u Kzinv Lx + 1j v Kzinv Ly)
 * modes packed as in the device mode list; eig out is (n, 2). */
void hx_eigval(int64_t m0, int64_t m1, const uint32_t *modes, int nlx, int nly, double valx, double valy,
               double lx_scale, double ly_scale, double Kx_top, double Ky_top, double Kz_top, double u_top,
               double v_top, double *eig)
{
    double Kzinv = 1.0 / Kz_top;
    double KxKzinv = Kx_top * Kzinv;
    double KyKzinv = Ky_top * Kzinv;
    double uK = u_top * Kzinv;
    double vK = v_top * Kzinv;
    for (int64_t m = m0; m < m1; ++m) {
        uint32_t e = modes[m];
        int c = (int)(e & 0x7fffu);
        int r = (int)((e >> 15) & 0x7fffu);
        int hx = (nlx - 1) / 2 + 1, hy = (nly - 1) / 2 + 1;
        int kx = c < hx ? c : c - nlx;
        int ky = r < hy ? r : r - nly;
        double lx = lx_scale * ((double)kx * valx);
        double ly = ly_scale * ((double)ky * valy);
        double wr = KxKzinv * (lx * lx) + KyKzinv * (ly * ly);
        double wi = uK * lx + vK * ly;
        double complex s = csqrt(CMPLX(wr, wi));
        eig[2 * m] = creal(s);
        eig[2 * m + 1] = cimag(s);
    }
}

/* 1 when Kx == Ky at every level and (u, v) keeps one direction (ex, ey):
 * then T = -K k^2 - i U (ex kx + ey ky) with U = u ex + v ey (all four
 * closures of vertical_profiles have this form). */
/* Input validation before any work: every z and profile value finite, z
 * strictly increasing, Kz > 0 and Kx, Ky >= 0 at every level.  The sweep
 * divides by Kz and by the top eigenvalue (src/bldfm/solver.py:164-174,
 * 357-364); the reference itself returns NaN fields for such inputs.
 * Returns 0 when the inputs are valid. */
int hx_check_profiles(int nz, const double *z, const double *prof)
{
    for (int i = 0; i < nz; ++i) {
        if (!isfinite(z[i])) return 1;
        if (i > 0 && !(z[i] > z[i - 1])) return 1;
        for (int k = 0; k < 5; ++k)
            if (!isfinite(prof[k * nz + i])) return 1;
        if (!(prof[4 * nz + i] > 0.0) || prof[2 * nz + i] < 0.0 || prof[3 * nz + i] < 0.0) return 1;
    }
    return 0;
}

int hx_profiles_iso(int nz, const double *prof, double *ex, double *ey)
{
    const double *u = prof, *v = prof + nz, *Kx = prof + 2 * nz, *Ky = prof + 3 * nz;
    int imax = 0;
    double best = -1.0;
    for (int i = 0; i < nz; ++i) {
        if (Kx[i] != Ky[i]) return 0;
        double m = u[i] * u[i] + v[i] * v[i];
        if (m > best) {
            best = m;
            imax = i;
        }
    }
    double n = sqrt(best);
    if (!(n > 0)) {
        *ex = 1.0;
        *ey = 0.0;
        return 1;
    }
    double dx = u[imax] / n, dy = v[imax] / n;
    for (int i = 0; i < nz; ++i) {
        double cross = u[i] * dy - v[i] * dx;
        double mag = sqrt(u[i] * u[i] + v[i] * v[i]);
        if (fabs(cross) > 1e-12 * mag + 1e-300) return 0;
    }
    *ex = dx;
    *ey = dy;
    return 1;
}

/* Compact FP32 level table for isotropic profiles with a fixed wind
 * direction (row layout of StepCoef<true> in sweep32.cuh); lvff (may be
 * NULL) receives the same rows unrounded as float pairs (hi, lo). */
void hx_level_table32_iso(int nz, const double *z, const double *prof, double ex, double ey, float *lv, float *lvff)
{
    const double *u = prof, *v = prof + nz, *Kx = prof + 2 * nz, *Kz = prof + 4 * nz;
    for (int i = 0; i < nz - 1; ++i) {
        double k = 1.0 / Kz[i];
        double h = z[i + 1] - z[i];
        double K = Kx[i];
        double U = u[i] * ex + v[i] * ey;
        double A = 0.5 * k * h * h, B0 = -k * h, B1 = k * k * h * h * h / 6.0, C1 = k * h * h * h / 6.0;
        double r[12];
        r[0] = A * K;
        r[1] = A * U;
        r[2] = B0;
        r[3] = B1 * K;
        r[4] = B1 * U;
        r[5] = -h * K;
        r[6] = -C1 * K * K;
        r[7] = C1 * U * U;
        r[8] = -h * U;
        r[9] = -2.0 * C1 * K * U;
        r[10] = 0.0;
        r[11] = 0.0;
        float *row = lv + (size_t)i * 12;
        for (int j = 0; j < 12; ++j) row[j] = (float)r[j];
        if (lvff)
            for (int j = 0; j < 12; ++j) {
                const float h = (float)r[j];
                lvff[((size_t)i * 12 + j) * 2] = h;
                lvff[((size_t)i * 12 + j) * 2 + 1] = (float)(r[j] - (double)h);
            }
    }
}

/* k = 0 mode of every output slot when the source spectrum's k = 0 value q0
 * is known on the host (footprint mode), exactly as solver.py:186-191 and
 * 237-251 evaluate it: p00 starts at p000 and loses (q0 dz_i) w_i per step,
 * w_i = 0.5/Kz[i] + 0.5/Kz[i+1] (level-table column 11).  dc receives
 * (p_s, q_s) as 4 doubles per slot s < nlvls; complex64 rounding when
 * single != 0.  Slots without a level keep p = 0 (slot 0: p000), q = q0. */
void hx_dc_values(int nz, const double *lv, const int *slot, double q0r, double q0i, double p000, int single,
                  int nlvls, int analytic, double *dc)
{
    double qr = q0r, qi = q0i;
    if (single) {
        qr = (double)(float)qr;
        qi = (double)(float)qi;
    }
    for (int s = 0; s < nlvls; ++s) {
        dc[4 * s + 0] = 0.0;
        dc[4 * s + 1] = 0.0;
        dc[4 * s + 2] = qr;
        dc[4 * s + 3] = qi;
    }
    dc[0] = single ? (double)(float)p000 : p000;
    if (analytic) return;
    double pr = p000, pi = 0.0;
    for (int i = 0; i < nz - 1; ++i) {
        if (slot[i] >= 0) {
            dc[4 * slot[i] + 0] = single ? (double)(float)pr : pr;
            dc[4 * slot[i] + 1] = single ? (double)(float)pi : pi;
        }
        const double dz = lv[(size_t)i * 12 + 10], w = lv[(size_t)i * 12 + 11];
        pr = pr - (q0r * dz) * w;
        pi = pi - (q0i * dz) * w;
    }
    if (slot[nz - 1] >= 0) {
        dc[4 * slot[nz - 1] + 0] = single ? (double)(float)pr : pr;
        dc[4 * slot[nz - 1] + 1] = single ? (double)(float)pi : pi;
    }
}
