/*
 * Host-side arithmetic that must round exactly as the reference's numpy code.
 * Compiled with -ffp-contract=off: every + - * / below is one IEEE operation,
 * pow() and csqrt() are the process's libm (numpy's scalar ** and complex
 * sqrt call the same libm).
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

/* FP32 level table of the Riccati sweep, from the same per-step scalars. */
void hx_level_table32(int nz, const double *z, const double *prof, float *lv)
{
    const double *u = prof, *v = prof + nz, *Kx = prof + 2 * nz, *Ky = prof + 3 * nz, *Kz = prof + 4 * nz;
    for (int i = 0; i < nz - 1; ++i) {
        double k = 1.0 / Kz[i];
        double h = z[i + 1] - z[i];
        float *row = lv + (size_t)i * 12;
        double c1 = k * h * h * h / 6.0;
        row[0] = (float)(-Kx[i]);
        row[1] = (float)(-Ky[i]);
        row[2] = (float)(-u[i]);
        row[3] = (float)(-v[i]);
        row[4] = (float)(0.5 * k * h * h);
        row[5] = (float)(-k * h);
        row[6] = (float)(k * k * h * h * h / 6.0);
        row[7] = (float)h;
        row[8] = (float)c1;
        row[9] = (float)(-2.0 * c1);
        row[10] = 0.f;
        row[11] = 0.f;
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
