#pragma once
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
void hx_level_table(int nz, const double *z, const double *prof, double *lv);
void hx_level_dz_w(int nz, const double *z, const double *prof, double *lv);
void hx_level_table32(int nz, const double *z, const double *prof, float *lv, float *lvff);
double hx_fftfreq_val(int n);
void hx_eigval(int64_t m0, int64_t m1, const uint32_t *modes, int nlx, int nly, double valx, double valy,
               double lx_scale, double ly_scale, double Kx_top, double Ky_top, double Kz_top, double u_top,
               double v_top, double *eig);
int hx_check_profiles(int nz, const double *z, const double *prof);
int hx_profiles_iso(int nz, const double *prof, double *ex, double *ey);
void hx_level_table32_iso(int nz, const double *z, const double *prof, double ex, double ey, float *lv,
                          float *lvff);
void hx_dc_values(int nz, const double *lv, const int *slot, double q0r, double q0i, double p000, int single,
                  int nlvls, int analytic, double *dc);
#ifdef __cplusplus
}
#endif
