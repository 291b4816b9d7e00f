// Geometry of one solve (geometry.h): the reference's grid arithmetic
// (src/bldfm/solver.py:94-131, 253-262, 264-290) in one heap-free place, used
// by the workspace, host, batched, surrogate and allocation-free entry points.
#include <math.h>
#include <string.h>

#include "geometry.h"
#include "host_exact.h"

int solved_in_column(int c, int nlx, int nly)
{
    const int kx = freq_of_index(c, nlx);
    const bool nyq_x = (nlx % 2 == 0) && kx == -(nlx / 2);
    const bool even_y = nly % 2 == 0;
    if (kx > 0 || nyq_x) return nly;
    if (kx == 0) return freq_max(nly) + (even_y ? 1 : 0);
    return even_y ? 1 : 0;
}

int band_columns(int nlx, int nfx, int4 *out)
{
    const int f0 = freq_min(nlx), f1 = freq_max(nlx);
    const int hmax = (-f0 > f1) ? -f0 : f1;
    int nb = 0;
    for (int f = -hmax; f <= hmax; ++f) {
        // 2 h <= nlx <= nfx, so only f = h can land on the position of f = -h
        // (when 2 h = nfx); the first occurrence is kept
        if (f > -hmax && f - (-hmax) == nfx) continue;
        const int pos = ((f % nfx) + nfx) % nfx;
        auto colof = [&](int p) -> int {
            if (p <= f1) return p;                      // non-negative frequencies
            if (p >= nfx + f0) return p - nfx + nlx;    // negative frequencies
            return -1;
        };
        const int a = colof(pos), b = colof((nfx - pos) % nfx);
        if (a < 0 && b < 0) continue;
        out[nb++] = make_int4(pos, a, b, 0);
    }
    return nb;
}

int solve_geometry(const bldfm_desc *d, const double *z, const double *prof, const int64_t *levels, int nlvls,
                   SolveGeom &g, int *slot, bool *shape_ok)
{
    if (!d) return BLDFM_ERR_ARG;
    if ((d->nlx % 2) != 0 || (d->nly % 2) != 0) return BLDFM_ERR_ODD_MODES;
    if (d->precision != BLDFM_PREC_SINGLE && d->precision != BLDFM_PREC_DOUBLE) return BLDFM_ERR_PRECISION;
    if (d->nx < 1 || d->ny < 1 || d->nz < 1 || d->nlx < 0 || d->nly < 0 || nlvls < 1) return BLDFM_ERR_ARG;
    if (d->mode != BLDFM_MODE_FP64 && d->mode != BLDFM_MODE_FP32 && d->mode != BLDFM_MODE_FP64R) return BLDFM_ERR_ARG;
    if (!(d->xmax > 0) || !(d->ymax > 0)) return BLDFM_ERR_ARG;
    if (d->nz > BLDFM_MAX_NZ) return BLDFM_ERR_UNSUPPORTED;
    memset(&g, 0, sizeof(g));
    g.nx = d->nx;
    g.ny = d->ny;
    g.nz = d->nz;
    const double dx = d->xmax / d->nx, dy = d->ymax / d->ny;
    const double halo = d->has_halo ? d->halo : (d->xmax > d->ymax ? d->xmax : d->ymax);
    if (!(halo >= 0)) return BLDFM_ERR_ARG;
    const double pxd = halo / dx, pyd = halo / dy;
    if (pxd > 1e7 || pyd > 1e7) return BLDFM_ERR_UNSUPPORTED;
    g.px = (int)pxd;
    g.py = (int)pyd;
    g.nxe = g.nx + 2 * g.px;
    g.nye = g.ny + 2 * g.py;
    int nlx = d->nlx, nly = d->nly;
    if (nlx > g.nxe || nly > g.nye) {  // clamp (solver.py:122-128)
        nlx = g.nxe;
        nly = g.nye;
    }
    if (nlx < 1 || nly < 1) return BLDFM_ERR_ARG;
    g.nlx = nlx;
    g.nly = nly;
    g.dlx = (g.nxe - nlx) / 2;
    g.dly = (g.nye - nly) / 2;
    g.nfx = nlx + 2 * g.dlx;
    g.nfy = nly + 2 * g.dly;
    g.out_ny = (g.nye - g.py < g.nfy ? g.nye - g.py : g.nfy) - g.py;
    g.out_nx = (g.nxe - g.px < g.nfx ? g.nxe - g.px : g.nfx) - g.px;
    if (g.out_ny < 0) g.out_ny = 0;
    if (g.out_nx < 0) g.out_nx = 0;
    if (nlx > 32767 || nly > 32767) return BLDFM_ERR_UNSUPPORTED;
    if (g.nfx > BLDFM_MAX_FFT_N || g.nfy > BLDFM_MAX_FFT_N) return BLDFM_ERR_UNSUPPORTED;
    if (!d->footprint && (g.nxe > BLDFM_MAX_FFT_N || g.nye > BLDFM_MAX_FFT_N)) return BLDFM_ERR_UNSUPPORTED;
    const bool ok = ((g.nxe - nlx) % 2 == 0) && ((g.nye - nly) % 2 == 0);
    if (shape_ok) *shape_ok = ok;
    if (!d->footprint && !ok) return BLDFM_ERR_SPECTRUM_SHAPE;
    if (d->analytic && nlvls != 1) return BLDFM_ERR_BROADCAST;

    g.nlvls = nlvls;
    g.footprint = d->footprint ? 1 : 0;
    g.analytic = d->analytic ? 1 : 0;
    g.precision = d->precision;
    g.mode = d->mode;
    g.out_sign = d->footprint ? -1 : +1;
    g.valx = hx_fftfreq_val(nlx);
    g.valy = hx_fftfreq_val(nly);
    g.lx_scale = 2.0 * M_PI / dx / g.nxe;
    g.ly_scale = 2.0 * M_PI / dy / g.nye;
    g.inv_nxe = 1.0 / g.nxe;
    g.inv_nye = 1.0 / g.nye;
    // numpy evaluates ones(complex128) / nxe / nye with Smith's reciprocal-scale
    // division, i.e. (1/nxe) * (1/nye) (solver.py:134)
    g.q0dc_fp = (1.0 / g.nxe) * (1.0 / g.nye);
    g.q0dc_f = (float)g.q0dc_fp;
    if (d->footprint) {
        g.do_shift = 1;
        g.sx = d->meas_x + halo;
        g.sy = d->meas_y + halo;
    } else if (d->meas_x * d->meas_x + d->meas_y * d->meas_y > 0.0) {
        g.do_shift = 1;
        g.sx = d->meas_x - d->xmax / 2;
        g.sy = d->meas_y - d->ymax / 2;
    }
    {
        // phase shift as fixed-point turns for the FP32 path
        const long double pi2 = 6.283185307179586476925286766559005768L;
        long double tx = (long double)g.lx_scale * g.valx * g.sx / pi2;
        long double ty = (long double)g.ly_scale * g.valy * g.sy / pi2;
        tx -= floorl(tx);
        ty -= floorl(ty);
        g.turn_x = (uint32_t)(uint64_t)llrintl(tx * 4294967296.0L);
        g.turn_y = (uint32_t)(uint64_t)llrintl(ty * 4294967296.0L);
    }
    const int nz = d->nz;
    if (z && prof) {
        if (hx_check_profiles(nz, z, prof) != 0) return BLDFM_ERR_PROFILE;
        const double *u = prof, *v = prof + nz, *Kx = prof + 2 * nz, *Ky = prof + 3 * nz, *Kz = prof + 4 * nz;
        const double kzinv = 1.0 / Kz[nz - 1];
        g.kz_top = Kz[nz - 1];
        g.kxk_top = Kx[nz - 1] * kzinv;
        g.kyk_top = Ky[nz - 1] * kzinv;
        g.uk_top = u[nz - 1] * kzinv;
        g.vk_top = v[nz - 1] * kzinv;
        g.kz_top_f = (float)g.kz_top;
        g.kxk_top_f = (float)g.kxk_top;
        g.kyk_top_f = (float)g.kyk_top;
        g.uk_top_f = (float)g.uk_top;
        g.vk_top_f = (float)g.vk_top;
        double ex = 1.0, ey = 0.0;
        g.iso = hx_profiles_iso(nz, prof, &ex, &ey);
        g.ex = (float)ex;
        g.ey = (float)ey;
    }
    // snapshot schedule (solver.py:350-372): slot s = s-th distinct level in [0, nz-1]
    int ns = 0;
    if (levels) {
        for (int k = 0; k < nlvls; ++k)
            if (levels[k] < -(int64_t)nz || levels[k] >= nz) return BLDFM_ERR_ARG;
        g.jmax = -1;
        for (int i = 0; i < nz; ++i) {
            int s = -1;
            for (int k = 0; k < nlvls; ++k)
                if (levels[k] == i) {
                    s = ns++;
                    break;
                }
            if (slot) slot[i] = s;
            if (s >= 0) g.jmax = i;
        }
    } else {
        g.jmax = -1;
        if (slot)
            for (int i = 0; i < nz; ++i) slot[i] = -1;
    }
    g.nsnap = ns;
    int64_t nsolved = 0;
    for (int c = 0; c < nlx; ++c) nsolved += solved_in_column(c, nlx, nly);
    g.nsolved = nsolved;
    return BLDFM_OK;
}
