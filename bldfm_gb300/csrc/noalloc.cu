// Allocation-free FP32 solve: bldfm_solve_noalloc (include/bldfm_gb300.h).
//
// Who needs it: callers that may not allocate GPU memory at solve time --
// code running inside a CUDA stream capture, embedded or real-time hosts that
// pre-reserve all device memory, and plugin hosts whose allocator policy
// forbids cudaMalloc from third-party libraries.  They pass inputs and
// outputs; every intermediate the solve needs (twiddle tables, mode list,
// band table, level tables, spectra, transform intermediate) lives in one
// file-scope device array of BLDFM_NOALLOC_SCRATCH_BYTES (16 MiB).  Every GPU
// that loads this library holds that array until the process exits.
//
// Rules of use:
//  - The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
//  - All calls share the one array and it keeps the previous call's contents;
//    this file clears what must start at zero.  Calls whose GPU work overlaps
//    (different streams, or different host threads without ordering) race on
//    the array: serialise them on one stream.
//  - FP32 mode only (the FP64 mode needs host-side libm values staged in
//    pinned memory); problems whose scratch exceeds the array are rejected
//    with BLDFM_ERR_WORKSPACE.
// Nothing here calls cudaMalloc, cudaFree, cudaHostAlloc or any other
// allocating routine, and the host side uses fixed static buffers.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "../../include/bldfm_gb300.h"
#include "common.h"
#include "host_exact.h"
#include "kernels.h"

#define BLDFM_NOALLOC_SCRATCH_BYTES (16u << 20)
#define NA_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[BLDFM_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex na_mutex;
void *na_scratch_dev[NA_MAX_DEVICES];  // device address of g_noalloc_scratch per device

// host-side staging (static, no heap): level tables, slot map, band table
struct NaHost {
    double lv64[(BLDFM_MAX_NZ - 1) * BLDFM_LV64];
    double dc[4 * BLDFM_MAX_NZ];
    float lv32[(BLDFM_MAX_NZ - 1) * BLDFM_LV32];
    int slot[BLDFM_MAX_NZ];
    int4 xband[BLDFM_MAX_FFT_N + 1];
    int colstart[BLDFM_MAX_FFT_N + 1];
};
NaHost na_host;

inline size_t na_al(size_t x) { return (x + 255) & ~(size_t)255; }

void na_factorize(int n, FftPlan &p)
{
    p.n = n;
    p.nstages = 0;
    int m = n;
    const int pref[] = {8, 4, 2, 3, 5};
    for (int r : pref)
        while (m % r == 0 && p.nstages < BLDFM_MAX_STAGES) {
            p.radix[p.nstages++] = r;
            m /= r;
        }
    for (int f = 7; m > 1 && f <= m; f += 2)
        while (m % f == 0 && p.nstages < BLDFM_MAX_STAGES) {
            p.radix[p.nstages++] = f;
            m /= f;
        }
    if (m > 1) p.radix[p.nstages++] = m;
    fft_plan_finalize(p);
}

// solved modes of column c (Hermitian representatives plus unpaired modes),
// in the order the workspace entry point lists them
int na_col_count(int c, int nlx, int nly)
{
    const int kx = freq_of_index(c, nlx);
    const bool nyq_x = (nlx % 2 == 0) && kx == -(nlx / 2);
    const bool even_y = nly % 2 == 0;
    if (kx > 0 || nyq_x) return nly;
    if (kx == 0) return freq_max(nly) + (even_y ? 1 : 0);
    return even_y ? 1 : 0;
}

}  // namespace

// One thread per (column, row): writes the packed mode entry of solved modes.
__global__ void na_modes_kernel(int nlx, int nly, const int *__restrict__ colstart, uint32_t *__restrict__ modes)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nlx * nly) return;
    const int c = (int)(t / nly), r = (int)(t - (int64_t)c * nly);
    const int kx = freq_of_index(c, nlx), ky = freq_of_index(r, nly);
    if (kx == 0 && ky == 0) return;
    const bool mirror =
        (-kx >= freq_min(nlx) && -kx <= freq_max(nlx) && -ky >= freq_min(nly) && -ky <= freq_max(nly));
    if (!(!mirror || kx > 0 || (kx == 0 && ky > 0))) return;
    int rank;
    const bool nyq_x = (nlx % 2 == 0) && kx == -(nlx / 2);
    if (kx > 0 || nyq_x)
        rank = r;
    else if (kx == 0)
        rank = ky > 0 ? r - 1 : freq_max(nly);  // the unpaired row -nly/2 follows ky > 0
    else
        rank = 0;
    modes[colstart[c] + rank] = (uint32_t)c | ((uint32_t)r << 15) | (mirror ? 0x80000000u : 0u);
}

// twiddle table tw[m] = exp(-2 pi i m / n) in FP32 (computed in FP64)
__global__ void na_twiddle_kernel(int n, float2 *__restrict__ tw)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    double s, c;
    sincospi(-2.0 * (double)m / (double)n, &s, &c);
    tw[m] = make_float2((float)c, (float)s);
}

extern "C" int bldfm_solve_noalloc(const bldfm_desc *d, const double *srf_flx_dev, const double *z_host,
                                   const double *prof_host, const int64_t *levels_host, int32_t nlvls,
                                   double *conc_dev, double *flx_dev, void *stream)
{
    std::lock_guard<std::mutex> lk(na_mutex);
    if (!d || !z_host || !prof_host || !levels_host || !conc_dev || !flx_dev) return BLDFM_ERR_ARG;
    if ((d->nlx % 2) != 0 || (d->nly % 2) != 0) return BLDFM_ERR_ODD_MODES;
    if (d->precision != BLDFM_PREC_SINGLE && d->precision != BLDFM_PREC_DOUBLE) return BLDFM_ERR_PRECISION;
    if (d->mode != BLDFM_MODE_FP32 || d->analytic) return BLDFM_ERR_UNSUPPORTED;
    if (d->nx < 1 || d->ny < 1 || d->nz < 2 || nlvls < 1 || !(d->xmax > 0) || !(d->ymax > 0))
        return BLDFM_ERR_ARG;
    if (d->nz > BLDFM_MAX_NZ || nlvls > BLDFM_MAX_NZ) return BLDFM_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;

    // per-device set-up: device address of the scratch array
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return BLDFM_ERR_CUDA;
    if (!na_scratch_dev[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return BLDFM_ERR_CUDA;
        na_scratch_dev[dev] = p;
    }
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return BLDFM_ERR_CUDA;

    // geometry (solver.py:94-131)
    SolveGeom g;
    memset(&g, 0, sizeof(g));
    g.nx = d->nx;
    g.ny = d->ny;
    g.nz = d->nz;
    const double dx = d->xmax / d->nx, dy = d->ymax / d->ny;
    const double halo = d->has_halo ? d->halo : (d->xmax > d->ymax ? d->xmax : d->ymax);
    if (!(halo >= 0) || halo / dx > 1e7 || halo / dy > 1e7) return BLDFM_ERR_ARG;
    g.px = (int)(halo / dx);
    g.py = (int)(halo / dy);
    g.nxe = g.nx + 2 * g.px;
    g.nye = g.ny + 2 * g.py;
    int nlx = d->nlx, nly = d->nly;
    if (nlx > g.nxe || nly > g.nye) {
        nlx = g.nxe;
        nly = g.nye;
    }
    if (nlx < 1 || nly < 1 || nlx > 32767 || nly > 32767) return BLDFM_ERR_ARG;
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
    if (g.nfx > BLDFM_MAX_FFT_N || g.nfy > BLDFM_MAX_FFT_N) return BLDFM_ERR_UNSUPPORTED;
    if (!d->footprint) {
        if (!srf_flx_dev) return BLDFM_ERR_ARG;
        if (g.nxe > BLDFM_MAX_FFT_N || g.nye > BLDFM_MAX_FFT_N) return BLDFM_ERR_UNSUPPORTED;
        if ((g.nxe - nlx) % 2 != 0 || (g.nye - nly) % 2 != 0) return BLDFM_ERR_SPECTRUM_SHAPE;
    }
    const int nz = g.nz;
    for (int k = 0; k < nlvls; ++k)
        if (levels_host[k] < -(int64_t)nz || levels_host[k] >= nz) return BLDFM_ERR_ARG;
    g.nlvls = nlvls;
    g.footprint = d->footprint ? 1 : 0;
    g.precision = d->precision;
    g.mode = BLDFM_MODE_FP32;
    g.out_sign = d->footprint ? -1 : +1;
    g.valx = hx_fftfreq_val(nlx);
    g.valy = hx_fftfreq_val(nly);
    g.lx_scale = 2.0 * M_PI / dx / g.nxe;
    g.ly_scale = 2.0 * M_PI / dy / g.nye;
    g.inv_nxe = 1.0 / g.nxe;
    g.inv_nye = 1.0 / g.nye;
    g.q0dc_fp = (1.0 / g.nxe) * (1.0 / g.nye);
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
        const long double pi2 = 6.283185307179586476925286766559005768L;
        long double tx = (long double)g.lx_scale * g.valx * g.sx / pi2;
        long double ty = (long double)g.ly_scale * g.valy * g.sy / pi2;
        tx -= floorl(tx);
        ty -= floorl(ty);
        g.turn_x = (uint32_t)(uint64_t)llrintl(tx * 4294967296.0L);
        g.turn_y = (uint32_t)(uint64_t)llrintl(ty * 4294967296.0L);
    }
    {
        const double *u = prof_host, *v = prof_host + nz, *Kx = prof_host + 2 * nz, *Ky = prof_host + 3 * nz,
                     *Kz = prof_host + 4 * nz;
        const double kzinv = 1.0 / Kz[nz - 1];
        g.kz_top = Kz[nz - 1];
        g.kxk_top = Kx[nz - 1] * kzinv;
        g.kyk_top = Ky[nz - 1] * kzinv;
        g.uk_top = u[nz - 1] * kzinv;
        g.vk_top = v[nz - 1] * kzinv;
        double ex = 1.0, ey = 0.0;
        g.iso = hx_profiles_iso(nz, prof_host, &ex, &ey);
        g.ex = (float)ex;
        g.ey = (float)ey;
    }
    int ns = 0;
    for (int i = 0; i < nz; ++i) {
        na_host.slot[i] = -1;
        for (int k = 0; k < nlvls; ++k)
            if (levels_host[k] == i) {
                na_host.slot[i] = ns++;
                break;
            }
    }
    g.nsnap = ns;
    g.jmax = -1;
    for (int i = 0; i < nz; ++i)
        if (na_host.slot[i] >= 0) g.jmax = i;
    int64_t nsolved = 0;
    for (int c = 0; c < nlx; ++c) {
        na_host.colstart[c] = (int)nsolved;
        nsolved += na_col_count(c, nlx, nly);
    }
    na_host.colstart[nlx] = (int)nsolved;
    g.nsolved = nsolved;
    // band columns of the output transform (positions of frequencies [-h, h])
    int nbx = 0;
    {
        const int f0 = freq_min(nlx), f1 = freq_max(nlx);
        const int hmax = (-f0 > f1) ? -f0 : f1;
        for (int f = -hmax; f <= hmax; ++f) {
            const int pos = ((f % g.nfx) + g.nfx) % g.nfx;
            bool dup = false;
            if (f == hmax && hmax == -f0 && ((-hmax % g.nfx) + g.nfx) % g.nfx == pos) dup = true;
            if (dup) continue;
            auto colof = [&](int p) -> int {
                if (p <= f1) return p;
                if (p >= g.nfx + f0) return p - g.nfx + nlx;
                return -1;
            };
            const int a = colof(pos), b = colof((g.nfx - pos) % g.nfx);
            if (a < 0 && b < 0) continue;
            na_host.xband[nbx++] = make_int4(pos, a, b, 0);
        }
    }
    g.nbx = nbx;
    FftPlan plx_out, ply_out, plx_fwd, ply_fwd;
    na_factorize(g.nfx, plx_out);
    na_factorize(g.nfy, ply_out);
    na_factorize(g.nxe, plx_fwd);
    na_factorize(g.nye, ply_fwd);

    // carve the scratch array
    const int L = nz - 1;
    size_t o = 0;
    const size_t o_err = o;
    o = na_al(o + 64);
    const size_t o_lv64 = o;
    o = na_al(o + (size_t)L * BLDFM_LV64 * 8);
    const size_t o_lv32 = o;
    o = na_al(o + (size_t)L * BLDFM_LV32 * 4);
    const size_t o_slot = o;
    o = na_al(o + (size_t)nz * 4);
    const size_t o_dc = o;
    o = na_al(o + (size_t)nlvls * 32);
    const size_t o_cs = o;
    o = na_al(o + (size_t)(nlx + 1) * 4);
    const size_t o_modes = o;
    o = na_al(o + (size_t)(nsolved > 0 ? nsolved : 1) * 4);
    const size_t o_xb = o;
    o = na_al(o + (size_t)(nbx > 0 ? nbx : 1) * 16);
    const size_t o_twxo = o;
    o = na_al(o + (size_t)g.nfx * 8);
    const size_t o_twyo = o;
    o = na_al(o + (size_t)g.nfy * 8);
    const size_t o_twxf = o;
    o = na_al(o + (d->footprint ? 0 : (size_t)g.nxe * 8));
    const size_t o_twyf = o;
    o = na_al(o + (d->footprint ? 0 : (size_t)g.nye * 8));
    const size_t o_snap = o;
    o = na_al(o + (ns > 1 ? (size_t)ns * 5 * nsolved * 4 : 0));
    const size_t o_q0 = o;
    o = na_al(o + (d->footprint ? 0 : (size_t)nlx * nly * 8));
    const size_t o_A = o;
    o = na_al(o + (d->footprint ? 0 : (size_t)nlx * g.ny * 8));
    const size_t specb = (size_t)nlvls * nlx * nly * 8;
    const size_t o_Xp = o;
    o = na_al(o + specb);
    const size_t o_Xq = o;
    o = na_al(o + specb);
    const size_t o_Cb = o;
    o = na_al(o + (size_t)nlvls * nbx * (g.out_ny > 0 ? g.out_ny : 1) * 8);
    if (o > BLDFM_NOALLOC_SCRATCH_BYTES) return BLDFM_ERR_WORKSPACE;

    char *w = (char *)na_scratch_dev[dev];
    if (d->footprint)
        hx_level_dz_w(nz, z_host, prof_host, na_host.lv64);  // the k = 0 values read only these columns
    else
        hx_level_table(nz, z_host, prof_host, na_host.lv64);
    if (g.iso)
        hx_level_table32_iso(nz, z_host, prof_host, g.ex, g.ey, na_host.lv32);
    else
        hx_level_table32(nz, z_host, prof_host, na_host.lv32);
#define NA_CK(x)                                                                                                       \
    do {                                                                                                               \
        if ((x) != cudaSuccess) return BLDFM_ERR_CUDA;                                                                 \
    } while (0)
    // pageable host -> device copies: they return once the host buffer is read
    NA_CK(cudaMemsetAsync(w + o_err, 0, 64, st));
    NA_CK(cudaMemcpyAsync(w + o_lv64, na_host.lv64, (size_t)L * BLDFM_LV64 * 8, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(w + o_lv32, na_host.lv32, (size_t)L * BLDFM_LV32 * 4, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(w + o_slot, na_host.slot, (size_t)nz * 4, cudaMemcpyHostToDevice, st));
    if (d->footprint) {
        hx_dc_values(nz, na_host.lv64, na_host.slot, g.q0dc_fp, 0.0, d->srf_bg_conc, d->precision == BLDFM_PREC_SINGLE,
                     nlvls, 0, na_host.dc);
        NA_CK(cudaMemcpyAsync(w + o_dc, na_host.dc, (size_t)nlvls * 32, cudaMemcpyHostToDevice, st));
    }
    NA_CK(cudaMemcpyAsync(w + o_cs, na_host.colstart, (size_t)(nlx + 1) * 4, cudaMemcpyHostToDevice, st));
    if (nbx > 0) NA_CK(cudaMemcpyAsync(w + o_xb, na_host.xband, (size_t)nbx * 16, cudaMemcpyHostToDevice, st));
    // the spectra start at zero when some output slot stays empty
    if (ns < nlvls) {
        NA_CK(cudaMemsetAsync(w + o_Xp, 0, specb, st));
        NA_CK(cudaMemsetAsync(w + o_Xq, 0, specb, st));
    }
    const int64_t nm = (int64_t)nlx * nly;
    na_modes_kernel<<<(unsigned)((nm + 255) / 256), 256, 0, st>>>(nlx, nly, (const int *)(w + o_cs),
                                                                  (uint32_t *)(w + o_modes));
    na_twiddle_kernel<<<(g.nfx + 255) / 256, 256, 0, st>>>(g.nfx, (float2 *)(w + o_twxo));
    na_twiddle_kernel<<<(g.nfy + 255) / 256, 256, 0, st>>>(g.nfy, (float2 *)(w + o_twyo));
    float2 *q0 = nullptr;
    if (!d->footprint) {
        na_twiddle_kernel<<<(g.nxe + 255) / 256, 256, 0, st>>>(g.nxe, (float2 *)(w + o_twxf));
        na_twiddle_kernel<<<(g.nye + 255) / 256, 256, 0, st>>>(g.nye, (float2 *)(w + o_twyf));
        q0 = (float2 *)(w + o_q0);
        NA_CK(launch_forward_fft<float>(g, plx_fwd, ply_fwd, (const float2 *)(w + o_twxf),
                                        (const float2 *)(w + o_twyf), srf_flx_dev, (float2 *)(w + o_A), q0, st));
    }
    NA_CK(cudaGetLastError());
    float2 *Xp = (float2 *)(w + o_Xp), *Xq = (float2 *)(w + o_Xq);
    const float ax = (float)(g.lx_scale * g.valx), ay = (float)(g.ly_scale * g.valy);
    if (nsolved > 0)
        NA_CK(launch_riccati32(g, (const float *)(w + o_lv32), (const int *)(w + o_slot),
                               (const uint32_t *)(w + o_modes), q0, (float *)(w + o_snap), Xp, Xq, ax, ay,
                               (int *)(w + o_err), nsm, 256, st));
    if (!d->footprint)
        NA_CK(launch_trapezoid32(g, (const double *)(w + o_lv64), (const int *)(w + o_slot), q0, d->srf_bg_conc,
                                 (double2 *)(w + o_dc), st));
    NA_CK(launch_output_fft<float>(g, plx_out, ply_out, (const float2 *)(w + o_twxo), (const float2 *)(w + o_twyo),
                                   (const int4 *)(w + o_xb), Xp, Xq, (const double2 *)(w + o_dc), (float2 *)(w + o_Cb),
                                   conc_dev, flx_dev, (int *)(w + o_err), st));
    return BLDFM_OK;
}
