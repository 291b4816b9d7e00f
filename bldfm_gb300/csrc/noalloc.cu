// Allocation-free FP32 solve: bldfm_solve_noalloc (include/bldfm_gb300.h).
//
// Who needs it: callers that may not allocate GPU memory at solve time --
// embedded or real-time hosts that reserve all device memory up front and
// treat a later cudaMalloc as a failure, and plugin hosts whose allocator
// policy forbids cudaMalloc from third-party libraries (the host owns every
// allocation and accounts for it).  They pass inputs and outputs; every
// intermediate the solve needs (twiddle tables, mode list, band table, level
// tables, spectra, transform intermediate) lives in one file-scope device
// array of BLDFM_NOALLOC_SCRATCH_BYTES (16 MiB).  Every GPU that loads this
// library holds that array until the process exits.
//
// Rules of use:
//  - The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current.
//  - Calls are not for stream capture: the small host tables are copied from
//    the static pageable buffer na_host, which every call rewrites (a graph
//    would replay the buffer's contents at replay time).
//  - All calls share the one array and it keeps the previous call's contents;
//    this file clears what must start at zero.  Calls whose GPU work overlaps
//    (different streams, or different host threads without ordering) race on
//    the array: serialise them on one stream.
//  - FP32 mode only (the FP64 mode needs host-side libm values staged in
//    pinned memory); problems whose scratch exceeds the array are rejected
//    with BLDFM_ERR_WORKSPACE.
//  - The device status of the call (a bounded wait that ran out, or a
//    non-finite output value) is copied to the caller's status word when the
//    stream reaches the end of the call.
// Nothing here calls cudaMalloc, cudaFree, cudaHostAlloc or any other
// allocating routine, and the host side uses fixed static buffers.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "../../include/bldfm_gb300.h"
#include "common.h"
#include "geometry.h"
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
                                   double *conc_dev, double *flx_dev, int32_t *status_dev, void *stream)
{
    std::lock_guard<std::mutex> lk(na_mutex);
    if (!d || !z_host || !prof_host || !levels_host || !conc_dev || !flx_dev) return BLDFM_ERR_ARG;
    if (d->nz > BLDFM_MAX_NZ || nlvls > BLDFM_MAX_NZ) return BLDFM_ERR_UNSUPPORTED;
    // geometry and input checks shared with every other entry point
    SolveGeom g;
    bool shape_ok = true;
    int rc = solve_geometry(d, z_host, prof_host, levels_host, nlvls, g, na_host.slot, &shape_ok);
    if (rc != BLDFM_OK) return rc;
    if (d->mode != BLDFM_MODE_FP32 || d->analytic) return BLDFM_ERR_UNSUPPORTED;
    if (d->nz < 2) return BLDFM_ERR_ARG;  // at least one sweep step
    if (!d->footprint && !srf_flx_dev) return BLDFM_ERR_ARG;
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

    const int nz = g.nz, nlx = g.nlx, nly = g.nly, ns = g.nsnap;
    const int64_t nsolved = g.nsolved;
    {
        int64_t acc = 0;
        for (int c = 0; c < nlx; ++c) {
            na_host.colstart[c] = (int)acc;
            acc += solved_in_column(c, nlx, nly);
        }
        na_host.colstart[nlx] = (int)acc;
    }
    const int nbx = band_columns(nlx, g.nfx, na_host.xband);
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
        hx_level_table32_iso(nz, z_host, prof_host, g.ex, g.ey, na_host.lv32, nullptr);
    else
        hx_level_table32(nz, z_host, prof_host, na_host.lv32, nullptr);
#define NA_CK(x)                                                                                                       \
    do {                                                                                                               \
        if ((x) != cudaSuccess) return BLDFM_ERR_CUDA;                                                                 \
    } while (0)
    // pageable host -> device copies: they return once the host buffer is read
    // (outside a stream capture)
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
    if (status_dev)
        NA_CK(cudaMemcpyAsync(status_dev, w + o_err, sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
    return BLDFM_OK;
}
