// C ABI of bldfm_gb300 (include/bldfm_gb300.h): host planning, per-device
// plan cache, workspace layout and the orchestration of one solve.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/bldfm_gb300.h"
#include "common.h"
#include "host_exact.h"
#include "kernels.h"

#ifndef BLDFM_VERSION_STR
#define BLDFM_VERSION_STR "bldfm_gb300 0.1 sm_103a"
#endif

namespace {

std::mutex g_mutex;

// ---------------------------------------------------------------------------
// geometry of one solve (solver.py:94-131, 264-290)
// ---------------------------------------------------------------------------
struct HostPlan {
    SolveGeom g;
    FftPlan plx_fwd, ply_fwd, plx_out, ply_out;
    std::vector<int> slot;  // nz entries
    std::vector<int4> xband;
    bool shape_ok;          // truncated source spectrum matches modes
};

void factorize(int n, FftPlan &p)
{
    p.n = n;
    p.nstages = 0;
    int m = n;
    const int pref[] = {8, 4, 2, 3, 5};
    for (int r : pref) {
        while (m % r == 0 && p.nstages < BLDFM_MAX_STAGES) {
            p.radix[p.nstages++] = r;
            m /= r;
        }
    }
    for (int f = 7; m > 1 && f <= m; f += 2) {
        while (m % f == 0 && p.nstages < BLDFM_MAX_STAGES) {
            p.radix[p.nstages++] = f;
            m /= f;
        }
    }
    if (m > 1) p.radix[p.nstages++] = m;
}

int64_t count_and_fill_modes(int nlx, int nly, std::vector<uint32_t> *out);

// number of solved modes per (nlx, nly), memoised (called under g_mutex)
int64_t solved_count(int nlx, int nly)
{
    static std::map<std::pair<int, int>, int64_t> memo;
    auto key = std::make_pair(nlx, nly);
    auto it = memo.find(key);
    if (it != memo.end()) return it->second;
    const int64_t n = count_and_fill_modes(nlx, nly, nullptr);
    memo[key] = n;
    return n;
}

int64_t count_and_fill_modes(int nlx, int nly, std::vector<uint32_t> *out)
{
    const int fx0 = freq_min(nlx), fx1 = freq_max(nlx), fy0 = freq_min(nly), fy1 = freq_max(nly);
    int64_t cnt = 0;
    for (int c = 0; c < nlx; ++c) {
        const int kx = freq_of_index(c, nlx);
        for (int r = 0; r < nly; ++r) {
            const int ky = freq_of_index(r, nly);
            if (kx == 0 && ky == 0) continue;
            const bool mirror = (-kx >= fx0 && -kx <= fx1 && -ky >= fy0 && -ky <= fy1);
            if (!mirror || kx > 0 || (kx == 0 && ky > 0)) {
                if (out) out->push_back((uint32_t)c | ((uint32_t)r << 15) | (mirror ? 0x80000000u : 0u));
                ++cnt;
            }
        }
    }
    return cnt;
}

int make_plan(const bldfm_desc *d, const double *z, const double *prof, const int64_t *levels, int nlvls,
              HostPlan &hp)
{
    if (!d) return BLDFM_ERR_ARG;
    if ((d->nlx % 2) != 0 || (d->nly % 2) != 0) return BLDFM_ERR_ODD_MODES;
    if (d->precision != BLDFM_PREC_SINGLE && d->precision != BLDFM_PREC_DOUBLE) return BLDFM_ERR_PRECISION;
    if (d->nx < 1 || d->ny < 1 || d->nz < 1 || d->nlx < 0 || d->nly < 0 || nlvls < 1) return BLDFM_ERR_ARG;
    if (d->mode != BLDFM_MODE_FP64 && d->mode != BLDFM_MODE_FP32) return BLDFM_ERR_ARG;
    if (!(d->xmax > 0) || !(d->ymax > 0)) return BLDFM_ERR_ARG;
    if (d->nz > BLDFM_MAX_NZ) return BLDFM_ERR_UNSUPPORTED;
    SolveGeom &g = hp.g;
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
    if (nlx > g.nxe || nly > g.nye) {
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
    g.out_ny = std::min(g.nye - g.py, g.nfy) - g.py;
    g.out_nx = std::min(g.nxe - g.px, g.nfx) - g.px;
    if (g.out_ny < 0) g.out_ny = 0;
    if (g.out_nx < 0) g.out_nx = 0;
    if (nlx > 32767 || nly > 32767) return BLDFM_ERR_UNSUPPORTED;
    if (g.nfx > BLDFM_MAX_FFT_N || g.nfy > BLDFM_MAX_FFT_N) return BLDFM_ERR_UNSUPPORTED;
    if (!d->footprint && (g.nxe > BLDFM_MAX_FFT_N || g.nye > BLDFM_MAX_FFT_N)) return BLDFM_ERR_UNSUPPORTED;
    hp.shape_ok = ((g.nxe - nlx) % 2 == 0) && ((g.nye - nly) % 2 == 0);
    if (!d->footprint && !hp.shape_ok) return BLDFM_ERR_SPECTRUM_SHAPE;
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
    if (d->footprint) {
        g.do_shift = 1;
        g.sx = d->meas_x + halo;
        g.sy = d->meas_y + halo;
    } else if (d->meas_x * d->meas_x + d->meas_y * d->meas_y > 0.0) {
        g.do_shift = 1;
        g.sx = d->meas_x - d->xmax / 2;
        g.sy = d->meas_y - d->ymax / 2;
    }
    // phase shift as fixed-point turns for the FP32 path
    {
        long double tx = (long double)g.lx_scale * g.valx * g.sx / (2.0L * 3.14159265358979323846264338327950288L);
        long double ty = (long double)g.ly_scale * g.valy * g.sy / (2.0L * 3.14159265358979323846264338327950288L);
        tx -= floorl(tx);
        ty -= floorl(ty);
        g.turn_x = (uint32_t)(uint64_t)llrintl(tx * 4294967296.0L);
        g.turn_y = (uint32_t)(uint64_t)llrintl(ty * 4294967296.0L);
    }
    const int nz = d->nz;
    if (z && prof) {
        const double *u = prof, *v = prof + nz, *Kx = prof + 2 * nz, *Ky = prof + 3 * nz, *Kz = prof + 4 * nz;
        const double kzinv = 1.0 / Kz[nz - 1];
        g.kz_top = Kz[nz - 1];
        g.kxk_top = Kx[nz - 1] * kzinv;
        g.kyk_top = Ky[nz - 1] * kzinv;
        g.uk_top = u[nz - 1] * kzinv;
        g.vk_top = v[nz - 1] * kzinv;
    }
    // snapshot schedule (solver.py:350-372): slot s = s-th distinct level in [0, nz-1]
    hp.slot.assign(nz, -1);
    int ns = 0;
    if (levels) {
        for (int i = 0; i < nz; ++i) {
            for (int k = 0; k < nlvls; ++k)
                if (levels[k] == i) {
                    hp.slot[i] = ns++;
                    break;
                }
        }
        for (int k = 0; k < nlvls; ++k)
            if (levels[k] < -(int64_t)nz || levels[k] >= nz) return BLDFM_ERR_ARG;
    }
    g.nsnap = ns;
    g.nsolved = solved_count(nlx, nly);
    // output band columns: positions of frequencies [-h, h] mod nfx
    hp.xband.clear();
    {
        const int f0 = freq_min(nlx), f1 = freq_max(nlx);
        const int hmax = std::max(-f0, f1);
        std::vector<char> seen(g.nfx, 0);
        for (int f = -hmax; f <= hmax; ++f) {
            const int pos = ((f % g.nfx) + g.nfx) % g.nfx;
            if (seen[pos]) continue;
            seen[pos] = 1;
            auto colof = [&](int p) -> int {
                if (p <= f1) return p;  // non-negative frequencies
                if (p >= g.nfx + f0) return p - g.nfx + nlx;
                return -1;
            };
            const int a = colof(pos);
            const int b = colof((g.nfx - pos) % g.nfx);
            if (a < 0 && b < 0) continue;
            hp.xband.push_back(make_int4(pos, a, b, 0));
        }
    }
    g.nbx = (int)hp.xband.size();
    factorize(g.nxe, hp.plx_fwd);
    factorize(g.nye, hp.ply_fwd);
    factorize(g.nfx, hp.plx_out);
    factorize(g.nfy, hp.ply_out);
    return BLDFM_OK;
}

// ---------------------------------------------------------------------------
// workspace layout
// ---------------------------------------------------------------------------
struct Layout {
    size_t err, lv64, lv32, slot, eig, snap, top, q0, A, Xp, Xq, Cb, scratch, total;
};

inline size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

Layout layout_for(const SolveGeom &g)
{
    Layout L;
    const bool f64 = g.mode == BLDFM_MODE_FP64 || g.analytic;
    const size_t ce = f64 ? 16 : 8;  // complex element size
    const size_t ns = (size_t)g.nsolved;
    size_t o = 0;
    L.err = o;
    o = al(o + 64);
    L.lv64 = o;
    o = al(o + (size_t)std::max(g.nz - 1, 1) * BLDFM_LV64 * 8);
    L.lv32 = o;
    o = al(o + (size_t)std::max(g.nz - 1, 1) * BLDFM_LV32 * 4);
    L.slot = o;
    o = al(o + (size_t)g.nz * 4);
    L.eig = o;
    o = al(o + (f64 ? ns * 16 : 0));
    L.snap = o;
    o = al(o + ((f64 && !g.analytic) ? (size_t)g.nsnap * 4 * ns * 16 : 0));
    L.top = o;
    o = al(o + ((f64 && !g.analytic) ? 4 * ns * 16 : 0));
    L.scratch = o;
    o = al(o + ((!f64 && g.nsnap > 1) ? (size_t)g.nsnap * 5 * ns * 4 : 0));
    L.q0 = o;
    o = al(o + (g.footprint ? 0 : (size_t)g.nlx * g.nly * ce));
    L.A = o;
    o = al(o + (g.footprint ? 0 : (size_t)g.nlx * g.ny * ce));
    L.Xp = o;
    o = al(o + (size_t)g.nlvls * g.nlx * g.nly * ce);
    L.Xq = o;
    o = al(o + (size_t)g.nlvls * g.nlx * g.nly * ce);
    L.Cb = o;
    o = al(o + (size_t)g.nlvls * g.nbx * std::max(g.out_ny, 1) * ce);
    L.total = o;
    return L;
}

// ---------------------------------------------------------------------------
// per-device cache: twiddle tables, mode lists, band tables, pinned staging
// ---------------------------------------------------------------------------
struct TwTable {
    double2 *d64 = nullptr;
    float2 *d32 = nullptr;
};
struct ModeList {
    uint32_t *dev = nullptr;
    std::vector<uint32_t> host;
};
struct HostBuffers {
    void *ws = nullptr;
    size_t ws_bytes = 0;
    double *srf = nullptr;
    size_t srf_bytes = 0;
    double *conc = nullptr, *flx = nullptr;
    size_t out_bytes = 0;
    cudaStream_t stream = nullptr;
};
// A pinned upload buffer; its event marks the last copy out of it.
struct StageSlot {
    void *buf = nullptr;
    size_t bytes = 0;
    cudaEvent_t ev = nullptr;
};
enum { NSTAGE = 8, NTIMER = 8, NTSETS = 1024 };
// CUDA events of one solve's stage boundaries
struct TimerSet {
    cudaEvent_t ev[NTIMER + 1] = {};
    int used = 0;
};
struct DeviceCache {
    int nsm = 0;
    std::map<int, TwTable> tw;
    std::map<std::pair<int, int>, ModeList> modes;
    std::map<std::vector<int>, int4 *> xband;
    StageSlot stage[NSTAGE];  // ring of pinned staging buffers
    int stage_next = 0;
    HostBuffers hb;
    bool timing = false;       // per-stage CUDA-event timers
    std::vector<TimerSet> tsets;
    TimerSet *cur = nullptr;   // timers of the solve being enqueued
    int tnext = 0, tpending = 0;
};

std::map<int, DeviceCache> g_cache;

DeviceCache &cache_for_current(int *status)
{
    int dev = 0;
    cudaGetDevice(&dev);
    DeviceCache &dc = g_cache[dev];
    if (dc.nsm == 0) {
        cudaDeviceGetAttribute(&dc.nsm, cudaDevAttrMultiProcessorCount, dev);
        if (dc.nsm <= 0) dc.nsm = 1;
        for (int i = 0; i < NSTAGE; ++i)
            if (cudaEventCreateWithFlags(&dc.stage[i].ev, cudaEventDisableTiming) != cudaSuccess)
                *status = BLDFM_ERR_CUDA;
    }
    return dc;
}

int get_tw(DeviceCache &dc, int n, TwTable **out)
{
    auto it = dc.tw.find(n);
    if (it != dc.tw.end()) {
        *out = &it->second;
        return BLDFM_OK;
    }
    std::vector<double2> h(n);
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (int m = 0; m < n; ++m) {
        long double a = -two_pi * (long double)m / (long double)n;
        h[m] = make_double2((double)cosl(a), (double)sinl(a));
    }
    TwTable t;
    if (cudaMalloc(&t.d64, sizeof(double2) * n) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (cudaMalloc(&t.d32, sizeof(float2) * n) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (cudaMemcpy(t.d64, h.data(), sizeof(double2) * n, cudaMemcpyHostToDevice) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (launch_tw_to_float(t.d64, t.d32, n, 0) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) return BLDFM_ERR_CUDA;
    dc.tw[n] = t;
    *out = &dc.tw[n];
    return BLDFM_OK;
}

int get_modes(DeviceCache &dc, int nlx, int nly, ModeList **out)
{
    auto key = std::make_pair(nlx, nly);
    auto it = dc.modes.find(key);
    if (it != dc.modes.end()) {
        *out = &it->second;
        return BLDFM_OK;
    }
    ModeList ml;
    count_and_fill_modes(nlx, nly, &ml.host);
    const size_t bytes = std::max<size_t>(ml.host.size(), 1) * sizeof(uint32_t);
    if (cudaMalloc(&ml.dev, bytes) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (!ml.host.empty() &&
        cudaMemcpy(ml.dev, ml.host.data(), ml.host.size() * sizeof(uint32_t), cudaMemcpyHostToDevice) != cudaSuccess)
        return BLDFM_ERR_CUDA;
    dc.modes[key] = std::move(ml);
    *out = &dc.modes[key];
    return BLDFM_OK;
}

int get_xband(DeviceCache &dc, const HostPlan &hp, int4 **out)
{
    std::vector<int> key;
    key.push_back(hp.g.nfx);
    key.push_back(hp.g.nlx);
    auto it = dc.xband.find(key);
    if (it != dc.xband.end()) {
        *out = it->second;
        return BLDFM_OK;
    }
    int4 *d = nullptr;
    const size_t bytes = std::max<size_t>(hp.xband.size(), 1) * sizeof(int4);
    if (cudaMalloc(&d, bytes) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (!hp.xband.empty() &&
        cudaMemcpy(d, hp.xband.data(), hp.xband.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess)
        return BLDFM_ERR_CUDA;
    dc.xband[key] = d;
    *out = d;
    return BLDFM_OK;
}

// Next slot of the staging ring, grown to `bytes`; waits only for the copies
// that last read this slot (NSTAGE solves ago), not for whole solves.
int acquire_stage(DeviceCache &dc, size_t bytes, StageSlot **out)
{
    StageSlot &sl = dc.stage[dc.stage_next];
    dc.stage_next = (dc.stage_next + 1) % NSTAGE;
    if (cudaEventSynchronize(sl.ev) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (bytes > sl.bytes) {
        if (sl.buf) cudaFreeHost(sl.buf);
        sl.buf = nullptr;
        sl.bytes = 0;
        size_t want = std::max(bytes, (size_t)1 << 20);
        if (cudaHostAlloc(&sl.buf, want, cudaHostAllocDefault) != cudaSuccess) return BLDFM_ERR_CUDA;
        sl.bytes = want;
    }
    *out = &sl;
    return BLDFM_OK;
}

// stage timers: event k is recorded before stage k
inline void tmark(DeviceCache &dc, cudaStream_t st)
{
    if (!dc.timing || !dc.cur || dc.cur->used > NTIMER) return;
    cudaEventRecord(dc.cur->ev[dc.cur->used++], st);
}

inline void timers_begin(DeviceCache &dc)
{
    dc.cur = nullptr;
    if (!dc.timing) return;
    if (dc.tsets.empty()) {
        dc.tsets.resize(NTSETS);
        for (auto &t : dc.tsets)
            for (int i = 0; i <= NTIMER; ++i) cudaEventCreate(&t.ev[i]);
    }
    if (dc.tpending >= NTSETS) return;  // full: further solves are not timed
    dc.cur = &dc.tsets[dc.tnext];
    dc.tnext = (dc.tnext + 1) % NTSETS;
    dc.tpending++;
    dc.cur->used = 0;
}

void eigval_parallel(const ModeList &ml, const SolveGeom &g, const double *prof, int nz, double *eig)
{
    const double *u = prof, *v = prof + nz, *Kx = prof + 2 * nz, *Ky = prof + 3 * nz, *Kz = prof + 4 * nz;
    const int64_t n = (int64_t)ml.host.size();
    unsigned hw = std::thread::hardware_concurrency();
    int nt = (int)std::min<int64_t>(std::max(1u, std::min(hw, 32u)), n / 16384 + 1);
    auto work = [&](int64_t a, int64_t b) {
        hx_eigval(a, b, ml.host.data(), g.nlx, g.nly, g.valx, g.valy, g.lx_scale, g.ly_scale, Kx[nz - 1],
                  Ky[nz - 1], Kz[nz - 1], u[nz - 1], v[nz - 1], eig);
    };
    if (nt <= 1) {
        work(0, n);
        return;
    }
    std::vector<std::thread> th;
    const int64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) {
        int64_t a = t * chunk, b = std::min(n, a + chunk);
        if (a < b) th.emplace_back(work, a, b);
    }
    for (auto &t : th) t.join();
}

#define CK(x)                                                                                                          \
    do {                                                                                                               \
        if ((x) != cudaSuccess) return BLDFM_ERR_CUDA;                                                                 \
    } while (0)

int solve_impl(const bldfm_desc *d, const double *srf_dev, const double *z, const double *prof,
               const int64_t *levels, int nlvls, double *conc, double *flx, void *ws, size_t ws_bytes,
               cudaStream_t st)
{
    if (!z || !prof || !levels || !conc || !flx || !ws) return BLDFM_ERR_ARG;
    HostPlan hp;
    int rc = make_plan(d, z, prof, levels, nlvls, hp);
    if (rc != BLDFM_OK) return rc;
    SolveGeom g = hp.g;
    if (!g.footprint && !srf_dev) return BLDFM_ERR_ARG;
    const Layout L = layout_for(g);
    if (ws_bytes < L.total) return BLDFM_ERR_WORKSPACE;
    if (((uintptr_t)ws & 255) != 0) return BLDFM_ERR_ARG;
    int status = BLDFM_OK;
    DeviceCache &dc = cache_for_current(&status);
    if (status != BLDFM_OK) return status;
    const bool f64 = g.mode == BLDFM_MODE_FP64 || g.analytic;
    ModeList *ml = nullptr;
    TwTable *twxo = nullptr, *twyo = nullptr, *twxf = nullptr, *twyf = nullptr;
    int4 *xband = nullptr;
    if ((rc = get_modes(dc, g.nlx, g.nly, &ml)) != BLDFM_OK) return rc;
    if ((rc = get_tw(dc, g.nfx, &twxo)) != BLDFM_OK) return rc;
    if ((rc = get_tw(dc, g.nfy, &twyo)) != BLDFM_OK) return rc;
    if (!g.footprint) {
        if ((rc = get_tw(dc, g.nxe, &twxf)) != BLDFM_OK) return rc;
        if ((rc = get_tw(dc, g.nye, &twyf)) != BLDFM_OK) return rc;
    }
    if ((rc = get_xband(dc, hp, &xband)) != BLDFM_OK) return rc;

    char *w = (char *)ws;
    int *err = (int *)(w + L.err);
    double *lv64 = (double *)(w + L.lv64);
    float *lv32 = (float *)(w + L.lv32);
    int *slot = (int *)(w + L.slot);
    const int nz = g.nz;

    // stage per-call host data: level tables and the snapshot schedule
    const size_t lv64b = (size_t)std::max(nz - 1, 0) * BLDFM_LV64 * 8;
    const size_t lv32b = (size_t)std::max(nz - 1, 0) * BLDFM_LV32 * 4;
    const size_t slotb = (size_t)nz * 4;
    const size_t eigb = f64 ? (size_t)g.nsolved * 16 : 0;
    const size_t off_lv32 = al(lv64b), off_slot = off_lv32 + al(lv32b), off_eig = off_slot + al(slotb);
    StageSlot *slt = nullptr;
    if ((rc = acquire_stage(dc, off_eig + al(eigb) + 256, &slt)) != BLDFM_OK) return rc;
    char *sg = (char *)slt->buf;
    timers_begin(dc);
    hx_level_table(nz, z, prof, (double *)sg);
    if (!f64) hx_level_table32(nz, z, prof, (float *)(sg + off_lv32));
    memcpy(sg + off_slot, hp.slot.data(), slotb);

    CK(cudaMemsetAsync(err, 0, 64, st));
    if (lv64b) CK(cudaMemcpyAsync(lv64, sg, lv64b, cudaMemcpyHostToDevice, st));
    if (!f64 && lv32b) CK(cudaMemcpyAsync(lv32, sg + off_lv32, lv32b, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(slot, sg + off_slot, slotb, cudaMemcpyHostToDevice, st));
    // every spectrum entry is written unless some output slot stays empty
    // (duplicate levels) or the analytic branch runs
    const size_t specb = (size_t)g.nlvls * g.nlx * g.nly * (f64 ? 16 : 8);
    if (g.nsnap < g.nlvls || g.analytic) {
        CK(cudaMemsetAsync(w + L.Xp, 0, specb, st));
        CK(cudaMemsetAsync(w + L.Xq, 0, specb, st));
    }
    tmark(dc, st);  // 0: before the forward transform

    const double p000 = d->srf_bg_conc;
    if (f64) {
        double2 *q0 = g.footprint ? nullptr : (double2 *)(w + L.q0);
        if (!g.footprint)
            CK(launch_forward_fft<double>(g, hp.plx_fwd, hp.ply_fwd, twxf->d64, twyf->d64, srf_dev,
                                          (double2 *)(w + L.A), q0, st));
        tmark(dc, st);  // 1: before the sweep
        double2 *eig = (double2 *)(w + L.eig);
        double2 *Xp = (double2 *)(w + L.Xp), *Xq = (double2 *)(w + L.Xq);
        if (g.analytic) {
            eigval_parallel(*ml, g, prof, nz, (double *)(sg + off_eig));
            if (eigb) CK(cudaMemcpyAsync(eig, sg + off_eig, eigb, cudaMemcpyHostToDevice, st));
            const int64_t lev = levels[0] < 0 ? levels[0] + nz : levels[0];
            const double hlev = z[lev] - z[0];
            const double kzinv = 1.0 / prof[4 * nz + nz - 1];
            CK(launch_analytic64(g, ml->dev, eig, q0, p000, kzinv, hlev, Xp, Xq, st));
        } else {
            double2 *snap = (double2 *)(w + L.snap), *top = (double2 *)(w + L.top);
            if (g.nsolved > 0) CK(launch_sweep64(g, lv64, slot, ml->dev, q0, snap, top, err, dc.nsm, st));
            tmark(dc, st);  // 2: after the sweep
            // the host evaluates libm csqrt for every mode while the device sweeps
            eigval_parallel(*ml, g, prof, nz, (double *)(sg + off_eig));
            if (eigb) CK(cudaMemcpyAsync(eig, sg + off_eig, eigb, cudaMemcpyHostToDevice, st));
            CK(cudaEventRecord(slt->ev, st));
            CK(launch_combine64(g, ml->dev, eig, snap, top, Xp, Xq, st));
            CK(launch_trapezoid64(g, lv64, slot, q0, p000, Xp, Xq, st));
        }
        tmark(dc, st);  // 3: before the output transform
        CK(launch_output_fft<double>(g, hp.plx_out, hp.ply_out, twxo->d64, twyo->d64, xband, Xp, Xq,
                                     (double2 *)(w + L.Cb), conc, flx, st));
    } else {
        float2 *q0 = g.footprint ? nullptr : (float2 *)(w + L.q0);
        if (!g.footprint)
            CK(launch_forward_fft<float>(g, hp.plx_fwd, hp.ply_fwd, twxf->d32, twyf->d32, srf_dev,
                                         (float2 *)(w + L.A), q0, st));
        CK(cudaEventRecord(slt->ev, st));
        tmark(dc, st);  // 1: before the sweep
        float2 *Xp = (float2 *)(w + L.Xp), *Xq = (float2 *)(w + L.Xq);
        const float ax = (float)(g.lx_scale * g.valx), ay = (float)(g.ly_scale * g.valy);
        if (g.nsolved > 0)
            CK(launch_riccati32(g, lv32, slot, ml->dev, q0, (float *)(w + L.scratch), Xp, Xq, ax, ay, err, dc.nsm,
                                256, st));
        tmark(dc, st);  // 2: after the sweep
        CK(launch_trapezoid32(g, lv64, slot, q0, p000, Xp, Xq, st));
        tmark(dc, st);  // 3: before the output transform
        CK(launch_output_fft<float>(g, hp.plx_out, hp.ply_out, twxo->d32, twyo->d32, xband, Xp, Xq,
                                    (float2 *)(w + L.Cb), conc, flx, st));
    }
    tmark(dc, st);  // 4: end
    if (f64 && g.analytic) CK(cudaEventRecord(slt->ev, st));
    return BLDFM_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// exported entry points
// ---------------------------------------------------------------------------
extern "C" {

const char *bldfm_status_str(int s)
{
    switch (s) {
    case BLDFM_OK: return "ok";
    case BLDFM_ERR_ODD_MODES: return "modes must consist of even numbers.";
    case BLDFM_ERR_PRECISION: return "precision must be single (default) or double.";
    case BLDFM_ERR_ARG: return "invalid argument";
    case BLDFM_ERR_SPECTRUM_SHAPE: return "truncated source spectrum does not match the number of modes";
    case BLDFM_ERR_BROADCAST: return "analytic solution supports a single output level";
    case BLDFM_ERR_UNSUPPORTED: return "grid larger than the supported transform length";
    case BLDFM_ERR_WORKSPACE: return "workspace too small";
    case BLDFM_ERR_CUDA: return "CUDA runtime error";
    case BLDFM_ERR_TIMEOUT: return "device wait timed out";
    case BLDFM_ERR_NONFINITE: return "non-finite values in the output";
    default: return "unknown status";
    }
}

const char *bldfm_version(void) { return BLDFM_VERSION_STR; }

int bldfm_set_stage_timing(int enable)
{
    std::lock_guard<std::mutex> lk(g_mutex);
    int status = BLDFM_OK;
    DeviceCache &dc = cache_for_current(&status);
    if (status != BLDFM_OK) return status;
    dc.timing = enable != 0;
    dc.tpending = 0;
    dc.tnext = 0;
    return BLDFM_OK;
}

int bldfm_stage_times(float *ms, int n)
{
    std::lock_guard<std::mutex> lk(g_mutex);
    int status = BLDFM_OK;
    DeviceCache &dc = cache_for_current(&status);
    if (status != BLDFM_OK) return status;
    if (!ms || n < 1) return BLDFM_ERR_ARG;
    for (int k = 0; k < n; ++k) ms[k] = 0.f;
    if (!dc.timing || dc.tpending == 0) return 0;
    // average over every solve timed since the last call
    std::vector<double> acc(NTIMER, 0.0);
    int nst = 0, cnt = 0;
    const int first = (dc.tnext - dc.tpending + NTSETS) % NTSETS;
    for (int j = 0; j < dc.tpending; ++j) {
        TimerSet &t = dc.tsets[(first + j) % NTSETS];
        if (t.used < 2) continue;
        CK(cudaEventSynchronize(t.ev[t.used - 1]));
        for (int k = 0; k + 1 < t.used && k < NTIMER; ++k) {
            float e = 0.f;
            CK(cudaEventElapsedTime(&e, t.ev[k], t.ev[k + 1]));
            acc[k] += e;
        }
        nst = std::max(nst, t.used - 1);
        ++cnt;
    }
    dc.tpending = 0;
    for (int k = 0; k < nst && k < n; ++k) ms[k] = (float)(acc[k] / std::max(cnt, 1));
    return std::min(nst, n);
}

int bldfm_fma_peak(int fp64, double *flops_per_s, void *stream)
{
    std::lock_guard<std::mutex> lk(g_mutex);
    if (!flops_per_s) return BLDFM_ERR_ARG;
    int status = BLDFM_OK;
    DeviceCache &dc = cache_for_current(&status);
    if (status != BLDFM_OK) return status;
    double v = 0;
    if (run_fma_peak(fp64 != 0, dc.nsm, (cudaStream_t)stream, &v) != cudaSuccess) return BLDFM_ERR_CUDA;
    *flops_per_s = v;
    return BLDFM_OK;
}

int bldfm_plan(const bldfm_desc *d, int nlvls, bldfm_plan_info *out)
{
    if (!out) return BLDFM_ERR_ARG;
    HostPlan hp;
    int rc = make_plan(d, nullptr, nullptr, nullptr, nlvls, hp);
    if (rc != BLDFM_OK) return rc;
    // without levels the snapshot count is bounded by nlvls
    hp.g.nsnap = std::min(nlvls, hp.g.nz);
    const SolveGeom &g = hp.g;
    out->nxe = g.nxe;
    out->nye = g.nye;
    out->nlx = g.nlx;
    out->nly = g.nly;
    out->px = g.px;
    out->py = g.py;
    out->nfx = g.nfx;
    out->nfy = g.nfy;
    out->out_nx = g.out_nx;
    out->out_ny = g.out_ny;
    out->nsolved = g.nsolved;
    out->workspace_bytes = (int64_t)layout_for(g).total;
    return BLDFM_OK;
}

int bldfm_solve(const bldfm_desc *d, const double *srf_flx_dev, const double *z_host, const double *prof_host,
                const int64_t *levels_host, int32_t nlvls, double *conc_dev, double *flx_dev, void *workspace_dev,
                size_t workspace_bytes, void *stream)
{
    std::lock_guard<std::mutex> lk(g_mutex);
    return solve_impl(d, srf_flx_dev, z_host, prof_host, levels_host, nlvls, conc_dev, flx_dev, workspace_dev,
                      workspace_bytes, (cudaStream_t)stream);
}

int bldfm_solve_host(const bldfm_desc *d, const double *srf_flx_host, const double *z_host, const double *prof_host,
                     const int64_t *levels_host, int32_t nlvls, double *conc_host, double *flx_host)
{
    std::lock_guard<std::mutex> lk(g_mutex);
    if (!d || !conc_host || !flx_host) return BLDFM_ERR_ARG;
    bldfm_plan_info pi;
    int rc;
    {
        HostPlan hp;
        rc = make_plan(d, z_host, prof_host, levels_host, nlvls, hp);
        if (rc != BLDFM_OK) return rc;
        pi.out_nx = hp.g.out_nx;
        pi.out_ny = hp.g.out_ny;
        pi.workspace_bytes = (int64_t)layout_for(hp.g).total;
    }
    int status = BLDFM_OK;
    DeviceCache &dc = cache_for_current(&status);
    if (status != BLDFM_OK) return status;
    HostBuffers &hb = dc.hb;
    if (!hb.stream) CK(cudaStreamCreateWithFlags(&hb.stream, cudaStreamNonBlocking));
    if ((size_t)pi.workspace_bytes > hb.ws_bytes) {
        if (hb.ws) cudaFree(hb.ws);
        hb.ws = nullptr;
        CK(cudaMalloc(&hb.ws, (size_t)pi.workspace_bytes));
        hb.ws_bytes = (size_t)pi.workspace_bytes;
    }
    const size_t outb = (size_t)nlvls * pi.out_ny * pi.out_nx * sizeof(double);
    if (outb > hb.out_bytes) {
        if (hb.conc) cudaFree(hb.conc);
        if (hb.flx) cudaFree(hb.flx);
        hb.conc = hb.flx = nullptr;
        CK(cudaMalloc(&hb.conc, std::max<size_t>(outb, 8)));
        CK(cudaMalloc(&hb.flx, std::max<size_t>(outb, 8)));
        hb.out_bytes = outb;
    }
    const double *srf_dev = nullptr;
    if (!d->footprint) {
        if (!srf_flx_host) return BLDFM_ERR_ARG;
        const size_t sb = (size_t)d->nx * d->ny * sizeof(double);
        if (sb > hb.srf_bytes) {
            if (hb.srf) cudaFree(hb.srf);
            hb.srf = nullptr;
            CK(cudaMalloc(&hb.srf, sb));
            hb.srf_bytes = sb;
        }
        CK(cudaMemcpyAsync(hb.srf, srf_flx_host, sb, cudaMemcpyHostToDevice, hb.stream));
        srf_dev = hb.srf;
    }
    rc = solve_impl(d, srf_dev, z_host, prof_host, levels_host, nlvls, hb.conc, hb.flx, hb.ws, hb.ws_bytes,
                    hb.stream);
    if (rc != BLDFM_OK) return rc;
    if (outb) {
        CK(cudaMemcpyAsync(conc_host, hb.conc, outb, cudaMemcpyDeviceToHost, hb.stream));
        CK(cudaMemcpyAsync(flx_host, hb.flx, outb, cudaMemcpyDeviceToHost, hb.stream));
    }
    int err = 0;
    CK(cudaMemcpyAsync(&err, hb.ws, sizeof(int), cudaMemcpyDeviceToHost, hb.stream));
    CK(cudaStreamSynchronize(hb.stream));
    if (err != 0) return BLDFM_ERR_TIMEOUT;
    return BLDFM_OK;
}

}  // extern "C"
