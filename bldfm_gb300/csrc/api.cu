// C ABI of bldfm_gb300 (include/bldfm_gb300.h): host planning, per-device
// plan cache, workspace layout and the orchestration of one solve.
#include <cuda_runtime.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <exception>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/bldfm_gb300.h"
#include "batch.h"
#include "common.h"
#include "geometry.h"
#include "guard.h"
#include "host_exact.h"
#include "kernels.h"
#include "serve.h"
#include "surrogate_phys.cuh"

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
    std::shared_ptr<const std::vector<int4>> xband;  // output band columns (memoised per size)
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
    fft_plan_finalize(p);
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
    const int nz = d ? std::max(d->nz, 1) : 1;
    hp.slot.assign(nz, -1);
    int rc = solve_geometry(d, z, prof, levels, nlvls, hp.g, levels ? hp.slot.data() : nullptr, &hp.shape_ok);
    if (rc != BLDFM_OK) return rc;
    SolveGeom &g = hp.g;
    // output band columns and the transform plans depend on sizes only and
    // are memoised
    static std::mutex memo_mutex;
    static std::map<std::pair<int, int>, std::shared_ptr<const std::vector<int4>>> xband_memo;
    static std::map<int, FftPlan> plan_memo;
    std::lock_guard<std::mutex> memo_lock(memo_mutex);
    auto &xb = xband_memo[std::make_pair(g.nlx, g.nfx)];
    if (!xb) {
        const int f0 = freq_min(g.nlx), f1 = freq_max(g.nlx);
        auto v = std::make_shared<std::vector<int4>>(2 * std::max(-f0, f1) + 1);
        v->resize(band_columns(g.nlx, g.nfx, v->data()));
        xb = v;
    }
    hp.xband = xb;
    g.nbx = (int)hp.xband->size();
    auto plan_of = [&](int n, FftPlan &p) {
        auto it = plan_memo.find(n);
        if (it != plan_memo.end()) {
            p = it->second;
            return;
        }
        factorize(n, p);
        plan_memo[n] = p;
    };
    plan_of(g.nxe, hp.plx_fwd);
    plan_of(g.nye, hp.ply_fwd);
    plan_of(g.nfx, hp.plx_out);
    plan_of(g.nfy, hp.ply_out);
    return BLDFM_OK;
}

// ---------------------------------------------------------------------------
// workspace layout
// ---------------------------------------------------------------------------
struct Layout {
    size_t err, lv64, lv32, slot, dc, eig, snap, top, q0, A, Xp, Xq, Cb, scratch, total;
};

inline size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

Layout layout_for(const SolveGeom &g)
{
    Layout L;
    const bool f64 = g.mode != BLDFM_MODE_FP32 || g.analytic;
    const bool shoot = g.mode == BLDFM_MODE_FP64 && !g.analytic;  // eigval, snapshots, top states
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
    L.dc = o;  // k = 0 values (p, q) per output level
    o = al(o + (size_t)g.nlvls * 32);
    L.eig = o;
    o = al(o + ((shoot || g.analytic) ? ns * 16 : 0));
    L.snap = o;
    o = al(o + (shoot ? (size_t)g.nsnap * 4 * ns * 16 : 0));
    L.top = o;
    o = al(o + (shoot ? 4 * ns * 16 : 0));
    L.scratch = o;  // multi-level Riccati snapshots (5 reals per mode and level)
    o = al(o + ((!shoot && !g.analytic && g.nsnap > 1) ? (size_t)g.nsnap * 5 * ns * (f64 ? 8 : 4) : 0));
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
    // a second stream per caller stream: the batch's accuracy check runs on
    // it beside the transform passes (fork and join by events)
    struct Aux {
        cudaStream_t s = nullptr;
        cudaEvent_t fork = nullptr, join = nullptr;
    };
    std::map<cudaStream_t, Aux> aux;
    std::map<std::vector<int>, int4 *> xband;
    StageSlot stage[NSTAGE];  // ring of pinned staging buffers
    int stage_next = 0;
    HostBuffers hb;
    // CUDA graphs of batches, keyed by the launch topology; each instance owns
    // the pinned buffer its upload node reads
    struct GraphInst {
        cudaGraphExec_t exec = nullptr;
        void *pinned = nullptr;
        size_t bytes = 0;
        cudaEvent_t done = nullptr;
    };
    std::map<std::vector<int64_t>, std::vector<GraphInst>> graphs;
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
        prepare_kernel_attributes();
        prepare_batch_attributes();
    }
    return dc;
}

// the auxiliary stream of caller stream st (created on first use)
int get_aux(DeviceCache &dc, cudaStream_t st, DeviceCache::Aux **out)
{
    auto it = dc.aux.find(st);
    if (it == dc.aux.end()) {
        DeviceCache::Aux a;
        if (cudaStreamCreateWithFlags(&a.s, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&a.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&a.join, cudaEventDisableTiming) != cudaSuccess)
            return BLDFM_ERR_CUDA;
        it = dc.aux.emplace(st, a).first;
    }
    *out = &it->second;
    return BLDFM_OK;
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
    const std::vector<int4> &xband = *hp.xband;
    const size_t bytes = std::max<size_t>(xband.size(), 1) * sizeof(int4);
    if (cudaMalloc(&d, bytes) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (!xband.empty() &&
        cudaMemcpy(d, xband.data(), xband.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess)
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

// Persistent host threads for the per-case work of a batch call (level
// tables, k = 0 values, plans, descriptor and CTA-map fills): fn(i) for
// i < n.  A call is a job whose items the calling thread and the workers
// claim through an atomic counter; the caller starts at once and spins only
// until the items have finished and the workers that took the job have left
// it (a worker that wakes after the job has finished finds none), so a call
// never waits for sleeping threads.  One call at a time: every entry point
// that uses it holds g_mutex.  The workers start on first use and are joined
// when the library unloads; a forked child (which has none of them) runs the
// items itself.
class HostPool {
  public:
    static HostPool &get()
    {
        static HostPool p;
        return p;
    }
    void run(int n, const std::function<void(int)> &fn)
    {
        // a few items: waking workers costs more than they save
        if (n < 4 || th_.empty() || getpid() != pid_) {
            for (int i = 0; i < n; ++i) fn(i);
            return;
        }
        Job job;
        job.fn = &fn;
        job.n = n;
        {
            std::lock_guard<std::mutex> lk(m_);
            job_ = &job;
            ++gen_;
        }
        // wake as many workers as there are items besides the caller's first
        const int wake = std::min<int>(n - 1, (int)th_.size());
        if (wake == (int)th_.size())
            cv_.notify_all();
        else
            for (int i = 0; i < wake; ++i) cv_.notify_one();
        work(job);
        while (job.done.load(std::memory_order_acquire) < n) std::this_thread::yield();
        {
            std::lock_guard<std::mutex> lk(m_);
            if (job_ == &job) job_ = nullptr;  // workers that wake from now on find no job
        }
        while (job.refs.load(std::memory_order_acquire) > 0) std::this_thread::yield();
        // an item that threw (std::bad_alloc in planning) rethrows in the caller
        if (job.failed.load(std::memory_order_acquire)) std::rethrow_exception(job.error);
    }
    ~HostPool()
    {
        if (getpid() != pid_) {  // a forked child: the threads are not its own
            for (auto &t : th_) t.detach();
            return;
        }
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }

  private:
    struct Job {
        const std::function<void(int)> *fn = nullptr;
        int n = 0;
        std::atomic<int> next{0}, done{0};
        std::atomic<int> refs{0};  // workers inside the job (taken under m_)
        std::atomic<bool> claim{false}, failed{false};
        std::exception_ptr error;  // the first item's exception, set before failed
    };
    HostPool() : pid_(getpid())
    {
        const unsigned hw = std::thread::hardware_concurrency();
        const int nt = (int)std::min(7u, hw > 1 ? hw - 1 : 0u);
        for (int i = 0; i < nt; ++i) th_.emplace_back([this] { loop(); });
    }
    static void work(Job &j)
    {
        for (int i = j.next.fetch_add(1); i < j.n; i = j.next.fetch_add(1)) {
            try {
                (*j.fn)(i);
            } catch (...) {
                bool expect = false;
                if (j.claim.compare_exchange_strong(expect, true)) {
                    j.error = std::current_exception();
                    j.failed.store(true, std::memory_order_release);
                }
            }
            j.done.fetch_add(1, std::memory_order_release);
        }
    }
    void loop()
    {
        uint64_t seen = 0;
        for (;;) {
            Job *j = nullptr;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                j = job_;
                if (!j) continue;
                j->refs.fetch_add(1);
            }
            work(*j);
            j->refs.fetch_sub(1, std::memory_order_release);
        }
    }
    pid_t pid_;
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable cv_;
    Job *job_ = nullptr;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

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
    const bool f64 = g.mode != BLDFM_MODE_FP32 || g.analytic;
    const bool shoot = g.mode == BLDFM_MODE_FP64 && !g.analytic;
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
    const size_t eigb = (shoot || g.analytic) ? (size_t)g.nsolved * 16 : 0;
    const size_t dcb = (size_t)g.nlvls * 32;
    const size_t off_lv32 = al(lv64b), off_slot = off_lv32 + al(lv32b), off_dc = off_slot + al(slotb),
                 off_eig = off_dc + al(dcb);
    StageSlot *slt = nullptr;
    if ((rc = acquire_stage(dc, off_eig + al(eigb) + 256, &slt)) != BLDFM_OK) return rc;
    char *sg = (char *)slt->buf;
    timers_begin(dc);
    if (!f64 && g.footprint)
        hx_level_dz_w(nz, z, prof, (double *)sg);  // the FP32 footprint reads only what the k = 0 values use
    else
        hx_level_table(nz, z, prof, (double *)sg);
    if (!f64) {
        if (g.iso)
            hx_level_table32_iso(nz, z, prof, g.ex, g.ey, (float *)(sg + off_lv32), nullptr);
        else
            hx_level_table32(nz, z, prof, (float *)(sg + off_lv32), nullptr);
    }
    memcpy(sg + off_slot, hp.slot.data(), slotb);
    double2 *dcv = (double2 *)(w + L.dc);
    if (g.footprint) {
        // the k = 0 values need only host data in footprint mode
        double *hdc = (double *)(sg + off_dc);
        const double q0r = g.q0dc_fp;
        if (g.analytic) {
            const int64_t lev = levels[0] < 0 ? levels[0] + nz : levels[0];
            const double hlev = z[lev] - z[0];
            const double kzinv = 1.0 / prof[4 * nz + nz - 1];
            double pr = d->srf_bg_conc - (q0r * kzinv) * hlev;
            double pi = 0.0 - (0.0 * kzinv) * hlev;
            double qr = q0r, qi = 0.0;
            if (g.precision == BLDFM_PREC_SINGLE) {
                pr = (double)(float)pr;
                pi = (double)(float)pi;
                qr = (double)(float)qr;
            }
            hdc[0] = pr;
            hdc[1] = pi;
            hdc[2] = qr;
            hdc[3] = qi;
        } else {
            hx_dc_values(nz, (const double *)sg, hp.slot.data(), q0r, 0.0, d->srf_bg_conc,
                         g.precision == BLDFM_PREC_SINGLE, g.nlvls, 0, hdc);
        }
    }

    CK(cudaMemsetAsync(err, 0, 64, st));
    if (lv64b) CK(cudaMemcpyAsync(lv64, sg, lv64b, cudaMemcpyHostToDevice, st));
    if (!f64 && lv32b) CK(cudaMemcpyAsync(lv32, sg + off_lv32, lv32b, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(slot, sg + off_slot, slotb, cudaMemcpyHostToDevice, st));
    if (g.footprint) CK(cudaMemcpyAsync(dcv, sg + off_dc, dcb, cudaMemcpyHostToDevice, st));
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
            CK(launch_analytic64(g, ml->dev, eig, q0, p000, kzinv, hlev, Xp, Xq, dcv, st));
        } else if (!shoot) {
            // accurate FP64 mode: invariant imbedding, no libm values needed
            CK(cudaEventRecord(slt->ev, st));
            CK(launch_riccati64(g, lv64, slot, ml->dev, q0, (double *)(w + L.scratch), Xp, Xq, err, dc.nsm, st));
            tmark(dc, st);  // 2: after the sweep
            if (!g.footprint) CK(launch_trapezoid64(g, lv64, slot, q0, p000, dcv, st));
        } else {
            double2 *snap = (double2 *)(w + L.snap), *top = (double2 *)(w + L.top);
            if (g.nsolved > 0) CK(launch_sweep64(g, lv64, slot, ml->dev, q0, snap, top, err, dc.nsm, st));
            tmark(dc, st);  // 2: after the sweep
            // the host evaluates libm csqrt for every mode while the device sweeps
            eigval_parallel(*ml, g, prof, nz, (double *)(sg + off_eig));
            if (eigb) CK(cudaMemcpyAsync(eig, sg + off_eig, eigb, cudaMemcpyHostToDevice, st));
            CK(cudaEventRecord(slt->ev, st));
            CK(launch_combine64(g, ml->dev, eig, snap, top, Xp, Xq, st));
            if (!g.footprint) CK(launch_trapezoid64(g, lv64, slot, q0, p000, dcv, st));
        }
        tmark(dc, st);  // 3: before the output transform
        CK(launch_output_fft<double>(g, hp.plx_out, hp.ply_out, twxo->d64, twyo->d64, xband, Xp, Xq, dcv,
                                     (double2 *)(w + L.Cb), conc, flx, err, st));
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
        // the k = 0 source value as the FP64 sum of the source (partials in
        // bytes 128..255 of the status region)
        if (!g.footprint)
            CK(launch_trapezoid32(g, lv64, slot, q0, p000, dcv, st, srf_dev, (double *)(w + L.err + 128)));
        tmark(dc, st);  // 3: before the output transform
        CK(launch_output_fft<float>(g, hp.plx_out, hp.ply_out, twxo->d32, twyo->d32, xband, Xp, Xq, dcv,
                                    (float2 *)(w + L.Cb), conc, flx, err, st));
    }
    tmark(dc, st);  // 4: end
    if (f64 && g.analytic) CK(cudaEventRecord(slt->ev, st));
    return BLDFM_OK;
}


// ---------------------------------------------------------------------------
// batches (bldfm_solve_batch)
// ---------------------------------------------------------------------------
enum { BATCH_MAX_CTAS = 16384 };

struct BatchBuild {
    std::vector<HostPlan> hp;
    std::vector<ModeList *> ml;
    std::vector<TwTable *> twxo, twyo, twxf, twyf;
    std::vector<int4 *> xb;
    size_t off_cases = 0, off_tile_case = 0, off_cta_tiles = 0, off_col_case = 0, off_row_case = 0;
    std::vector<size_t> off_lv32, off_lv64, off_lvd, off_slot, off_dc;
    size_t blob_bytes = 0, blob_at = 0, extra_off = 0;
    std::vector<size_t> d_q0, d_A, d_dcp, d_scratch, d_Xp, d_Xq, d_Cb;
    size_t total = 0;
    int64_t ntiles = 0;
    int G = 0, threads = 256, ncol = 0, nrow = 0, rpc = 2, cpc = 1;
    size_t sweep_smem = 0, col_smem = 0, row_smem = 0;
    // persistent one-line transforms (lines per CTA 1)
    int persist = 0, col_grid = 0, row_grid = 0, maxnfy = 0, maxnfx = 0, maxnly = 0;
    // register-resident transform passes: rx_col >= 0 when they run, with
    // one column and one row launch per group of cases sharing their line
    // configs (xg); -1 for the shared-memory passes (one group)
    int rx_col = -1, rx_row = -1;
    int nxg = 1;
    XGroup xg[BATCH_MAX_XGROUPS] = {};
    int check = 1;  // run the accuracy check
    std::vector<int64_t> tile0, col0, row0;  // col0 / row0 from the case's group start
    std::vector<int64_t> colbase, rowbase;   // the group start of each case
    std::vector<int> cpck, rpck;             // lines per column / row CTA of each case
};

int batch_build(const bldfm_case *cs, int n, const bldfm_batch_opts *opts, DeviceCache *dc, BatchBuild &B,
                size_t extra_blob = 0)
{
    if (!cs || n < 1) return BLDFM_ERR_ARG;
    B.threads = (opts && opts->threads > 0) ? opts->threads : 256;
    B.check = !(opts && opts->skip_check);
    if (B.threads != 128 && B.threads != 256) return BLDFM_ERR_ARG;
    B.hp.resize(n);
    size_t o = 0;
    B.off_cases = o;
    o = al(o + sizeof(BatchCase) * n);
    B.tile0.resize(n);
    B.col0.resize(n);
    B.row0.resize(n);
    B.colbase.assign(n, 0);
    B.rowbase.assign(n, 0);
    B.cpck.assign(n, 1);
    B.rpck.assign(n, 1);
    int maxL = 0, maxnz = 0, maxnfy = 0, maxnfx = 0;
    // every case's checks and plan on the host pool; the first failing case
    // (lowest index) gives the status
    std::vector<int> status(n, BLDFM_OK);
    HostPool::get().run(n, [&](int k) {
        const bldfm_case &c = cs[k];
        if (c.desc.mode != BLDFM_MODE_FP32 || c.desc.analytic)
            status[k] = BLDFM_ERR_UNSUPPORTED;
        else if (!c.z_host || !c.prof_host || !c.levels_host || !c.conc_dev || !c.flx_dev ||
                 (!c.desc.footprint && !c.srf_flx_dev))
            status[k] = BLDFM_ERR_ARG;
        else
            status[k] = make_plan(&c.desc, c.z_host, c.prof_host, c.levels_host, c.nlvls, B.hp[k]);
    });
    for (int k = 0; k < n; ++k)
        if (status[k] != BLDFM_OK) return status[k];
    for (int k = 0; k < n; ++k) {
        const SolveGeom &g = B.hp[k].g;
        B.tile0[k] = B.ntiles;
        const int64_t tm = (int64_t)B.threads * BATCH_MODES_PER_THREAD;
        B.ntiles += (g.nsolved + tm - 1) / tm;
        maxL = std::max(maxL, g.nz - 1);
        maxnz = std::max(maxnz, g.nz);
        maxnfy = std::max(maxnfy, g.nfy);
        maxnfx = std::max(maxnfx, g.nfx);
        B.maxnly = std::max(B.maxnly, g.nly);
    }
    B.maxnfy = maxnfy;
    B.maxnfx = maxnfx;
    int xl = opts ? opts->xform_lines : 0;
    if (xl != 0 && xl != 1 && xl != 2 && xl != 4 && xl != 8 && xl != 16) return BLDFM_ERR_ARG;
    // register-resident passes (xform_lines 0, 8 or 16) when every case has
    // supported column and row line lengths, one launch per group of cases
    // sharing their configs (at most BATCH_MAX_XGROUPS groups); otherwise the
    // shared-memory passes.  0 and 16 take the zoomed column pass for the
    // cases whose band and kept window allow it (3 M lines, the default halo).
    std::vector<int> grp(n, 0);
    B.nxg = 1;
    if (xl == 0 || xl == 8 || xl == 16) {
        std::vector<int> cc(n), rc(n);
        bool ok = true;
        for (int k = 0; k < n && ok; ++k) {
            const SolveGeom &g = B.hp[k].g;
            cc[k] = rx_config(g.nfy);
            rc[k] = rx_config(g.nfx);
            ok = cc[k] >= 0 && rc[k] >= 0;
            if (ok && xl != 8) {
                const int hy = std::max(-freq_min(g.nly), freq_max(g.nly));
                const int z = rx_zoom_config(g.nfy, hy, g.out_ny);
                if (z >= 0) cc[k] = z;
            }
        }
        int ng = 0;
        for (int k = 0; k < n && ok; ++k) {
            int gi = 0;
            while (gi < ng && !(B.xg[gi].rx_col == cc[k] && B.xg[gi].rx_row == rc[k])) ++gi;
            if (gi == ng) {
                if (ng == BATCH_MAX_XGROUPS) {
                    ok = false;
                    break;
                }
                B.xg[ng].rx_col = cc[k];
                B.xg[ng].rx_row = rc[k];
                ++ng;
            }
            grp[k] = gi;
            B.cpck[k] = rx_lines_per_cta(cc[k], true);
            B.rpck[k] = rx_lines_per_cta(rc[k], false);
        }
        if (ok) {
            B.nxg = ng;
            B.rx_col = B.xg[0].rx_col;
            B.rx_row = B.xg[0].rx_row;
        } else {
            B.rx_col = B.rx_row = -1;
            std::fill(grp.begin(), grp.end(), 0);
        }
        xl = 0;
    }
    B.rpc = xl > 0 ? xl : 2;
    while (B.rpc > 1 && (2 * (size_t)B.rpc + 1) * maxnfx * 8 > 190 * 1024) --B.rpc;
    // column pass: (2 cpc + 1) lines of maxnfy in shared memory
    auto col_bytes = [&](int c) { return (2 * (size_t)c + 1) * maxnfy * 8; };
    B.cpc = xl > 0 ? xl : out_cols_per_cta(maxnfy, 8);
    while (B.cpc > 1 && col_bytes(B.cpc) > 190 * 1024) B.cpc >>= 1;
    if (B.rx_col < 0) {
        B.nxg = 1;
        for (int k = 0; k < n; ++k) {
            B.cpck[k] = B.cpc;
            B.rpck[k] = B.rpc;
        }
    }
    B.ncol = B.nrow = 0;
    for (int gi = 0; gi < B.nxg; ++gi) {
        XGroup &x = B.xg[gi];
        x.col_start = B.ncol;
        x.row_start = B.nrow;
        for (int k = 0; k < n; ++k) {
            if (grp[k] != gi) continue;
            const SolveGeom &g = B.hp[k].g;
            B.colbase[k] = x.col_start;
            B.rowbase[k] = x.row_start;
            B.col0[k] = B.ncol - x.col_start;
            B.row0[k] = B.nrow - x.row_start;
            B.ncol += g.nlvls * ((g.nbx + B.cpck[k] - 1) / B.cpck[k]);
            B.nrow += g.nlvls * ((g.out_ny + B.rpck[k] - 1) / B.rpck[k]);
        }
        x.col_ctas = B.ncol - x.col_start;
        x.row_ctas = B.nrow - x.row_start;
    }
    B.off_tile_case = o;
    o = al(o + 4 * (size_t)std::max<int64_t>(B.ntiles, 1));
    B.off_cta_tiles = o;
    o = al(o + 8 * (size_t)(BATCH_MAX_CTAS + 1));
    B.off_col_case = o;
    o = al(o + 4 * (size_t)std::max(B.ncol, 1));
    B.off_row_case = o;
    o = al(o + 4 * (size_t)std::max(B.nrow, 1));
    B.off_lv32.resize(n);
    B.off_lv64.resize(n);
    B.off_lvd.resize(n);
    B.off_slot.resize(n);
    B.off_dc.resize(n);
    for (int k = 0; k < n; ++k) {
        const SolveGeom &g = B.hp[k].g;
        B.off_lv32[k] = o;
        o = al(o + (size_t)std::max(g.nz - 1, 1) * BLDFM_LV32 * 4);
        B.off_lvd[k] = o;
        o = al(o + (size_t)std::max(g.nz - 1, 1) * BLDFM_LV32 * 8);
        B.off_lv64[k] = o;
        o = al(o + (size_t)std::max(g.nz - 1, 1) * BLDFM_LV64 * 8);
        B.off_slot[k] = o;
        o = al(o + (size_t)g.nz * 4);
        B.off_dc[k] = o;
        o = al(o + (size_t)g.nlvls * 32);
    }
    B.extra_off = o;  // caller's region at the end of the blob
    o = al(o + extra_blob);
    B.blob_bytes = o;
    // workspace: status word, the accuracy check's per-case sums (16 bytes
    // per case from byte 64), blob, per-case device regions
    size_t w = 0;
    w = al(w + 64 + 16 * (size_t)n);
    B.blob_at = w;
    w = al(w + B.blob_bytes);
    B.d_q0.resize(n);
    B.d_A.resize(n);
    B.d_dcp.resize(n);
    B.d_scratch.resize(n);
    B.d_Xp.resize(n);
    B.d_Xq.resize(n);
    B.d_Cb.resize(n);
    for (int k = 0; k < n; ++k) {
        const SolveGeom &g = B.hp[k].g;
        const size_t specb = (size_t)g.nlvls * g.nlx * g.nly * 8;
        B.d_q0[k] = w;
        w = al(w + (g.footprint ? 0 : (size_t)g.nlx * g.nly * 8));
        B.d_A[k] = w;
        w = al(w + (g.footprint ? 0 : (size_t)g.nlx * g.ny * 8));
        B.d_dcp[k] = w;  // FP64 partial sums of the source (the k = 0 source value)
        w = al(w + (g.footprint ? 0 : DC_PARTS * sizeof(double)));
        B.d_scratch[k] = w;
        w = al(w + (g.nsnap > 1 ? (size_t)g.nsnap * 5 * g.nsolved * 4 : 0));
        B.d_Xp[k] = w;
        w = al(w + specb);
        B.d_Xq[k] = w;
        w = al(w + specb);
        B.d_Cb[k] = w;
        w = al(w + (size_t)g.nlvls * g.nbx * std::max(g.out_ny, 1) * 8);
    }
    B.total = w;
    B.sweep_smem = (size_t)maxL * BLDFM_LV32 * 4 + (size_t)maxnz * 4 + 16;
    B.col_smem = col_bytes(B.cpc);
    B.row_smem = (2 * (size_t)B.rpc + 1) * maxnfx * 8;
    B.persist = B.cpc == 1 && B.rpc == 1;
    if (B.rx_col >= 0) {
        B.col_smem = B.row_smem = 0;
        for (int gi = 0; gi < B.nxg; ++gi) {
            B.col_smem = std::max(B.col_smem, rx_smem(B.xg[gi].rx_col, true));
            B.row_smem = std::max(B.row_smem, rx_smem(B.xg[gi].rx_row, false));
        }
        B.persist = 0;
    }
    if (B.persist) {
        B.col_smem = (3 * (size_t)maxnfy + 4 * (size_t)B.maxnly) * 8;
        B.row_smem = 3 * (size_t)maxnfx * 8;
        if (B.col_smem > 200 * 1024 || B.row_smem > 200 * 1024) return BLDFM_ERR_UNSUPPORTED;
        // SMs of the current device (planning calls come without a device cache)
        int nsm = dc ? dc->nsm : 0;
        if (nsm <= 0) {
            int dev = 0;
            if (cudaGetDevice(&dev) != cudaSuccess ||
                cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
                nsm = 1;
        }
        B.col_grid = (int)std::min<int64_t>(B.ncol, (int64_t)nsm * batch_xform_occupancy(1, B.col_smem));
        B.row_grid = (int)std::min<int64_t>(B.nrow, (int64_t)nsm * batch_xform_occupancy(0, B.row_smem));
    }
    if (B.sweep_smem > 200 * 1024) return BLDFM_ERR_UNSUPPORTED;
    if (!dc) return BLDFM_OK;
    // persistent sweep grid
    int per_sm = (opts && opts->ctas_per_sm > 0) ? opts->ctas_per_sm : batch_sweep_occupancy(B.threads, B.sweep_smem);
    B.G = (int)std::min<int64_t>(std::min<int64_t>((int64_t)dc->nsm * per_sm, BATCH_MAX_CTAS),
                                 std::max<int64_t>(B.ntiles, 1));
    B.ml.resize(n);
    B.twxo.resize(n);
    B.twyo.resize(n);
    B.twxf.assign(n, nullptr);
    B.twyf.assign(n, nullptr);
    B.xb.resize(n);
    for (int k = 0; k < n; ++k) {
        const SolveGeom &g = B.hp[k].g;
        int rc;
        if ((rc = get_modes(*dc, g.nlx, g.nly, &B.ml[k])) != BLDFM_OK) return rc;
        if ((rc = get_tw(*dc, g.nfx, &B.twxo[k])) != BLDFM_OK) return rc;
        if ((rc = get_tw(*dc, g.nfy, &B.twyo[k])) != BLDFM_OK) return rc;
        if (!g.footprint) {
            if ((rc = get_tw(*dc, g.nxe, &B.twxf[k])) != BLDFM_OK) return rc;
            if ((rc = get_tw(*dc, g.nye, &B.twyf[k])) != BLDFM_OK) return rc;
        }
        if ((rc = get_xband(*dc, B.hp[k], &B.xb[k])) != BLDFM_OK) return rc;
    }
    return BLDFM_OK;
}

// Fill the upload blob: case descriptors with device pointers into ws, the
// tile / CTA maps, and every case's level tables, slot map and k = 0 values.
void batch_fill_blob(const bldfm_case *cs, int n, BatchBuild &B, char *ws, char *blob)
{
    BatchCase *bc = (BatchCase *)(blob + B.off_cases);
    int *tile_case = (int *)(blob + B.off_tile_case);
    int64_t *cta_tiles = (int64_t *)(blob + B.off_cta_tiles);
    int *col_case = (int *)(blob + B.off_col_case);
    int *row_case = (int *)(blob + B.off_row_case);
    char *wb = ws + B.blob_at;  // device address of the blob
    // every case writes its own regions of the blob: the cases run on the
    // host pool (a 16-footprint step's tables and maps took ~0.1 ms on one
    // core of the Arm host, a fifth of the step)
    auto one_case = [&](int k) {
        const HostPlan &hp = B.hp[k];
        const SolveGeom &g = hp.g;
        const bldfm_case &c = cs[k];
        const int nz = g.nz;
        BatchCase &x = bc[k];
        memset(&x, 0, sizeof(x));
        x.g = g;
        x.plx = hp.plx_out;
        x.ply = hp.ply_out;
        x.lv32 = (const float *)(wb + B.off_lv32[k]);
        x.slot = (const int *)(wb + B.off_slot[k]);
        x.modes = B.ml[k]->dev;
        x.q0 = g.footprint ? nullptr : (const float2 *)(ws + B.d_q0[k]);
        x.scratch = (float *)(ws + B.d_scratch[k]);
        x.Xp = (float2 *)(ws + B.d_Xp[k]);
        x.Xq = (float2 *)(ws + B.d_Xq[k]);
        x.dc = (const double2 *)(wb + B.off_dc[k]);
        x.Cb = (float2 *)(ws + B.d_Cb[k]);
        x.twx = B.twxo[k]->d32;
        x.twy = B.twyo[k]->d32;
        x.xband = B.xb[k];
        x.conc = c.conc_dev;
        x.flx = c.flx_dev;
        x.lvff = (const float2 *)(wb + B.off_lvd[k]);
        x.ax = (float)(g.lx_scale * g.valx);
        x.ay = (float)(g.ly_scale * g.valy);
        x.tile0 = B.tile0[k];
        x.col0 = B.col0[k];
        x.row0 = B.row0[k];
        x.rpc = B.rpck[k];
        x.cpc = B.cpck[k];
        double *lv64 = (double *)(blob + B.off_lv64[k]);
        if (g.footprint)
            hx_level_dz_w(nz, c.z_host, c.prof_host, lv64);  // all the k = 0 values need (no trapezoid pass)
        else
            hx_level_table(nz, c.z_host, c.prof_host, lv64);
        // FP32 table of the sweep; the accuracy check's float-pair table always
        // in the generic row layout (u, v themselves, no rounded wind direction)
        float *lvd = (float *)(blob + B.off_lvd[k]);
        if (g.iso) {
            hx_level_table32_iso(nz, c.z_host, c.prof_host, g.ex, g.ey, (float *)(blob + B.off_lv32[k]), nullptr);
            hx_level_table32(nz, c.z_host, c.prof_host, nullptr, lvd);
        } else {
            hx_level_table32(nz, c.z_host, c.prof_host, (float *)(blob + B.off_lv32[k]), lvd);
        }
        memcpy(blob + B.off_slot[k], hp.slot.data(), (size_t)nz * 4);
        if (g.footprint)
            hx_dc_values(nz, lv64, hp.slot.data(), g.q0dc_fp, 0.0, c.desc.srf_bg_conc,
                         g.precision == BLDFM_PREC_SINGLE, g.nlvls, 0, (double *)(blob + B.off_dc[k]));
        const int64_t tm = (int64_t)B.threads * BATCH_MODES_PER_THREAD;
        const int64_t nt = (g.nsolved + tm - 1) / tm;
        for (int64_t t = 0; t < nt; ++t) tile_case[B.tile0[k] + t] = k;
        const int64_t ncb = (g.nbx + B.cpck[k] - 1) / B.cpck[k];
        for (int64_t i = 0; i < (int64_t)g.nlvls * ncb; ++i) col_case[B.colbase[k] + B.col0[k] + i] = k;
        const int nblk = (g.out_ny + B.rpck[k] - 1) / B.rpck[k];
        for (int64_t i = 0; i < (int64_t)g.nlvls * nblk; ++i) row_case[B.rowbase[k] + B.row0[k] + i] = k;
    };
    HostPool::get().run(n, one_case);
    // cost-weighted contiguous partition of the tiles over G persistent CTAs
    std::vector<double> tile_cost;
    tile_cost.reserve((size_t)B.ntiles);
    for (int k = 0; k < n; ++k) {
        const SolveGeom &g = B.hp[k].g;
        const int64_t tm = (int64_t)B.threads * BATCH_MODES_PER_THREAD;
        const int64_t nt = (g.nsolved + tm - 1) / tm;
        for (int64_t t = 0; t < nt; ++t) tile_cost.push_back((double)std::max(g.nz - 1, 1));
    }
    double total = 0;
    for (double c : tile_cost) total += c;
    int64_t t = 0;
    double acc = 0;
    cta_tiles[0] = 0;
    for (int b = 0; b < B.G; ++b) {
        const double target = total * (b + 1) / B.G;
        while (t < B.ntiles && acc + 0.5 * tile_cost[(size_t)t] <= target) acc += tile_cost[(size_t)t++];
        if (b == B.G - 1) t = B.ntiles;
        cta_tiles[b + 1] = t;
    }
}

int batch_enqueue(const bldfm_case *cs, int n, BatchBuild &B, char *ws, const void *blob_host, cudaStream_t st,
                  DeviceCache *tdc, DeviceCache::Aux *aux)
{
    if (tdc) tmark(*tdc, st);  // 0: upload and per-case forward transforms
    CK(cudaMemcpyAsync(ws + B.blob_at, blob_host, B.blob_bytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(ws, 0, 64 + 16 * (size_t)n, st));  // status word and the check's sums
    char *wb = ws + B.blob_at;
    for (int k = 0; k < n; ++k) {
        const SolveGeom &g = B.hp[k].g;
        if (g.nsnap < g.nlvls) {
            const size_t specb = (size_t)g.nlvls * g.nlx * g.nly * 8;
            CK(cudaMemsetAsync(ws + B.d_Xp[k], 0, specb, st));
            CK(cudaMemsetAsync(ws + B.d_Xq[k], 0, specb, st));
        }
        if (!g.footprint) {
            float2 *q0 = (float2 *)(ws + B.d_q0[k]);
            CK(launch_forward_fft<float>(g, B.hp[k].plx_fwd, B.hp[k].ply_fwd, B.twxf[k]->d32, B.twyf[k]->d32,
                                         cs[k].srf_flx_dev, (float2 *)(ws + B.d_A[k]), q0, st));
            CK(launch_trapezoid32(g, (const double *)(wb + B.off_lv64[k]), (const int *)(wb + B.off_slot[k]), q0,
                                  cs[k].desc.srf_bg_conc, (double2 *)(wb + B.off_dc[k]), st, cs[k].srf_flx_dev,
                                  (double *)(ws + B.d_dcp[k])));
        }
    }
    BatchLaunch bl;
    bl.cases = (const BatchCase *)(wb + B.off_cases);
    bl.tile_case = (const int *)(wb + B.off_tile_case);
    bl.cta_tiles = (const int64_t *)(wb + B.off_cta_tiles);
    bl.col_case = (const int *)(wb + B.off_col_case);
    bl.row_case = (const int *)(wb + B.off_row_case);
    bl.err = (int *)ws;
    bl.sweep_ctas = B.ntiles > 0 ? B.G : 0;
    bl.threads = B.threads;
    bl.sweep_smem = B.sweep_smem;
    bl.col_ctas = B.ncol;
    bl.col_smem = B.col_smem;
    bl.row_ctas = B.nrow;
    bl.row_smem = B.row_smem;
    bl.persist = B.persist;
    bl.col_grid = B.col_grid;
    bl.row_grid = B.row_grid;
    bl.maxn_col = B.maxnfy;
    bl.maxnly = B.maxnly;
    bl.maxn_row = B.maxnfx;
    bl.rx_col = B.rx_col;
    bl.rx_row = B.rx_row;
    bl.nxg = B.nxg;
    for (int i = 0; i < B.nxg; ++i) bl.xg[i] = B.xg[i];
    if (tdc) tmark(*tdc, st);  // 1: the sweep
    CK(launch_batch_kernels(bl, st, 0));
    // the accuracy check reads the spectra, as the transform passes do: it
    // runs beside them on the auxiliary stream (after them when the stages
    // are timed, so that each stage's time is its own)
    const bool fork = B.check && aux && !tdc;
    if (fork) {
        CK(cudaEventRecord(aux->fork, st));
        CK(cudaStreamWaitEvent(aux->s, aux->fork, 0));
        CK(launch_fp32_check(bl.cases, n, (float4 *)(ws + 64), aux->s));
        CK(cudaEventRecord(aux->join, aux->s));
    }
    if (tdc) tmark(*tdc, st);  // 2: the output transform
    CK(launch_batch_kernels(bl, st, 1));
    if (tdc) tmark(*tdc, st);  // 3: the accuracy check
    if (fork)
        CK(cudaStreamWaitEvent(st, aux->join, 0));
    else if (B.check)
        CK(launch_fp32_check(bl.cases, n, (float4 *)(ws + 64), st));
    if (tdc) tmark(*tdc, st);  // 4: end
    return BLDFM_OK;
}

std::vector<int64_t> batch_key(const bldfm_case *cs, int n, const BatchBuild &B, const void *ws)
{
    std::vector<int64_t> k;
    k.push_back((int64_t)(uintptr_t)ws);
    k.push_back(n);
    k.push_back((int64_t)B.blob_bytes);
    k.push_back(B.G);
    k.push_back(B.threads);
    k.push_back((int64_t)B.sweep_smem);
    k.push_back(B.ncol);
    k.push_back((int64_t)B.col_smem);
    k.push_back(B.nrow);
    k.push_back((int64_t)B.row_smem);
    k.push_back(B.persist);
    k.push_back(B.rx_col);
    k.push_back(B.rx_row);
    k.push_back(B.nxg);
    for (int i = 0; i < B.nxg; ++i) {
        const XGroup &x = B.xg[i];
        k.push_back(x.rx_col);
        k.push_back(x.rx_row);
        k.push_back(x.col_start);
        k.push_back(x.col_ctas);
        k.push_back(x.row_start);
        k.push_back(x.row_ctas);
    }
    k.push_back(B.check);
    k.push_back(B.col_grid);
    k.push_back(B.row_grid);
    for (int i = 0; i < n; ++i) {
        const SolveGeom &g = B.hp[i].g;
        k.push_back(g.footprint);
        k.push_back(g.nsnap < g.nlvls);
        k.push_back(g.nlvls);
        k.push_back(g.nlx);
        k.push_back(g.nly);
        k.push_back(g.nz);
        if (!g.footprint) {
            k.push_back(g.nx);
            k.push_back(g.ny);
            k.push_back(g.nxe);
            k.push_back(g.nye);
            k.push_back(g.px);
            k.push_back(g.py);
            k.push_back(g.precision);
            k.push_back((int64_t)(uintptr_t)cs[i].srf_flx_dev);
        }
    }
    return k;
}


// ---------------------------------------------------------------------------
// surrogate serving (bldfm_surrogate_solve): FP32 footprint solve whose
// per-mode sweep is replaced by the MLP's transfer at z_m
// ---------------------------------------------------------------------------
struct SurLayout {
    Layout L;
    size_t X, Y, steps, tcase, lbcase, total;
    int64_t npad;
};

SurLayout sur_layout(const SolveGeom &g)
{
    SurLayout S;
    S.L = layout_for(g);
    S.npad = std::max<int64_t>((g.nsolved + 255) / 256 * 256, 256);
    size_t o = S.L.total;
    S.X = o;
    o = al(o + (size_t)S.npad * 32);
    S.Y = o;
    o = al(o + (size_t)S.npad * 16);
    S.steps = o;
    o = al(o + (size_t)std::max(g.nz - 1, 1) * 16);
    S.tcase = o;  // TransferCase (exact variant) or SurCase (fused kernel)
    o = al(o + std::max(sizeof(TransferCase), sizeof(SurCase)));
    S.lbcase = o;  // LowBandCase of the exact low band
    o = al(o + sizeof(LowBandCase));
    S.total = o;
    return S;
}

int sur_check_desc(const bldfm_desc *d, int nlvls)
{
    if (!d) return BLDFM_ERR_ARG;
    if (d->mode != BLDFM_MODE_FP32 || !d->footprint || d->analytic || nlvls != 1) return BLDFM_ERR_UNSUPPORTED;
    return BLDFM_OK;
}

int sur_solve_impl(void *net, const bldfm_desc *d, const bldfm_surrogate_case *met, const double *z,
                   const double *prof, const int64_t *levels, int nlvls, double *conc, double *flx, void *ws,
                   size_t ws_bytes, cudaStream_t st)
{
    if (!met || !z || !prof || !levels || !conc || !flx || !ws || (met->variant != 1 && !net) || met->variant < 0 ||
        met->variant > 2 || !(met->exact_kz >= 0))
        return BLDFM_ERR_ARG;
    int rc = sur_check_desc(d, nlvls);
    if (rc != BLDFM_OK) return rc;
    HostPlan hp;
    if ((rc = make_plan(d, z, prof, levels, nlvls, hp)) != BLDFM_OK) return rc;
    const SolveGeom g = hp.g;
    if (!g.iso) return BLDFM_ERR_UNSUPPORTED;
    const int nz = g.nz;
    const int64_t lev = levels[0] < 0 ? levels[0] + nz : levels[0];
    if (!(met->zm > 0) || !(met->wind > 0) || fabs(z[lev] - met->zm) > 1e-6 * met->zm) return BLDFM_ERR_ARG;
    const SurLayout S = sur_layout(g);
    if (ws_bytes < S.total) return BLDFM_ERR_WORKSPACE;
    if (((uintptr_t)ws & 255) != 0) return BLDFM_ERR_ARG;
    int status = BLDFM_OK;
    DeviceCache &dc = cache_for_current(&status);
    if (status != BLDFM_OK) return status;
    ModeList *ml = nullptr;
    TwTable *twxo = nullptr, *twyo = nullptr;
    int4 *xband = nullptr;
    if ((rc = get_modes(dc, g.nlx, g.nly, &ml)) != BLDFM_OK) return rc;
    if ((rc = get_tw(dc, g.nfx, &twxo)) != BLDFM_OK) return rc;
    if ((rc = get_tw(dc, g.nfy, &twyo)) != BLDFM_OK) return rc;
    if ((rc = get_xband(dc, hp, &xband)) != BLDFM_OK) return rc;

    char *w = (char *)ws;
    // host data: FP64 level table (for the k = 0 values), k = 0 values, and
    // in the check mode the nondimensional step table of this case
    const size_t lv64b = (size_t)std::max(nz - 1, 0) * BLDFM_LV64 * 8;
    const size_t dcb = 32, stb = (size_t)std::max(nz - 1, 1) * 16;
    const size_t off_dc = al(lv64b), off_st = off_dc + al(dcb), off_tc = off_st + al(stb);
    const size_t tcb = std::max(sizeof(TransferCase), sizeof(SurCase));
    // the exact low band (network variants): FP32 level table and band record
    const size_t lv32b = (size_t)std::max(nz - 1, 0) * BLDFM_LV32 * 4;
    const size_t off_lv32 = off_tc + al(tcb), off_lb = off_lv32 + al(lv32b);
    StageSlot *slt = nullptr;
    if ((rc = acquire_stage(dc, off_lb + al(sizeof(LowBandCase)) + 256, &slt)) != BLDFM_OK) return rc;
    char *sg = (char *)slt->buf;
    hx_level_table(nz, z, prof, (double *)sg);
    hx_dc_values(nz, (const double *)sg, hp.slot.data(), g.q0dc_fp, 0.0, d->srf_bg_conc, 1, 1, 0,
                 (double *)(sg + off_dc));
    const float zm = (float)met->zm;
    const double *u_ = prof, *v_ = prof + nz, *Kz_ = prof + 4 * nz;
    const float ktop = (float)(Kz_[nz - 1] / (met->wind * met->zm));
    const float utop = (float)((u_[nz - 1] * g.ex + v_[nz - 1] * g.ey) / met->wind);
    const bool exact = met->variant == 1;
    if (exact) {
        surrogate_steps_from_profiles(nz, z, prof, met->zm, met->wind, g.ex, g.ey, (float4 *)(sg + off_st));
        TransferCase *tc = (TransferCase *)(sg + off_tc);
        tc->nz = nz;
        tc->jm = (int)lev;
        tc->ktop = ktop;
        tc->utop = utop;
        tc->s1 = (float)met->s1;
        tc->s2 = (float)met->s2;
        tc->s3 = (float)met->s3;
        tc->pad = 0;
    }
    const float ax = (float)(g.lx_scale * g.valx), ay = (float)(g.ly_scale * g.valy);
    float2 *Xp = (float2 *)(w + S.L.Xp), *Xq = (float2 *)(w + S.L.Xq);
    const float inv_wind = (float)(1.0 / met->wind);
    if (met->variant == 0) {
        SurCase *c = (SurCase *)(sg + off_tc);
        memset(c, 0, sizeof(SurCase));
        c->g = g;
        c->modes = ml->dev;
        c->Xp = Xp;
        c->Xq = Xq;
        c->ax = ax;
        c->ay = ay;
        c->zm = zm;
        c->s1 = (float)met->s1;
        c->s2 = (float)met->s2;
        c->s3 = (float)met->s3;
        c->inv_wind = inv_wind;
        c->ktop = ktop;
        c->utop = utop;
        c->tile0 = 0;
    }
    int lb_total = 0;
    if (!exact && lv32b > 0) {
        hx_level_table32_iso(nz, z, prof, g.ex, g.ey, (float *)(sg + off_lv32), nullptr);
        LowBandCase *lb = (LowBandCase *)(sg + off_lb);
        memset(lb, 0, sizeof(LowBandCase));
        lb->g = g;
        lb->lv32 = (const float *)(w + S.L.lv32);
        lb->Xp = Xp;
        lb->Xq = Xq;
        lb->ax = ax;
        lb->ay = ay;
        lb_total = sur_lowband_setup(*lb, met->exact_kz, met->zm);
    }
    double2 *dcv = (double2 *)(w + S.L.dc);
    CK(cudaMemsetAsync(w + S.L.err, 0, 64, st));
    if (lb_total > 0) {
        CK(cudaMemcpyAsync(w + S.L.lv32, sg + off_lv32, lv32b, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(w + S.lbcase, sg + off_lb, sizeof(LowBandCase), cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemcpyAsync(dcv, sg + off_dc, dcb, cudaMemcpyHostToDevice, st));
    if (exact) {
        CK(cudaMemcpyAsync(w + S.steps, sg + off_st, stb, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(w + S.tcase, sg + off_tc, sizeof(TransferCase), cudaMemcpyHostToDevice, st));
    } else if (met->variant == 0) {
        CK(cudaMemcpyAsync(w + S.tcase, sg + off_tc, sizeof(SurCase), cudaMemcpyHostToDevice, st));
    }
    CK(cudaEventRecord(slt->ev, st));
    float *X = (float *)(w + S.X), *Y = (float *)(w + S.Y);
    if (met->variant == 0) {
        MlpServing view;
        if ((rc = mlp_serving_view(net, &view)) != BLDFM_OK) return rc;
        CK(launch_sur_serve((const SurCase *)(w + S.tcase), 1, (g.nsolved + 127) / 128, view, (int *)(w + S.L.err),
                            dc.nsm, st));
    } else {
        if (exact) {
            CK(launch_sur_exact(g, ml->dev, ax, ay, zm, (const TransferCase *)(w + S.tcase),
                                (const float4 *)(w + S.steps), Y, st));
        } else {
            CK(launch_sur_features(g, ml->dev, ax, ay, zm, (float)met->s1, (float)met->s2, (float)met->s3, X,
                                   S.npad, st));
            const int cap = bldfm_surrogate_batch(net);
            if (cap < 256) return BLDFM_ERR_ARG;
            for (int64_t off = 0; off < S.npad; off += cap) {
                const int n = (int)std::min<int64_t>(cap, S.npad - off);
                if ((rc = bldfm_surrogate_forward(net, X + off * 8, Y + off * 4, n, st)) != BLDFM_OK) return rc;
            }
        }
        CK(launch_sur_spectra(g, ml->dev, Y, ax, ay, zm, inv_wind, ktop, utop, Xp, Xq, st));
    }
    CK(launch_sur_lowband((const LowBandCase *)(w + S.lbcase), 1, lb_total, nz, st));
    CK(launch_output_fft<float>(g, hp.plx_out, hp.ply_out, twxo->d32, twyo->d32, xband, Xp, Xq, dcv,
                                (float2 *)(w + S.L.Cb), conc, flx, (int *)(w + S.L.err), st));
    return BLDFM_OK;
}

// ---------------------------------------------------------------------------
// batched surrogate serving (bldfm_surrogate_solve_batch): every case's
// 128-mode tiles in one persistent fused launch, then the batched output
// transform of the FP32 batch path
// ---------------------------------------------------------------------------
int sur_batch_check(const bldfm_case *cs, const bldfm_surrogate_case *mets, int n)
{
    if (!cs || !mets || n < 1) return BLDFM_ERR_ARG;
    for (int k = 0; k < n; ++k) {
        const int rc = sur_check_desc(&cs[k].desc, cs[k].nlvls);
        if (rc != BLDFM_OK) return rc;
        if (mets[k].variant != 0 || !(mets[k].zm > 0) || !(mets[k].wind > 0) || !(mets[k].exact_kz >= 0))
            return BLDFM_ERR_ARG;
    }
    return BLDFM_OK;
}

// Accuracy guard of the batched surrogate: a stratified sample of each case
// (the k = 0 mode, the modes with |kx|, |ky| <= 2, every SUR_GUARD_STRIDE-th
// solved mode) re-solved exactly (FP32 sweep) and compared with the served
// spectra.  The blob's extra region holds the SurCase records, then
// the guard's sample offsets; the per-case sums (4 floats) sit in the last
// sur_guard_bytes(n) bytes of the planned workspace.
enum { SUR_GUARD_STRIDE = 61 };  // prime: no alignment with the rows of a column
size_t sur_prefix_off(int n) { return (sizeof(SurCase) * (size_t)n + 15) & ~(size_t)15; }
size_t sur_lowband_off(int n) { return (sur_prefix_off(n) + 8 * ((size_t)n + 1) + 15) & ~(size_t)15; }
size_t sur_extra_bytes(int n) { return sur_lowband_off(n) + sizeof(LowBandCase) * (size_t)n; }
size_t sur_guard_bytes(int n) { return al(16 * (size_t)n); }

int sur_solve_batch_impl(void *net, const bldfm_case *cs, const bldfm_surrogate_case *mets, int n, void *ws,
                         size_t ws_bytes, cudaStream_t st)
{
    int rc = sur_batch_check(cs, mets, n);
    if (rc != BLDFM_OK) return rc;
    if (!net || !ws) return BLDFM_ERR_ARG;
    if (((uintptr_t)ws & 255) != 0) return BLDFM_ERR_ARG;
    int status = BLDFM_OK;
    DeviceCache &dc = cache_for_current(&status);
    if (status != BLDFM_OK) return status;
    BatchBuild B;
    bldfm_batch_opts opts = {256, 0, 0, 0, 1};
    if ((rc = batch_build(cs, n, &opts, &dc, B, sur_extra_bytes(n))) != BLDFM_OK) return rc;
    if (ws_bytes < B.total + sur_guard_bytes(n)) return BLDFM_ERR_WORKSPACE;
    for (int k = 0; k < n; ++k) {
        const SolveGeom &g = B.hp[k].g;
        const int nz = g.nz;
        const int64_t lev = cs[k].levels_host[0] < 0 ? cs[k].levels_host[0] + nz : cs[k].levels_host[0];
        if (!g.iso) return BLDFM_ERR_UNSUPPORTED;
        if (fabs(cs[k].z_host[lev] - mets[k].zm) > 1e-6 * mets[k].zm) return BLDFM_ERR_ARG;
    }
    StageSlot *slt = nullptr;
    if ((rc = acquire_stage(dc, B.blob_bytes + 256, &slt)) != BLDFM_OK) return rc;
    char *blob = (char *)slt->buf;
    char *w = (char *)ws;
    batch_fill_blob(cs, n, B, w, blob);
    SurCase *sc = (SurCase *)(blob + B.extra_off);
    int64_t t = 0;
    for (int k = 0; k < n; ++k) {
        const SolveGeom &g = B.hp[k].g;
        const int nz = g.nz;
        const double *prof = cs[k].prof_host;
        const bldfm_surrogate_case &m = mets[k];
        SurCase &c = sc[k];
        memset(&c, 0, sizeof(c));
        c.g = g;
        c.modes = B.ml[k]->dev;
        c.Xp = (float2 *)(w + B.d_Xp[k]);
        c.Xq = (float2 *)(w + B.d_Xq[k]);
        c.ax = (float)(g.lx_scale * g.valx);
        c.ay = (float)(g.ly_scale * g.valy);
        c.zm = (float)m.zm;
        c.s1 = (float)m.s1;
        c.s2 = (float)m.s2;
        c.s3 = (float)m.s3;
        c.inv_wind = (float)(1.0 / m.wind);
        c.ktop = (float)(prof[4 * nz + nz - 1] / (m.wind * m.zm));
        c.utop = (float)((prof[nz - 1] * g.ex + prof[nz + nz - 1] * g.ey) / m.wind);
        c.tile0 = t;
        t += (g.nsolved + 127) / 128;
    }
    // the exact low band of each case: the case's level table and spectra
    // from its BatchCase record in the blob
    LowBandCase *lbc = (LowBandCase *)(blob + B.extra_off + sur_lowband_off(n));
    const BatchCase *bcs = (const BatchCase *)(blob + B.off_cases);
    int lb_total = 0, lb_maxnz = 2;
    for (int k = 0; k < n; ++k) {
        LowBandCase &c = lbc[k];
        memset(&c, 0, sizeof(c));
        c.g = B.hp[k].g;
        c.lv32 = bcs[k].lv32;
        c.Xp = sc[k].Xp;
        c.Xq = sc[k].Xq;
        c.ax = sc[k].ax;
        c.ay = sc[k].ay;
        c.block0 = lb_total;
        const int nb = sur_lowband_setup(c, mets[k].exact_kz, mets[k].zm);
        if (nb > INT_MAX - lb_total) return BLDFM_ERR_ARG;
        lb_total += nb;
        lb_maxnz = std::max(lb_maxnz, c.g.nz);
    }
    int64_t *prefix = (int64_t *)(blob + B.extra_off + sur_prefix_off(n));
    prefix[0] = 0;
    for (int k = 0; k < n; ++k) {
        // the k = 0 mode, the low-wavenumber box, every stride-th solved mode
        const int64_t s = 1 + SUR_GUARD_BOX + (B.hp[k].g.nsolved + SUR_GUARD_STRIDE - 1) / SUR_GUARD_STRIDE;
        prefix[k + 1] = prefix[k] + (s + SUR_GUARD_CTA - 1) / SUR_GUARD_CTA * SUR_GUARD_CTA;
    }
    timers_begin(dc);
    tmark(dc, st);  // 0: upload
    CK(cudaMemcpyAsync(w + B.blob_at, blob, B.blob_bytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(w, 0, 64, st));
    CK(cudaEventRecord(slt->ev, st));
    MlpServing view;
    if ((rc = mlp_serving_view(net, &view)) != BLDFM_OK) return rc;
    char *wb = w + B.blob_at;
    tmark(dc, st);  // 1: the fused features -> MLP -> spectra kernel
    CK(launch_sur_serve((const SurCase *)(wb + B.extra_off), n, t, view, (int *)w, dc.nsm, st));
    tmark(dc, st);  // 2: the exact low band
    CK(launch_sur_lowband((const LowBandCase *)(wb + B.extra_off + sur_lowband_off(n)), n, lb_total, lb_maxnz, st));
    tmark(dc, st);  // 3: the accuracy guard
    float4 *acc = (float4 *)(w + B.total);
    CK(cudaMemsetAsync(acc, 0, 16 * (size_t)n, st));
    CK(launch_sur_guard((const BatchCase *)(wb + B.off_cases), n,
                        (const int64_t *)(wb + B.extra_off + sur_prefix_off(n)), prefix[n], SUR_GUARD_STRIDE, lb_maxnz,
                        acc, st));
    tmark(dc, st);  // 4: the output transform
    BatchLaunch bl;
    memset(&bl, 0, sizeof(bl));
    bl.cases = (const BatchCase *)(wb + B.off_cases);
    bl.tile_case = (const int *)(wb + B.off_tile_case);
    bl.cta_tiles = (const int64_t *)(wb + B.off_cta_tiles);
    bl.col_case = (const int *)(wb + B.off_col_case);
    bl.row_case = (const int *)(wb + B.off_row_case);
    bl.err = (int *)w;
    bl.threads = B.threads;
    bl.col_ctas = B.ncol;
    bl.col_smem = B.col_smem;
    bl.row_ctas = B.nrow;
    bl.row_smem = B.row_smem;
    bl.persist = B.persist;
    bl.col_grid = B.col_grid;
    bl.row_grid = B.row_grid;
    bl.maxn_col = B.maxnfy;
    bl.maxnly = B.maxnly;
    bl.maxn_row = B.maxnfx;
    bl.rx_col = B.rx_col;
    bl.rx_row = B.rx_row;
    bl.nxg = B.nxg;
    for (int i = 0; i < B.nxg; ++i) bl.xg[i] = B.xg[i];
    CK(launch_batch_kernels(bl, st, 1));
    tmark(dc, st);  // 5: end
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
    case BLDFM_ERR_PROFILE:
        return "z must be strictly increasing and the profiles finite with Kz > 0 and Kx, Ky >= 0";
    case BLDFM_ERR_HOST: return "host-side failure (memory allocation or thread start)";
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

int bldfm_memcpy_async(void *dst, const void *src, size_t bytes, void *stream)
{
    if (bytes == 0) return BLDFM_OK;
    if (!dst || !src) return BLDFM_ERR_ARG;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, (cudaStream_t)stream) == cudaSuccess ? BLDFM_OK
                                                                                                 : BLDFM_ERR_CUDA;
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

int bldfm_sweep32_flops(int32_t nz, const double *prof_host, const int64_t *levels_host, int32_t nlvls,
                        double *flops_per_mode)
{
    if (nz < 2 || !prof_host || !levels_host || nlvls < 1 || !flops_per_mode) return BLDFM_ERR_ARG;
    int64_t jmax = -1;
    for (int k = 0; k < nlvls; ++k) {
        if (levels_host[k] < 0 || levels_host[k] >= nz) return BLDFM_ERR_ARG;
        jmax = std::max(jmax, levels_host[k]);
    }
    double ex, ey;
    const bool iso = hx_profiles_iso(nz, prof_host, &ex, &ey) != 0;
    // flops per step (FMA 2, MUL/ADD/RCP 1): step coefficients, ratio update,
    // flux product (StepCoef::eval_row, ricc_step, flux_step)
    const double coef = iso ? 14.0 : 21.0, ratio = 28.0, flux = 14.0;
    const double L = nz - 1;
    *flops_per_mode = (L - (double)jmax) * (coef + ratio) + (double)jmax * (coef + ratio + flux);
    return BLDFM_OK;
}

int bldfm_fma_peak(int kind, double *flops_per_s, void *stream)
{
    std::lock_guard<std::mutex> lk(g_mutex);
    if (!flops_per_s || kind < 0 || kind > 2) return BLDFM_ERR_ARG;
    int status = BLDFM_OK;
    DeviceCache &dc = cache_for_current(&status);
    if (status != BLDFM_OK) return status;
    double v = 0;
    if (run_fma_peak(kind, dc.nsm, (cudaStream_t)stream, &v) != cudaSuccess) return BLDFM_ERR_CUDA;
    *flops_per_s = v;
    return BLDFM_OK;
}

int bldfm_plan(const bldfm_desc *d, int nlvls, bldfm_plan_info *out)
{
    return bldfm_guarded([&]() -> int {
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
    });
}

int bldfm_solve(const bldfm_desc *d, const double *srf_flx_dev, const double *z_host, const double *prof_host,
                const int64_t *levels_host, int32_t nlvls, double *conc_dev, double *flx_dev, void *workspace_dev,
                size_t workspace_bytes, void *stream)
{
    return bldfm_guarded([&]() -> int {
        std::lock_guard<std::mutex> lk(g_mutex);
        return solve_impl(d, srf_flx_dev, z_host, prof_host, levels_host, nlvls, conc_dev, flx_dev, workspace_dev,
                          workspace_bytes, (cudaStream_t)stream);
    });
}

int bldfm_solve_host(const bldfm_desc *d, const double *srf_flx_host, const double *z_host, const double *prof_host,
                     const int64_t *levels_host, int32_t nlvls, double *conc_host, double *flx_host)
{
    return bldfm_guarded([&]() -> int {
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
        if (err != 0) return err == BLDFM_ERR_NONFINITE ? BLDFM_ERR_NONFINITE : BLDFM_ERR_TIMEOUT;
        return BLDFM_OK;
    });
}

int bldfm_batch_plan(const bldfm_case *cases, int32_t ncases, const bldfm_batch_opts *opts, int64_t *workspace_bytes)
{
    return bldfm_guarded([&]() -> int {
        std::lock_guard<std::mutex> lk(g_mutex);
        if (!workspace_bytes) return BLDFM_ERR_ARG;
        BatchBuild B;
        int rc = batch_build(cases, ncases, opts, nullptr, B);
        if (rc != BLDFM_OK) return rc;
        *workspace_bytes = (int64_t)B.total;
        return BLDFM_OK;
    });
}

int bldfm_solve_batch(const bldfm_case *cases, int32_t ncases, const bldfm_batch_opts *opts, void *workspace,
                      size_t workspace_bytes, void *stream)
{
    return bldfm_guarded([&]() -> int {
        std::lock_guard<std::mutex> lk(g_mutex);
        if (!workspace) return BLDFM_ERR_ARG;
        if (((uintptr_t)workspace & 255) != 0) return BLDFM_ERR_ARG;
        int status = BLDFM_OK;
        DeviceCache &dc = cache_for_current(&status);
        if (status != BLDFM_OK) return status;
        BatchBuild B;
        int rc = batch_build(cases, ncases, opts, &dc, B);
        if (rc != BLDFM_OK) return rc;
        if (workspace_bytes < B.total) return BLDFM_ERR_WORKSPACE;
        cudaStream_t st = (cudaStream_t)stream;
        char *ws = (char *)workspace;
        const bool graph =
            opts && opts->use_graph && st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread;
        DeviceCache::Aux *aux = nullptr;
        if ((rc = get_aux(dc, st, &aux)) != BLDFM_OK) return rc;
        if (!graph) {
            StageSlot *slt = nullptr;
            if ((rc = acquire_stage(dc, B.blob_bytes + 256, &slt)) != BLDFM_OK) return rc;
            batch_fill_blob(cases, ncases, B, ws, (char *)slt->buf);
            timers_begin(dc);
            if ((rc = batch_enqueue(cases, ncases, B, ws, slt->buf, st, dc.timing ? &dc : nullptr, aux)) != BLDFM_OK)
                return rc;
            CK(cudaEventRecord(slt->ev, st));
            return BLDFM_OK;
        }
        // graph path: an instance whose previous replay has finished, else a new
        // capture (up to two instances per topology), else wait for the oldest
        std::vector<int64_t> key = batch_key(cases, ncases, B, ws);
        auto &insts = dc.graphs[key];
        DeviceCache::GraphInst *gi = nullptr;
        for (auto &x : insts)
            if (cudaEventQuery(x.done) == cudaSuccess) {
                gi = &x;
                break;
            }
        if (!gi && insts.size() < 2) {
            DeviceCache::GraphInst x;
            if (cudaHostAlloc(&x.pinned, B.blob_bytes, cudaHostAllocDefault) != cudaSuccess) return BLDFM_ERR_CUDA;
            x.bytes = B.blob_bytes;
            CK(cudaEventCreateWithFlags(&x.done, cudaEventDisableTiming));
            batch_fill_blob(cases, ncases, B, ws, (char *)x.pinned);
            // capture the whole batch once; a failure leaves the stream usable
            cudaGraph_t graph_h = nullptr;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            rc = batch_enqueue(cases, ncases, B, ws, x.pinned, st, nullptr, aux);
            cudaError_t ce = cudaStreamEndCapture(st, &graph_h);
            if (rc != BLDFM_OK || ce != cudaSuccess) {
                if (graph_h) cudaGraphDestroy(graph_h);
                return rc != BLDFM_OK ? rc : BLDFM_ERR_CUDA;
            }
            ce = cudaGraphInstantiate(&x.exec, graph_h, 0);
            cudaGraphDestroy(graph_h);
            if (ce != cudaSuccess) return BLDFM_ERR_CUDA;
            CK(cudaGraphLaunch(x.exec, st));
            CK(cudaEventRecord(x.done, st));
            insts.push_back(x);
            return BLDFM_OK;
        }
        if (!gi) {
            gi = &insts[0];
            CK(cudaEventSynchronize(gi->done));
        }
        batch_fill_blob(cases, ncases, B, ws, (char *)gi->pinned);
        CK(cudaGraphLaunch(gi->exec, st));
        CK(cudaEventRecord(gi->done, st));
        return BLDFM_OK;
    });
}

int bldfm_surrogate_plan(const bldfm_desc *d, int32_t nlvls, int64_t *workspace_bytes)
{
    return bldfm_guarded([&]() -> int {
        if (!workspace_bytes) return BLDFM_ERR_ARG;
        int rc = sur_check_desc(d, nlvls);
        if (rc != BLDFM_OK) return rc;
        std::lock_guard<std::mutex> lk(g_mutex);
        HostPlan hp;
        if ((rc = make_plan(d, nullptr, nullptr, nullptr, nlvls, hp)) != BLDFM_OK) return rc;
        *workspace_bytes = (int64_t)sur_layout(hp.g).total;
        return BLDFM_OK;
    });
}

int bldfm_surrogate_solve(void *net, const bldfm_desc *d, const bldfm_surrogate_case *met, const double *z_host,
                          const double *prof_host, const int64_t *levels_host, int32_t nlvls, double *conc_dev,
                          double *flx_dev, void *workspace_dev, size_t workspace_bytes, void *stream)
{
    return bldfm_guarded([&]() -> int {
        std::lock_guard<std::mutex> lk(g_mutex);
        return sur_solve_impl(net, d, met, z_host, prof_host, levels_host, nlvls, conc_dev, flx_dev, workspace_dev,
                              workspace_bytes, (cudaStream_t)stream);
    });
}

int bldfm_surrogate_batch_plan(const bldfm_case *cases, const bldfm_surrogate_case *mets, int32_t ncases,
                               int64_t *workspace_bytes)
{
    return bldfm_guarded([&]() -> int {
        if (!workspace_bytes) return BLDFM_ERR_ARG;
        int rc = sur_batch_check(cases, mets, ncases);
        if (rc != BLDFM_OK) return rc;
        std::lock_guard<std::mutex> lk(g_mutex);
        BatchBuild B;
        bldfm_batch_opts opts = {256, 0, 0, 0, 1};
        if ((rc = batch_build(cases, ncases, &opts, nullptr, B, sur_extra_bytes(ncases))) != BLDFM_OK) return rc;
        *workspace_bytes = (int64_t)(B.total + sur_guard_bytes(ncases));
        return BLDFM_OK;
    });
}

int bldfm_surrogate_solve_batch(void *net, const bldfm_case *cases, const bldfm_surrogate_case *mets,
                                int32_t ncases, void *workspace, size_t workspace_bytes, void *stream)
{
    return bldfm_guarded([&]() -> int {
        std::lock_guard<std::mutex> lk(g_mutex);
        return sur_solve_batch_impl(net, cases, mets, ncases, workspace, workspace_bytes, (cudaStream_t)stream);
    });
}

}  // extern "C"
