// Footprint-weighted point measurement (reference: point_measurement,
// src/bldfm/utils.py:80-92, np.sum(f * g)) for a batch of (footprint, flux)
// pairs: out[b] = sum_i f[b][i] g[b][i] in FP64.
//
// The field is HBM-bound (16 bytes read per point, nothing written): each
// batch entry is split over the CTAs of one grid row, every thread keeps a
// Kahan-compensated FP64 sum of its grid-stride points (16-byte vector loads
// where the arrays allow), the CTA combines its threads in a fixed tree
// order, and a second kernel adds the per-CTA partials in index order, so the
// result is deterministic (no atomics) and carries about eps of error
// independent of n; numpy's pairwise sum differs from it at the level of its
// own rounding (about log2(n) eps).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bldfm_gb300.h"
#include "tc.cuh"

namespace {

const int MEAS_THREADS = 256;

struct Kahan {
    double s = 0.0, c = 0.0;
    __device__ __forceinline__ void add(double x)
    {
        const double y = __dsub_rn(x, c);
        const double t = __dadd_rn(s, y);
        c = __dsub_rn(__dsub_rn(t, s), y);
        s = t;
    }
};

__global__ void __launch_bounds__(MEAS_THREADS) meas_partial_kernel(const double *__restrict__ f,
                                                                    const double *__restrict__ g, int64_t n,
                                                                    int64_t stride, double *__restrict__ part)
{
    const int b = blockIdx.y;
    const double *fb = f + (size_t)b * stride, *gb = g + (size_t)b * stride;
    Kahan k;
    const int64_t t0 = (int64_t)blockIdx.x * MEAS_THREADS + threadIdx.x;
    const int64_t step = (int64_t)gridDim.x * MEAS_THREADS;
    const bool vec = ((((uintptr_t)fb) | ((uintptr_t)gb)) & 15) == 0;
    if (vec) {
        const int64_t n2 = n / 2;
        const double2 *f2 = (const double2 *)fb, *g2 = (const double2 *)gb;
        for (int64_t i = t0; i < n2; i += step) {
            const double2 a = __ldg(f2 + i), c = __ldg(g2 + i);
            k.add(__dmul_rn(a.x, c.x));
            k.add(__dmul_rn(a.y, c.y));
        }
        if ((n & 1) && t0 == 0) k.add(__dmul_rn(fb[n - 1], gb[n - 1]));
    } else {
        for (int64_t i = t0; i < n; i += step) k.add(__dmul_rn(__ldg(fb + i), __ldg(gb + i)));
    }
    __shared__ double ss[MEAS_THREADS];
    ss[threadIdx.x] = __dadd_rn(k.s, -k.c);
    __syncthreads();
    for (int w = MEAS_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ss[threadIdx.x] = __dadd_rn(ss[threadIdx.x], ss[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(size_t)b * gridDim.x + blockIdx.x] = ss[0];
}

__global__ void meas_final_kernel(const double *__restrict__ part, int nparts, int nbatch, double *__restrict__ out)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbatch) return;
    Kahan k;
    for (int i = 0; i < nparts; ++i) k.add(part[(size_t)b * nparts + i]);
    out[b] = __dadd_rn(k.s, -k.c);
}

// One CTA waits on an mbarrier that nothing arrives at, with an iteration
// limit: the bounded-wait path every waiting kernel takes on a timeout.  The
// elapsed global-timer nanoseconds of the wait go to ns[0].
__global__ void wait_timeout_kernel(long limit, int *status, long long *ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tc_mbar_init(&bar, 1);
        tc_fence_init();
    }
    __syncthreads();
    unsigned long long t0, t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    const uint32_t a = tc_smem(&bar);
    uint32_t done = 0;
    for (long it = 0; it < limit && !done; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(0u)
            : "memory");
    }
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    if (__syncthreads_or(!done) && threadIdx.x == 0) {
        *status = BLDFM_ERR_TIMEOUT;
        *ns = (long long)(t1 - t0);
    }
}

}  // namespace

extern "C" {

// Self-check of the failure-detection path (no reference counterpart): a
// kernel whose wait can never complete gives up after `limit` polls and
// reports BLDFM_ERR_TIMEOUT in *status_host, with the time the wait took in
// *wait_ns_host; the context stays usable.
int bldfm_selftest_wait_timeout(int64_t limit, int32_t *status_host, int64_t *wait_ns_host)
{
    if (!status_host || !wait_ns_host || limit < 1 || limit > ((int64_t)1 << 20)) return BLDFM_ERR_ARG;
    void *d = nullptr;
    if (cudaMalloc(&d, 16) != cudaSuccess) return BLDFM_ERR_CUDA;
    int rc = BLDFM_OK;
    if (cudaMemset(d, 0, 16) != cudaSuccess) rc = BLDFM_ERR_CUDA;
    if (rc == BLDFM_OK) {
        wait_timeout_kernel<<<1, 64>>>((long)limit, (int *)d, (long long *)((char *)d + 8));
        if (cudaDeviceSynchronize() != cudaSuccess) rc = BLDFM_ERR_CUDA;
    }
    long long h[2] = {0, 0};
    if (rc == BLDFM_OK && cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost) != cudaSuccess) rc = BLDFM_ERR_CUDA;
    *status_host = (int32_t)(int)h[0];
    *wait_ns_host = (int64_t)h[1];
    cudaFree(d);
    return rc;
}

// Scratch bytes bldfm_point_measurement needs for nbatch entries of n points.
int64_t bldfm_point_measurement_workspace(int64_t n, int32_t nbatch)
{
    if (n < 0 || nbatch < 1) return -1;
    int dev = 0, nsm = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int64_t per = (n + MEAS_THREADS * 8 - 1) / (MEAS_THREADS * 8);
    const int64_t want = (int64_t)nsm * 4 / nbatch + 1;
    if (per > want) per = want;
    if (per < 1) per = 1;
    if (per > 65535) per = 65535;
    return per * nbatch * (int64_t)sizeof(double);
}

int bldfm_point_measurement(const double *f_dev, const double *g_dev, int64_t n, int64_t stride, int32_t nbatch,
                            double *out_dev, void *workspace_dev, size_t workspace_bytes, void *stream)
{
    if (!f_dev || !g_dev || !out_dev || n < 0 || stride < n || nbatch < 1 || nbatch > 65535) return BLDFM_ERR_ARG;
    const int64_t need = bldfm_point_measurement_workspace(n, nbatch);
    if (!workspace_dev || need < 0 || (int64_t)workspace_bytes < need) return BLDFM_ERR_WORKSPACE;
    if (((uintptr_t)workspace_dev & 7) != 0) return BLDFM_ERR_ARG;
    const int per = (int)(need / ((int64_t)nbatch * (int64_t)sizeof(double)));
    cudaStream_t st = (cudaStream_t)stream;
    double *part = (double *)workspace_dev;
    meas_partial_kernel<<<dim3(per, nbatch), MEAS_THREADS, 0, st>>>(f_dev, g_dev, n, stride, part);
    meas_final_kernel<<<(nbatch + 127) / 128, 128, 0, st>>>(part, per, nbatch, out_dev);
    return cudaGetLastError() == cudaSuccess ? BLDFM_OK : BLDFM_ERR_CUDA;
}

}  // extern "C"
