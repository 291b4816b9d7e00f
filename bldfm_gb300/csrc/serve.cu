// Serving path of the learned surrogate (footprint mode, MOST profiles): the
// per-mode sweep of the FP32 solver is replaced by the MLP's transfer at z_m.
// One thread per solved mode in each kernel; the spectra kernel writes the
// same (Xp, Xq) slots and Hermitian mirrors as the sweep, so the output
// transform is the solver's own.
#include "../../include/bldfm_gb300.h"
#include "devmath.cuh"
#include "mlp_common.cuh"
#include "serve.h"
#include "surrogate_phys.cuh"
#include "tc.cuh"

#include <algorithm>

namespace {

// rotated, scaled wavenumbers of mode m: k_par (signed), |k_perp|, |k|
__device__ __forceinline__ void mode_k(const SolveGeom &g, uint32_t e, float ax, float ay, float zm, int &r, int &c,
                                       bool &paired, float &kpar, float &kperp, float &k)
{
    unpack_mode(e, r, c, paired);
    const float lx = ax * (float)freq_of_index(c, g.nlx), ly = ay * (float)freq_of_index(r, g.nly);
    kpar = zm * fmaf(g.ex, lx, g.ey * ly);
    kperp = fabsf(zm * fmaf(-g.ey, lx, g.ex * ly));
    k = sqrtf(fmaf(kpar, kpar, kperp * kperp));
}

__global__ void sur_features_kernel(const SolveGeom g, const uint32_t *__restrict__ modes, float ax, float ay,
                                    float zm, float s1, float s2, float s3, float *__restrict__ X, int64_t npad)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npad) return;
    float kpar = 1.f, kperp = 0.f;
    if (m < g.nsolved) {
        int r, c;
        bool paired;
        float k;
        mode_k(g, modes[m], ax, ay, zm, r, c, paired, kpar, kperp, k);
        kpar = fabsf(kpar);
    }
    feature_row(X + (size_t)m * 8, kpar, kperp, s1, s2, s3);
}

__global__ void sur_exact_kernel(const SolveGeom g, const uint32_t *__restrict__ modes, float ax, float ay, float zm,
                                 const TransferCase *__restrict__ tc, const float4 *__restrict__ steps,
                                 float *__restrict__ Y)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= g.nsolved) return;
    int r, c;
    bool paired;
    float kpar, kperp, k;
    mode_k(g, modes[m], ax, ay, zm, r, c, paired, kpar, kperp, k);
    transfer_one(*tc, steps, fabsf(kpar), kperp, Y + (size_t)m * 4);
}

// (Xp, Xq) of solved mode e and its Hermitian mirror from the targets y
__device__ __forceinline__ void emit_spectrum(const SolveGeom &g, uint32_t e, const float *y, float ax, float ay,
                                              float zm, float inv_wind, float ktop, float utop,
                                              float2 *__restrict__ Xp, float2 *__restrict__ Xq)
{
    int r, c;
    bool paired;
    float kpar, kperp, k;
    mode_k(g, e, ax, ay, zm, r, c, paired, kpar, kperp, k);
    float2 Tq, Rt;
    decode_transfer(y, k, Tq, Rt);
    Rt = sp_cmul(Rt, top_ratio(ktop, utop, fabsf(kpar), kperp));
    if (kpar < 0.f) {
        Tq.y = -Tq.y;
        Rt.y = -Rt.y;
    }
    const float q0 = (float)g.q0dc_fp;
    float2 q = make_float2(q0 * Tq.x, q0 * Tq.y);
    float2 p = sp_cmul(make_float2(Rt.x * inv_wind, Rt.y * inv_wind), q);
    if (g.do_shift) {
        const int kx = freq_of_index(c, g.nlx), ky = freq_of_index(r, g.nly);
        const uint32_t turns = (uint32_t)kx * g.turn_x + (uint32_t)ky * g.turn_y;
        float sn, cs;
        sincospif((float)(int32_t)turns * 4.656612873077393e-10f, &sn, &cs);
        const float2 sh = make_float2(cs, sn);
        p = sp_cmul(p, sh);
        q = sp_cmul(q, sh);
    }
    Xp[spec_idx(g, 0, r, c)] = p;
    Xq[spec_idx(g, 0, r, c)] = q;
    if (paired) {
        const int rm = index_of_freq(-freq_of_index(r, g.nly), g.nly);
        const int cm = index_of_freq(-freq_of_index(c, g.nlx), g.nlx);
        Xp[spec_idx(g, 0, rm, cm)] = make_float2(p.x, -p.y);
        Xq[spec_idx(g, 0, rm, cm)] = make_float2(q.x, -q.y);
    }
}

__global__ void sur_spectra_kernel(const SolveGeom g, const uint32_t *__restrict__ modes, const float *__restrict__ Y,
                                   float ax, float ay, float zm, float inv_wind, float ktop, float utop,
                                   float2 *__restrict__ Xp, float2 *__restrict__ Xq)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= g.nsolved) return;
    emit_spectrum(g, modes[m], Y + (size_t)m * 4, ax, ay, zm, inv_wind, ktop, utop, Xp, Xq);
}

// ---------------------------------------------------------------------------
// Fused serving kernel: features -> MLP -> spectra for 128 modes per tile,
// one persistent CTA of 256 threads per SM.  The tile's activations stay in
// shared memory (BF16, core-matrix K-major layout: the A operand of the next
// layer), the hidden 256 x 256 layers run as one tcgen05 MMA chain each
// (M = 128, N = 256, K = 256) into a 256-column TMEM accumulator, and the
// next layer's BF16 weights stream into the single 128 KB weight buffer by
// bulk copy while the epilogue (bias + GELU from TMEM) runs.  The input and
// output layers are FP32 on the CUDA cores.  Every mbarrier wait is bounded;
// on a timeout the kernel records BLDFM_ERR_TIMEOUT, waits (bounded) for its
// own copies and MMAs in flight, frees TMEM and returns.
// ---------------------------------------------------------------------------
struct SvSmem {
    uint16_t A[128 * MLP_H];    // activations (A operand)
    uint16_t W[MLP_H * MLP_H];  // Wt_j (B operand)
    float W0[MLP_IN * MLP_H];
    float bias[4][MLP_H];
    float W4[MLP_H * MLP_OUT];
    float4 Yp[2][128];  // output-layer partial sums of the two column halves
    float X[128][8];    // features
    float b4[4];
};

__device__ __forceinline__ void sv_put8(uint16_t *st, int r, int c, const float *v)
{
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] = (uint32_t)f2bf(v[2 * q]) | ((uint32_t)f2bf(v[2 * q + 1]) << 16);
    *(uint4 *)(st + tc_core_offset(r, c, MLP_H) / 2) = make_uint4(w[0], w[1], w[2], w[3]);
}

__global__ void __launch_bounds__(256, 1)
    sur_serve_kernel(const SolveGeom g, const uint32_t *__restrict__ modes, float ax, float ay, float zm, float s1,
                     float s2, float s3, float inv_wind, float ktop, float utop, const MlpServing net,
                     float2 *__restrict__ Xp, float2 *__restrict__ Xq, int *err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    SvSmem &S = *reinterpret_cast<SvSmem *>(smem_raw);
    __shared__ uint64_t bar_w, bar_mma;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tc_tmem_alloc(&tmem_slot, 256);
    if (tid == 0) {
        tc_mbar_init(&bar_w, 1);
        tc_mbar_init(&bar_mma, 1);
        tc_fence_init();
    }
    for (int i = tid; i < MLP_IN * MLP_H; i += 256) S.W0[i] = net.P[MLP_OFF_W0 + i];
    for (int i = tid; i < MLP_H; i += 256) {
        S.bias[0][i] = net.P[MLP_OFF_B0 + i];
#pragma unroll
        for (int j = 1; j <= 3; ++j) S.bias[j][i] = net.P[MLP_OFF_B(j) + i];
    }
    for (int i = tid; i < MLP_H * MLP_OUT; i += 256) S.W4[i] = net.P[MLP_OFF_W4 + i];
    if (tid < MLP_OUT) S.b4[tid] = net.P[MLP_OFF_B4 + tid];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const int64_t ntiles = (g.nsolved + 127) / 128;
    const uint32_t WBYTES = MLP_H * MLP_H * 2;
    const uint32_t idesc = tc_idesc_bf16(128, MLP_H);
    const uint32_t sbo = (MLP_H / 8) * 128;
    uint32_t wph = 0, mph = 0;
    bool pend_w = false, pend_mma = false;  // thread 0: copies / MMAs not yet waited for
    if (tid == 0 && (int64_t)blockIdx.x < ntiles) {
        tc_expect_tx(&bar_w, WBYTES);
        tc_bulk_load(S.W, net.Wt[0], WBYTES, &bar_w);
        pend_w = true;
    }
    bool failed = false;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        if (tid < 128) {
            const int64_t m = tile * 128 + tid;
            float kpar = 1.f, kperp = 0.f;
            if (m < g.nsolved) {
                int r, c;
                bool pr;
                float k;
                mode_k(g, modes[m], ax, ay, zm, r, c, pr, kpar, kperp, k);
                kpar = fabsf(kpar);
            }
            feature_row(S.X[tid], kpar, kperp, s1, s2, s3);
        }
        __syncthreads();
        {   // input layer: thread = (row, half of the 256 features)
            const int r = tid & 127, f0 = (tid >> 7) * 128;
            const float4 xa = *(const float4 *)&S.X[r][0], xb = *(const float4 *)&S.X[r][4];
            const float x[8] = {xa.x, xa.y, xa.z, xa.w, xb.x, xb.y, xb.z, xb.w};
#pragma unroll 1
            for (int fb = 0; fb < 128; fb += 8) {
                float h[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int f = f0 + fb + q;
                    float z = S.bias[0][f];
#pragma unroll
                    for (int i = 0; i < MLP_IN; ++i) z = fmaf(x[i], S.W0[i * MLP_H + f], z);
                    h[q] = gelu_f(z);
                }
                sv_put8(S.A, r, f0 + fb, h);
            }
        }
        tc_fence_proxy_async();
        __syncthreads();
        for (int j = 0; j < 3; ++j) {
            bool bad = !tc_mbar_wait(&bar_w, wph);
            if (__syncthreads_or(bad)) {
                failed = true;
                break;
            }
            wph ^= 1;
            if (tid == 0) {
                pend_w = false;
                tc_fence_after();
                const uint32_t a0 = tc_smem(S.A), b0 = tc_smem(S.W);
#pragma unroll 1
                for (int s = 0; s < MLP_H / 16; ++s)
                    tc_mma(tmem, tc_desc(a0 + s * 256, 128, sbo), tc_desc(b0 + s * 256, 128, sbo), idesc,
                           s > 0 ? 1u : 0u);
                tc_commit(&bar_mma);
                pend_mma = true;
            }
            bad = !tc_mbar_wait(&bar_mma, mph);
            if (__syncthreads_or(bad)) {
                failed = true;
                break;
            }
            mph ^= 1;
            if (tid == 0) {
                pend_mma = false;
                // the weights are free: stream in the next layer's (or the next tile's first)
                const uint16_t *next = j < 2 ? net.Wt[j + 1] : (tile + gridDim.x < ntiles ? net.Wt[0] : nullptr);
                if (next) {
                    tc_expect_tx(&bar_w, WBYTES);
                    tc_bulk_load(S.W, next, WBYTES, &bar_w);
                    pend_w = true;
                }
            }
            tc_fence_after();
            // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (its rows), columns 128 (w / 4) .. +127
            const int qd = warp & 3, hf = warp >> 2;
            const int row = 32 * qd + lane;
            const uint32_t tb = tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(128 * hf);
            if (j < 2) {
#pragma unroll 1
                for (int cc = 0; cc < 4; ++cc) {
                    float v[32];
                    tc_ld32(tb + 32 * cc, v);
                    const int c0 = 128 * hf + 32 * cc;
#pragma unroll
                    for (int i = 0; i < 32; ++i) v[i] = gelu_f(v[i] + S.bias[j + 1][c0 + i]);
#pragma unroll
                    for (int q = 0; q < 4; ++q) sv_put8(S.A, row, c0 + 8 * q, v + 8 * q);
                }
                tc_fence_proxy_async();
            } else {
                float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
                for (int cc = 0; cc < 4; ++cc) {
                    float v[32];
                    tc_ld32(tb + 32 * cc, v);
                    const int c0 = 128 * hf + 32 * cc;
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const float h = gelu_f(v[i] + S.bias[3][c0 + i]);
                        const float4 w4 = *(const float4 *)&S.W4[(c0 + i) * MLP_OUT];
                        y.x = fmaf(h, w4.x, y.x);
                        y.y = fmaf(h, w4.y, y.y);
                        y.z = fmaf(h, w4.z, y.z);
                        y.w = fmaf(h, w4.w, y.w);
                    }
                }
                S.Yp[hf][row] = y;
            }
            tc_fence_before();
            __syncthreads();
        }
        if (failed) break;
        if (tid < 128) {
            const int64_t m = tile * 128 + tid;
            if (m < g.nsolved) {
                const float4 a = S.Yp[0][tid], b = S.Yp[1][tid];
                const float y[4] = {a.x + b.x + S.b4[0], a.y + b.y + S.b4[1], a.z + b.z + S.b4[2],
                                    a.w + b.w + S.b4[3]};
                emit_spectrum(g, modes[m], y, ax, ay, zm, inv_wind, ktop, utop, Xp, Xq);
            }
        }
    }
    if (failed && tid == 0) {
        atomicExch(err, BLDFM_ERR_TIMEOUT);
        if (pend_mma) tc_mbar_wait(&bar_mma, mph);
        if (pend_w) tc_mbar_wait(&bar_w, wph);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_tmem_free(tmem, 256);
}

inline unsigned blocks_for(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

cudaError_t launch_sur_features(const SolveGeom &g, const uint32_t *modes, float ax, float ay, float zm, float s1,
                                float s2, float s3, float *X, int64_t npad, cudaStream_t st)
{
    if (npad <= 0) return cudaSuccess;
    sur_features_kernel<<<blocks_for(npad), 256, 0, st>>>(g, modes, ax, ay, zm, s1, s2, s3, X, npad);
    return cudaGetLastError();
}

cudaError_t launch_sur_exact(const SolveGeom &g, const uint32_t *modes, float ax, float ay, float zm,
                             const TransferCase *tc, const float4 *steps, float *Y, cudaStream_t st)
{
    if (g.nsolved <= 0) return cudaSuccess;
    sur_exact_kernel<<<blocks_for(g.nsolved), 256, 0, st>>>(g, modes, ax, ay, zm, tc, steps, Y);
    return cudaGetLastError();
}

cudaError_t launch_sur_serve(const SolveGeom &g, const uint32_t *modes, float ax, float ay, float zm, float s1,
                             float s2, float s3, float inv_wind, float ktop, float utop, const MlpServing &net,
                             float2 *Xp, float2 *Xq, int *err, int nsm, cudaStream_t st)
{
    if (g.nsolved <= 0) return cudaSuccess;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(sur_serve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(SvSmem));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int64_t ntiles = (g.nsolved + 127) / 128;
    const int grid = (int)std::min<int64_t>(ntiles, std::max(nsm, 1));
    sur_serve_kernel<<<grid, 256, sizeof(SvSmem), st>>>(g, modes, ax, ay, zm, s1, s2, s3, inv_wind, ktop, utop, net,
                                                        Xp, Xq, err);
    return cudaGetLastError();
}

cudaError_t launch_sur_spectra(const SolveGeom &g, const uint32_t *modes, const float *Y, float ax, float ay,
                               float zm, float inv_wind, float ktop, float utop, float2 *Xp, float2 *Xq,
                               cudaStream_t st)
{
    if (g.nsolved <= 0) return cudaSuccess;
    sur_spectra_kernel<<<blocks_for(g.nsolved), 256, 0, st>>>(g, modes, Y, ax, ay, zm, inv_wind, ktop, utop, Xp,
                                                              Xq);
    return cudaGetLastError();
}
