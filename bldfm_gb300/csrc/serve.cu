// Serving path of the learned surrogate (footprint mode, MOST profiles): the
// per-mode sweep of the FP32 solver is replaced by the MLP's transfer at z_m.
// One thread per solved mode in each kernel; the spectra kernel writes the
// same (Xp, Xq) slots and Hermitian mirrors as the sweep, so the output
// transform is the solver's own.
#include "devattr.h"
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
// one persistent CTA of 256 threads per SM.  All four matrix layers run on
// the tensor cores (tcgen05.mma, M = 128, N = 256, FP32 accumulator in a
// 256-column TMEM allocation); the epilogues (bias + GELU, from TMEM) and the
// 256 -> 4 output layer run on the CUDA cores in FP32.
//
// Input layer in BF16 at FP32 accuracy: x = xh + xl and W0 = wh + wl split
// into BF16 parts, K = 32 columns [xh | xl | xh | 0] x [wh | wh | wl | 0]
// give x.W0 up to the xl.wl term (relative 2^-16).
//
// Shared memory: the tile's activations (BF16, core-matrix K-major layout: the
// A operand of the next layer; the first 8 KB hold the input-layer operand
// before its MMA), one 256 x 256 BF16 weight matrix streamed by bulk copy
// while the previous layer's epilogue runs, the split W0, biases, W4.  Every
// mbarrier wait is bounded; on a timeout the kernel records
// BLDFM_ERR_TIMEOUT, waits (bounded) for its own copies and MMAs in flight,
// frees TMEM and returns.
// ---------------------------------------------------------------------------
#define SV_K0 32     // K of the split input layer
#define SV_WARPS 16  // 4 warps per TMEM lane quarter, each a quarter of the 256 columns

struct SvSmem {
    uint16_t A[128 * MLP_H];    // activations (A operand)
    uint16_t W[MLP_H * MLP_H];  // Wt_j (B operand)
    uint16_t B0[MLP_H * SV_K0]; // split W0 (B operand of the input layer)
    float bias[4][MLP_H];
    float W4[MLP_H * MLP_OUT];
    float4 Yp[SV_WARPS / 4][128];  // output-layer partial sums of the column quarters
    float b4[4];
};

__device__ __forceinline__ void sv_put8(uint16_t *st, int r, int c, const float *v)
{
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] = (uint32_t)f2bf(v[2 * q]) | ((uint32_t)f2bf(v[2 * q + 1]) << 16);
    *(uint4 *)(st + tc_core_offset(r, c, MLP_H) / 2) = make_uint4(w[0], w[1], w[2], w[3]);
}

// epilogue of a hidden layer: this thread's row, 64 columns from c0, bias,
// GELU, BF16 into the A tile
__device__ __forceinline__ void sv_epilogue_hidden(uint32_t tb, int row, int c0, const float *bias, uint16_t *A)
{
#pragma unroll 1
    for (int cc = 0; cc < 2; ++cc) {
        float v[32];
        tc_ld32(tb + 32 * cc, v);
        const int cb = c0 + 32 * cc;
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = gelu_f(v[i] + bias[cb + i]);
#pragma unroll
        for (int q = 0; q < 4; ++q) sv_put8(A, row, cb + 8 * q, v + 8 * q);
    }
}

__global__ void __launch_bounds__(32 * SV_WARPS, 1)
    sur_serve_kernel(const SurCase *__restrict__ cases, int ncases, int64_t ntiles, const MlpServing net, int *err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    SvSmem &S = *reinterpret_cast<SvSmem *>(smem_raw);
    __shared__ uint64_t bar_w, bar_mma;
    __shared__ uint32_t tmem_slot;
    __shared__ SurCase sc;  // the current tile's case
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tc_tmem_alloc(&tmem_slot, 256);
    if (tid == 0) {
        tc_mbar_init(&bar_w, 1);
        tc_mbar_init(&bar_mma, 1);
        tc_fence_init();
    }
    // split W0 [in][out] into the B operand [out][K = 32]
    for (int e = tid; e < MLP_H * SV_K0; e += blockDim.x) {
        const int f = e / SV_K0, k = e % SV_K0, grp = k >> 3, i = k & 7;
        const float w = net.P[MLP_OFF_W0 + i * MLP_H + f];
        const uint16_t wh = f2bf(w);
        const uint16_t wl = f2bf(w - bf2f(wh));
        S.B0[tc_core_offset(f, k, SV_K0) / 2] = grp < 2 ? wh : (grp == 2 ? wl : (uint16_t)0);
    }
    for (int i = tid; i < MLP_H; i += blockDim.x) {
        S.bias[0][i] = net.P[MLP_OFF_B0 + i];
#pragma unroll
        for (int j = 1; j <= 3; ++j) S.bias[j][i] = net.P[MLP_OFF_B(j) + i];
    }
    for (int i = tid; i < MLP_H * MLP_OUT; i += blockDim.x) S.W4[i] = net.P[MLP_OFF_W4 + i];
    if (tid < MLP_OUT) S.b4[tid] = net.P[MLP_OFF_B4 + tid];
    tc_fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t WBYTES = MLP_H * MLP_H * 2;
    const uint32_t idesc = tc_idesc_bf16(128, MLP_H);
    const uint32_t sbo = (MLP_H / 8) * 128, sbo0 = (SV_K0 / 8) * 128;
    uint32_t wph = 0, mph = 0;
    bool pend_w = false, pend_mma = false;  // thread 0: copies / MMAs not yet waited for
    if (tid == 0 && (int64_t)blockIdx.x < ntiles) {
        tc_expect_tx(&bar_w, WBYTES);
        tc_bulk_load(S.W, net.Wt[0], WBYTES, &bar_w);
        pend_w = true;
    }
    // epilogue geometry: warp w reads TMEM lanes 32 (w % 4) .. +31 (its rows), columns 64 (w / 4) .. +63
    const int qd = warp & 3, hf = warp >> 2;
    const int row = 32 * qd + lane;
    const uint32_t tb = tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(64 * hf);
    bool failed = false;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        if (tid < 32) {
            // the tile's case: last case with tile0 <= tile, copied to shared memory
            int lo = 0, hi = ncases - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (cases[mid].tile0 <= tile) lo = mid;
                else hi = mid - 1;
            }
            const uint32_t *src = (const uint32_t *)(cases + lo);
            uint32_t *dst = (uint32_t *)&sc;
            for (int i = tid; i < (int)(sizeof(SurCase) / 4); i += 32) dst[i] = src[i];
        }
        __syncthreads();
        const SolveGeom &g = sc.g;
        const int64_t lt = tile - sc.tile0;  // tile within the case
        if (tid < 128) {
            // features -> [xh | xl | xh | 0] of row tid (input-layer A operand, K = 32)
            const int64_t m = lt * 128 + tid;
            float kpar = 1.f, kperp = 0.f;
            if (m < g.nsolved) {
                int r, c;
                bool pr;
                float k;
                mode_k(g, sc.modes[m], sc.ax, sc.ay, sc.zm, r, c, pr, kpar, kperp, k);
                kpar = fabsf(kpar);
            }
            float x[8], xl[8];
            feature_row(x, kpar, kperp, sc.s1, sc.s2, sc.s3);
#pragma unroll
            for (int i = 0; i < 8; ++i) xl[i] = x[i] - bf2f(f2bf(x[i]));
            uint16_t *A0 = S.A;
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = (uint32_t)f2bf(x[2 * q]) | ((uint32_t)f2bf(x[2 * q + 1]) << 16);
            const uint4 hi = make_uint4(w[0], w[1], w[2], w[3]);
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = (uint32_t)f2bf(xl[2 * q]) | ((uint32_t)f2bf(xl[2 * q + 1]) << 16);
            const uint4 lo = make_uint4(w[0], w[1], w[2], w[3]);
            *(uint4 *)(A0 + tc_core_offset(tid, 0, SV_K0) / 2) = hi;
            *(uint4 *)(A0 + tc_core_offset(tid, 8, SV_K0) / 2) = lo;
            *(uint4 *)(A0 + tc_core_offset(tid, 16, SV_K0) / 2) = hi;
            *(uint4 *)(A0 + tc_core_offset(tid, 24, SV_K0) / 2) = make_uint4(0u, 0u, 0u, 0u);
        }
        tc_fence_proxy_async();
        __syncthreads();
        // layers 0..3: input layer (split W0 in S.B0), then Wt_1..3 streamed through S.W
        for (int j = 0; j < 4; ++j) {
            bool bad = false;
            if (j > 0) {
                bad = !tc_mbar_wait(&bar_w, wph);
                if (__syncthreads_or(bad)) {
                    failed = true;
                    break;
                }
                wph ^= 1;
            }
            if (tid == 0) {
                if (j > 0) pend_w = false;
                tc_fence_after();
                const uint32_t a0 = tc_smem(S.A);
                if (j == 0) {
                    const uint32_t b0 = tc_smem(S.B0);
#pragma unroll 1
                    for (int s = 0; s < SV_K0 / 16; ++s)
                        tc_mma(tmem, tc_desc(a0 + s * 256, 128, sbo0), tc_desc(b0 + s * 256, 128, sbo0), idesc,
                               s > 0 ? 1u : 0u);
                } else {
                    const uint32_t b0 = tc_smem(S.W);
#pragma unroll 1
                    for (int s = 0; s < MLP_H / 16; ++s)
                        tc_mma(tmem, tc_desc(a0 + s * 256, 128, sbo), tc_desc(b0 + s * 256, 128, sbo), idesc,
                               s > 0 ? 1u : 0u);
                }
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
                // after layer j >= 1 the weights are free: stream in the next
                // layer's (or, after the last, the next tile's first)
                if (j >= 1) {
                    const uint16_t *next =
                        j < 3 ? net.Wt[j] : (tile + gridDim.x < ntiles ? net.Wt[0] : nullptr);
                    if (next) {
                        tc_expect_tx(&bar_w, WBYTES);
                        tc_bulk_load(S.W, next, WBYTES, &bar_w);
                        pend_w = true;
                    }
                }
            }
            tc_fence_after();
            if (j < 3) {
                sv_epilogue_hidden(tb, row, 64 * hf, S.bias[j], S.A);
                tc_fence_proxy_async();
            } else {
                float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
                for (int cc = 0; cc < 2; ++cc) {
                    float v[32];
                    tc_ld32(tb + 32 * cc, v);
                    const int c0 = 64 * hf + 32 * cc;
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
            const int64_t m = lt * 128 + tid;
            if (m < g.nsolved) {
                float4 a = S.Yp[0][tid];
#pragma unroll
                for (int qq = 1; qq < SV_WARPS / 4; ++qq) {
                    const float4 b = S.Yp[qq][tid];
                    a = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
                }
                const float y[4] = {a.x + S.b4[0], a.y + S.b4[1], a.z + S.b4[2], a.w + S.b4[3]};
                emit_spectrum(g, sc.modes[m], y, sc.ax, sc.ay, sc.zm, sc.inv_wind, sc.ktop, sc.utop, sc.Xp, sc.Xq);
            }
        }
        __syncthreads();  // sc is rewritten by the next tile
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

cudaError_t launch_sur_serve(const SurCase *cases, int ncases, int64_t ntiles, const MlpServing &net, int *err,
                             int nsm, cudaStream_t st)
{
    if (ntiles <= 0 || ncases <= 0) return cudaSuccess;
    static uint64_t attr = 0;
    if (first_on_device(attr)) {
        cudaError_t e = cudaFuncSetAttribute(sur_serve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(SvSmem));
        if (e != cudaSuccess) {
            attr = 0;
            return e;
        }
    }
    const int grid = (int)std::min<int64_t>(ntiles, std::max(nsm, 1));
    sur_serve_kernel<<<grid, 32 * SV_WARPS, sizeof(SvSmem), st>>>(cases, ncases, ntiles, net, err);
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
