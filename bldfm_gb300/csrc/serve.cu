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
    const float q0 = g.q0dc_f;
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
// Fused serving kernel (sur_serve_kernel) and its helpers
// ---------------------------------------------------------------------------
#define SV_K0 32     // K of the split input layer
#define SV_WARPS 8  // epilogue warps: 2 per TMEM lane quarter, each 2 x 32 columns of a half
#define SV_THREADS (32 * SV_WARPS + 32)  // + one control warp (copies and MMAs)
#define SV_AB(i) (256u + 64u * (uint32_t)(i))  // TMEM column of activation K-half buffer i

struct SvSmem {
    uint16_t Wq[4][128 * 128];   // Wt_j quarters (N half, K half), B operands
    uint16_t A0[128 * SV_K0];    // input-layer A operand (split features)
    uint16_t B0[MLP_H * SV_K0];  // split W0 (B operand of the input layer)
    float bias[4][MLP_H];
    float W4[MLP_H * MLP_OUT];
    float4 Yp[SV_WARPS / 4][128];  // output-layer partial sums of the column groups
    float b4[4];
};

// Quarter q = 2 nh + kh of Wt_j (Wq_j: four contiguous 32 KB quarters in the
// layout of a 128 x 128 operand) into shared memory: one bulk copy.
__device__ __forceinline__ void sv_load_quarter(uint16_t *dst, const uint16_t *Wq, int q, uint64_t *bar)
{
    const uint32_t bytes = 128 * 128 * 2;
    tc_expect_tx(bar, bytes);
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     tc_smem(dst)),
                 "l"((const char *)Wq + (size_t)q * bytes), "r"(bytes), "r"(tc_smem(bar))
                 : "memory");
}

// D[dcol .. +127] (+)= A[TMEM acol .. +63] (K = 128) x quarter^T: 8 MMAs of
// K = 16; bdesc is the quarter's descriptor (each K step advances the start
// address by 256 bytes, 16 in the descriptor's address field)
__device__ __forceinline__ void sv_mma_quarter(uint32_t dt, uint32_t at, uint64_t bdesc, uint32_t idesc,
                                               bool accumulate)
{
    tc_mma_ts(dt, at, bdesc, idesc, accumulate ? 1u : 0u);
#pragma unroll
    for (int s = 1; s < 8; ++s) tc_mma_ts(dt, at + 8 * s, bdesc + (uint64_t)(16 * s), idesc, 1u);
}

// K steps s0 .. s0 + 3 of a quarter MMA (K = 64 of the 128)
__device__ __forceinline__ void sv_mma_quarter_part(uint32_t dt, uint32_t at, uint64_t bdesc, uint32_t idesc, int s0)
{
#pragma unroll
    for (int s = 0; s < 4; ++s)
        tc_mma_ts(dt, at + 8 * (s0 + s), bdesc + (uint64_t)(16 * (s0 + s)), idesc, 1u);
}

// Bounded wait for phase `parity` of an mbarrier that also gives up as soon
// as another warp has recorded a failure in *fail.
__device__ __forceinline__ bool sv_wait(uint64_t *bar, uint32_t parity, const volatile int *fail)
{
    const uint32_t a = tc_smem(bar);
    for (long it = 0; it < BLDFM_WAIT_POLLS; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 63) == 63 && *fail) return false;
    }
    return false;
}

__device__ __forceinline__ void sv_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(tc_smem(bar)) : "memory");
}

// barrier of the epilogue warps only (the control warp does not take part)
__device__ __forceinline__ void sv_epi_sync() { asm volatile("bar.sync 1, %0;" ::"n"(32 * SV_WARPS) : "memory"); }
// barrier of the feature / emit warps 0..3
__device__ __forceinline__ void sv_row_sync() { asm volatile("bar.sync 2, 128;" ::: "memory"); }

// mode word of row r of a tile (0 past the case's last mode)
__device__ __forceinline__ uint32_t sv_mode_word(const SurCase &c, int64_t tile, int r)
{
    const int64_t m = (tile - c.tile0) * 128 + r;
    return m < c.g.nsolved ? c.modes[m] : 0u;
}

// features of row r of a tile (mode word e) -> [xh | xl | xh | 0] (input-layer
// A operand, K = 32)
__device__ __forceinline__ void sv_features(const SurCase &c, int64_t tile, int r, uint32_t e, uint16_t *A0)
{
    const int64_t m = (tile - c.tile0) * 128 + r;
    float kpar = 1.f, kperp = 0.f;
    if (m < c.g.nsolved) {
        int rr, cc;
        bool pr;
        float k;
        mode_k(c.g, e, c.ax, c.ay, c.zm, rr, cc, pr, kpar, kperp, k);
        kpar = fabsf(kpar);
    }
    float x[8], xl[8];
    feature_row(x, kpar, kperp, c.s1, c.s2, c.s3);
#pragma unroll
    for (int i = 0; i < 8; ++i) xl[i] = x[i] - bf2f(f2bf(x[i]));
    const uint4 hi = make_uint4(pack_bf16x2(x[0], x[1]), pack_bf16x2(x[2], x[3]), pack_bf16x2(x[4], x[5]),
                                pack_bf16x2(x[6], x[7]));
    const uint4 lo = make_uint4(pack_bf16x2(xl[0], xl[1]), pack_bf16x2(xl[2], xl[3]), pack_bf16x2(xl[4], xl[5]),
                                pack_bf16x2(xl[6], xl[7]));
    *(uint4 *)(A0 + tc_core_offset(r, 0, SV_K0) / 2) = hi;
    *(uint4 *)(A0 + tc_core_offset(r, 8, SV_K0) / 2) = lo;
    *(uint4 *)(A0 + tc_core_offset(r, 16, SV_K0) / 2) = hi;
    *(uint4 *)(A0 + tc_core_offset(r, 24, SV_K0) / 2) = make_uint4(0u, 0u, 0u, 0u);
}

// hidden-layer epilogue of two 32-column groups of this thread's row
// (accumulator columns td0, td1, both TMEM loads in flight together): bias,
// GELU in f32x2 lanes, BF16 pairs into 16 activation columns each (ta0,
// ta1); when bar0 is given, the first group's activations are announced on
// it (one arrival per warp) before the second group is computed
__device__ __forceinline__ void sv_epilogue_hidden2(uint32_t td0, uint32_t td1, uint32_t ta0, uint32_t ta1,
                                                    const float *bias0, const float *bias1, uint64_t *bar0)
{
    float v[64];
    tc_ld32x2(td0, td1, v);
    uint32_t w[16];
#pragma unroll
    for (int p = 0; p < 16; ++p) {
        const float2 g = gelu2_bias(make_float2(v[2 * p], v[2 * p + 1]), *(const float2 *)(bias0 + 2 * p));
        w[p] = pack_bf16x2(g.x, g.y);
    }
    tc_st16(ta0, w);
    if (bar0) {
        tc_wait_st();
        tc_fence_before();
        __syncwarp();
        if ((threadIdx.x & 31) == 0) sv_arrive(bar0);
    }
#pragma unroll
    for (int p = 0; p < 16; ++p) {
        const float2 g =
            gelu2_bias(make_float2(v[32 + 2 * p], v[32 + 2 * p + 1]), *(const float2 *)(bias1 + 2 * p));
        w[p] = pack_bf16x2(g.x, g.y);
    }
    tc_st16(ta1, w);
}

// last hidden layer's epilogue of 32 columns, folded into the 256 -> 4 output
// layer: y += gelu(v + b) . W4 rows
__device__ __forceinline__ void sv_epilogue_out(uint32_t td, const float *bias, const float *W4, float2 &y01,
                                                float2 &y23)
{
    float v[32];
    tc_ld32(td, v);
#pragma unroll
    for (int i = 0; i < 32; i += 2) {
        const float2 h = gelu2_bias(make_float2(v[i], v[i + 1]), *(const float2 *)&bias[i]);
        const float4 wa = *(const float4 *)&W4[i * MLP_OUT];
        const float4 wb = *(const float4 *)&W4[(i + 1) * MLP_OUT];
        y01 = __ffma2_rn(make_float2(h.x, h.x), make_float2(wa.x, wa.y), y01);
        y23 = __ffma2_rn(make_float2(h.x, h.x), make_float2(wa.z, wa.w), y23);
        y01 = __ffma2_rn(make_float2(h.y, h.y), make_float2(wb.x, wb.y), y01);
        y23 = __ffma2_rn(make_float2(h.y, h.y), make_float2(wb.z, wb.w), y23);
    }
}

// Fused serving kernel: features -> MLP -> spectra for 128 modes per tile,
// one persistent CTA per SM: 8 epilogue warps and one control warp.
//
// All four matrix layers run on the tensor cores (tcgen05.mma, M = 128, FP32
// accumulators in TMEM); the epilogues (bias + GELU) and the 256 -> 4 output
// layer run on the CUDA cores in FP32.  Input layer in BF16 at FP32 accuracy:
// x = xh + xl and W0 = wh + wl split into BF16 parts, K = 32 columns
// [xh | xl | xh | 0] x [wh | wh | wl | 0] give x.W0 up to the xl.wl term
// (relative 2^-16).
//
// Overlap of tensor cores and epilogues: every layer's 256 outputs are two
// N = 128 halves with their own accumulator (TMEM columns 0 and 128) and
// completion barrier.  The epilogue of half 0 writes the low K half of the
// next layer's activations (BF16 pairs in TMEM: the A operand of the next
// MMAs) while the tensor cores finish half 1; the next layer's first quarter
// MMA (half 0, low K) then runs during the epilogue of half 1.  Activations
// rotate through three K-half TMEM buffers so that no buffer is rewritten
// while an MMA reads it.  The hidden weights stream through shared memory as
// four 32 KB quarters (N half x K half), each reloaded with the next layer's
// as soon as the MMAs reading it have completed.  The control warp issues
// every copy and MMA and hands work to the epilogue warps through mbarriers
// only, so a blocked MMA issue never holds an epilogue back.  Every wait is
// bounded; on a timeout the kernel records BLDFM_ERR_TIMEOUT, all warps leave
// their loops, the control warp waits (bounded) for its copies and MMAs in
// flight, and TMEM is freed.
__global__ void __launch_bounds__(SV_THREADS, 1)
    sur_serve_kernel(const SurCase *__restrict__ cases, int ncases, int64_t ntiles, const MlpServing net, int *err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    SvSmem &S = *reinterpret_cast<SvSmem *>(smem_raw);
    // bar_m[h]: MMAs of accumulator half h done; bar_e[h]: epilogue of half h
    // done (one arrival per epilogue warp); bar_f: input operand written (128 thread
    // arrivals); bar_q[q]: weight quarter q loaded
    // bar_p: the first 64 columns of half 1 done (one arrival per epilogue warp)
    __shared__ uint64_t bar_m[2], bar_e[2], bar_p, bar_f, bar_q[4];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    __shared__ SurCase sc[2];         // cases of the current and the next tile (warps 0..3)
    __shared__ int64_t s_case_t1[2];  // first tile after each
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const volatile int *fail = &s_fail;
    if (warp == 0) tc_tmem_alloc(&tmem_slot, 512);
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            tc_mbar_init(&bar_m[i], 1);
            tc_mbar_init(&bar_e[i], SV_WARPS);
        }
        tc_mbar_init(&bar_f, 128);
        tc_mbar_init(&bar_p, SV_WARPS);
        for (int i = 0; i < 4; ++i) tc_mbar_init(&bar_q[i], 1);
        tc_fence_init();
        s_fail = 0;
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
    // activation K-half buffers of layers 1..3: (lo, hi) = (0, 1), (2, 0), (1, 2)
    auto buf_lo = [](int j) { return j == 0 ? 0 : (j == 1 ? 2 : 1); };
    auto buf_hi = [](int j) { return j == 0 ? 1 : (j == 1 ? 0 : 2); };

    if (warp == SV_WARPS) {
        // ---------------- control warp: copies and MMAs (lane 0) ----------------
        if (lane == 0) {
            const uint32_t idesc = tc_idesc_bf16(128, 128);
            uint64_t bq[4];  // descriptors of the weight quarters
            for (int q = 0; q < 4; ++q) bq[q] = tc_desc(tc_smem(S.Wq[q]), 128, 2048);
            const uint64_t da0 = tc_desc(tc_smem(S.A0), 128, 512), db0 = tc_desc(tc_smem(S.B0), 128, 512);
            uint32_t ph_m[2] = {0u, 0u}, ph_e[2] = {0u, 0u}, ph_p = 0u, ph_f = 0u, ph_q[4] = {0u, 0u, 0u, 0u};
            bool pend_m[2] = {false, false}, pend_q[4] = {false, false, false, false};
            bool ok = true;
            if ((int64_t)blockIdx.x < ntiles)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    sv_load_quarter(S.Wq[q], net.Wq[0], q, &bar_q[q]);
                    pend_q[q] = true;
                }
            for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                // input layer, both halves (B0 rows 128 h .. +127 start 8 KB
                // apart); the previous tile's last epilogue has released both
                // accumulator halves (its bar_e phases were waited below)
                ok = sv_wait(&bar_f, ph_f, fail);
                if (!ok) break;
                ph_f ^= 1u;
                tc_fence_after();
                for (int h = 0; h < 2; ++h) {
                    tc_mma(tmem + 128u * h, da0, db0 + (uint64_t)(512 * h), idesc, 0u);
                    tc_mma(tmem + 128u * h, da0 + 16u, db0 + (uint64_t)(512 * h + 16), idesc, 1u);
                    tc_commit(&bar_m[h]);
                    pend_m[h] = true;
                }
                for (int j = 0; j < 4 && ok; ++j) {
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        if (!ok) break;
                        // layer j's half h is complete: the quarters of Wt_j in N
                        // half h are free for the next layer's (after the last
                        // layer, the next tile's first)
                        ok = sv_wait(&bar_m[h], ph_m[h], fail);
                        if (!ok) break;
                        ph_m[h] ^= 1u;
                        pend_m[h] = false;
                        if (j >= 1) {
                            const uint16_t *next =
                                j < 3 ? net.Wq[j] : (tile + gridDim.x < ntiles ? net.Wq[0] : nullptr);
                            if (next)
#pragma unroll
                                for (int q = 2 * h; q < 2 * h + 2; ++q) {
                                    sv_load_quarter(S.Wq[q], next, q, &bar_q[q]);
                                    pend_q[q] = true;
                                }
                        }
                        const uint32_t alo = tmem + SV_AB(j < 3 ? buf_lo(j) : 0),
                                       ahi = tmem + SV_AB(j < 3 ? buf_hi(j) : 0);
                        if (h == 1 && j < 3) {
                            // the first 64 activations of the high K half: the
                            // first half of quarter 1 (layer j + 1, N half 0)
                            ok = sv_wait(&bar_p, ph_p, fail) && sv_wait(&bar_q[1], ph_q[1], fail);
                            if (!ok) break;
                            ph_p ^= 1u;
                            ph_q[1] ^= 1u;
                            pend_q[1] = false;
                            tc_fence_after();
                            sv_mma_quarter_part(tmem, ahi, bq[1], idesc, 0);
                        }
                        // the epilogue of half h has read the accumulator (and
                        // written the activations it feeds)
                        ok = sv_wait(&bar_e[h], ph_e[h], fail);
                        if (!ok) break;
                        ph_e[h] ^= 1u;
                        if (j == 3) continue;
                        tc_fence_after();
                        if (h == 1) {
                            sv_mma_quarter_part(tmem, ahi, bq[1], idesc, 4);
                            tc_commit(&bar_m[0]);
                            pend_m[0] = true;
                        }
#pragma unroll
                        for (int q = h == 0 ? 0 : 2; q < (h == 0 ? 1 : 4); ++q) {
                            if (!ok) break;
                            ok = sv_wait(&bar_q[q], ph_q[q], fail);
                            if (!ok) break;
                            ph_q[q] ^= 1u;
                            pend_q[q] = false;
                            sv_mma_quarter(tmem + 128u * (q >> 1), (q & 1) ? ahi : alo, bq[q], idesc, (q & 1) != 0);
                            if (q & 1) {
                                tc_commit(&bar_m[q >> 1]);
                                pend_m[q >> 1] = true;
                            }
                        }
                    }
                }
            }
            if (!ok) {
                s_fail = 1;
                atomicExch(err, BLDFM_ERR_TIMEOUT);
                const int never = 0;  // drain without the early exit on s_fail
                for (int h = 0; h < 2; ++h)
                    if (pend_m[h] && sv_wait(&bar_m[h], ph_m[h], &never)) ph_m[h] ^= 1u;
                // MMAs issued after the last commit: one more commit tracks them all
                tc_commit(&bar_m[0]);
                sv_wait(&bar_m[0], ph_m[0], &never);
                for (int q = 0; q < 4; ++q)
                    if (pend_q[q]) sv_wait(&bar_q[q], ph_q[q], &never);
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue warps ----------------
        // warp w owns TMEM lanes 32 (w % 4) .. +31 (its rows) and columns
        // 32 (w / 4) .. +31 of each accumulator half.  Warps 0..3 (one thread
        // per row) also compute the features of the next tile (as soon as the
        // input layer of the current one has read its operand) and write the
        // spectra; the tile's case sits in one of two shared slots, so that a
        // new case can be loaded while the previous one is still read.
        const int qd = warp & 3, cg = warp >> 2;
        const int row = 32 * qd + lane;
        const uint32_t lane_off = (uint32_t)(32 * qd) << 16;
        uint32_t ph_m[2] = {0u, 0u};
        int slot = 0;
        bool ok = true;
        // the case of `tile` into slot `to` unless slot `from` already holds it
        auto locate = [&](int64_t tile, int from, int to) -> int {
            if (from >= 0 && tile >= sc[from].tile0 && tile < s_case_t1[from]) return from;
            if (warp == 0) {
                int lo = 0, hi = ncases - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (cases[mid].tile0 <= tile) lo = mid;
                    else hi = mid - 1;
                }
                const uint32_t *src = (const uint32_t *)(cases + lo);
                uint32_t *dst = (uint32_t *)&sc[to];
                for (int i = lane; i < (int)(sizeof(SurCase) / 4); i += 32) dst[i] = src[i];
                if (lane == 0) s_case_t1[to] = lo + 1 < ncases ? cases[lo + 1].tile0 : ntiles;
            }
            sv_row_sync();
            return to;
        };
        uint32_t mw = 0u;  // warps 0..3: mode word of this thread's row of the current tile
        if (warp < 4 && (int64_t)blockIdx.x < ntiles) {
            slot = locate(blockIdx.x, -1, 0);
            mw = sv_mode_word(sc[slot], blockIdx.x, tid);
            sv_features(sc[slot], blockIdx.x, tid, mw, S.A0);
            tc_fence_proxy_async();
            sv_arrive(&bar_f);
        }
        for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
            float2 y01 = make_float2(0.f, 0.f), y23 = make_float2(0.f, 0.f);
            const bool has_next = tile + gridDim.x < ntiles;
            int next_slot = slot;
            uint32_t mw_next = 0u;
            if (warp < 4 && has_next) {
                // the next tile's case and mode words, in flight while this tile runs
                next_slot = locate(tile + gridDim.x, slot, slot ^ 1);
                mw_next = sv_mode_word(sc[next_slot], tile + gridDim.x, tid);
            }
            for (int j = 0; j < 4 && ok; ++j) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (!ok) break;
                    ok = sv_wait(&bar_m[h], ph_m[h], fail);
                    if (!ok) break;
                    ph_m[h] ^= 1u;
                    tc_fence_after();
                    // this warp's 32-column groups c = cg, cg + 2 of the half
                    const uint32_t td = tmem + lane_off + 128u * h + 32u * cg;
                    const float *bias = S.bias[j] + 128 * h + 32 * cg;
                    if (j < 3) {
                        const uint32_t ta = tmem + lane_off + SV_AB(h == 0 ? buf_lo(j) : buf_hi(j)) + 16u * cg;
                        sv_epilogue_hidden2(td, td + 64u, ta, ta + 32u, bias, bias + 64, h == 1 ? &bar_p : nullptr);
                        tc_wait_st();
                    } else {
                        const float *w4 = S.W4 + (128 * h + 32 * cg) * MLP_OUT;
                        sv_epilogue_out(td, bias, w4, y01, y23);
                        sv_epilogue_out(td + 64u, bias + 64, w4 + 64 * MLP_OUT, y01, y23);
                    }
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) sv_arrive(&bar_e[h]);
                    if (j == 0 && h == 1 && warp < 4 && has_next) {
                        // the input layer of this tile is complete: the next
                        // tile's features into its operand
                        sv_features(sc[next_slot], tile + gridDim.x, tid, mw_next, S.A0);
                        tc_fence_proxy_async();
                        sv_arrive(&bar_f);
                    }
                }
            }
            if (!ok) {
                s_fail = 1;
                break;
            }
            S.Yp[cg][row] = make_float4(y01.x, y01.y, y23.x, y23.y);
            sv_epi_sync();  // every column group's partial sums are in Yp
            if (warp < 4) {
                const SurCase &c = sc[slot];
                const int64_t m = (tile - c.tile0) * 128 + tid;
                if (m < c.g.nsolved) {
                    float4 a = S.Yp[0][tid];
#pragma unroll
                    for (int qq = 1; qq < SV_WARPS / 4; ++qq) {
                        const float4 b = S.Yp[qq][tid];
                        a = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
                    }
                    const float y[4] = {a.x + S.b4[0], a.y + S.b4[1], a.z + S.b4[2], a.w + S.b4[3]};
                    emit_spectrum(c.g, mw, y, c.ax, c.ay, c.zm, c.inv_wind, c.ktop, c.utop, c.Xp, c.Xq);
                }
            }
            slot = next_slot;
            mw = mw_next;
            // Yp is rewritten only after this emit: the next tile's layer-1
            // MMAs wait for the layer-0 epilogue of warps 0..3, which follows it
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_tmem_free(tmem, 512);
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
    sur_serve_kernel<<<grid, SV_THREADS, sizeof(SvSmem), st>>>(cases, ncases, ntiles, net, err);
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
