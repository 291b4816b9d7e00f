// Learned surrogate of the per-mode transfer function: a BF16 MLP whose hidden
// 256 x 256 layers run on the tcgen05 tensor cores (tcgemm.cuh).
#include "devattr.h"
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "../../include/bldfm_gb300.h"
#include "common.h"
#include "guard.h"
#include "mlp_common.cuh"
#include "profiles.h"
#include "surrogate_phys.cuh"
#include "tcgemm.cuh"

namespace {

// row-major R x K bf16 -> blocks [R / rows_per_block][K / KC] in core-matrix order
void host_block(const uint16_t *src, int R, int K, int rows_per_block, int KC, std::vector<uint16_t> &dst)
{
    dst.assign((size_t)R * K, 0);
    const int nb = R / rows_per_block, nc = K / KC;
    for (int b = 0; b < nb; ++b)
        for (int c = 0; c < nc; ++c) {
            uint16_t *blk = dst.data() + ((size_t)b * nc + c) * rows_per_block * KC;
            for (int r = 0; r < rows_per_block; ++r)
                for (int k = 0; k < KC; ++k)
                    blk[tc_core_offset(r, k, KC) / 2] = src[(size_t)(b * rows_per_block + r) * K + c * KC + k];
        }
}

struct StoreF32 {
    float *D;
    int ld;
    __device__ void row(int r, int col0, const float *v, uint16_t *) const
    {
        float *o = D + (size_t)r * ld + col0;
#pragma unroll
        for (int i = 0; i < 32; ++i) o[i] = v[i];
    }
    __device__ void finish(int, uint16_t *) const {}
};

}  // namespace

// D (M x 256, fp32) = A (M x K) * B (256 x K)^T, bf16 operands given row-major
// on the host; M a multiple of 128, K a multiple of 16.  Validates the tensor
// core path against a reference GEMM; allocates its own device buffers.
extern "C" int bldfm_tc_gemm_check(const uint16_t *A, const uint16_t *B, float *D, int32_t M, int32_t K)
{
    return bldfm_guarded([&]() -> int {
        if (!A || !B || !D || M <= 0 || K <= 0 || M % 128 != 0 || K % 16 != 0) return BLDFM_ERR_ARG;
        int KC = K <= 256 ? K : 256;
        if (K % KC != 0) return BLDFM_ERR_ARG;
        std::vector<uint16_t> Ab, Bb;
        host_block(A, M, K, 128, KC, Ab);
        host_block(B, 256, K, 256, KC, Bb);
        uint16_t *dA = nullptr, *dB = nullptr;
        float *dD = nullptr;
        int *derr = nullptr;
        int rc = BLDFM_OK;
        if (cudaMalloc(&dA, Ab.size() * 2) != cudaSuccess || cudaMalloc(&dB, Bb.size() * 2) != cudaSuccess ||
            cudaMalloc(&dD, (size_t)M * 256 * 4) != cudaSuccess || cudaMalloc(&derr, 4) != cudaSuccess)
            rc = BLDFM_ERR_CUDA;
        if (rc == BLDFM_OK) {
            cudaMemcpy(dA, Ab.data(), Ab.size() * 2, cudaMemcpyHostToDevice);
            cudaMemcpy(dB, Bb.data(), Bb.size() * 2, cudaMemcpyHostToDevice);
            cudaMemset(derr, 0, 4);
            const size_t smem = tc_gemm_smem(KC);
            cudaFuncSetAttribute(tc_gemm_kernel<StoreF32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            StoreF32 epi{dD, 256};
            tc_gemm_kernel<StoreF32><<<M / 128, 128, smem>>>(dA, dB, K, KC, epi, derr);
            int herr = 0;
            if (cudaDeviceSynchronize() != cudaSuccess) rc = BLDFM_ERR_CUDA;
            if (rc == BLDFM_OK && cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
                rc = BLDFM_ERR_CUDA;
            if (rc == BLDFM_OK && herr != 0) rc = BLDFM_ERR_TIMEOUT;
            if (rc == BLDFM_OK) cudaMemcpy(D, dD, (size_t)M * 256 * 4, cudaMemcpyDeviceToHost);
        }
        cudaFree(dA);
        cudaFree(dB);
        cudaFree(dD);
        cudaFree(derr);
        return rc;
    });
}

// ===========================================================================
// The MLP: 8 -> 256 -> 256 -> 256 -> 256 -> 4, GELU after each hidden layer.
// Hidden 256 x 256 layers on tensor cores (BF16 operands, FP32 accumulation),
// input and output layers on CUDA cores (FP32); the last hidden layer is kept
// in FP32 for the output layer (fused into the last GEMM's epilogue when only
// the forward pass runs).  Parameters are FP32 masters updated by Adam; the
// tensor-core layers read BF16 copies.
//
// Flat parameter vector: W0 [8][256] (in, out), b0 [256], then for j = 1..3
// Wt_j [256][256] (out, in) and b_j [256], then W4 [256][4] (in, out), b4 [4].
// ===========================================================================


namespace {

// A CTA's 128 x 256 bf16 tile in core-matrix order (tc_core_offset) is copied
// to the row blocks of its tile (contiguous 64 KB), and scattered into the
// transposed layouts used as operands of the weight-gradient GEMM:
//   mode 0 (B operand, H^T): blocks [chunk = sample / 256] of 256 x 256,
//          element (feature, sample % 256)
//   mode 1 (A operand, dZ^T): blocks [feature / 128][chunk] of 128 x 256,
//          element (feature % 128, sample % 256)
__device__ void emit_tile(int tile, const uint16_t *st, uint16_t *rows_dst, uint16_t *T_dst, int mode, int nchunks)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    if (rows_dst) {
        const uint4 *s = (const uint4 *)st;
        uint4 *d = (uint4 *)(rows_dst + (size_t)tile * 128 * MLP_H);
        for (int i = tid; i < 128 * MLP_H / 8; i += nt) d[i] = s[i];
    }
    if (!T_dst) return;
    const int chunk = tile >> 1, half = tile & 1;
    // one 16-byte store per (feature, group of 8 samples): 256 x 16 per tile
    for (int i = tid; i < MLP_H * 16; i += nt) {
        const int f = i & (MLP_H - 1), g = i >> 8;  // consecutive threads: consecutive features
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int s0 = g * 8 + 2 * q;
            const uint32_t lo = st[tc_core_offset(s0, f, MLP_H) / 2];
            const uint32_t hi = st[tc_core_offset(s0 + 1, f, MLP_H) / 2];
            w[q] = lo | (hi << 16);
        }
        const int s256 = half * 128 + g * 8;
        size_t off;
        if (mode == 0)
            off = (size_t)chunk * MLP_H * 256 + tc_core_offset(f, s256, 256) / 2;
        else
            off = ((size_t)(f >> 7) * nchunks + chunk) * 128 * 256 + tc_core_offset(f & 127, s256, 256) / 2;
        *(uint4 *)(T_dst + off) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// 8 consecutive values of one row into the smem tile (one 16-byte store)
__device__ __forceinline__ void put8(uint16_t *st, int r, int c, const float *v)
{
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] = (uint32_t)f2bf(v[2 * q]) | ((uint32_t)f2bf(v[2 * q + 1]) << 16);
    *(uint4 *)(st + tc_core_offset(r, c, MLP_H) / 2) = make_uint4(w[0], w[1], w[2], w[3]);
}

// forward hidden layer: Z = acc + b, H = gelu(Z); written as the bf16 rows
// and transposed blocks of the next GEMM (rows_dst, T_dst), gelu'(Z) as bf16
// (G_dst), H in FP32 row-major (h32_dst), or straight into the output layer:
// Y[r] = b4 + sum_f H[r][f] W4[f] in FP32 (Y != null).  Null pointers skip.
struct EpiFwd {
    const float *bias;
    uint16_t *rows_dst, *T_dst, *G_dst;
    float *h32_dst;
    const float *W4, *b4;
    float *Y;
    int nchunks;
    __device__ void row(int r, int c0, const float *v, uint16_t *st) const
    {
        float h[32], gd[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            const float z = v[i] + bias[c0 + i];
            h[i] = gelu_f(z);
            gd[i] = G_dst ? gelu_d(z) : 0.f;
        }
        if (rows_dst || T_dst) {
            const int rl = r & 127;
#pragma unroll
            for (int q = 0; q < 4; ++q) put8(st, rl, c0 + 8 * q, h + 8 * q);
        }
        if (G_dst) {
            uint32_t w[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) w[i] = (uint32_t)f2bf(gd[2 * i]) | ((uint32_t)f2bf(gd[2 * i + 1]) << 16);
            uint4 *g = (uint4 *)(G_dst + (size_t)r * MLP_H + c0);
#pragma unroll
            for (int q = 0; q < 4; ++q) g[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
        }
        if (h32_dst) {
            float4 *o = (float4 *)(h32_dst + (size_t)r * MLP_H + c0);
#pragma unroll
            for (int q = 0; q < 8; ++q) o[q] = make_float4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
        }
        if (Y) {
            // this thread owns row r for every column slice, in order
            float4 y = c0 == 0 ? make_float4(b4[0], b4[1], b4[2], b4[3]) : *(const float4 *)(Y + (size_t)r * 4);
            const float4 *w4 = (const float4 *)(W4 + (size_t)c0 * MLP_OUT);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const float4 wv = w4[i];
                y.x = fmaf(h[i], wv.x, y.x);
                y.y = fmaf(h[i], wv.y, y.y);
                y.z = fmaf(h[i], wv.z, y.z);
                y.w = fmaf(h[i], wv.w, y.w);
            }
            *(float4 *)(Y + (size_t)r * 4) = y;
        }
    }
    __device__ void finish(int tile, uint16_t *st) const
    {
        if (rows_dst || T_dst) emit_tile(tile, st, rows_dst, T_dst, 0, nchunks);
    }
};

// backward data: dZ = bf16(acc * G); db += sum over rows of dZ
struct EpiBwd {
    const uint16_t *G;
    uint16_t *rows_dst, *T_dst;
    float *rowmajor_f32;  // dZ1 for the input layer's gradient
    float *dbias;
    int nchunks;
    __device__ void row(int r, int c0, const float *v, uint16_t *st) const
    {
        float dz[32];
        const uint4 *g4 = (const uint4 *)(G + (size_t)r * MLP_H + c0);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint4 u = g4[q];
            const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                dz[8 * q + 2 * k] = bf2f(f2bf(v[8 * q + 2 * k] * bf2f((uint16_t)(w[k] & 0xFFFF))));
                dz[8 * q + 2 * k + 1] = bf2f(f2bf(v[8 * q + 2 * k + 1] * bf2f((uint16_t)(w[k] >> 16))));
            }
        }
        if (rows_dst || T_dst) {
            const int rl = r & 127;
#pragma unroll
            for (int q = 0; q < 4; ++q) put8(st, rl, c0 + 8 * q, dz + 8 * q);
        }
        if (rowmajor_f32) {
            float4 *o = (float4 *)(rowmajor_f32 + (size_t)r * MLP_H + c0);
#pragma unroll
            for (int q = 0; q < 8; ++q) o[q] = make_float4(dz[4 * q], dz[4 * q + 1], dz[4 * q + 2], dz[4 * q + 3]);
        }
        // bias gradient: sum the warp's 32 rows per column, one atomic per column
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            float s = dz[i];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
            if ((threadIdx.x & 31) == 0) atomicAdd(dbias + c0 + i, s);
        }
    }
    __device__ void finish(int tile, uint16_t *st) const
    {
        if (rows_dst || T_dst) emit_tile(tile, st, rows_dst, T_dst, 1, nchunks);
    }
};

// weight gradient partial sums: grad[out][in] += acc
struct EpiGrad {
    float *grad;
    __device__ void row(int r, int c0, const float *v, uint16_t *) const
    {
        float *o = grad + (size_t)r * MLP_H + c0;
#pragma unroll
        for (int i = 0; i < 32; ++i) atomicAdd(o + i, v[i]);
    }
    __device__ void finish(int, uint16_t *) const {}
};

// input layer forward: one CTA per 128-sample tile, thread = feature
__global__ void __launch_bounds__(256) mlp_in_fwd_kernel(const float *__restrict__ X, const float *__restrict__ P,
                                                         uint16_t *rows_dst, uint16_t *T_dst, uint16_t *G_dst,
                                                         int nchunks)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint16_t *st = (uint16_t *)smem_raw;
    const int f = threadIdx.x, tile = blockIdx.x;
    float w[MLP_IN];
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) w[i] = P[MLP_OFF_W0 + i * MLP_H + f];
    const float b = P[MLP_OFF_B0 + f];
    for (int s = 0; s < 128; ++s) {
        const int r = tile * 128 + s;
        const float *x = X + (size_t)r * MLP_XS;
        float z = b;
#pragma unroll
        for (int i = 0; i < MLP_IN; ++i) z = fmaf(x[i], w[i], z);
        st[tc_core_offset(s, f, MLP_H) / 2] = f2bf(gelu_f(z));
        if (G_dst) G_dst[(size_t)r * MLP_H + f] = f2bf(gelu_d(z));
    }
    __syncthreads();
    emit_tile(tile, st, rows_dst, T_dst, 0, nchunks);
}

// Output layer forward, loss and the start of the backward pass: one CTA per
// 128-sample tile.  Phase 1, thread = sample: y = H4 W4 + b4, the weighted
// error and dY (kept in shared memory).  Phase 2, thread = two features:
// dW4 = H4^T dY and dZ4 = bf16(dY W4^T * gelu'), db3 = sum dZ4, reduced over
// the tile's rows in registers (one global atomic per parameter and CTA).
__global__ void __launch_bounds__(128) mlp_out_kernel(const float *__restrict__ H4, const uint16_t *__restrict__ G4,
                                                      const float *__restrict__ P, const float *__restrict__ T,
                                                      const float *__restrict__ wts, float inv_n, float *Y,
                                                      float *grad, float *loss, uint16_t *rows_dst, uint16_t *T_dst,
                                                      int nchunks, int n)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint16_t *st = (uint16_t *)smem_raw;                // dZ4 tile (64 KB)
    float *sW = (float *)(smem_raw + 128 * MLP_H * 2);  // W4 [256][4]
    float4 *sDY = (float4 *)(sW + MLP_H * MLP_OUT);     // dY [128]
    __shared__ float sdb4[MLP_OUT], sloss;
    const int t = threadIdx.x, tile = blockIdx.x;
    for (int i = t; i < MLP_H * MLP_OUT; i += blockDim.x) sW[i] = P[MLP_OFF_W4 + i];
    if (t < MLP_OUT) sdb4[t] = 0.f;
    if (t == 0) sloss = 0.f;
    __syncthreads();
    const int r = tile * 128 + t;
    const bool live = r < n;
    const float4 *h4 = (const float4 *)(H4 + (size_t)(live ? r : 0) * MLP_H);
    float y[MLP_OUT];
#pragma unroll
    for (int o = 0; o < MLP_OUT; ++o) y[o] = P[MLP_OFF_B4 + o];
    for (int q = 0; q < MLP_H / 4; ++q) {
        const float4 u = h4[q];
        const float hq[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int f = q * 4 + k;
#pragma unroll
            for (int o = 0; o < MLP_OUT; ++o) y[o] = fmaf(hq[k], sW[f * MLP_OUT + o], y[o]);
        }
    }
    if (Y && live)
        for (int o = 0; o < MLP_OUT; ++o) Y[(size_t)r * MLP_OUT + o] = y[o];
    if (!T) return;
    float dy[MLP_OUT];
    float l = 0.f;
#pragma unroll
    for (int o = 0; o < MLP_OUT; ++o) {
        const float wb = live ? wts[(size_t)r * MLP_OUT + o] : 0.f;
        const float e = live ? (y[o] - T[(size_t)r * MLP_OUT + o]) : 0.f;
        l = fmaf(wb * e, e, l);
        dy[o] = 2.f * wb * e * inv_n;
    }
    sDY[t] = make_float4(dy[0], dy[1], dy[2], dy[3]);
    // tile sums of the loss and db4: warp reductions, one shared atomic per warp
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        l += __shfl_xor_sync(0xffffffffu, l, off);
#pragma unroll
        for (int o = 0; o < MLP_OUT; ++o) dy[o] += __shfl_xor_sync(0xffffffffu, dy[o], off);
    }
    if ((t & 31) == 0) {
        atomicAdd(&sloss, l * inv_n);
#pragma unroll
        for (int o = 0; o < MLP_OUT; ++o) atomicAdd(&sdb4[o], dy[o]);
    }
    __syncthreads();
    // phase 2: features f0 = 2 t, f0 + 1
    const int f0 = 2 * t;
    float gW[2][MLP_OUT] = {};
    float db[2] = {0.f, 0.f};
    float w4[2][MLP_OUT];
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int o = 0; o < MLP_OUT; ++o) w4[k][o] = sW[(f0 + k) * MLP_OUT + o];
    const int rows = min(128, n - tile * 128);
    for (int rr = 0; rr < rows; ++rr) {
        const size_t gr = (size_t)(tile * 128 + rr) * MLP_H + f0;
        const float2 h = *(const float2 *)(H4 + gr);
        const uint32_t gw = *(const uint32_t *)(G4 + gr);
        const float4 d = sDY[rr];
        const float hk[2] = {h.x, h.y};
        const float gk[2] = {bf2f((uint16_t)(gw & 0xFFFF)), bf2f((uint16_t)(gw >> 16))};
        uint16_t zb[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            gW[k][0] = fmaf(hk[k], d.x, gW[k][0]);
            gW[k][1] = fmaf(hk[k], d.y, gW[k][1]);
            gW[k][2] = fmaf(hk[k], d.z, gW[k][2]);
            gW[k][3] = fmaf(hk[k], d.w, gW[k][3]);
            const float dh = fmaf(d.x, w4[k][0], fmaf(d.y, w4[k][1], fmaf(d.z, w4[k][2], d.w * w4[k][3])));
            zb[k] = f2bf(dh * gk[k]);
            db[k] += bf2f(zb[k]);
        }
        // f0 is even, so the pair is one aligned 32-bit word of the core-matrix row
        *(uint32_t *)(st + tc_core_offset(rr, f0, MLP_H) / 2) = (uint32_t)zb[0] | ((uint32_t)zb[1] << 16);
    }
    for (int rr = rows; rr < 128; ++rr) *(uint32_t *)(st + tc_core_offset(rr, f0, MLP_H) / 2) = 0u;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
#pragma unroll
        for (int o = 0; o < MLP_OUT; ++o) atomicAdd(grad + MLP_OFF_W4 + (f0 + k) * MLP_OUT + o, gW[k][o]);
        atomicAdd(grad + MLP_OFF_B(3) + f0 + k, db[k]);
    }
    if (t < MLP_OUT) atomicAdd(grad + MLP_OFF_B4 + t, sdb4[t]);
    if (t == 0) atomicAdd(loss, sloss);
    __syncthreads();
    emit_tile(tile, st, rows_dst, T_dst, 1, nchunks);
}

// input layer weight gradient: dW0[i][f] += sum_b X[b][i] dZ1[b][f]
__global__ void __launch_bounds__(256) mlp_in_grad_kernel(const float *__restrict__ X, const float *__restrict__ dZ1,
                                                          float *grad, int n)
{
    const int f = threadIdx.x;
    float acc[MLP_IN];
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) acc[i] = 0.f;
    const int r0 = blockIdx.x * 128, r1 = min(n, r0 + 128);
    for (int r = r0; r < r1; ++r) {
        const float d = dZ1[(size_t)r * MLP_H + f];
#pragma unroll
        for (int i = 0; i < MLP_IN; ++i) acc[i] = fmaf(X[(size_t)r * MLP_XS + i], d, acc[i]);
    }
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) atomicAdd(grad + MLP_OFF_W0 + i * MLP_H + f, acc[i]);
}

__global__ void adam_kernel(float *P, const float *G, float *m, float *v, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// BF16 operand blocks of the hidden weights: Wt_j (rows out, K in) for the
// forward GEMM, W_j (rows in, K out) for the backward-data GEMM, and Wq_j, Wt_j
// as four contiguous 128 x 128 quarters (N half, K half) for the serving kernel
struct WBlocks {
    uint16_t *Wt[3], *W[3], *Wq[3];
};

__global__ void weights_to_blocks_kernel(const float *__restrict__ P, WBlocks wb)
{
    const int j = blockIdx.y + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;  // out * 256 + in
    if (e >= MLP_H * MLP_H) return;
    const int out = e >> 8, in = e & 255;
    const uint16_t b = f2bf(P[MLP_OFF_WT(j) + e]);
    wb.Wt[j - 1][tc_core_offset(out, in, MLP_H) / 2] = b;
    wb.W[j - 1][tc_core_offset(in, out, MLP_H) / 2] = b;
    const int q = (out >> 7) * 2 + (in >> 7);
    wb.Wq[j - 1][(size_t)q * 128 * 128 + tc_core_offset(out & 127, in & 127, 128) / 2] = b;
}

struct Mlp {
    int B = 0;  // batch capacity, multiple of 256
    int step = 0;
    float *P = nullptr, *G = nullptr, *m = nullptr, *v = nullptr;
    uint16_t *Wt[3] = {}, *W[3] = {}, *Wq[3] = {};
    uint16_t *Hrows[3] = {}, *HT[3] = {};
    float *H4 = nullptr;  // last hidden layer, FP32 row-major (training)
    uint16_t *Gz[4] = {};
    uint16_t *dZrows[3] = {}, *dZT[3] = {};  // index j-2 for dZ_j, j = 2..4
    float *dZ1 = nullptr, *Y = nullptr, *loss = nullptr;
    int *err = nullptr;
    std::vector<void *> allocs;  // every device allocation, freed with the object
    Mlp() = default;
    Mlp(const Mlp &) = delete;
    Mlp &operator=(const Mlp &) = delete;
    ~Mlp()
    {
        for (void *p : allocs) cudaFree(p);
    }
};

template <typename T>
bool mlp_alloc(Mlp &M, T **p, size_t count)
{
    M.allocs.push_back(nullptr);  // may throw: nothing is held yet
    if (cudaMalloc(&M.allocs.back(), count * sizeof(T)) != cudaSuccess) return false;
    *p = (T *)M.allocs.back();
    return true;
}

WBlocks mlp_blocks(const Mlp &M)
{
    WBlocks b;
    for (int j = 0; j < 3; ++j) {
        b.Wt[j] = M.Wt[j];
        b.W[j] = M.W[j];
        b.Wq[j] = M.Wq[j];
    }
    return b;
}

void mlp_free(Mlp *M) { delete M; }

template <class Epi>
cudaError_t gemm(const uint16_t *A, const uint16_t *Bop, int tiles, int K, int splits, Epi epi, int *err,
                 cudaStream_t st)
{
    const size_t smem = tc_gemm_smem(256);
    static uint64_t attr = 0;
    if (first_on_device(attr))
        cudaFuncSetAttribute(tc_gemm_kernel<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    tc_gemm_kernel<Epi><<<dim3(tiles, splits), 128, smem, st>>>(A, Bop, K, 256, epi, err);
    return cudaGetLastError();
}

// Forward pass.  train: keep what the backward pass reads (transposed blocks,
// gelu'(Z), the FP32 last hidden layer H4) and leave the output layer to
// mlp_out_kernel; otherwise the output layer runs in the last epilogue -> Y.
cudaError_t mlp_forward(Mlp &M, const float *X, int n, bool train, float *Y, cudaStream_t st)
{
    const int tiles = n / 128, nchunks = n / 256;
    cudaFuncSetAttribute(mlp_in_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 128 * MLP_H * 2);
    mlp_in_fwd_kernel<<<tiles, 256, 128 * MLP_H * 2, st>>>(X, M.P, M.Hrows[0], train ? M.HT[0] : nullptr,
                                                            train ? M.Gz[0] : nullptr, nchunks);
    for (int j = 1; j <= 3; ++j) {
        EpiFwd e;
        e.bias = M.P + MLP_OFF_B(j);
        e.rows_dst = j < 3 ? M.Hrows[j] : nullptr;
        e.T_dst = train && j < 3 ? M.HT[j] : nullptr;
        e.G_dst = train ? M.Gz[j] : nullptr;
        e.h32_dst = train && j == 3 ? M.H4 : nullptr;
        e.W4 = M.P + MLP_OFF_W4;
        e.b4 = M.P + MLP_OFF_B4;
        e.Y = !train && j == 3 ? Y : nullptr;
        e.nchunks = nchunks;
        cudaError_t c = gemm(M.Hrows[j - 1], M.Wt[j - 1], tiles, MLP_H, 1, e, M.err, st);
        if (c != cudaSuccess) return c;
    }
    return cudaGetLastError();
}

const size_t OUT_SMEM = 128 * MLP_H * 2 + MLP_H * MLP_OUT * 4 + 128 * 16;

}  // namespace

extern "C" {

int bldfm_surrogate_create(int32_t batch, uint64_t seed, void **handle)
{
    return bldfm_guarded([&]() -> int {
        if (!handle || batch < 256 || batch % 256 != 0) return BLDFM_ERR_ARG;
        std::unique_ptr<Mlp> own(new Mlp());  // freed on every early return
        Mlp *M = own.get();
        M->B = batch;
        const size_t B = (size_t)batch;
        bool ok = mlp_alloc(*M, &M->P, MLP_NPARAM) && mlp_alloc(*M, &M->G, MLP_NPARAM) &&
                  mlp_alloc(*M, &M->m, MLP_NPARAM) && mlp_alloc(*M, &M->v, MLP_NPARAM) &&
                  mlp_alloc(*M, &M->H4, B * MLP_H) && mlp_alloc(*M, &M->dZ1, B * MLP_H) &&
                  mlp_alloc(*M, &M->Y, B * MLP_OUT) && mlp_alloc(*M, &M->loss, 1) && mlp_alloc(*M, &M->err, 1);
        for (int j = 0; j < 3 && ok; ++j)
            ok = mlp_alloc(*M, &M->Wt[j], (size_t)MLP_H * MLP_H) && mlp_alloc(*M, &M->W[j], (size_t)MLP_H * MLP_H) &&
                 mlp_alloc(*M, &M->Wq[j], (size_t)MLP_H * MLP_H) &&
                 mlp_alloc(*M, &M->Hrows[j], B * MLP_H) && mlp_alloc(*M, &M->HT[j], B * MLP_H) &&
                 mlp_alloc(*M, &M->dZrows[j], B * MLP_H) && mlp_alloc(*M, &M->dZT[j], B * MLP_H);
        for (int j = 0; j < 4 && ok; ++j) ok = mlp_alloc(*M, &M->Gz[j], B * MLP_H);
        if (!ok) return BLDFM_ERR_CUDA;
        // He-scaled normal weights (Box-Muller on a 64-bit LCG), zero biases
        std::vector<float> p(MLP_NPARAM, 0.f);
        uint64_t s = seed * 6364136223846793005ULL + 1442695040888963407ULL;
        auto unif = [&]() {
            s = s * 6364136223846793005ULL + 1442695040888963407ULL;
            return ((s >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        };
        auto normal = [&]() { return sqrt(-2.0 * log(unif())) * cos(6.283185307179586 * unif()); };
        for (int i = 0; i < MLP_IN * MLP_H; ++i) p[MLP_OFF_W0 + i] = (float)(normal() * sqrt(2.0 / MLP_IN));
        for (int j = 1; j <= 3; ++j)
            for (int i = 0; i < MLP_H * MLP_H; ++i) p[MLP_OFF_WT(j) + i] = (float)(normal() * sqrt(2.0 / MLP_H));
        for (int i = 0; i < MLP_H * MLP_OUT; ++i) p[MLP_OFF_W4 + i] = (float)(normal() * sqrt(1.0 / MLP_H));
        cudaMemcpy(M->P, p.data(), MLP_NPARAM * 4, cudaMemcpyHostToDevice);
        cudaMemset(M->m, 0, MLP_NPARAM * 4);
        cudaMemset(M->v, 0, MLP_NPARAM * 4);
        cudaMemset(M->G, 0, MLP_NPARAM * 4);
        cudaMemset(M->err, 0, 4);
        weights_to_blocks_kernel<<<dim3(MLP_H * MLP_H / 256, 3), 256>>>(M->P, mlp_blocks(*M));
        if (cudaDeviceSynchronize() != cudaSuccess) return BLDFM_ERR_CUDA;
        *handle = own.release();
        return BLDFM_OK;
    });
}

int bldfm_surrogate_destroy(void *handle)
{
    if (!handle) return BLDFM_ERR_ARG;
    cudaDeviceSynchronize();
    mlp_free((Mlp *)handle);
    return BLDFM_OK;
}

int bldfm_surrogate_nparams(void) { return MLP_NPARAM; }

int bldfm_surrogate_batch(void *handle) { return handle ? ((Mlp *)handle)->B : BLDFM_ERR_ARG; }

// get (host_out != NULL) and/or set (host_in != NULL) the FP32 parameters
int bldfm_surrogate_params(void *handle, float *host_out, const float *host_in)
{
    Mlp *M = (Mlp *)handle;
    if (!M) return BLDFM_ERR_ARG;
    if (cudaDeviceSynchronize() != cudaSuccess) return BLDFM_ERR_CUDA;
    if (host_out && cudaMemcpy(host_out, M->P, MLP_NPARAM * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return BLDFM_ERR_CUDA;
    if (host_in) {
        if (cudaMemcpy(M->P, host_in, MLP_NPARAM * 4, cudaMemcpyHostToDevice) != cudaSuccess) return BLDFM_ERR_CUDA;
        weights_to_blocks_kernel<<<dim3(MLP_H * MLP_H / 256, 3), 256>>>(M->P, mlp_blocks(*M));
        if (cudaDeviceSynchronize() != cudaSuccess) return BLDFM_ERR_CUDA;
    }
    return BLDFM_OK;
}

// gradients of the last training step and its loss
int bldfm_surrogate_grads(void *handle, float *host_grads, float *host_loss)
{
    Mlp *M = (Mlp *)handle;
    if (!M) return BLDFM_ERR_ARG;
    if (cudaDeviceSynchronize() != cudaSuccess) return BLDFM_ERR_CUDA;
    if (host_grads && cudaMemcpy(host_grads, M->G, MLP_NPARAM * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return BLDFM_ERR_CUDA;
    if (host_loss && cudaMemcpy(host_loss, M->loss, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BLDFM_ERR_CUDA;
    int e = 0;
    if (cudaMemcpy(&e, M->err, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BLDFM_ERR_CUDA;
    return e != 0 ? BLDFM_ERR_TIMEOUT : BLDFM_OK;
}

// One Adam step on n samples (n <= batch, n % 256 == 0): X [n][8] inputs,
// T [n][4] targets, w [n][4] loss weights, all device pointers.
// loss = sum_b sum_o w_bo (y_bo - t_bo)^2 / n.  lr = 0 computes gradients only.
int bldfm_surrogate_train_step(void *handle, const float *X, const float *T, const float *w, int32_t n, float lr,
                               void *stream)
{
    Mlp *M = (Mlp *)handle;
    if (!M || !X || !T || !w || n < 256 || n > M->B || n % 256 != 0) return BLDFM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int tiles = n / 128, nchunks = n / 256;
    if (cudaMemsetAsync(M->G, 0, MLP_NPARAM * 4, st) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (cudaMemsetAsync(M->loss, 0, 4, st) != cudaSuccess) return BLDFM_ERR_CUDA;
    if (mlp_forward(*M, X, n, true, nullptr, st) != cudaSuccess) return BLDFM_ERR_CUDA;
    cudaFuncSetAttribute(mlp_out_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OUT_SMEM);
    mlp_out_kernel<<<tiles, 128, OUT_SMEM, st>>>(M->H4, M->Gz[3], M->P, T, w, 1.0f / n, M->Y, M->G, M->loss,
                                                 M->dZrows[2], M->dZT[2], nchunks, n);
    // hidden layers, last to first: dW_j from dZ_{j+1}^T and H_j^T, dH_j from dZ_{j+1} and W_j
    for (int j = 3; j >= 1; --j) {
        EpiGrad eg;
        eg.grad = M->G + MLP_OFF_WT(j);
        const int splits = nchunks < 64 ? nchunks : 64;
        if (gemm(M->dZT[j - 1], M->HT[j - 1], 2, n, splits, eg, M->err, st) != cudaSuccess) return BLDFM_ERR_CUDA;
        EpiBwd eb;
        eb.G = M->Gz[j - 1];
        eb.rows_dst = j > 1 ? M->dZrows[j - 2] : nullptr;
        eb.T_dst = j > 1 ? M->dZT[j - 2] : nullptr;
        eb.rowmajor_f32 = j == 1 ? M->dZ1 : nullptr;
        eb.dbias = M->G + (j > 1 ? MLP_OFF_B(j - 1) : MLP_OFF_B0);
        eb.nchunks = nchunks;
        if (gemm(M->dZrows[j - 1], M->W[j - 1], tiles, MLP_H, 1, eb, M->err, st) != cudaSuccess) return BLDFM_ERR_CUDA;
    }
    mlp_in_grad_kernel<<<tiles, 256, 0, st>>>(X, M->dZ1, M->G, n);
    if (lr != 0.f) {
        M->step += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f / (1.f - powf(b1, (float)M->step)), c2 = 1.f / (1.f - powf(b2, (float)M->step));
        adam_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(M->P, M->G, M->m, M->v, MLP_NPARAM, lr, b1, b2, 1e-8f,
                                                              c1, c2);
        weights_to_blocks_kernel<<<dim3(MLP_H * MLP_H / 256, 3), 256, 0, st>>>(M->P, mlp_blocks(*M));
    }
    return cudaGetLastError() == cudaSuccess ? BLDFM_OK : BLDFM_ERR_CUDA;
}

// Y [n][4] = MLP(X [n][8]), n % 256 == 0, device pointers (forward only: the
// output layer is fused into the last tensor-core GEMM)
int bldfm_surrogate_forward(void *handle, const float *X, float *Y, int32_t n, void *stream)
{
    Mlp *M = (Mlp *)handle;
    if (!M || !X || !Y || n < 256 || n > M->B || n % 256 != 0) return BLDFM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (mlp_forward(*M, X, n, false, Y, st) != cudaSuccess) return BLDFM_ERR_CUDA;
    return BLDFM_OK;
}

}  // extern "C"

int mlp_serving_view(void *handle, MlpServing *out)
{
    Mlp *M = (Mlp *)handle;
    if (!M || !out) return BLDFM_ERR_ARG;
    out->P = M->P;
    for (int j = 0; j < 3; ++j) {
        out->Wt[j] = M->Wt[j];
        out->Wq[j] = M->Wq[j];
    }
    return BLDFM_OK;
}

// ===========================================================================
// Training data: nondimensional transfer functions (surrogate_phys.cuh) of a
// pool of MOST met cases, sampled on the device.
// ===========================================================================
namespace {

struct TransferPool {
    int ncases = 0, lmax = 0, n = 0;
    TransferCase *cases = nullptr;  // device
    float4 *steps = nullptr;        // device [case][lmax]: (h~, K~, U~, 0) of step i
    std::vector<TransferCase> host_cases;
    TransferPool() = default;
    TransferPool(const TransferPool &) = delete;
    TransferPool &operator=(const TransferPool &) = delete;
    ~TransferPool()
    {
        cudaFree(cases);
        cudaFree(steps);
    }
};

// counter-based uniform in (0, 1): splitmix64 of (seed, index, stream)
__device__ __forceinline__ float hash_unif(uint64_t seed, uint64_t idx, uint32_t k)
{
    uint64_t z = seed + 0x9E3779B97F4A7C15ULL * (idx * 4 + k + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return ((float)(z >> 40) + 0.5f) * (1.0f / 16777216.0f);
}

// Random samples: case uniform over the pool, |k~| log-uniform in
// [kmin, kmax], direction uniform in the first quadrant (k_par, k_perp >= 0).
// W [m][4]: loss weights for the footprint's relative L2 error, with the
// importance factor k^2 of the log-uniform draw: flux term
// k^2 |Tq|^2 / Eq(case), concentration term k^2 |R~ Tq|^2 / Ep(case);
// outputs 0, 1 weigh (1 + k)^2 (flux + conc), outputs 2, 3 weigh conc, each
// plus `floor`.  norm == null: W = raw (k^2 |Tq|^2, -, k^2 |R~ Tq|^2, -)
// for estimating the per-case energies.  cid_out (optional) gets the case ids.
__global__ void transfer_samples_kernel(const TransferCase *__restrict__ cases, const float4 *__restrict__ steps,
                                        int lmax, int ncases, uint64_t seed, float kmin, float lratio,
                                        const float2 *__restrict__ norm, float floor_w, float *X, float *Tg,
                                        float *W, int *cid_out, int m)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    const int c = min((int)(hash_unif(seed, s, 0) * (float)ncases), ncases - 1);
    // (|k|, direction) on the additive-recurrence sequence with plastic-number
    // steps (a stratified 2D point set), shifted at random per call
    // (fractional parts in 32-bit fixed point: frac(a s + r) = (A s + R) / 2^32)
    const uint32_t r1 = (uint32_t)(hash_unif(seed, 0, 1) * 4294967296.0f);
    const uint32_t r2 = (uint32_t)(hash_unif(seed, 0, 2) * 4294967296.0f);
    const float u1 = ((uint32_t)s * 3242174890u + r1) * 2.3283064365386963e-10f;
    const float u2 = ((uint32_t)s * 2447445414u + r2) * 2.3283064365386963e-10f;
    const float k = kmin * expf(lratio * u1);
    float sn, cs;
    sincospif(0.5f * u2, &sn, &cs);
    const float kpar = k * cs, kperp = k * sn;
    const TransferCase tc = cases[c];
    float out[4];
    transfer_one(tc, steps + (size_t)c * lmax, kpar, kperp, out);
    feature_row(X + (size_t)s * 8, kpar, kperp, tc.s1, tc.s2, tc.s3);
#pragma unroll
    for (int o = 0; o < 4; ++o) Tg[(size_t)s * 4 + o] = out[o];
    if (cid_out) cid_out[s] = c;
    const float kk = 1.f + k;
    const float imp = k * k;
    const float q2 = imp * expf(fmaxf(2.f * out[0] * kk, -80.f));
    const float2 rt = top_ratio(tc.ktop, tc.utop, kpar, kperp);
    const float p2 = q2 * expf(fminf(2.f * out[2], 80.f)) * fmaf(rt.x, rt.x, rt.y * rt.y);
    float *w = W + (size_t)s * 4;
    if (!norm) {
        w[0] = q2;
        w[1] = 0.f;
        w[2] = p2;
        w[3] = 0.f;
        return;
    }
    const float2 nm = norm[c];
    const float fq = q2 * nm.x, fp = p2 * nm.y;
    w[0] = w[1] = kk * kk * (fq + fp) + floor_w;
    w[2] = w[3] = fp + floor_w;
}

// targets of given samples (case ids and wavenumbers), for checks
__global__ void transfer_eval_kernel(const TransferCase *__restrict__ cases, const float4 *__restrict__ steps,
                                     int lmax, const int *__restrict__ cid, const float *__restrict__ kpar,
                                     const float *__restrict__ kperp, float *Tg, int m)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    float out[4];
    transfer_one(cases[cid[s]], steps + (size_t)cid[s] * lmax, kpar[s], kperp[s], out);
#pragma unroll
    for (int o = 0; o < 4; ++o) Tg[(size_t)s * 4 + o] = out[o];
}

}  // namespace

// Nondimensional step table of a case given its dimensional grid and profiles
// (u, v, Kx, Ky, Kz rows of nz): h~ = dz / zm, K~ = Kz / (U zm), U~ = u_par / U
// with u_par the speed along (ex, ey).  Shared with the serving path.
void surrogate_steps_from_profiles(int nz, const double *z, const double *prof, double zm, double wind, double ex,
                                   double ey, float4 *st)
{
    const double *u = prof, *v = prof + nz, *Kz = prof + 4 * nz;
    for (int i = 0; i < nz - 1; ++i)
        st[i] = make_float4((float)((z[i + 1] - z[i]) / zm), (float)(Kz[i] / (wind * zm)),
                            (float)((u[i] * ex + v[i] * ey) / wind), 0.f);
}

extern "C" {

int bldfm_transfer_pool_create(const double *s1, const double *s2, int32_t ncases, int32_t n, void **pool)
{
    return bldfm_guarded([&]() -> int {
        if (!s1 || !s2 || ncases < 1 || n < 2 || !pool) return BLDFM_ERR_ARG;
        std::unique_ptr<TransferPool> own(new TransferPool());  // freed on every early return
        TransferPool *P = own.get();
        P->ncases = ncases;
        P->n = n;
        std::vector<std::vector<float4>> st(ncases);
        P->host_cases.resize(ncases);
        for (int c = 0; c < ncases; ++c) {
            // z_m = 1 and unit wind at z_m: z0 = exp(-s2), L = 1 / s1, u* from the log-law
            const double mol = fabs(s1[c]) < 1e-12 ? 1e12 : 1.0 / s1[c];
            ProfileCase pc;
            const int rc = profile_scalars(n, 1.0, 1.0, 0.0, -1.0, exp(-s2[c]), mol, 1.0, 0, -1.0, -1.0, -1.0, &pc);
            if (rc != BLDFM_OK || pc.nz > BLDFM_MAX_NZ) return rc != BLDFM_OK ? rc : BLDFM_ERR_UNSUPPORTED;
            std::vector<double> z(pc.nz), prof(5 * (size_t)pc.nz);
            profile_levels_host(pc, z.data(), prof.data());
            TransferCase &tc = P->host_cases[c];
            tc.nz = pc.nz;
            tc.jm = n;
            tc.ktop = (float)prof[4 * (size_t)pc.nz + pc.nz - 1];
            tc.utop = (float)prof[pc.nz - 1];
            tc.s1 = (float)s1[c];
            tc.s2 = (float)s2[c];
            tc.s3 = (float)pc.ustar;
            tc.pad = 0;
            st[c].resize(pc.nz - 1);
            surrogate_steps_from_profiles(pc.nz, z.data(), prof.data(), 1.0, 1.0, 1.0, 0.0, st[c].data());
            P->lmax = std::max(P->lmax, pc.nz - 1);
        }
        std::vector<float4> flat((size_t)ncases * P->lmax, make_float4(0.f, 1.f, 0.f, 0.f));
        for (int c = 0; c < ncases; ++c) std::copy(st[c].begin(), st[c].end(), flat.begin() + (size_t)c * P->lmax);
        if (cudaMalloc(&P->cases, sizeof(TransferCase) * ncases) != cudaSuccess ||
            cudaMalloc(&P->steps, sizeof(float4) * flat.size()) != cudaSuccess)
            return BLDFM_ERR_CUDA;
        if (cudaMemcpy(P->cases, P->host_cases.data(), sizeof(TransferCase) * ncases, cudaMemcpyHostToDevice) !=
                cudaSuccess ||
            cudaMemcpy(P->steps, flat.data(), sizeof(float4) * flat.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return BLDFM_ERR_CUDA;
        *pool = own.release();
        return BLDFM_OK;
    });
}

int bldfm_transfer_pool_destroy(void *pool)
{
    TransferPool *P = (TransferPool *)pool;
    if (!P) return BLDFM_ERR_ARG;
    cudaDeviceSynchronize();
    delete P;
    return BLDFM_OK;
}

int bldfm_transfer_pool_case(void *pool, int32_t c, double *s3, int32_t *nz)
{
    TransferPool *P = (TransferPool *)pool;
    if (!P || c < 0 || c >= P->ncases) return BLDFM_ERR_ARG;
    if (s3) *s3 = P->host_cases[c].s3;
    if (nz) *nz = P->host_cases[c].nz;
    return BLDFM_OK;
}

int bldfm_transfer_samples(void *pool, uint64_t seed, int32_t m, float kmin, float kmax, const float *norm,
                           float floor_w, float *X, float *T, float *W, int32_t *cid, void *stream)
{
    TransferPool *P = (TransferPool *)pool;
    if (!P || !X || !T || !W || m < 1 || !(kmin > 0.f) || !(kmax > kmin)) return BLDFM_ERR_ARG;
    transfer_samples_kernel<<<(m + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
        P->cases, P->steps, P->lmax, P->ncases, seed, kmin, logf(kmax / kmin), (const float2 *)norm, floor_w, X, T,
        W, cid, m);
    return cudaGetLastError() == cudaSuccess ? BLDFM_OK : BLDFM_ERR_CUDA;
}

int bldfm_transfer_eval(void *pool, const int32_t *cid, const float *kpar, const float *kperp, float *T, int32_t m,
                        void *stream)
{
    TransferPool *P = (TransferPool *)pool;
    if (!P || !cid || !kpar || !kperp || !T || m < 1) return BLDFM_ERR_ARG;
    transfer_eval_kernel<<<(m + 127) / 128, 128, 0, (cudaStream_t)stream>>>(P->cases, P->steps, P->lmax, cid, kpar,
                                                                           kperp, T, m);
    return cudaGetLastError() == cudaSuccess ? BLDFM_OK : BLDFM_ERR_CUDA;
}

}  // extern "C"
