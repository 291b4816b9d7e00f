// Parameter layout and activation of the surrogate MLP, shared by the
// training kernels (surrogate.cu) and the fused serving kernel (serve.cu).
//
// The MLP: 8 -> 256 -> 256 -> 256 -> 256 -> 4, GELU after each hidden layer.
// Flat FP32 parameter vector: W0 [8][256] (in, out), b0 [256], then for
// j = 1..3 Wt_j [256][256] (out, in) and b_j [256], then W4 [256][4]
// (in, out), b4 [4].
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#define MLP_IN 8
#define MLP_XS 8  // stride of the input rows
#define MLP_H 256
#define MLP_OUT 4
#define MLP_OFF_W0 0
#define MLP_OFF_B0 (MLP_IN * MLP_H)
#define MLP_OFF_WT(j) (MLP_OFF_B0 + MLP_H + ((j)-1) * (MLP_H * MLP_H + MLP_H))
#define MLP_OFF_B(j) (MLP_OFF_WT(j) + MLP_H * MLP_H)
#define MLP_OFF_W4 (MLP_OFF_WT(4))
#define MLP_OFF_B4 (MLP_OFF_W4 + MLP_H * MLP_OUT)
#define MLP_NPARAM (MLP_OFF_B4 + MLP_OUT)

__device__ __forceinline__ uint16_t f2bf(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }
__device__ __forceinline__ float bf2f(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// GELU in its tanh form (Hendrycks & Gimpel, 2016):
//   gelu(z) = z/2 (1 + tanh(u)), u = sqrt(2/pi) (z + 0.044715 z^3)
#define GELU_C 0.7978845608028654f
#define GELU_A 0.044715f
__device__ __forceinline__ float gelu_f(float z)
{
    // u = z (c + c a z^2), gelu = z/2 + z/2 tanh(u)
    const float u = z * fmaf(GELU_C * GELU_A, z * z, GELU_C);
    const float hz = 0.5f * z;
    return fmaf(hz, tanh_approx(u), hz);
}
// gelu_f(v + b) for two values in the lanes of packed f32x2 operations (the
// same operations and rounding as the scalar form, lane by lane)
__device__ __forceinline__ float2 gelu2_bias(float2 v, float2 b)
{
    const float2 z = __fadd2_rn(v, b);
    const float2 p = __ffma2_rn(make_float2(GELU_C * GELU_A, GELU_C * GELU_A), __fmul2_rn(z, z),
                                make_float2(GELU_C, GELU_C));
    const float2 u = __fmul2_rn(z, p);
    const float2 hz = __fmul2_rn(make_float2(0.5f, 0.5f), z);
    return __ffma2_rn(hz, make_float2(tanh_approx(u.x), tanh_approx(u.y)), hz);
}

// two floats -> BF16x2 (round to nearest even; first value in the low half)
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ float gelu_d(float z)
{
    const float z2 = z * z;
    const float t = tanh_approx(GELU_C * fmaf(GELU_A * z2, z, z));
    return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * GELU_C * fmaf(3.0f * GELU_A, z2, 1.0f);
}

// device views of a trained MLP for the fused serving kernel: FP32
// parameters and the BF16 core-matrix blocks of Wt_1..3 (256 x 256 each)
struct MlpServing {
    const float *P;
    const uint16_t *Wt[3];  // 256 x 256 core-matrix blocks
    const uint16_t *Wq[3];  // the same as four contiguous 128 x 128 quarters (N half, K half)
};
int mlp_serving_view(void *handle, MlpServing *out);
