// Device helpers shared by the kernels: numpy-exact complex128 arithmetic,
// mode unpacking, the spectrum index, and the bounded TMA bulk load.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.h"
#include "kernels.h"

// ---------------------------------------------------------------------------
// numpy-exact complex128 arithmetic
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 np_cmul(double2 a, double2 b)
{
    return make_double2(__fma_rn(a.x, b.x, -__dmul_rn(a.y, b.y)), __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 np_cadd(double2 a, double2 b)
{
    return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}
__device__ __forceinline__ double2 np_csub(double2 a, double2 b)
{
    return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y));
}
// Smith's method, reciprocal-scale form (numpy complex128 divide).
__device__ __forceinline__ double2 np_cdiv(double2 a, double2 b)
{
    double2 o;
    if (fabs(b.x) >= fabs(b.y)) {
        double rat = __ddiv_rn(b.y, b.x);
        double scl = __ddiv_rn(1.0, __dadd_rn(b.x, __dmul_rn(b.y, rat)));
        o.x = __dmul_rn(__dadd_rn(a.x, __dmul_rn(a.y, rat)), scl);
        o.y = __dmul_rn(__dsub_rn(a.y, __dmul_rn(a.x, rat)), scl);
    } else {
        double rat = __ddiv_rn(b.x, b.y);
        double scl = __ddiv_rn(1.0, __dadd_rn(b.y, __dmul_rn(b.x, rat)));
        o.x = __dmul_rn(__dadd_rn(__dmul_rn(a.x, rat), a.y), scl);
        o.y = __dmul_rn(__dsub_rn(__dmul_rn(a.y, rat), a.x), scl);
    }
    return o;
}
__device__ __forceinline__ double2 round_c64(double2 a)
{
    return make_double2((double)__double2float_rn(a.x), (double)__double2float_rn(a.y));
}

// wavenumber of fftfreq index (solver.py:148-155): scale * (k * val)
__device__ __forceinline__ double wavenumber(int k, double val, double scale)
{
    return __dmul_rn(scale, __dmul_rn((double)k, val));
}

__device__ __forceinline__ void unpack_mode(uint32_t e, int &r, int &c, bool &paired)
{
    c = (int)(e & 0x7fffu);
    r = (int)((e >> 15) & 0x7fffu);
    paired = (e >> 31) != 0;
}

// ---------------------------------------------------------------------------
// bulk (TMA) copy of a table into shared memory with a bounded wait
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Copies `bytes` (multiple of 16, both addresses 16-byte aligned) from global
// to shared memory with cp.async.bulk, completing on an mbarrier.  Returns
// false (and sets *err) if the wait runs out; never spins without a limit.
__device__ __noinline__ static bool bulk_load_to_smem(void *dst, const void *src, uint32_t bytes, uint64_t *bar, int *err)
{
    const uint32_t bar_a = smem_u32(bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar_a), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(bytes) : "memory");
        const uint32_t chunk = 32768;
        for (uint32_t off = 0; off < bytes; off += chunk) {
            uint32_t n = bytes - off < chunk ? bytes - off : chunk;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32((char *)dst + off)),
                "l"((const char *)src + off), "r"(n), "r"(bar_a)
                : "memory");
        }
    }
    uint32_t done = 0;
    for (long it = 0; it < BLDFM_WAIT_POLLS; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar_a), "r"(0)
            : "memory");
        if (done) break;
    }
    if (!done) {
        atomicExch(err, BLDFM_ERR_TIMEOUT_DEV);
        return false;
    }
    return true;
}

// Spectrum layout shared by all writers: [lvl][col c][row r], complex.
__device__ __forceinline__ size_t spec_idx(const SolveGeom &g, int lvl, int r, int c)
{
    return ((size_t)lvl * g.nlx + c) * g.nly + r;
}

