// Internal definitions shared by the host planner and the device kernels.
#pragma once

#include <stdint.h>
#include <vector_types.h>

// complex vector type of a real type
template <typename R> struct cvec;
template <> struct cvec<double> { typedef double2 T; };
template <> struct cvec<float> { typedef float2 T; };

#define BLDFM_MAX_FFT_N 4096    // longest transform held in shared memory
#define BLDFM_MAX_STAGES 16
#define BLDFM_MAX_NZ 2048       // level table must fit in shared memory
#define BLDFM_LV64 12           // doubles per FP64 level-table row
#define BLDFM_LV32 12           // floats per FP32 level-table row
// Polls of an mbarrier wait before it gives up and reports a timeout.  A
// failed poll suspends the thread for about 4 us on GB300 (measured by
// bldfm_selftest_wait_timeout), so a wait that never completes ends after
// about 1 s; every copy or MMA waited on completes in well under 1 ms.
#define BLDFM_WAIT_POLLS (1L << 18)

// Columns of the FP64 level table (same layout as the CPU oracle's).
enum {
    LV_KX = 0, LV_KY, LV_U, LV_V, LV_S1, LV_H2, LV_S2, LV_H3, LV_S3, LV_S4, LV_H, LV_PAD
};

// Columns of the FP32 level table (Riccati sweep), generic profiles.  Isotropic
// profiles with a fixed wind direction use the compact row of StepCoef<true>.
enum {
    L32_NKX = 0,  // -Kx
    L32_NKY,      // -Ky
    L32_NU,       // -u
    L32_NV,       // -v
    L32_A,        // 0.5 * h^2 / Kz
    L32_B0,       // -h / Kz
    L32_B1,       // h^3 / (6 Kz^2)
    L32_H,        // h
    L32_C1,       // h^3 / (6 Kz)
    L32_C2,       // -2 * C1
    L32_P0, L32_P1
};

// Plan of one mixed-radix transform length.
// floor(x / d) for 0 <= x < 2^31 as umulhi(x, m) >> s (Granlund-Montgomery
// round-up multiplier, l = ceil(log2 d), m = ceil(2^(31 + l) / d) < 2^32,
// s = l - 1); s < 0 marks d == 1.
struct FDiv {
    uint32_t m;
    int32_t s;
};

inline FDiv fdiv_make(uint32_t d)
{
    FDiv f;
    if (d <= 1) {
        f.m = 0;
        f.s = -1;
        return f;
    }
    int l = 0;
    while ((1ull << l) < d) ++l;
    f.m = (uint32_t)(((1ull << (31 + l)) + d - 1) / d);
    f.s = l - 1;
    return f;
}

struct FftPlan {
    int32_t n;
    int32_t nstages;
    int32_t radix[BLDFM_MAX_STAGES];
    int32_t rq[BLDFM_MAX_STAGES];   // stride of stage q: n / (L_{q-1} p_q)
    FDiv drq[BLDFM_MAX_STAGES];     // division by rq
    FDiv dnb[BLDFM_MAX_STAGES];     // division by n / p_q (butterflies per line)
};

// per-stage strides and division multipliers of a factorised plan
inline void fft_plan_finalize(FftPlan &p)
{
    int L1 = 1;
    for (int q = 0; q < p.nstages; ++q) {
        const int P = p.radix[q];
        p.rq[q] = p.n / (L1 * P);
        p.drq[q] = fdiv_make((uint32_t)p.rq[q]);
        p.dnb[q] = fdiv_make((uint32_t)(p.n / P));
        L1 *= P;
    }
}

// columns per CTA of the column pass for transform length n: a power of two,
// as many as fit (2 cpc + 1) n complex in ~110 KB of shared memory, at most 4
inline int out_cols_per_cta(int n, size_t csize)
{
    int cpc = 4;
    while (cpc > 1 && (2 * (size_t)cpc + 1) * n * csize > 110 * 1024) cpc >>= 1;
    return cpc;
}

// Everything a kernel needs to know about one solve (passed by value).
struct SolveGeom {
    int32_t nx, ny, nz;
    int32_t nlx, nly;       // effective modes
    int32_t nxe, nye;
    int32_t px, py, dlx, dly;
    int32_t nfx, nfy;       // output transform size
    int32_t out_nx, out_ny;
    int32_t nlvls, nsnap;
    int32_t footprint, analytic, precision, mode;
    int32_t do_shift;
    int32_t out_sign;       // -1: fft2 (footprint), +1: ifft2 norm=forward
    int32_t nbx;            // number of band columns of the output transform
    int64_t nsolved;
    double lx_scale, ly_scale;  // Lx = lx_scale * (kx * valx)
    double valx, valy;
    double sx, sy;              // phase shift offsets
    double kz_top;
    double q0dc_fp;             // footprint source spectrum 1/nxe/nye
    double inv_nxe, inv_nye;    // forward-FFT normalisation
    // top-level coefficients for the FP32 eigenvalue
    double kxk_top, kyk_top, uk_top, vk_top;
    uint32_t turn_x, turn_y;    // phase shift as 32-bit fixed-point turns per unit k
    int32_t iso;                // Kx == Ky and (u, v) along one direction at every level
    int32_t jmax;               // highest output level (slot level), -1 if none
    float ex, ey;               // wind direction unit vector (iso tables)
    // the FP32 path's copies of kxk_top, kyk_top, uk_top, vk_top, kz_top and
    // q0dc_fp, rounded once on the host: the per-mode setup of the FP32
    // sweeps then needs no FP64 conversion (FP64 runs at 1/64 of the FP32
    // rate on GB300)
    float kxk_top_f, kyk_top_f, uk_top_f, vk_top_f, kz_top_f, q0dc_f;
};

// fftfreq ordering helpers: index <-> signed frequency.
__host__ __device__ inline int freq_of_index(int idx, int n)
{
    int half = (n - 1) / 2 + 1;
    return idx < half ? idx : idx - n;
}
__host__ __device__ inline int index_of_freq(int f, int n)
{
    return f >= 0 ? f : f + n;
}
// lowest / highest signed frequency of fftfreq(n)
__host__ __device__ inline int freq_min(int n) { return -(n / 2); }
__host__ __device__ inline int freq_max(int n) { return (n - 1) / 2; }
