// Serving kernels of the learned surrogate: per-mode features, the exact
// nondimensional transfer (for checks), and the spectra at z_m.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.h"
#include "mlp_common.cuh"

struct TransferCase;

cudaError_t launch_sur_features(const SolveGeom &g, const uint32_t *modes, float ax, float ay, float zm, float s1,
                                float s2, float s3, float *X, int64_t npad, cudaStream_t st);
cudaError_t launch_sur_exact(const SolveGeom &g, const uint32_t *modes, float ax, float ay, float zm,
                             const TransferCase *tc, const float4 *steps, float *Y, cudaStream_t st);
// One footprint of a surrogate launch as the fused kernel sees it.
struct __align__(16) SurCase {
    SolveGeom g;
    const uint32_t *modes;
    float2 *Xp, *Xq;
    float ax, ay;                  // wavenumber scales (Lx = ax * kx)
    float zm, s1, s2, s3;          // z_m, z_m / L, ln(z_m / z0), u* / U
    float inv_wind, ktop, utop;    // 1 / U, K~ and U~ of the top level
    float pad;
    int64_t tile0;                 // first 128-mode tile of this case in the launch
};

// fused features -> MLP (tcgen05) -> spectra over every 128-mode tile of
// ncases cases (device table, tile0 ascending), one persistent CTA per SM
cudaError_t launch_sur_serve(const SurCase *cases, int ncases, int64_t ntiles, const MlpServing &net, int *err,
                             int nsm, cudaStream_t st);
// ktop, utop: K~ and U~ of the top level (the radiation ratio R~top)
cudaError_t launch_sur_spectra(const SolveGeom &g, const uint32_t *modes, const float *Y, float ax, float ay,
                               float zm, float inv_wind, float ktop, float utop, float2 *Xp, float2 *Xq,
                               cudaStream_t st);
void surrogate_steps_from_profiles(int nz, const double *z, const double *prof, double zm, double wind, double ex,
                                   double ey, float4 *st);
