// Launchers of the device kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.h"

#define BLDFM_ERR_TIMEOUT_DEV (-9)
#define BLDFM_ERR_NONFINITE_DEV (-10)


cudaError_t launch_sweep64(const SolveGeom &g, const double *lvtab, const int *slot, const uint32_t *modes,
                           const double2 *q0spec, double2 *snap, double2 *top, int *err, int nsm, cudaStream_t st);
cudaError_t launch_combine64(const SolveGeom &g, const uint32_t *modes, const double2 *eig, const double2 *snap,
                             const double2 *top, double2 *Xp, double2 *Xq, cudaStream_t st);
// k = 0 mode from a device-resident q0 (dispersion mode) into dc[2 s], dc[2 s + 1]
cudaError_t launch_trapezoid64(const SolveGeom &g, const double *lvtab, const int *slot, const double2 *q0spec,
                               double p000, double2 *dc, cudaStream_t st);
// FP32 spectra: with src and dcp (DC_PARTS doubles of scratch), the k = 0
// source value is the FP64 sum of the source field (dc_partial_kernel), not
// the FP32 transform's k = 0 output, whose rounding (~1e-6 relative) would
// dominate the mean of the concentration field
#define DC_PARTS 16
cudaError_t launch_trapezoid32(const SolveGeom &g, const double *lvtab, const int *slot, const float2 *q0spec,
                               double p000, double2 *dc, cudaStream_t st, const double *src = nullptr,
                               double *dcp = nullptr);
cudaError_t launch_analytic64(const SolveGeom &g, const uint32_t *modes, const double2 *eig, const double2 *q0spec,
                              double p000, double kzinv, double hlev, double2 *Xp, double2 *Xq, double2 *dc,
                              cudaStream_t st);
cudaError_t launch_riccati32(const SolveGeom &g, const float *lv32, const int *slot, const uint32_t *modes,
                             const float2 *q0spec, float *scratch, float2 *Xp, float2 *Xq, float ax, float ay,
                             int *err, int nsm, int threads, cudaStream_t st);
template <typename R>
cudaError_t launch_forward_fft(const SolveGeom &g, const FftPlan &plx, const FftPlan &ply,
                               const typename cvec<R>::T *twx, const typename cvec<R>::T *twy, const double *src,
                               typename cvec<R>::T *A, typename cvec<R>::T *Q0, cudaStream_t st);
template <typename R>
cudaError_t launch_output_fft(const SolveGeom &g, const FftPlan &plx, const FftPlan &ply,
                              const typename cvec<R>::T *twx, const typename cvec<R>::T *twy, const int4 *xband,
                              const typename cvec<R>::T *Xp, const typename cvec<R>::T *Xq, const double2 *dc,
                              typename cvec<R>::T *Cbuf, double *conc, double *flx, int *err, cudaStream_t st);
cudaError_t launch_tw_to_float(const double2 *src, float2 *dst, int n, cudaStream_t st);
cudaError_t launch_spec_to_float(const double2 *src, float2 *dst, int64_t n, cudaStream_t st);
cudaError_t launch_nonfinite(const double *a, const double *b, int64_t n, int *flag, int nsm, cudaStream_t st);
cudaError_t run_fma_peak(int kind, int nsm, cudaStream_t st, double *flops_per_s);
void prepare_kernel_attributes();
cudaError_t launch_riccati64(const SolveGeom &g, const double *lvtab, const int *slot, const uint32_t *modes,
                             const double2 *q0spec, double *scratch, double2 *Xp, double2 *Xq, int *err, int nsm,
                             cudaStream_t st);
