// Batched FP32 solve: device descriptors and launch parameters.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.h"

// solved modes per thread of the batched sweep (a tile is this many blocks)
#define BATCH_MODES_PER_THREAD 2

// One case of a batch as the device kernels see it.
struct __align__(16) BatchCase {
    SolveGeom g;
    FftPlan plx, ply;  // output transform plans
    const float *lv32;
    const int *slot;
    const uint32_t *modes;
    const float2 *q0;
    float *scratch;
    float2 *Xp, *Xq;
    const double2 *dc;
    float2 *Cb;
    const float2 *twx, *twy;
    const int4 *xband;
    double *conc, *flx;
    const float2 *lvff;  // the level table's FP64 rows as float pairs hi + lo (accuracy check)
    float ax, ay;
    int64_t tile0;  // first sweep tile of this case
    int64_t col0;   // first column-transform CTA
    int64_t row0;   // first row-transform CTA
    int32_t rpc;    // rows per row-transform CTA
    int32_t cpc;    // band columns per column-transform CTA
};

// A group of a batch's cases that share the register-resident transform
// configs: one column-pass and one row-pass launch each, over its CTAs
// [col_start, col_start + col_ctas) and [row_start, row_start + row_ctas) of
// the CTA-to-case maps (each case's col0 / row0 counts from its group's start)
#define BATCH_MAX_XGROUPS 8
struct XGroup {
    int rx_col, rx_row;
    int col_start, col_ctas, row_start, row_ctas;
};

struct BatchLaunch {
    const BatchCase *cases;
    const int *tile_case;
    const int64_t *cta_tiles;
    const int *col_case;
    const int *row_case;
    int *err;
    int sweep_ctas, threads;
    size_t sweep_smem;
    int col_ctas;
    size_t col_smem;
    int row_ctas;
    size_t row_smem;
    // persistent one-line transforms (col_ctas / row_ctas count items, launched
    // on col_grid / row_grid CTAs); shared-memory sizes from the largest case
    int persist, col_grid, row_grid, maxn_col, maxnly, maxn_row;
    // register-resident transform passes (xform.cu): rx_col >= 0 when they
    // run (one launch per group of xg), -1 for the shared-memory passes
    int rx_col, rx_row;
    int nxg;
    XGroup xg[BATCH_MAX_XGROUPS];
};

cudaError_t launch_batch_kernels(const BatchLaunch &bl, cudaStream_t st, int part);

// Accuracy check of a batched FP32 solve (batch.cu: fp32_check_kernel): a
// stratified sample of 32 modes per case evaluated in float-float arithmetic
// and compared with the FP32 spectra at every output level; per case
// acc[k] = weighted (sum |dXp|^2, sum |Xp|^2, sum |dXq|^2, sum |Xq|^2).
cudaError_t launch_fp32_check(const BatchCase *cases, int n, float4 *acc, cudaStream_t st);

// Accuracy guard of a surrogate batch (batch.cu: sur_guard_kernel): exact
// FP32 values of every stride-th solved mode against the served spectra,
// per-case sums into acc[k] = (|dXp|^2, |Xp|^2, |dXq|^2, |Xq|^2); prefix:
// n + 1 sample offsets, each case's count padded to a multiple of
// SUR_GUARD_CTA (a CTA's samples belong to one case); max_nz: the largest
// level count (the level table is staged in shared memory).
#define SUR_GUARD_BOX 12  // solved modes with |kx|, |ky| <= 2, sampled by the guard
#define SUR_GUARD_THREADS 256
#define SUR_GUARD_CTA (2 * SUR_GUARD_THREADS)  // samples per CTA, two per thread
cudaError_t launch_sur_guard(const BatchCase *cases, int n, const int64_t *prefix, int64_t nsamples, int stride,
                             int max_nz, float4 *acc, cudaStream_t st);

// Exact low band of a surrogate footprint (batch.cu: sur_lowband_kernel):
// the solved modes with |k| < kmax are re-solved by the exact FP32 sweep and
// written over the served spectra, mirrors included, before the output
// transform.  The band's modes are enumerated over the half box kx in
// [0, bx], ky in [-by, by] (kx = 0: ky in [1, by]), then, when the box
// reaches an even mode count's Nyquist frequency, the unpaired modes of the
// Nyquist column kx = -nlx/2 and row ky = -nly/2; two per thread, 512 per
// CTA; modes outside the disc are skipped.
#define SUR_LOWBAND_THREADS 256
#define SUR_LOWBAND_MODES (2 * SUR_LOWBAND_THREADS)  // box positions per CTA
struct __align__(16) LowBandCase {
    SolveGeom g;
    const float *lv32;  // the case's FP32 level table (layout of g.iso)
    float2 *Xp, *Xq;    // the served spectra
    float ax, ay;       // wavenumber scales (Lx = ax kx, Ly = ay ky)
    float kmax2;        // squared wavenumber bound (1/m^2)
    int bx, by;         // index half-widths of the band's box
    int nbox, ncol, nrow, ncorner;  // positions: half box, Nyquist column, row, corner
    int count;          // nbox + ncol + nrow + ncorner
    int block0;         // the case's first CTA in the launch
};
// Fill the band of a case for |k| z_m < exact_kz (count = 0 when exact_kz
// <= 0) and return its CTA count; g, lv32, Xp, Xq, ax, ay must be set.
int sur_lowband_setup(LowBandCase &c, double exact_kz, double zm);
// nblocks: the CTAs of all cases; max_nz: the largest level count (the
// level table is staged in shared memory)
cudaError_t launch_sur_lowband(const LowBandCase *cases, int n, int nblocks, int max_nz, cudaStream_t st);

// register-resident transform passes (xform.cu), for line lengths 512, 768,
// 1024, 1536, 2048, 3072: config id of a length (-1 if unsupported), lines
// per 256-thread CTA and dynamic shared memory per CTA of the column (col)
// or row pass, one-time attributes,
// and the launch of the column (col) or row pass over nctas CTAs
int rx_config(int n);
// zoomed column pass (xform_zoom.cuh) for a line of length n = 3 M (M = 256,
// 512) whose band has at most 2 band_half + 1 <= M + 1 frequencies and whose
// kept window nout <= M positions: config id RX_ZOOM_BASE + k, or -1
#define RX_ZOOM_BASE 16
int rx_zoom_config(int n, int band_half, int nout);
int rx_lines_per_cta(int cfg, bool col);
size_t rx_smem(int cfg, bool col);
void prepare_rx_attributes();
cudaError_t launch_rx_pass(int cfg, bool col, const BatchLaunch &bl, int nctas, cudaStream_t st);
int batch_sweep_occupancy(int threads, size_t smem);
int batch_xform_occupancy(int col, size_t smem);
void prepare_batch_attributes();
