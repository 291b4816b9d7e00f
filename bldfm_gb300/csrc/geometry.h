// Geometry of one solve, shared by every entry point (heap-free).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bldfm_gb300.h"
#include "common.h"

// Grid arithmetic of the reference (solver.py:94-131, 253-262, 264-290) and
// the per-call scalars of the sweep.  Fills every SolveGeom field that does
// not depend on a device: extended grid, clamped modes, transform sizes, crop,
// phase shift (also as 32-bit fixed-point turns), top-level coefficients,
// snapshot schedule (slot[i] = output slot of level i or -1; slot may be null
// when levels is null) and the number of solved modes.  z, prof and levels
// may be null (sizes only: bldfm_plan).  *shape_ok reports whether the
// truncated source spectrum matches the modes (non-footprint solves need it).
// Returns BLDFM_OK or a BLDFM_ERR_* code.
int solve_geometry(const bldfm_desc *d, const double *z, const double *prof, const int64_t *levels, int nlvls,
                   SolveGeom &g, int *slot, bool *shape_ok);

// Solved modes of column c (one of each Hermitian pair plus the unpaired
// Nyquist row/column), in the order the sweep kernels list them.
int solved_in_column(int c, int nlx, int nly);

// Band columns of the output transform: positions of the frequencies
// [-h, h] mod nfx (h = max(-fmin, fmax) of nlx), each as (position, column
// of X at P, column of X at -P, 0).  out holds at least 2 h + 1 entries.
// Returns the count.
int band_columns(int nlx, int nfx, int4 *out);
