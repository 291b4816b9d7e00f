#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// Per-case scalars of vertical_profiles (closures 0 MOST, 1 CONSTANT, 2 MOSTM, 3 OAAHOC).
struct ProfileCase {
    int nz, closure;
    double zm, um, vm, absum, ustar, z0, mol, prsc, h, aa, bb, dzeta, tke;
};

int profile_scalars(int n, double zm, double um, double vm, double ustar, double z0, double mol, double prsc,
                    int closure, double domain_height, double stretch, double tke, ProfileCase *pc);
// z and the five profile rows (stride nz) of every level, on the host
void profile_levels_host(const ProfileCase &pc, double *z, double *prof);
cudaError_t launch_profiles_batch(const ProfileCase *pcs_dev, const int64_t *zoff_dev, int ncases, double *z,
                                  double *prof, cudaStream_t st);
