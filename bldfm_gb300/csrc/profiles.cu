// Device evaluation of vertical_profiles (src/bldfm/pbl_model.py:8-204) for the
// MOST (0), CONSTANT (1), MOSTM (2) and OAAHOC (3) closures, with the
// Businger-Dyer functions psi and phi (pbl_model.py:207-250).  Per-case scalars (roughness length or friction
// velocity, grid constants, number of levels) are computed on the host; every
// level is one device thread.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "../../include/bldfm_gb300.h"
#include "guard.h"
#include "profiles.h"

namespace {
const double KAP = 0.4;

__host__ __device__ inline double psi_bd(double x)
{
    if (x > 0.0) return 5.0 * x;
    const double xi = pow(1.0 - 16.0 * x, 0.25);
    return -2.0 * log(0.5 * (1.0 + xi)) - log(0.5 * (1.0 + xi * xi)) + 2.0 * atan(xi) - 0.5 * M_PI;
}

__host__ __device__ inline double phi_bd(double x)
{
    if (x > 0.0) return 1.0 + 5.0 * x;
    return pow(1.0 - 16.0 * x, -0.5);
}
}  // namespace

// Host part: per-case scalars and the number of levels.
// OAAHOC constants (pbl_model.py:83-86)
const double OA_CL = 0.845, OA_CM = 0.0856, OA_CH = 0.204;

int profile_scalars(int n, double zm, double um, double vm, double ustar, double z0, double mol, double prsc,
                    int closure, double domain_height, double stretch, double tke, ProfileCase *pc)
{
    if (n < 1 || !(zm > 0) || !(prsc > 0)) return BLDFM_ERR_ARG;
    if (closure < 0 || closure > 3) return BLDFM_ERR_ARG;
    const double absum = sqrt(um * um + vm * vm);
    const bool have_u = ustar > 0, have_z0 = z0 > 0;
    if (closure == 3) {
        // one-and-a-half order closure: z0 from ustar and tke (pbl_model.py:79-98)
        if (!have_u) return BLDFM_ERR_ARG;
        if (!(tke > 0)) tke = 1.0;
        z0 = zm * exp(-OA_CM * OA_CL * absum * sqrt(tke) / (ustar * ustar));
    } else {
        if (have_u == have_z0) return BLDFM_ERR_ARG;  // reference: "Either z0 or ustar must be provided."
        if (!have_z0)
            z0 = zm * exp(-KAP * absum / ustar + psi_bd(zm / mol));
        else
            ustar = absum * KAP / (log(zm / z0) + psi_bd(zm / mol));
    }
    const double h = stretch > 0 ? stretch : 2.0 * zm;
    const double zmx = domain_height > 0 ? domain_height : 2.0 * zm;
    const double bb = zm / (exp(-z0 / h) - exp(-zm / h));
    const double aa = bb * exp(-z0 / h);
    const double zetamx = aa - bb * exp(-zmx / h);
    const double dzeta = zm / n;
    const double len = ceil((zetamx + dzeta - 0.0) / dzeta);
    if (!(len >= 1) || len > 1e6) return BLDFM_ERR_ARG;
    pc->nz = (int)len;
    pc->zm = zm;
    pc->um = um;
    pc->vm = vm;
    pc->absum = absum;
    pc->ustar = ustar;
    pc->z0 = z0;
    pc->mol = mol;
    pc->prsc = prsc;
    pc->closure = closure;
    pc->h = h;
    pc->aa = aa;
    pc->bb = bb;
    pc->dzeta = dzeta;
    pc->tke = tke;
    return BLDFM_OK;
}

__host__ __device__ void profile_level(const ProfileCase &pc, int i, double *z, double *prof, int stride)
{
    const double zeta = (double)i * pc.dzeta;
    const double zi = -pc.h * log(-(zeta - pc.aa) / pc.bb);
    double u, v, K, Kx, Ky;
    if (pc.closure == 1) {  // CONSTANT
        u = pc.um;
        v = pc.vm;
        K = KAP * pc.ustar * pc.zm / pc.prsc;
        Kx = Ky = K;
    } else if (pc.closure == 3) {  // OAAHOC
        const double st = sqrt(pc.tke);
        const double absu = pc.ustar * pc.ustar / OA_CM / OA_CL / st * log(zi / pc.z0);
        u = pc.um / pc.absum * absu;
        v = pc.vm / pc.absum * absu;
        K = OA_CH * OA_CL * zi * st;
        Kx = Ky = K;
    } else {  // MOST, MOSTM
        const double absu = pc.ustar / KAP * (log(zi / pc.z0) + psi_bd(zi / pc.mol));
        u = pc.um / pc.absum * absu;
        v = pc.vm / pc.absum * absu;
        K = KAP * pc.ustar * zi / phi_bd(zi / pc.mol) / pc.prsc;
        Kx = Ky = K;
        if (pc.closure == 2) {  // no diffusion along the flow (pbl_model.py:152-164)
            Kx = K * v * v / (u * u + v * v);
            Ky = K * u * u / (u * u + v * v);
        }
    }
    z[i] = zi;
    prof[i] = u;
    prof[stride + i] = v;
    prof[2 * stride + i] = Kx;
    prof[3 * stride + i] = Ky;
    prof[4 * stride + i] = K;
}

// host evaluation of every level (training data of the surrogate)
void profile_levels_host(const ProfileCase &pc, double *z, double *prof)
{
    for (int i = 0; i < pc.nz; ++i) profile_level(pc, i, z, prof, pc.nz);
}

__global__ void profiles_kernel(ProfileCase pc, double *z, double *prof)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < pc.nz) profile_level(pc, i, z, prof, pc.nz);
}

// Batched: one block per case; case k writes z at zoff[k] and profiles at
// prof + 5 * zoff[k] (stride nz of that case).
__global__ void profiles_batch_kernel(const ProfileCase *__restrict__ pcs, const int64_t *__restrict__ zoff,
                                      double *z, double *prof)
{
    const ProfileCase pc = pcs[blockIdx.x];
    const int64_t o = zoff[blockIdx.x];
    for (int i = threadIdx.x; i < pc.nz; i += blockDim.x) profile_level(pc, i, z + o, prof + 5 * o, pc.nz);
}

cudaError_t launch_profiles_batch(const ProfileCase *pcs_dev, const int64_t *zoff_dev, int ncases, double *z,
                                  double *prof, cudaStream_t st)
{
    if (ncases <= 0) return cudaSuccess;
    profiles_batch_kernel<<<ncases, 128, 0, st>>>(pcs_dev, zoff_dev, z, prof);
    return cudaGetLastError();
}

extern "C" int bldfm_vertical_profiles(int32_t n, double meas_height, double um, double vm, double ustar,
                                       double z0, double mol, double prsc, int32_t closure, double domain_height,
                                       double stretch, double tke, int32_t *nz_out, double *z_dev,
                                       double *prof_dev, void *stream)
{
    ProfileCase pc;
    int rc = profile_scalars(n, meas_height, um, vm, ustar, z0, mol, prsc, closure, domain_height, stretch, tke,
                             &pc);
    if (rc != BLDFM_OK) return rc;
    if (nz_out) *nz_out = pc.nz;
    if (!z_dev) return BLDFM_OK;
    if (!prof_dev) return BLDFM_ERR_ARG;
    profiles_kernel<<<(pc.nz + 127) / 128, 128, 0, (cudaStream_t)stream>>>(pc, z_dev, prof_dev);
    return cudaGetLastError() == cudaSuccess ? BLDFM_OK : BLDFM_ERR_CUDA;
}

extern "C" int bldfm_vertical_profiles_batch(int32_t ncases, const bldfm_profile_params *params, int32_t *nz_out,
                                             int64_t *zoff_out, size_t *ws_bytes_out, double *z_dev,
                                             double *prof_dev, void *ws_dev, size_t ws_bytes, void *stream)
{
    return bldfm_guarded([&]() -> int {
        if (ncases < 1 || !params || !nz_out || !zoff_out) return BLDFM_ERR_ARG;
        std::vector<ProfileCase> pcs((size_t)ncases);
        std::vector<int64_t> zoff((size_t)ncases);
        int64_t total = 0;
        for (int k = 0; k < ncases; ++k) {
            const bldfm_profile_params &a = params[k];
            const int rc = profile_scalars(a.n, a.meas_height, a.um, a.vm, a.ustar, a.z0, a.mol, a.prsc, a.closure,
                                           a.domain_height, a.stretch, a.tke, &pcs[(size_t)k]);
            if (rc != BLDFM_OK) return rc;
            nz_out[k] = pcs[(size_t)k].nz;
            zoff[(size_t)k] = zoff_out[k] = total;
            total += pcs[(size_t)k].nz;
        }
        const size_t table = ((sizeof(ProfileCase) * (size_t)ncases + 255) & ~(size_t)255);
        const size_t need = table + sizeof(int64_t) * (size_t)ncases;
        if (ws_bytes_out) *ws_bytes_out = need;
        if (!z_dev) return BLDFM_OK;
        if (!prof_dev || !ws_dev || ws_bytes < need || ((uintptr_t)ws_dev & 15)) return BLDFM_ERR_ARG;
        cudaStream_t st = (cudaStream_t)stream;
        char *w = (char *)ws_dev;
        // pageable sources: the copies have read them when the calls return
        if (cudaMemcpyAsync(w, pcs.data(), sizeof(ProfileCase) * (size_t)ncases, cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaMemcpyAsync(w + table, zoff.data(), sizeof(int64_t) * (size_t)ncases, cudaMemcpyHostToDevice, st) !=
                cudaSuccess)
            return BLDFM_ERR_CUDA;
        if (launch_profiles_batch((const ProfileCase *)w, (const int64_t *)(w + table), ncases, z_dev, prof_dev, st) !=
            cudaSuccess)
            return BLDFM_ERR_CUDA;
        return BLDFM_OK;
    });
}
