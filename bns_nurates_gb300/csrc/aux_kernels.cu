// Small per-point kernels: distribution parameters from M1 moments and the
// equilibrium distribution with its M1 densities.  One thread per point;
// both are memory/latency bound and cheap next to the opacity kernels.

#include <cuda_runtime.h>

#include "bnsn_fp64.cuh"
#include "bnsn_internal.h"

namespace bnsn {
namespace {

using namespace fp64;

// CalculateDistrParamsFromM1 (distribution.hpp:323-333) per point.
__global__ void distr_from_m1_kernel(const __grid_constant__ DistrLaunch L)
{
    const int64_t npts = L.npts;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npts;
         p += (int64_t)gridDim.x * blockDim.x)
    {
#pragma unroll 1
        for (int s = 0; s < 4; ++s)
        {
            double v[7];
            distr_species(L.m1[s][p], L.m1[4 + s][p], L.m1[8 + s][p], L.gamma36, &v[0],
                          &v[1], &v[2], &v[3], &v[4], &v[5], &v[6]);
#pragma unroll
            for (int q = 0; q < 7; ++q)
                L.out[q * 4 + s][p] = v[q];
        }
    }
}

// NuEquilibriumParams + ComputeM1DensitiesEq (distribution.hpp:253-290,
// 447-473), chi = 1/3 as in tests/tests.hpp:328-331.
__global__ void nu_equilibrium_kernel(const __grid_constant__ EquilLaunch L)
{
    const int64_t npts = L.npts;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npts;
         p += (int64_t)gridDim.x * blockDim.x)
    {
        const double T    = L.eos[1][p];
        const double mu_p = L.eos[5][p], mu_n = L.eos[6][p], mu_e = L.eos[7][p];
        double eta[4];
        eta[0] = (mu_e - mu_n + mu_p) / T;
        eta[1] = -eta[0];
        eta[2] = 0.;
        eta[3] = 0.;
        const double npre = k::FourPiHc3 * (T * T * T);
        const double jpre = npre * T;
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            L.distr[0 + s][p]  = 1.;
            L.distr[4 + s][p]  = T;
            L.distr[8 + s][p]  = eta[s];
            L.distr[12 + s][p] = 0.;
            L.distr[16 + s][p] = T;
            L.distr[20 + s][p] = k::CF;
            L.distr[24 + s][p] = 1.;
            double f[2];
            fdi_orders<2, 3>(eta[s], f);
            L.m1[0 + s][p] = npre * f[0];
            L.m1[4 + s][p] = jpre * f[1];
            L.m1[8 + s][p] = 1. / 3.;
        }
    }
}

int grid_for(int64_t npts, int threads, int num_sms)
{
    const int64_t need = (npts + threads - 1) / threads;
    const int64_t cap  = (int64_t)num_sms * 16;
    return (int)(need < cap ? need : cap);
}

} // namespace

cudaError_t launch_distr_from_m1(const DistrLaunch& L, cudaStream_t stream, int num_sms)
{
    if (L.npts <= 0)
        return cudaSuccess;
    phase_mark(kPhAux, 0, stream);
    distr_from_m1_kernel<<<grid_for(L.npts, 128, num_sms), 128, 0, stream>>>(L);
    phase_mark(kPhAux, 1, stream);
    return cudaGetLastError();
}

cudaError_t launch_nu_equilibrium(const EquilLaunch& L, cudaStream_t stream, int num_sms)
{
    if (L.npts <= 0)
        return cudaSuccess;
    phase_mark(kPhAux, 0, stream);
    nu_equilibrium_kernel<<<grid_for(L.npts, 128, num_sms), 128, 0, stream>>>(L);
    phase_mark(kPhAux, 1, stream);
    return cudaGetLastError();
}

} // namespace bnsn
