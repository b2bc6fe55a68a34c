// Grey opacities on a host code's own grid: boxes of 3-D arrays, one device
// array per field, with ghost zones (the layout of a THC / Cactus grid-function
// component, where the reference's exported headers are called point by point
// inside the host code's loops; utils/export_thc.py of the reference exports
// them for the Weakrates2 thorn).
//
// The interiors of all boxes are gathered into one point batch (coalesced:
// consecutive points are consecutive x), evaluated by the batched entry point
// and scattered back into the boxes' output arrays; cells outside the
// interiors are not touched.  Optional per-field factors convert units on the
// way in and out (the host code's units to MeV / nm^-3 and back).

#include <cuda_runtime.h>

#include "../../include/bns_nurates_gb300.h"
#include "bnsn_internal.h"

using namespace bnsn;

namespace {

constexpr int kBoxBatch = 32;  // boxes per gather / scatter launch (kernel parameters)
constexpr int kIn       = 23;  // 11 eos + 12 m1 fields
constexpr int kOut      = 20;

struct BoxDims
{
    int nb;                        // boxes in this launch
    int64_t first[kBoxBatch + 1];  // first point of each box in the launch's batch
    int64_t nx[kBoxBatch], ny[kBoxBatch];
    int64_t s1[kBoxBatch], s2[kBoxBatch]; // strides of y and z (x is contiguous)
    int64_t base[kBoxBatch];             // linear index of the interior's first cell
};

struct GatherArgs
{
    BoxDims D;
    const double* in[kBoxBatch][kIn];
    double scale[kIn];
    int use_scale;
};

struct ScatterArgs
{
    BoxDims D;
    double* out[kBoxBatch][kOut];
    double scale[kOut];
    int use_scale;
};

__device__ __forceinline__ int64_t cell_of(const BoxDims& D, int64_t q, int* box)
{
    int b = 0;
    while (b + 1 < D.nb && q >= D.first[b + 1])
        ++b;
    const int64_t r = q - D.first[b];
    const int64_t i = r % D.nx[b], jk = r / D.nx[b];
    const int64_t j = jk % D.ny[b], k = jk / D.ny[b];
    *box = b;
    return D.base[b] + k * D.s2[b] + j * D.s1[b] + i;
}

// staging[f * npts + off + q] = in[box][f][cell] (x scale[f])
__global__ void __launch_bounds__(256)
    box_gather_kernel(const __grid_constant__ GatherArgs A, double* __restrict__ staging,
                      int64_t npts, int64_t off)
{
    const int64_t n = A.D.first[A.D.nb];
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x)
    {
        int b;
        const int64_t c = cell_of(A.D, q, &b);
#pragma unroll 1
        for (int f = 0; f < kIn; ++f)
        {
            const double* src = A.in[b][f];
            const double v    = src ? src[c] : 0.; // mu_mu may be absent
            staging[f * npts + off + q] = A.use_scale ? v * A.scale[f] : v;
        }
    }
}

__global__ void __launch_bounds__(256)
    box_scatter_kernel(const __grid_constant__ ScatterArgs A, const double* __restrict__ staging,
                       int64_t npts, int64_t off)
{
    const int64_t n = A.D.first[A.D.nb];
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x)
    {
        int b;
        const int64_t c = cell_of(A.D, q, &b);
#pragma unroll 1
        for (int f = 0; f < kOut; ++f)
        {
            const double v = staging[f * npts + off + q];
            A.out[b][f][c] = A.use_scale ? v * A.scale[f] : v;
        }
    }
}

int64_t interior(const bnsn_grid_box& B)
{
    return (B.hi[0] - B.lo[0]) * (B.hi[1] - B.lo[1]) * (B.hi[2] - B.lo[2]);
}

int check_box(const bnsn_grid_box& B)
{
    for (int d = 0; d < 3; ++d)
        if (B.shape[d] < 1 || B.lo[d] < 0 || B.lo[d] > B.hi[d] || B.hi[d] > B.shape[d])
            return capi_fail(BNSN_ERR_ARG, "box extents: need 0 <= lo <= hi <= shape");
    if (interior(B) == 0)
        return BNSN_OK;
    for (int f = 0; f < 11; ++f)
        if (!B.eos[f] && f != 8)
            return capi_fail(BNSN_ERR_ARG, "a box eos field pointer is NULL");
    for (int f = 0; f < 12; ++f)
        if (!B.m1[f])
            return capi_fail(BNSN_ERR_ARG, "a box m1 field pointer is NULL");
    for (int f = 0; f < kOut; ++f)
        if (!B.out[f])
            return capi_fail(BNSN_ERR_ARG, "a box output pointer is NULL");
    return BNSN_OK;
}

// The launches' box dimensions for boxes [b0, b0 + nb) with first point off.
void dims_of(const bnsn_grid_box* boxes, int b0, int nb, BoxDims* D)
{
    D->nb       = nb;
    D->first[0] = 0;
    for (int b = 0; b < nb; ++b)
    {
        const bnsn_grid_box& B = boxes[b0 + b];
        D->nx[b]       = B.hi[0] - B.lo[0];
        D->ny[b]       = B.hi[1] - B.lo[1];
        D->s1[b]       = B.shape[0];
        D->s2[b]       = B.shape[0] * B.shape[1];
        D->base[b]     = B.lo[2] * D->s2[b] + B.lo[1] * D->s1[b] + B.lo[0];
        D->first[b + 1] = D->first[b] + interior(B);
    }
}

} // namespace

extern "C" int bnsn_m1_opacities_grid_boxes(const MyQuadrature* quad_1d,
                                            const MyQuadrature* quad_2d,
                                            const OpacityFlags* flags,
                                            const OpacityParams* params,
                                            const bnsn_grid_box* boxes, int nboxes,
                                            const double* in_scale, const double* out_scale,
                                            int stim_abs, int precision, void* stream)
{
    if (nboxes < 0 || (nboxes > 0 && !boxes))
        return capi_fail(BNSN_ERR_ARG, "boxes is NULL or nboxes < 0");
    int64_t npts = 0;
    for (int b = 0; b < nboxes; ++b)
    {
        int rc = check_box(boxes[b]);
        if (rc)
            return rc;
        npts += interior(boxes[b]);
    }
    if (precision != BNSN_FP64 && precision != BNSN_MIXED)
        return capi_fail(BNSN_ERR_ARG, "unknown precision");
    if (npts == 0)
        return BNSN_OK;
    DeviceInfo info;
    int rc = capi_device_info(&info);
    if (rc)
        return rc;
    const cudaStream_t st = (cudaStream_t)stream;
    double* stg = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&stg, sizeof(double) * (kIn + kOut) * npts, st);
    if (e != cudaSuccess)
        return capi_cuda_fail(e, "grid-box staging allocation");
    const int grid = info.num_sms * 8;
    GatherArgs G;
    G.use_scale = in_scale != nullptr;
    for (int f = 0; f < kIn; ++f)
        G.scale[f] = in_scale ? in_scale[f] : 1.;
    int64_t off = 0;
    for (int b0 = 0; b0 < nboxes && e == cudaSuccess; b0 += kBoxBatch)
    {
        const int nb = nboxes - b0 < kBoxBatch ? nboxes - b0 : kBoxBatch;
        dims_of(boxes, b0, nb, &G.D);
        for (int b = 0; b < nb; ++b)
        {
            for (int f = 0; f < 11; ++f)
                G.in[b][f] = boxes[b0 + b].eos[f];
            for (int f = 0; f < 12; ++f)
                G.in[b][11 + f] = boxes[b0 + b].m1[f];
        }
        if (G.D.first[nb] > 0)
            box_gather_kernel<<<grid, 256, 0, st>>>(G, stg, npts, off);
        off += G.D.first[nb];
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
    {
        const double* in  = stg;
        double* o         = stg + kIn * npts;
        bnsn_eos_soa eos  = {in,            in + npts,     in + 2 * npts, in + 3 * npts,
                             in + 4 * npts, in + 5 * npts, in + 6 * npts, in + 7 * npts,
                             in + 8 * npts, in + 9 * npts, in + 10 * npts};
        bnsn_m1_soa m1;
        bnsn_m1_opacities_soa out;
        for (int s = 0; s < 4; ++s)
        {
            m1.n[s]           = in + (11 + s) * npts;
            m1.J[s]           = in + (15 + s) * npts;
            m1.chi[s]         = in + (19 + s) * npts;
            out.eta_0[s]      = o + s * npts;
            out.kappa_0_a[s]  = o + (4 + s) * npts;
            out.eta[s]        = o + (8 + s) * npts;
            out.kappa_a[s]    = o + (12 + s) * npts;
            out.kappa_s[s]    = o + (16 + s) * npts;
        }
        rc = bnsn_m1_opacities(quad_1d, quad_2d, flags, params, &eos, &m1, nullptr, stim_abs,
                               precision, &out, npts, stream);
        if (rc == BNSN_OK)
        {
            ScatterArgs S;
            S.use_scale = out_scale != nullptr;
            for (int f = 0; f < kOut; ++f)
                S.scale[f] = out_scale ? out_scale[f] : 1.;
            off = 0;
            for (int b0 = 0; b0 < nboxes && e == cudaSuccess; b0 += kBoxBatch)
            {
                const int nb = nboxes - b0 < kBoxBatch ? nboxes - b0 : kBoxBatch;
                dims_of(boxes, b0, nb, &S.D);
                for (int b = 0; b < nb; ++b)
                    for (int f = 0; f < kOut; ++f)
                        S.out[b][f] = boxes[b0 + b].out[f];
                if (S.D.first[nb] > 0)
                    box_scatter_kernel<<<grid, 256, 0, st>>>(S, o, npts, off);
                off += S.D.first[nb];
                e = cudaGetLastError();
            }
        }
    }
    const cudaError_t ef = cudaFreeAsync(stg, st);
    if (rc)
        return rc;
    if (e != cudaSuccess)
        return capi_cuda_fail(e, "grid-box gather/scatter");
    return ef == cudaSuccess ? BNSN_OK : capi_cuda_fail(ef, "grid-box staging release");
}
