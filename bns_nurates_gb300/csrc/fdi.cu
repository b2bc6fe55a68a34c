// Batched Fermi-Dirac integrals of the reference's family (functions.hpp:442-4375):
// F_j(x) = integral_0^inf t^j / (exp(t - x) + 1) dt without the 1 / Gamma(j + 1)
// normalisation, j = k2 / 2 for k2 = -9, -7, -5, -3, -1 (FDI_m92 .. FDI_m12,
// continued below j = -1 by dF_{j+1}/dx = (j + 1) F_j) and k2 = 0 .. 21
// (FDI_0, FDI_p12, FDI_p1, ..., FDI_p10, FDI_p212).
//
// Integer orders 0..5 run the restatement of the reference's rational
// approximations (fdi_orders).  Every other order reads the tables of
// bnsn_fdi_tab.h (made by fdi_tables.py from mpmath): an alternating series
// in e^x below x = -4, one Chebyshev expansion per interval of [-4, 100) and
// the Sommerfeld expansion above.  The tables agree with the reference's
// approximations to a few 1e-16 (relative, away from the zeros of the
// negative orders).
//
// Non-finite arguments follow the reference: NaN gives NaN for the
// half-integer orders and 0 for the integer ones; -inf gives 0; +inf gives
// +inf for j > -1 and -0 or +0 (the sign of x^(j+1) / (j+1)) below.
//
// One thread per argument, grid-stride, the order's coefficients staged in
// shared memory per CTA; FP64-pipe bound (about 60 FP64 operations per
// argument against 16 bytes of traffic).

#include <cuda_runtime.h>

#include "bnsn_fdi_tab.h"
#include "bnsn_fp64.cuh"
#include "bnsn_internal.h"

namespace bnsn {
namespace {

using namespace fp64;

// Table slot of a twice-order (kTwice[slot] == k2), -1 when not tabulated.
constexpr int slot_of(int k2)
{
    for (int s = 0; s < fdit::kNumOrders; ++s)
        if (fdit::kTwice[s] == k2)
            return s;
    return -1;
}

// One order's coefficients staged in shared memory; the Chebyshev table is
// transposed to [term][interval] so that the lanes of a warp, which read the
// same term of different intervals, hit consecutive words.
struct FdiShared
{
    double series[fdit::kSeriesTerms];
    double cheb[fdit::kChebTerms][fdit::kPieces];
    double asym[fdit::kAsymTerms];
};

// x^(h/2) for x >= 100 (or +inf) and |h| <= 23: an integer power by repeated
// squaring, times sqrt(x) for odd h, inverted for negative h (far cheaper
// than pow, within a few ulp).
__device__ __forceinline__ double pow_half(double x, int h)
{
    const int a = h < 0 ? -h : h;
    int q       = a >> 1;
    double v = 1., b = x;
    while (q)
    {
        if (q & 1)
            v *= b;
        q >>= 1;
        if (q)
            b *= b;
    }
    if (a & 1)
        v *= sqrt(x);
    return h < 0 ? 1. / v : v;
}

__device__ __forceinline__ double fdi_table(const FdiShared& S, int h, bool integer, double x)
{
    const double j1 = 0.5 * h; // j + 1
    using namespace fdit;
    if (x < kXlo)
    {
        // sum_n (-1)^(n+1) c_n e^(n x) = e^x sum_m c_(m+1) (-e^x)^m
        const double e = exp(x);
        const double z = -e;
        double p       = S.series[kSeriesTerms - 1];
#pragma unroll
        for (int n = kSeriesTerms - 2; n >= 0; --n)
            p = fma(p, z, S.series[n]);
        return e * p;
    }
    if (x < kXhi)
    {
        int i;
        double cen, sc;
        if (x < kXmid)
        {
            i   = (int)floor((x - kXlo) * (1. / kWidth));
            i   = i < 0 ? 0 : (i > kNarrow - 1 ? kNarrow - 1 : i);
            cen = kXlo + kWidth * i + 0.5 * kWidth;
            sc  = 2. / kWidth;
        }
        else
        {
            int k = (int)floor((x - kXmid) * (1. / kWide));
            k     = k < 0 ? 0 : (k > kPieces - kNarrow - 1 ? kPieces - kNarrow - 1 : k);
            i     = kNarrow + k;
            cen   = kXmid + kWide * k + 0.5 * kWide;
            sc    = 2. / kWide;
        }
        const double t  = (x - cen) * sc;
        const double t2 = 2. * t;
        // Clenshaw recurrence for sum_m c_m T_m(t) (c_0 stored halved)
        double b1 = 0., b2 = 0.;
#pragma unroll
        for (int m = kChebTerms - 1; m >= 1; --m)
        {
            const double b0 = fma(t2, b1, S.cheb[m][i] - b2);
            b2              = b1;
            b1              = b0;
        }
        return fma(t, b1, S.cheb[0][i] - b2);
    }
    if (x != x) // NaN fails both regime tests above
        return integer ? 0. : x;
    // x^(j+1) / (j+1) (1 + sum_k a_k x^(-2k))
    const double u = 1. / (x * x);
    double s       = S.asym[kAsymTerms - 1];
#pragma unroll
    for (int k = kAsymTerms - 2; k >= 0; --k)
        s = fma(s, u, S.asym[k]);
    s = fma(s, u, 1.);
    return pow_half(x, h) / j1 * s;
}

template <int K>
__global__ void fdi_int_kernel(const double* __restrict__ x, double* __restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = fdi<K>(x[i]);
}

__global__ void fdi_table_kernel(int slot, int h, int integer, const double* __restrict__ x,
                                 double* __restrict__ out, int64_t n)
{
    using namespace fdit;
    __shared__ FdiShared S;
    for (int k = threadIdx.x; k < kSeriesTerms; k += blockDim.x)
        S.series[k] = kSeries[slot][k];
    for (int k = threadIdx.x; k < kPieces * kChebTerms; k += blockDim.x)
    {
        const int i = k / kChebTerms, m = k - i * kChebTerms;
        S.cheb[m][i] = kCheb[slot][i][m];
    }
    for (int k = threadIdx.x; k < kAsymTerms; k += blockDim.x)
        S.asym[k] = kAsym[slot][k];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = fdi_table(S, h, integer != 0, x[i]);
}

} // namespace

// Twice-orders the family defines: -9, -7, -5, -3, -1 and 0 .. 21.
bool fdi_order_valid(int k2) { return (k2 >= 0 && k2 <= 21) || (k2 < 0 && k2 >= -9 && (k2 & 1)); }

cudaError_t launch_fdi(int k2, const double* x, double* out, int64_t n, cudaStream_t stream,
                       int num_sms)
{
    if (n <= 0)
        return cudaSuccess;
    constexpr int threads = 256;
    const int64_t need    = (n + threads - 1) / threads;
    const int64_t cap     = (int64_t)num_sms * 8;
    const int grid        = (int)(need < cap ? need : cap);
    const int slot        = slot_of(k2);
    if (slot < 0 && !(k2 >= 0 && k2 <= 10 && (k2 & 1) == 0))
        return cudaErrorInvalidValue;
    phase_mark(kPhAux, 0, stream);
    switch (k2)
    {
    case 0: fdi_int_kernel<0><<<grid, threads, 0, stream>>>(x, out, n); break;
    case 2: fdi_int_kernel<1><<<grid, threads, 0, stream>>>(x, out, n); break;
    case 4: fdi_int_kernel<2><<<grid, threads, 0, stream>>>(x, out, n); break;
    case 6: fdi_int_kernel<3><<<grid, threads, 0, stream>>>(x, out, n); break;
    case 8: fdi_int_kernel<4><<<grid, threads, 0, stream>>>(x, out, n); break;
    case 10: fdi_int_kernel<5><<<grid, threads, 0, stream>>>(x, out, n); break;
    default:
        fdi_table_kernel<<<grid, threads, 0, stream>>>(slot, k2 + 2, (k2 & 1) == 0, x, out, n);
    }
    phase_mark(kPhAux, 1, stream);
    return cudaGetLastError();
}

} // namespace bnsn
