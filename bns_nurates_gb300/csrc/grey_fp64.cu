// FP64 grey M1 opacity kernel (sm_103a).
//
// One warp computes one thermodynamic point; warps stride over the points of
// a persistent grid.  Within a point the 32 lanes split
//   * the 2n energies of the pair/brem grid (distribution values and the
//     Fermi integrals F_k(eta +- w/T) staged in shared memory),
//   * the M(M+1)/2 unordered (w, w') cells of the pair + brem double integral
//     (one kernel evaluation fills both (w, w') and (w', w)),
//   * the 2 n^2 (nu, nubar) pairs of the NES/NPS double integral (one pair of
//     Fermi-integral sets serves both directions and all four species),
//   * the nodes of the 1-D beta and iso-scattering integrals,
// and accumulate the quadrature sums directly; the reference's 2n x 2n
// integrand matrices (m1_opacities.hpp:774-1057) are never materialised.
// Sums are reduced with warp shuffles and lanes 0..19 write the 20 outputs.
//
// Restates ComputeM1OpacitiesGenericFormalism (m1_opacities.hpp:1062-1295)
// with the integration rules of integration.hpp:608-844.

#include <cuda_runtime.h>

#include "bnsn_fp64.cuh"
#include "bnsn_internal.h"

namespace bnsn {
namespace {

using namespace fp64;

constexpr int kWarps = 4; // warps per CTA

// Per-warp staging area in shared memory.
struct WarpScratch
{
    Distr d;
    double nu[kMaxM];
    double y[kMaxM];
    double g[kMaxM][4];
    double fm[kMaxM][5]; // F_1..F_5 at eta - nu/T
    double fp[kMaxM][5]; // F_1..F_5 at eta + nu/T
    double fe[2][6];     // F_0..F_5 at eta_e and -eta_e
    double fd0[2];       // FermiDistr(0, 1, +-eta_e)
    Hr98Point hr;
    double brt06_pre;
    double eta_pp, eta_nn;
    double tot[44];
    int same_cf;
};

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double total_nu_f1(double omega, const Distr& d, int s)
{
    const double ft = fermi_distr(omega, d.temp_t[s], d.temp_t[s] * d.eta_t[s]);
    const double fn = d.beta_f[s] * pow(omega, d.c_f[s]) * exp(-omega / d.temp_f[s]);
    return d.w_t[s] * ft + d.w_f[s] * fn;
}

__global__ void __launch_bounds__(kWarps * 32)
    grey_fp64_kernel(const __grid_constant__ OpacityLaunch L)
{
    __shared__ double s_A1[kMaxM], s_A2[kMaxM], s_B1[kMaxM];
    __shared__ double s_x1[kMaxQ], s_x2[kMaxQ], s_w2[kMaxQ], s_wx[kMaxQ], s_wx3[kMaxQ];
    __shared__ uint32_t s_cells[kMaxCells];
    __shared__ WarpScratch s_ws[kWarps];

    for (int k = threadIdx.x; k < kMaxM; k += blockDim.x)
    {
        s_A1[k] = L.A1[k];
        s_A2[k] = L.A2[k];
        s_B1[k] = L.B1[k];
    }
    for (int k = threadIdx.x; k < kMaxQ; k += blockDim.x)
    {
        s_x1[k]  = L.x1[k];
        s_x2[k]  = L.x2[k];
        s_w2[k]  = L.w2[k];
        s_wx[k]  = L.wx[k];
        s_wx3[k] = L.wx3[k];
    }
    for (int k = threadIdx.x; k < L.ncell; k += blockDim.x)
        s_cells[k] = L.cells[k];
    __syncthreads();

    const int lane      = threadIdx.x & 31;
    WarpScratch& W      = s_ws[threadIdx.x >> 5];
    const int64_t nwarp = (int64_t)gridDim.x * kWarps;
    const int n1 = L.n1, n2 = L.n2, M = 2 * n2;
    const bool nb_block = L.neglect_blocking != 0;

    for (int64_t p = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5); p < L.npts; p += nwarp)
    {
        // ---------------- point inputs (broadcast loads) -----------------
        const double nb = L.eos[0][p], T = L.eos[1][p], ye = L.eos[2][p];
        const double yp = L.eos[3][p], yn = L.eos[4][p];
        const double mu_p = L.eos[5][p], mu_n = L.eos[6][p], mu_e = L.eos[7][p];
        const double dU = L.eos[9][p], dm_eff = L.eos[10][p];
        double n[4], J[4];
#pragma unroll
        for (int s = 0; s < 4; ++s)
        {
            n[s] = L.m1[s][p];
            J[s] = L.m1[4 + s][p];
        }
        const double eta_e = mu_e / T;

        // ------------- per-point constants, spread over lanes ------------
        if (L.has_distr)
        {
            if (lane < 28)
                (&W.d.w_t[0])[lane] = L.distr[lane][p];
        }
        else if (lane < 4)
        {
            const int s = lane;
            distr_species(n[s], J[s], L.m1[8 + s][p], L.gamma36, &W.d.w_t[s],
                          &W.d.temp_t[s], &W.d.eta_t[s], &W.d.w_f[s], &W.d.temp_f[s],
                          &W.d.c_f[s], &W.d.beta_f[s]);
        }
        if (lane == 4 || lane == 5)
        {
            const int e     = lane - 4;
            const double et = e ? -mu_e / T : eta_e;
            fdi_orders<0, 5>(et, W.fe[e]);
            W.fd0[e] = fermi_distr(0., 1., et);
        }
        if (L.use_brem && L.brem_impl == 0)
        {
            if (lane >= 6 && lane < 9)
                W.hr.ch[lane - 6] = hr98_channel(nb, yn, yp, T, lane - 6);
            if (lane == 9)
                hr98_point_common(nb, T, L.use_medium != 0, &W.hr);
        }
        if (lane == 10 && L.use_brem && L.brem_impl == 1)
            W.brt06_pre = brt06_point(nb, T, yn, yp);
        if (lane == 11 && L.use_iso)
        {
            W.eta_pp = eta_nn_sc(nb, T, yp);
            W.eta_nn = eta_nn_sc(nb, T, yn);
        }
        __syncwarp();
        if (lane == 0)
        {
            const double c0 = W.d.c_f[0];
            W.same_cf = (W.d.c_f[1] == c0) && (W.d.c_f[2] == c0) && (W.d.c_f[3] == c0);
        }
        __syncwarp();
        const bool same_cf = W.same_cf != 0;

        // ---------------- pair + bremsstrahlung double integral ----------
        const double t2d = k::TempMultiple * T;
        if (L.use_pair || L.use_brem)
        {
            for (int a = lane; a < M; a += 32)
            {
                const int i     = a < n2 ? a : a - n2;
                const double nu = a < n2 ? t2d * s_x2[i] : t2d / s_x2[i];
                W.nu[a]         = nu;
                W.y[a]          = nu / T;
                total_nu_f4(nu, W.d, same_cf, W.g[a]);
            }
            if (L.use_pair)
            {
                for (int q = lane; q < 2 * M; q += 32)
                {
                    const int a     = q >> 1;
                    const int i     = a < n2 ? a : a - n2;
                    const double nu = a < n2 ? t2d * s_x2[i] : t2d / s_x2[i];
                    const double y  = nu / T;
                    if (q & 1)
                        fdi_orders<1, 5>(eta_e + y, W.fp[a]);
                    else
                        fdi_orders<1, 5>(eta_e - y, W.fm[a]);
                }
            }
            __syncwarp();
            double acc[16];
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                acc[kk] = 0.;
            const double f3e = W.fe[0][3], f4e = W.fe[0][4];
            for (int c = lane; c < L.ncell; c += 32)
            {
                const uint32_t ab = s_cells[c];
                const int a = ab & 0xffffu, b = ab >> 16;
                const double nua = W.nu[a], nub = W.nu[b];
                double pe[4] = {0., 0., 0., 0.}, pa[4] = {0., 0., 0., 0.};
                double be = 0., ba = 0.;
                if (L.use_pair)
                    pair_kernel(T, eta_e, nua, nub, W.y[a], W.y[b], W.fm[a], W.fp[a],
                                W.fm[b], W.fp[b], f3e, f4e, pe, pa);
                if (L.use_brem)
                {
                    if (L.brem_impl == 0)
                        hr98_kernel(W.hr, nua, nub, &be, &ba);
                    else if (L.brem_impl == 1)
                        brt06_kernel(W.brt06_pre, T, nua, nub, &be, &ba);
                    else
                    {
                        const Gp19Table G = {L.gp19.d0,   L.gp19.d1,    L.gp19.d2,
                                             L.gp19.d3,   L.gp19.nb,    L.gp19.ye,
                                             L.gp19.t,    L.gp19.w,     L.gp19.lognb,
                                             L.gp19.logw, L.gp19.data};
                        gp19_kernel(G, nb, ye, T, nua, nub, &be, &ba);
                    }
                }
                const double* ga = W.g[a];
                const double* gb = W.g[b];
                const double w4  = (nua * nua) * (nub * nub);
                const double W1  = s_A1[a] * s_A1[b];
                const double W2  = s_A2[a] * s_A1[b];
#pragma unroll
                for (int s = 0; s < 4; ++s)
                {
                    const int ps  = s ^ 1;
                    const double em = (pe[s] + be) * (nb_block ? 1. : 1. - gb[ps]);
                    const double am = (pa[s] + ba) * gb[ps];
                    double EM, AB;
                    if (L.stim)
                    {
                        AB = w4 * ga[s] * (em + am);
                        EM = em * w4;
                    }
                    else
                    {
                        AB = am * (w4 * ga[s]);
                        EM = em * (w4 * (1. - ga[s]));
                    }
                    acc[s] += EM * W1;
                    acc[4 + s] += AB * W1;
                    acc[8 + s] += EM * W2;
                    acc[12 + s] += AB * W2;
                }
                if (a != b)
                {
                    const double W2b = s_A2[b] * s_A1[a];
#pragma unroll
                    for (int s = 0; s < 4; ++s)
                    {
                        const int ps  = s ^ 1;
                        const double em = (pe[ps] + be) * (nb_block ? 1. : 1. - ga[ps]);
                        const double am = (pa[ps] + ba) * ga[ps];
                        double EM, AB;
                        if (L.stim)
                        {
                            AB = w4 * gb[s] * (em + am);
                            EM = em * w4;
                        }
                        else
                        {
                            AB = am * (w4 * gb[s]);
                            EM = em * (w4 * (1. - gb[s]));
                        }
                        acc[s] += EM * W1;
                        acc[4 + s] += AB * W1;
                        acc[8 + s] += EM * W2b;
                        acc[12 + s] += AB * W2b;
                    }
                }
            }
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                acc[kk] = warp_sum(acc[kk]);
            if (lane == 0)
            {
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    W.tot[kk] = acc[kk];
            }
        }

        // ---------------- NES / NPS double integral ----------------------
        if (L.use_inel)
        {
            NepsPoint P;
            P.T     = T;
            P.pre   = k::NepsConst * (T * T);
            P.eta0  = eta_e;
            P.eta1  = -mu_e / T;
            P.fd00  = W.fd0[0];
            P.fd01  = W.fd0[1];
            P.fe0   = W.fe[0];
            P.fe1   = W.fe[1];
            const double tn = 4. * (k::TempMultiple * T);
            double acc[16];
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                acc[kk] = 0.;
            const int nn2 = n2 * n2;
            for (int it = lane; it < 2 * nn2; it += 32)
            {
                const int r = it >= nn2;
                const int rem = it - r * nn2;
                const int i = rem / n2, j = rem - (rem / n2) * n2;
                const double xi = s_x2[i], xj = s_x2[j];
                double nu, nub;
                if (!r)
                {
                    nu  = 0.5 * tn * xi * (1. - xj);
                    nub = 0.5 * tn * xi * (1. + xj);
                }
                else
                {
                    nu  = 0.5 * tn * (1. - xj) / xi;
                    nub = 0.5 * tn * (1. + xj) / xi;
                }
                const double w4 = (nu * nu) * (nub * nub);
                double g[4], gb[4];
                total_nu_f4(nu, W.d, same_cf, g);
                total_nu_f4(nub, W.d, same_cf, gb);
                double em1[4], ab1[4], em2[4], ab2[4];
                neps_pair(P, nu, nub, em1, ab1, em2, ab2);
                const double Wr = (r ? s_wx3[i] : s_wx[i]) * s_w2[j];
#pragma unroll
                for (int s = 0; s < 4; ++s)
                {
                    const double e1 = em1[s] * gb[s];
                    const double a1 = ab1[s] * (nb_block ? 1. : 1. - gb[s]);
                    const double e2 = em2[s] * g[s];
                    const double a2 = ab2[s] * (nb_block ? 1. : 1. - g[s]);
                    double EM1, AB1, EM2, AB2;
                    if (L.stim)
                    {
                        AB1 = w4 * g[s] * (e1 + a1);
                        EM1 = w4 * e1;
                        AB2 = w4 * gb[s] * (e2 + a2);
                        EM2 = w4 * e2;
                    }
                    else
                    {
                        AB1 = w4 * g[s] * a1;
                        EM1 = w4 * (1. - g[s]) * e1;
                        AB2 = w4 * gb[s] * a2;
                        EM2 = w4 * (1. - gb[s]) * e2;
                    }
                    acc[s] += Wr * (EM1 + EM2);
                    acc[4 + s] += Wr * (AB1 + AB2);
                    acc[8 + s] += Wr * (nu * EM1 + nub * EM2);
                    acc[12 + s] += Wr * (nu * AB1 + nub * AB2);
                }
            }
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
                acc[kk] = warp_sum(acc[kk]);
            if (lane == 0)
            {
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                    W.tot[16 + kk] = acc[kk];
            }
        }

        // ---------------- beta processes (1-D) ---------------------------
        double s_beta[2] = {0., 0.};
        if (eta_e > -30. && eta_e < 30.)
        {
            s_beta[0] = T * W.fe[0][5] / W.fe[0][4];
            s_beta[1] = T * W.fe[1][5] / W.fe[1][4];
        }
        else if (eta_e > 30.)
        {
            s_beta[0] = T * eta_e * 0.8333333333333333;
            s_beta[1] = T * 5.;
        }
        else
        {
            s_beta[0] = T * 5.;
            s_beta[1] = T * eta_e * 0.8333333333333333;
        }
        if (L.use_abs_em)
        {
            const BetaPoint bp = beta_point(nb, T, yp, yn, mu_p, mu_n, mu_e, dU, dm_eff,
                                            L.use_dU, L.use_dm_eff, L.use_WM_ab,
                                            L.use_decay);
            double acc[8];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                acc[kk] = 0.;
            const int m1n = 2 * n1;
            for (int it = lane; it < 2 * m1n; it += 32)
            {
                const int s = it >= m1n;
                const int a = it - s * m1n;
                const int i = a < n1 ? a : a - n1;
                const double t  = s_beta[s];
                const double nu = a < n1 ? t * s_x1[i] : t / s_x1[i];
                const double g  = total_nu_f1(nu, W.d, s);
                double ab, em;
                beta_rates(bp, nu, s, &ab, &em);
                if (L.stim)
                    ab = ab + em;
                const double nu2 = nu * nu;
                const double ev  = nu2 * em;
                const double av  = nu2 * g * ab;
                const double wn  = s_B1[a];
                const double wj  = wn * nu;
                if (s == 0)
                {
                    acc[0] += wn * ev;
                    acc[2] += wj * ev;
                    acc[4] += wn * av;
                    acc[6] += wj * av;
                }
                else
                {
                    acc[1] += wn * ev;
                    acc[3] += wj * ev;
                    acc[5] += wn * av;
                    acc[7] += wj * av;
                }
            }
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                acc[kk] = warp_sum(acc[kk]);
            if (lane == 0)
            {
#pragma unroll
                for (int kk = 0; kk < 8; ++kk)
                    W.tot[32 + kk] = acc[kk];
            }
        }

        // ---------------- iso-energetic scattering (1-D) -----------------
        double s_iso[4];
#pragma unroll
        for (int s = 0; s < 4; ++s)
            s_iso[s] = (n[s] > k::ThresholdN) ? (J[s] / n[s]) : 1.5 * T;
        if (L.use_iso)
        {
            double acc[4] = {0., 0., 0., 0.};
            const int m1n = 2 * n1;
            for (int it = lane; it < 4 * m1n; it += 32)
            {
                const int s = it / m1n;
                const int a = it - s * m1n;
                const int i = a < n1 ? a : a - n1;
                const double t  = s_iso[s];
                const double nu = a < n1 ? t * s_x1[i] : t / s_x1[i];
                const double g  = total_nu_f1(nu, W.d, s);
                const double iso = iso_scatt_total(nu, W.eta_pp, W.eta_nn, L.use_WM_sc != 0);
                const double aux = 4. * k::Pi * (nu * nu) * (nu * nu) * nu * iso;
                const double v   = g * aux * s_B1[a];
                if (s == 0) acc[0] += v;
                else if (s == 1) acc[1] += v;
                else if (s == 2) acc[2] += v;
                else acc[3] += v;
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                acc[kk] = warp_sum(acc[kk]);
            if (lane == 0)
            {
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    W.tot[40 + kk] = acc[kk];
            }
        }
        __syncwarp();

        // ---------------- assemble (m1_opacities.hpp:1172-1294) ----------
        if (lane < 20)
        {
            const int q = lane >> 2, s = lane & 3;
            const bool has2d = L.use_pair || L.use_brem;
            const double t2 = t2d * t2d;
            const double tn = 4. * (k::TempMultiple * T);
            const double hn = 0.5 * (tn * tn);
            const double n2d_em = has2d ? W.tot[s] * t2 : 0.;
            const double n2d_ab = has2d ? W.tot[4 + s] * t2 : 0.;
            const double e2d_em = has2d ? W.tot[8 + s] * t2d * t2 : 0.;
            const double e2d_ab = has2d ? W.tot[12 + s] * t2d * t2 : 0.;
            const double nne_em = L.use_inel ? W.tot[16 + s] * hn : 0.;
            const double nne_ab = L.use_inel ? W.tot[20 + s] * hn : 0.;
            const double ene_em = L.use_inel ? W.tot[24 + s] * hn : 0.;
            const double ene_ab = L.use_inel ? W.tot[28 + s] * hn : 0.;
            double bne = 0., bje = 0., bna = 0., bja = 0., iso = 0.;
            if (s < 2 && L.use_abs_em)
            {
                bne = W.tot[32 + s] * s_beta[s];
                bje = W.tot[34 + s] * s_beta[s];
                bna = W.tot[36 + s] * s_beta[s];
                bja = W.tot[38 + s] * s_beta[s];
            }
            if (L.use_iso)
                iso = W.tot[40 + s] * s_iso[s];
            const double F = k::FourPiHc3, F2 = k::FourPiHc3Sqr, c = k::Clight;
            double v = 0.;
            if (s < 2)
            {
                if (q == 0)
                    v = F * (F * (n2d_em + nne_em) + bne);
                else if (q == 2)
                    v = F * (F * (e2d_em + ene_em) + bje);
                else if (q == 1)
                    v = (n[s] > k::ThresholdN) ? F / (c * n[s]) * (F * (n2d_ab + nne_ab) + bna) : 0.;
                else if (q == 3)
                    v = (J[s] > k::ThresholdJ) ?
                            ((s == 0 && n[s] == 0.) ? 0. :
                                                      F / (c * J[s]) * (F * (e2d_ab + ene_ab) + bja)) :
                            0.;
                else
                    v = (J[s] > k::ThresholdJ) ? F / (c * J[s]) * iso : 0.;
            }
            else
            {
                if (q == 0)
                    v = F2 * (n2d_em + nne_em);
                else if (q == 2)
                    v = F2 * (e2d_em + ene_em);
                else if (q == 1)
                    v = (n[s] > k::ThresholdN) ?
                            ((s == 3 && n[s] == 0.) ? 0. : F2 / (c * n[s]) * (n2d_ab + nne_ab)) :
                            0.;
                else if (q == 3)
                    v = (J[s] > k::ThresholdJ) ? F2 / (c * J[s]) * (e2d_ab + ene_ab) : 0.;
                else
                    v = (J[s] > k::ThresholdJ) ? F / (c * J[s]) * iso : 0.;
            }
            L.out[lane][p] = v;
        }
        __syncwarp();
    }
}

} // namespace

cudaError_t launch_grey_fp64(const OpacityLaunch& L, cudaStream_t stream, int num_sms)
{
    if (L.npts <= 0)
        return cudaSuccess;
    const int64_t need = (L.npts + kWarps - 1) / kWarps;
    int blocks_per_sm  = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &blocks_per_sm, grey_fp64_kernel, kWarps * 32, 0);
    if (err != cudaSuccess)
        return err;
    if (blocks_per_sm < 1)
        blocks_per_sm = 1;
    const int64_t cap = (int64_t)num_sms * blocks_per_sm;
    const int grid    = (int)(need < cap ? need : cap);
    grey_fp64_kernel<<<grid, kWarps * 32, 0, stream>>>(L);
    return cudaGetLastError();
}

} // namespace bnsn
