// Test infrastructure only: a C-ABI driver around the reference bns_nurates
// headers, compiled in their no-Kokkos shim mode (include/bns_nurates.hpp:39-53)
// straight from the reference checkout by oracle/build_ref.py.  The product
// never links or loads it; tests use it to pin the oracle restatement
// (oracle/bnsn_oracle.c) and to generate golden fixtures.
//
// Per point it builds a GreyOpacityParams the way the reference drivers do
// (tests/tests.hpp:272-343, mwe.cpp:74-160) and calls the reference functions:
//   ComputeM1Opacities / ComputeM1OpacitiesNotStimulated  m1_opacities.hpp:1297-1313
//   ComputeSpectralOpacities{Not,}StimulatedAbs           m1_opacities.hpp:1506-1660
//   CalculateDistrParamsFromM1                            distribution.hpp:323-333
// plus thin wrappers of the individual kernels for unit-level pinning.
//
// Array conventions (shared with the oracle restatement):
//   eos   : double[11][npts] = nb, temp, ye, yp, yn, mu_p, mu_n, mu_e, mu_mu, dU, dm_eff
//   m1    : double[12][npts] = n[4], J[4], chi[4]
//   distr : double[28][npts] = w_t[4], temp_t[4], eta_t[4], w_f[4], temp_f[4], c_f[4], beta_f[4]
//   grey  : double[20][npts] = eta_0[4], kappa_0_a[4], eta[4], kappa_a[4], kappa_s[4]
//   spec  : double[16][npts*ne] = j[4], kappa[4], j_s[4], kappa_s[4]; entry p*ne+e
//   flags : int[5] = use_abs_em, use_pair, use_brem, use_inelastic_scatt, use_iso
//   pars  : int[8] = use_dU, use_dm_eff, use_WM_ab, use_WM_sc, use_decay,
//                    brem_implementation, use_NN_medium_corr, neglect_blocking

#include <stdint.h>
#include <string.h>

#include "m1_opacities.hpp"

static void set_flags(GreyOpacityParams* g, const int* flags, const int* pars)
{
    g->opacity_flags.use_abs_em          = flags[0];
    g->opacity_flags.use_pair            = flags[1];
    g->opacity_flags.use_brem            = flags[2];
    g->opacity_flags.use_inelastic_scatt = flags[3];
    g->opacity_flags.use_iso             = flags[4];
    g->opacity_pars.use_dU               = pars[0] != 0;
    g->opacity_pars.use_dm_eff           = pars[1] != 0;
    g->opacity_pars.use_WM_ab            = pars[2] != 0;
    g->opacity_pars.use_WM_sc            = pars[3] != 0;
    g->opacity_pars.use_decay            = pars[4] != 0;
    g->opacity_pars.brem_implementation  = (BremImpl)pars[5];
    g->opacity_pars.use_NN_medium_corr   = pars[6] != 0;
    g->opacity_pars.neglect_blocking     = pars[7] != 0;
}

static void set_eos(MyEOSParams* e, const double* eos, int64_t np, int64_t p)
{
    e->nb     = eos[0 * np + p];
    e->temp   = eos[1 * np + p];
    e->ye     = eos[2 * np + p];
    e->yp     = eos[3 * np + p];
    e->yn     = eos[4 * np + p];
    e->mu_p   = eos[5 * np + p];
    e->mu_n   = eos[6 * np + p];
    e->mu_e   = eos[7 * np + p];
    e->mu_mu  = eos[8 * np + p];
    e->dU     = eos[9 * np + p];
    e->dm_eff = eos[10 * np + p];
}

static void set_m1(M1Quantities* m, const double* m1, int64_t np, int64_t p)
{
    memset(m, 0, sizeof(*m));
    for (int s = 0; s < 4; ++s)
    {
        m->n[s]   = m1[(0 + s) * np + p];
        m->J[s]   = m1[(4 + s) * np + p];
        m->chi[s] = m1[(8 + s) * np + p];
    }
}

static void get_distr(NuDistributionParams* d, const double* distr, int64_t np,
                      int64_t p)
{
    for (int s = 0; s < 4; ++s)
    {
        d->w_t[s]    = distr[(0 + s) * np + p];
        d->temp_t[s] = distr[(4 + s) * np + p];
        d->eta_t[s]  = distr[(8 + s) * np + p];
        d->w_f[s]    = distr[(12 + s) * np + p];
        d->temp_f[s] = distr[(16 + s) * np + p];
        d->c_f[s]    = distr[(20 + s) * np + p];
        d->beta_f[s] = distr[(24 + s) * np + p];
    }
}

static void put_distr(const NuDistributionParams* d, double* distr, int64_t np,
                      int64_t p)
{
    for (int s = 0; s < 4; ++s)
    {
        distr[(0 + s) * np + p]  = d->w_t[s];
        distr[(4 + s) * np + p]  = d->temp_t[s];
        distr[(8 + s) * np + p]  = d->eta_t[s];
        distr[(12 + s) * np + p] = d->w_f[s];
        distr[(16 + s) * np + p] = d->temp_f[s];
        distr[(20 + s) * np + p] = d->c_f[s];
        distr[(24 + s) * np + p] = d->beta_f[s];
    }
}

static void make_quad(MyQuadrature* q, int nx, const double* x, const double* w)
{
    memset(q, 0, sizeof(*q));
    q->type = kGauleg;
    q->dim  = 1;
    q->nx   = nx;
    q->ny   = 1;
    q->nz   = 1;
    q->x1   = 0.;
    q->x2   = 1.;
    q->y1 = q->y2 = q->z1 = q->z2 = -42.;
    for (int i = 0; i < nx; ++i)
    {
        q->points[i] = x[i];
        q->w[i]      = w[i];
    }
}

static void build_point(GreyOpacityParams* g, const double* eos,
                        const double* m1, const double* distr, const int* flags,
                        const int* pars, int64_t np, int64_t p)
{
    memset(g, 0, sizeof(*g));
    set_flags(g, flags, pars);
    set_eos(&g->eos_pars, eos, np, p);
    set_m1(&g->m1_pars, m1, np, p);
    if (distr)
        get_distr(&g->distr_pars, distr, np, p);
    else
        g->distr_pars = CalculateDistrParamsFromM1(&g->m1_pars, &g->eos_pars);
}

extern "C" {

int ref_bs_n_max(void) { return BS_N_MAX; }

void ref_gauss_legendre(int n, double* x, double* w)
{
    MyQuadrature q = quadrature_default;
    q.nx           = n;
    GaussLegendre(&q);
    for (int i = 0; i < n; ++i)
    {
        x[i] = q.points[i];
        w[i] = q.w[i];
    }
}

int ref_m1_opacities_batch(int64_t npts, const double* eos, const double* m1,
                           const double* distr, const int* flags,
                           const int* pars, int nx1, const double* x1,
                           const double* w1, int nx2, const double* x2,
                           const double* w2, int stim_abs, double* out,
                           int nthreads)
{
    if (2 * nx1 > BS_N_MAX || 2 * nx2 > BS_N_MAX)
        return 2;
    MyQuadrature q1, q2;
    make_quad(&q1, nx1, x1, w1);
    make_quad(&q2, nx2, x2, w2);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int64_t p = 0; p < npts; ++p)
    {
        GreyOpacityParams g;
        build_point(&g, eos, m1, distr, flags, pars, npts, p);
        M1Opacities o = stim_abs ? ComputeM1Opacities(&q1, &q2, &g) :
                                   ComputeM1OpacitiesNotStimulated(&q1, &q2, &g);
        for (int s = 0; s < 4; ++s)
        {
            out[(0 + s) * npts + p]  = o.eta_0[s];
            out[(4 + s) * npts + p]  = o.kappa_0_a[s];
            out[(8 + s) * npts + p]  = o.eta[s];
            out[(12 + s) * npts + p] = o.kappa_a[s];
            out[(16 + s) * npts + p] = o.kappa_s[s];
        }
    }
    return 0;
}

int ref_spectral_batch(int64_t npts, const double* eos, const double* m1,
                       const double* distr, const int* flags, const int* pars,
                       int nx, const double* x, const double* w, int ne,
                       const double* energies, int stimulated, double* out,
                       int nthreads)
{
    if (2 * nx > BS_N_MAX)
        return 2;
    MyQuadrature q;
    make_quad(&q, nx, x, w);
    const int64_t tot = npts * (int64_t)ne;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (int64_t p = 0; p < npts; ++p)
    {
        GreyOpacityParams g0;
        build_point(&g0, eos, m1, distr, flags, pars, npts, p);
        for (int e = 0; e < ne; ++e)
        {
            GreyOpacityParams g = g0;
            MyQuadrature qq     = q;
            SpectralOpacities s =
                stimulated ?
                    ComputeSpectralOpacitiesStimulatedAbs(energies[e], &qq, &g) :
                    ComputeSpectralOpacitiesNotStimulatedAbs(energies[e], &qq,
                                                             &g);
            const int64_t k = p * ne + e;
            for (int sp = 0; sp < 4; ++sp)
            {
                out[(0 + sp) * tot + k]  = s.j[sp];
                out[(4 + sp) * tot + k]  = s.kappa[sp];
                out[(8 + sp) * tot + k]  = s.j_s[sp];
                out[(12 + sp) * tot + k] = s.kappa_s[sp];
            }
        }
    }
    return 0;
}

void ref_distr_from_m1_batch(int64_t npts, const double* eos, const double* m1,
                             double* distr)
{
    for (int64_t p = 0; p < npts; ++p)
    {
        MyEOSParams e;
        M1Quantities m;
        set_eos(&e, eos, npts, p);
        set_m1(&m, m1, npts, p);
        NuDistributionParams d = CalculateDistrParamsFromM1(&m, &e);
        put_distr(&d, distr, npts, p);
    }
}

void ref_nu_equilibrium_batch(int64_t npts, const double* eos, double* distr,
                              double* m1)
{
    for (int64_t p = 0; p < npts; ++p)
    {
        MyEOSParams e;
        set_eos(&e, eos, npts, p);
        NuDistributionParams d = NuEquilibriumParams(&e);
        M1Quantities m;
        memset(&m, 0, sizeof(m));
        ComputeM1DensitiesEq(&e, &d, &m);
        put_distr(&d, distr, npts, p);
        for (int s = 0; s < 4; ++s)
        {
            m1[(0 + s) * npts + p] = m.n[s];
            m1[(4 + s) * npts + p] = m.J[s];
            m1[(8 + s) * npts + p] = 1. / 3.;
        }
    }
}

// k = 0..5 selects FDI_0 .. FDI_p5
void ref_fdi(int k, int64_t n, const double* x, double* out)
{
    for (int64_t i = 0; i < n; ++i)
    {
        switch (k)
        {
        case 0: out[i] = FDI_0(x[i]); break;
        case 1: out[i] = FDI_p1(x[i]); break;
        case 2: out[i] = FDI_p2(x[i]); break;
        case 3: out[i] = FDI_p3(x[i]); break;
        case 4: out[i] = FDI_p4(x[i]); break;
        default: out[i] = FDI_p5(x[i]); break;
        }
    }
}

// The whole family of functions.hpp:442-4375 by twice the order,
// k2 = -9, -7, ..., -1 (FDI_m92 .. FDI_m12) and 0..21 (FDI_0, FDI_p12, FDI_p1,
// ..., FDI_p10, FDI_p212).  Returns -1 for an order the reference lacks.
int ref_fdi_family(int k2, int64_t n, const double* x, double* out)
{
    double (*f)(double) = nullptr;
    switch (k2)
    {
    case -9: f = FDI_m92; break;
    case -7: f = FDI_m72; break;
    case -5: f = FDI_m52; break;
    case -3: f = FDI_m32; break;
    case -1: f = FDI_m12; break;
    case 0: f = FDI_0; break;
    case 1: f = FDI_p12; break;
    case 2: f = FDI_p1; break;
    case 3: f = FDI_p32; break;
    case 4: f = FDI_p2; break;
    case 5: f = FDI_p52; break;
    case 6: f = FDI_p3; break;
    case 7: f = FDI_p72; break;
    case 8: f = FDI_p4; break;
    case 9: f = FDI_p92; break;
    case 10: f = FDI_p5; break;
    case 11: f = FDI_p112; break;
    case 12: f = FDI_p6; break;
    case 13: f = FDI_p132; break;
    case 14: f = FDI_p7; break;
    case 15: f = FDI_p152; break;
    case 16: f = FDI_p8; break;
    case 17: f = FDI_p172; break;
    case 18: f = FDI_p9; break;
    case 19: f = FDI_p192; break;
    case 20: f = FDI_p10; break;
    case 21: f = FDI_p212; break;
    default: return -1;
    }
    for (int64_t i = 0; i < n; ++i)
        out[i] = f(x[i]);
    return 0;
}

// Pair kernel at (omega, omega_prime) for one EOS state: out[8] = em[4], abs[4]
void ref_pair_kernel(double temp, double mu_e, double omega, double omega_prime,
                     double* out)
{
    MyEOSParams e;
    memset(&e, 0, sizeof(e));
    e.temp = temp;
    e.mu_e = mu_e;
    PairKernelParams k;
    memset(&k, 0, sizeof(k));
    k.omega       = omega;
    k.omega_prime = omega_prime;
    k.cos_theta   = 1.;
    k.mu = k.mu_prime = 1.;
    MyKernelOutput o = PairKernels(&e, &k);
    for (int s = 0; s < 4; ++s)
    {
        out[s]     = o.em[s];
        out[4 + s] = o.abs[s];
    }
}

// Brem kernel: impl 0 = HR98 (l = 0), 1 = BRT06, 2 = GP19; out[2] = em, abs
void ref_brem_kernel(int impl, const double* eos11, double omega,
                     double omega_prime, int use_medium_corr, double* out)
{
    MyEOSParams e;
    set_eos(&e, eos11, 1, 0);
    BremKernelParams k;
    memset(&k, 0, sizeof(k));
    k.omega              = omega;
    k.omega_prime        = omega_prime;
    k.l                  = 0;
    k.use_NN_medium_corr = use_medium_corr != 0;
    MyKernelOutput o;
    if (impl == 0)
        o = BremKernelsLegCoeff(&k, &e);
    else if (impl == 1)
        o = BremKernelsBRT06(&k, &e);
    else
        o = BremKernelAbsGP19(&k, &e);
    out[0] = o.em[0];
    out[1] = o.abs[0];
}

// Inelastic NES+NPS kernel: out[8] = em[4], abs[4]
void ref_inelastic_kernel(double temp, double mu_e, double omega,
                          double omega_prime, double* out)
{
    MyEOSParams e;
    memset(&e, 0, sizeof(e));
    e.temp = temp;
    e.mu_e = mu_e;
    InelasticScattKernelParams k;
    k.omega          = omega;
    k.omega_prime    = omega_prime;
    MyKernelOutput o = InelasticScattKernels(&k, &e);
    for (int s = 0; s < 4; ++s)
    {
        out[s]     = o.em[s];
        out[4 + s] = o.abs[s];
    }
}

// Beta processes: out[4] = abs_nue, em_nue, abs_anue, em_anue (AbsOpacity)
void ref_abs_opacity(const double* eos11, const int* pars, double omega,
                     int stimulated, double* out)
{
    MyEOSParams e;
    set_eos(&e, eos11, 1, 0);
    GreyOpacityParams g;
    memset(&g, 0, sizeof(g));
    const int flags[5] = {0, 0, 0, 0, 0};
    set_flags(&g, flags, pars);
    MyOpacity o = stimulated ? StimAbsOpacity(omega, &g.opacity_pars, &e) :
                               AbsOpacity(omega, &g.opacity_pars, &e);
    out[0] = o.abs[id_nue];
    out[1] = o.em[id_nue];
    out[2] = o.abs[id_anue];
    out[3] = o.em[id_anue];
}

// Iso scattering: out[2] = IsoScattTotal, IsoScattLegCoeff(l)
void ref_iso_scatt(const double* eos11, const int* pars, double omega, int l,
                   double* out)
{
    MyEOSParams e;
    set_eos(&e, eos11, 1, 0);
    GreyOpacityParams g;
    memset(&g, 0, sizeof(g));
    const int flags[5] = {0, 0, 0, 0, 0};
    set_flags(&g, flags, pars);
    out[0] = IsoScattTotal(omega, &g.opacity_pars, &e);
    out[1] = IsoScattLegCoeff(omega, &g.opacity_pars, &e, l);
}

// Weak magnetism factors: out[6] = R, Rbar, R0_p, R1_p, R0_n, R1_n
void ref_weak_magnetism(double omega, double* out)
{
    WMAbsEm(omega, &out[0], &out[1]);
    WMScatt(omega, &out[2], &out[3], 1);
    WMScatt(omega, &out[4], &out[5], 2);
}

// TotalNuF for one distribution (28 values in the distr order) at energies
void ref_total_nu_f(const double* distr28, int64_t n, const double* omega,
                    double* out /* [4][n] */)
{
    NuDistributionParams d;
    get_distr(&d, distr28, 1, 0);
    for (int s = 0; s < 4; ++s)
        for (int64_t i = 0; i < n; ++i)
            out[s * n + i] = TotalNuF(omega[i], &d, s);
}

// Misc special functions: out[k] for k = 0..: SafeExp, FermiDistr, NEPSExpFunc,
// bessk1, GammaStirling
void ref_special(int which, int64_t n, const double* a, const double* b,
                 const double* c, double* out)
{
    for (int64_t i = 0; i < n; ++i)
    {
        switch (which)
        {
        case 0: out[i] = SafeExp(a[i]); break;
        case 1: out[i] = FermiDistr(a[i], b[i], c[i]); break;
        case 2: out[i] = NEPSExpFunc(a[i]); break;
        case 3: out[i] = bessk1(a[i]); break;
        default: out[i] = GammaStirling(a[i]); break;
        }
    }
}

} // extern "C"
