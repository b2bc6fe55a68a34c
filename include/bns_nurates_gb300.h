/* bns_nurates_gb300.h -- C ABI of the GB300 opacity library.
 *
 * Drop-in for the per-point opacity path of bns_nurates: the grey M1
 * emissivities/opacities (ComputeM1Opacities) and the spectral opacities
 * (ComputeSpectralOpacities*), computed on one GB300 (sm_103a) GPU.
 *
 * Part 1 restates the reference's public structs with the same names and the
 * same memory layout (BS_REAL = double, BS_N_MAX = 20), so caller code that
 * fills MyQuadrature / GreyOpacityParams keeps working.  Part 2 is the batched
 * device API (structure-of-arrays over points).  Part 3 holds per-point host
 * drop-ins and utilities.  Every entry point returns a bnsn_status.
 */
#ifndef BNS_NURATES_GB300_H_
#define BNS_NURATES_GB300_H_

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ======================================================================
 * Part 1: structs of include/bns_nurates.hpp (layout-identical)
 * ====================================================================== */

#define id_nue 0
#define id_anue 1
#define id_nux 2
#define id_anux 3
#define total_num_species 4
#define BS_N_MAX 20 /* capacity of MyQuadrature::points / w */

typedef double BS_REAL;

/* bns_nurates.hpp:80-84 */
enum Quadrature { kGauleg, kGaulag };

/* bns_nurates.hpp:106-130: n Gauss-Legendre nodes/weights on [0,1] in
 * points[0..nx-1], w[0..nx-1].  Only nx, points and w are read. */
typedef struct MyQuadrature
{
    enum Quadrature type;
    BS_REAL alpha;
    int dim;
    int nx;
    int ny;
    int nz;
    BS_REAL x1, x2, y1, y2, z1, z2;
    BS_REAL points[BS_N_MAX];
    BS_REAL w[BS_N_MAX];
} MyQuadrature;

/* bns_nurates.hpp:199-250 */
typedef struct BremKernelParams
{
    BS_REAL omega;
    BS_REAL omega_prime;
    int l;
    bool use_NN_medium_corr;
} BremKernelParams;

typedef struct PairKernelParams
{
    BS_REAL omega, omega_prime, cos_theta, mu, mu_prime, lmax, filter;
} PairKernelParams;

typedef struct InelasticScattKernelParams
{
    BS_REAL omega, omega_prime;
} InelasticScattKernelParams;

typedef struct MyKernelParams
{
    PairKernelParams pair_kernel_params;
    BremKernelParams brem_kernel_params;
    InelasticScattKernelParams inelastic_kernel_params;
} MyKernelParams;

/* bns_nurates.hpp:259-264 */
typedef struct MyKernelOutput
{
    BS_REAL em[total_num_species];
    BS_REAL abs[total_num_species];
} MyKernelOutput;

/* bns_nurates.hpp:289-306: chemical potentials include rest masses */
typedef struct MyEOSParams
{
    BS_REAL nb;     /* baryon number density [nm^-3] */
    BS_REAL temp;   /* temperature [MeV] */
    BS_REAL ye, yp, yn;
    BS_REAL mu_p, mu_n, mu_e, mu_mu; /* [MeV] (mu_mu unused) */
    BS_REAL dU;     /* mean-field potential difference [MeV] */
    BS_REAL dm_eff; /* effective mass difference [MeV] */
} MyEOSParams;

/* bns_nurates.hpp:324-329 */
typedef struct MyOpacity
{
    BS_REAL abs[total_num_species];
    BS_REAL em[total_num_species];
} MyOpacity;

/* bns_nurates.hpp:332 */
enum BremImpl { BREM_HR98 = 0, BREM_BRT06 = 1, BREM_GP19 = 2 };

/* bns_nurates.hpp:338-352 */
typedef struct OpacityParams
{
    bool use_dU;
    bool use_dm_eff;
    bool use_WM_ab;
    bool use_WM_sc;
    bool use_decay;
    enum BremImpl brem_implementation;
    bool use_NN_medium_corr;
    bool neglect_blocking;
} OpacityParams;

/* bns_nurates.hpp:387-401 */
typedef struct NuDistributionParams
{
    BS_REAL w_t[total_num_species];
    BS_REAL temp_t[total_num_species];
    BS_REAL eta_t[total_num_species];
    BS_REAL w_f[total_num_species];
    BS_REAL temp_f[total_num_species];
    BS_REAL c_f[total_num_species];
    BS_REAL beta_f[total_num_species];
} NuDistributionParams;

/* bns_nurates.hpp:409-416: n [nm^-3], J [MeV nm^-3]; H unused */
typedef struct M1Quantities
{
    BS_REAL n[total_num_species];
    BS_REAL J[total_num_species];
    BS_REAL H[total_num_species][4];
    BS_REAL chi[total_num_species];
} M1Quantities;

/* bns_nurates.hpp:418-426 */
typedef struct OpacityFlags
{
    int use_abs_em;
    int use_pair;
    int use_brem;
    int use_inelastic_scatt;
    int use_iso;
} OpacityFlags;

/* bns_nurates.hpp:444-454 */
typedef struct GreyOpacityParams
{
    OpacityParams opacity_pars;
    MyKernelParams kernel_pars;
    MyEOSParams eos_pars;
    NuDistributionParams distr_pars;
    M1Quantities m1_pars;
    OpacityFlags opacity_flags;
} GreyOpacityParams;

/* bns_nurates.hpp:463-474: eta_0 [nm^-3 s^-1], eta [MeV nm^-3 s^-1],
 * kappa_* [nm^-1] */
typedef struct M1Opacities
{
    BS_REAL eta_0[total_num_species];
    BS_REAL kappa_0_a[total_num_species];
    BS_REAL eta[total_num_species];
    BS_REAL kappa_a[total_num_species];
    BS_REAL kappa_s[total_num_species];
} M1Opacities;

/* bns_nurates.hpp:517-524 */
typedef struct SpectralOpacities
{
    BS_REAL j[total_num_species];
    BS_REAL kappa[total_num_species];
    BS_REAL j_s[total_num_species];
    BS_REAL kappa_s[total_num_species];
} SpectralOpacities;

/* ======================================================================
 * Part 2: batched device API
 *
 * Points are independent.  Every per-point quantity is a separate device
 * array of length npts (structure of arrays, one pointer per struct field),
 * so callers can pass their own grid-function storage.  Calls are
 * stream-ordered on `stream` (a cudaStream_t; NULL = default stream) and do
 * not synchronise the host.
 *
 * Device memory: bnsn_m1_opacities keeps a per-point scratch record (6.4 KB)
 * for at most 8192 points at a time (two such chunks for larger batches).
 * It takes that scratch from a library-owned stream-ordered memory pool (one
 * per device, created on the first call), allocating and freeing it in order
 * on `stream`, so calls on different streams never share scratch.  The pool
 * keeps its memory for later calls.  bnsn_spectral_opacities takes its
 * scratch (256 B per (point, energy) record, about 131,072 records per chunk,
 * two chunks for larger batches) from the same pool; bnsn_m1_opacities_noalloc
 * uses a static device array; the host-buffer calls copy through a
 * library-owned staging buffer.  The other batched calls allocate nothing.
 * ====================================================================== */

typedef enum bnsn_status
{
    BNSN_OK = 0,
    BNSN_ERR_ARG = 1,      /* null pointer, npts < 0, bad enum or flag */
    BNSN_ERR_NQUAD = 2,    /* quadrature order outside 1..BNSN_NQUAD_MAX */
    BNSN_ERR_CUDA = 3,     /* a CUDA call failed (see bnsn_last_error) */
    BNSN_ERR_NO_TABLE = 4, /* GP19 requested but no table loaded */
    BNSN_ERR_NO_DEVICE = 5 /* no usable sm_103 device */
} bnsn_status;

/* Quadrature nodes per half-interval supported by the kernels (2x energy
 * nodes); the reference build is limited to BS_N_MAX/2 = 10. */
#define BNSN_NQUAD_MAX 20

typedef enum bnsn_precision
{
    BNSN_FP64 = 0, /* all arithmetic in double precision */
    BNSN_MIXED = 1 /* FP32 kernel tiles, FP64 where stability needs it */
} bnsn_precision;

/* MyEOSParams, one device array per field (mu_mu may be NULL). */
typedef struct bnsn_eos_soa
{
    const double *nb, *temp, *ye, *yp, *yn, *mu_p, *mu_n, *mu_e, *mu_mu, *dU,
        *dm_eff;
} bnsn_eos_soa;

/* M1Quantities n, J, chi per species. */
typedef struct bnsn_m1_soa
{
    const double* n[total_num_species];
    const double* J[total_num_species];
    const double* chi[total_num_species];
} bnsn_m1_soa;

/* NuDistributionParams per species (input of the opacity calls, output of
 * bnsn_distr_from_m1). */
typedef struct bnsn_distr_soa
{
    double* w_t[total_num_species];
    double* temp_t[total_num_species];
    double* eta_t[total_num_species];
    double* w_f[total_num_species];
    double* temp_f[total_num_species];
    double* c_f[total_num_species];
    double* beta_f[total_num_species];
} bnsn_distr_soa;

/* M1Opacities per species. */
typedef struct bnsn_m1_opacities_soa
{
    double* eta_0[total_num_species];
    double* kappa_0_a[total_num_species];
    double* eta[total_num_species];
    double* kappa_a[total_num_species];
    double* kappa_s[total_num_species];
} bnsn_m1_opacities_soa;

/* SpectralOpacities per species; each array is [npts][n_energies]
 * (entry p * n_energies + e). */
typedef struct bnsn_spectral_soa
{
    double* j[total_num_species];
    double* kappa[total_num_species];
    double* j_s[total_num_species];
    double* kappa_s[total_num_species];
} bnsn_spectral_soa;

/* Grey M1 opacities of npts points.
 * Replaces ComputeM1Opacities (stim_abs = 1, m1_opacities.hpp:1306-1313) and
 * ComputeM1OpacitiesNotStimulated (stim_abs = 0, m1_opacities.hpp:1297-1304)
 * called once per point, e.g. from the Kokkos loop of tests/tests.hpp:272-343.
 * quad_1d drives the beta and iso integrals, quad_2d the pair, brem and
 * inelastic double integrals, exactly as in the reference.  `distr` = NULL
 * reconstructs the distribution from `m1` on the device
 * (CalculateDistrParamsFromM1, distribution.hpp:323-333) before use; otherwise
 * the given parameters are used as GreyOpacityParams::distr_pars. */
int bnsn_m1_opacities(const MyQuadrature* quad_1d, const MyQuadrature* quad_2d,
                      const OpacityFlags* flags, const OpacityParams* params,
                      const bnsn_eos_soa* eos, const bnsn_m1_soa* m1,
                      const bnsn_distr_soa* distr, int stim_abs, int precision,
                      const bnsn_m1_opacities_soa* out, int64_t npts,
                      void* stream);

/* One box of a host code's 3-D grid (a THC / Cactus grid-function component,
 * where the reference's exported headers -- utils/export_thc.py -- are called
 * point by point inside the host code's loops): every field a separate device
 * array of shape[0] x shape[1] x shape[2] doubles, x fastest.  The interior
 * lo <= (i, j, k) < hi (ghost zones excluded) is evaluated; the rest of the
 * output arrays is not touched.  Field order as in bnsn_eos_soa (mu_mu may
 * be NULL), bnsn_m1_soa and bnsn_m1_opacities_soa. */
typedef struct bnsn_grid_box
{
    int64_t shape[3];
    int64_t lo[3];
    int64_t hi[3];
    const double* eos[11]; /* nb temp ye yp yn mu_p mu_n mu_e mu_mu dU dm_eff */
    const double* m1[12];  /* n[4] J[4] chi[4] */
    double* out[20];       /* eta_0[4] kappa_0_a[4] eta[4] kappa_a[4] kappa_s[4] */
} bnsn_grid_box;

/* Grey M1 opacities of the interiors of nboxes boxes (no counterpart in the
 * reference, whose host codes loop over their grids calling
 * ComputeM1Opacities per cell, m1_opacities.hpp:1172-1294): the interiors are
 * gathered into one batch, evaluated as by bnsn_m1_opacities (distribution
 * reconstructed from the M1 moments) and scattered back.  in_scale (23
 * factors, eos then m1 fields) and out_scale (20) multiply the fields on the
 * way in and out, converting the host code's units; NULL means 1.  Stream
 * ordered; allocates a staging buffer of 43 doubles per interior cell from
 * the device's default pool.  Invalid extents (lo > hi, hi > shape) and NULL
 * field pointers of a non-empty box are rejected before any device work. */
int bnsn_m1_opacities_grid_boxes(const MyQuadrature* quad_1d,
                                 const MyQuadrature* quad_2d,
                                 const OpacityFlags* flags, const OpacityParams* params,
                                 const bnsn_grid_box* boxes, int nboxes,
                                 const double* in_scale, const double* out_scale,
                                 int stim_abs, int precision, void* stream);

/* Grey M1 opacities without any device allocation (no counterpart in the
 * reference).  Same arguments and results as bnsn_m1_opacities, but the
 * per-point scratch records live in a static device array inside the library
 * (room for BNSN_NOALLOC_MAX_POINTS points, 25 MiB) instead of the
 * stream-ordered pool.  It is meant for callers that must not allocate device
 * memory inside the call: codes whose device memory is owned by their own
 * allocator (hydro/AMR frameworks that reserve most of HBM at start-up, where
 * an extra driver allocation can fail or fragment it), and codes that keep
 * driver allocation calls out of their time step.
 *   - npts > BNSN_NOALLOC_MAX_POINTS is rejected with BNSN_ERR_ARG (split the
 *     batch, or call bnsn_m1_opacities).
 *   - The first call on each device looks up the array's address with that
 *     device current (cudaGetSymbolAddress, which may load a module); make
 *     that first call (npts may be 0) before any stream capture.
 *   - The array's 25 MiB are taken on a device when the library's module is
 *     loaded there: at that first call under lazy module loading (the CUDA
 *     default), but at context creation for every process that loads the
 *     library when CUDA_MODULE_LOADING=EAGER, whether or not it ever calls
 *     this entry point.
 *   - Nothing in the array needs to start at zero: every scratch value a
 *     kernel reads is written earlier in the same call.
 *   - There is one array per device: calls that overlap in time on one device
 *     (different streams or host threads without ordering between them) race
 *     on it and give wrong results.  Order such calls on one stream or with
 *     events. */
#define BNSN_NOALLOC_MAX_POINTS 4096
int bnsn_m1_opacities_noalloc(const MyQuadrature* quad_1d, const MyQuadrature* quad_2d,
                              const OpacityFlags* flags, const OpacityParams* params,
                              const bnsn_eos_soa* eos, const bnsn_m1_soa* m1,
                              const bnsn_distr_soa* distr, int stim_abs,
                              int precision, const bnsn_m1_opacities_soa* out,
                              int64_t npts, void* stream);

/* ----------------------------------------------------------------------
 * Batched AMR blocks (no counterpart in the reference, whose callers loop
 * over points): many blocks of uneven size, each with its own reactions,
 * bremsstrahlung variant and quadrature order, computed by one planned
 * execution.  A block is points [first, first + count) of the SoA arrays.
 * ---------------------------------------------------------------------- */
typedef struct bnsn_block
{
    int64_t first;
    int64_t count;
    OpacityFlags flags;      /* reactions of the block */
    int brem_implementation; /* BremImpl of the block */
    int nquad;               /* Gauss-Legendre nodes per half-interval (1d and 2d) */
} bnsn_block;

typedef struct bnsn_blocks_plan* bnsn_blocks_plan_t;

/* Plan the blocks: group them by configuration, upload each group's point
 * list and descriptor, split the points into steps (each step takes the same
 * fraction of every group's points; steps alternate between two streams) and
 * allocate the per-point scratch of two steps.  The step size is chosen by
 * the tuner (tune != 0: candidate step sizes and persistent-grid scales --
 * points per CTA -- timed on the first steps of the given arrays, keeping the
 * fastest; the tuning runs write `out`), else a default or the size set by
 * bnsn_blocks_set_options, with smaller steps where the scratch limit needs
 * them.  Allocates device memory and synchronises; the GP19 table, when a
 * block uses it, must be loaded before and not replaced while the plan
 * lives. */
int bnsn_blocks_plan_create(const bnsn_block* blocks, int nblocks,
                            const OpacityParams* params, int stim_abs, int precision,
                            int tune, const bnsn_eos_soa* eos, const bnsn_m1_soa* m1,
                            const bnsn_m1_opacities_soa* out, void* stream,
                            bnsn_blocks_plan_t* plan);
/* Grey opacities of every block of the plan on `stream`: per step, each phase
 * kernel is launched once for all configuration groups.  Kernel launches only
 * (no allocation, host synchronisation or copy), so a run can be captured in
 * a CUDA graph and replayed; the arrays may differ from the ones given to the
 * plan but must hold the same points.  Runs of one plan are ordered on the
 * streams they are given: two runs of the same plan must not execute
 * concurrently (they share the plan's scratch and descriptors). */
int bnsn_blocks_run(bnsn_blocks_plan_t plan, const bnsn_eos_soa* eos,
                    const bnsn_m1_soa* m1, const bnsn_m1_opacities_soa* out,
                    void* stream);
/* Number of configuration groups, and the configuration, size and launch
 * shape of group g (reactions: bit 0 abs/em, 1 pair, 2 brem, 3 NES, 4 iso;
 * chunk: the group's points per step).  Output pointers may be NULL. */
int bnsn_blocks_plan_groups(bnsn_blocks_plan_t plan);
int bnsn_blocks_plan_info(bnsn_blocks_plan_t plan, int group, int* nquad, int* reactions,
                          int* brem, int64_t* npts, int64_t* chunk, double* grid_scale);
/* The plan's steps per run, points per step (over all groups) and scratch
 * bytes.  Output pointers may be NULL. */
int bnsn_blocks_plan_layout(bnsn_blocks_plan_t plan, int* steps, int64_t* step_points,
                            int64_t* scratch_bytes);
/* Options of plans created afterwards (process-wide): scratch_bytes, the
 * scratch limit (0: a quarter of the device memory free at plan creation; a
 * plan holds at least two steps of one point per group); step_points, the
 * points per step over all groups (0: the tuner's choice, or the default
 * without tuning). */
int bnsn_blocks_set_options(int64_t scratch_bytes, int64_t step_points);
int bnsn_blocks_plan_destroy(bnsn_blocks_plan_t plan);

/* Spectral opacities of npts points at n_energies neutrino energies
 * (`energies` is a host array, MeV).  Replaces
 * ComputeSpectralOpacitiesStimulatedAbs (stimulated = 1,
 * m1_opacities.hpp:1641-1660) and ComputeSpectralOpacitiesNotStimulatedAbs
 * (stimulated = 0, m1_opacities.hpp:1506-1637) called per (point, energy). */
int bnsn_spectral_opacities(const MyQuadrature* quad_1d,
                            const OpacityFlags* flags,
                            const OpacityParams* params,
                            const bnsn_eos_soa* eos, const bnsn_m1_soa* m1,
                            const bnsn_distr_soa* distr, const double* energies,
                            int n_energies, int stimulated, int precision,
                            const bnsn_spectral_soa* out, int64_t npts,
                            void* stream);

/* Distribution parameters from M1 moments; replaces CalculateDistrParamsFromM1
 * (distribution.hpp:323-333) per point. */
int bnsn_distr_from_m1(const bnsn_m1_soa* m1, const bnsn_distr_soa* out,
                       int64_t npts, void* stream);

/* Equilibrium distribution and its M1 densities (chi = 1/3); replaces
 * NuEquilibriumParams + ComputeM1DensitiesEq (distribution.hpp:253-290,
 * 447-473) as used by the reference drivers (tests/tests.hpp:318-332). */
int bnsn_nu_equilibrium(const bnsn_eos_soa* eos, const bnsn_distr_soa* distr_out,
                        double* const n_out[total_num_species],
                        double* const J_out[total_num_species],
                        double* const chi_out[total_num_species], int64_t npts,
                        void* stream);

/* Load the 4-D GP19 response table (kernel_brem_GP19.hpp:75-139 layout:
 * data[((i_nb * d1 + i_ye) * d2 + i_T) * d3 + i_w], MeV^-1) onto the current
 * device.  lognb / logw may be NULL (computed as log of the axes).  Host
 * pointers; synchronous.  Required before any call with BREM_GP19. */
int bnsn_gp19_set_table(const int dims[4], const double* nb_axis,
                        const double* ye_axis, const double* t_axis,
                        const double* w_axis, const double* lognb_axis,
                        const double* logw_axis, const double* data);

/* The same from a table header in the reference's format (the GP19Table.hpp
 * that kernel_brem_GP19.hpp includes: GP19_{nb,Ye,T,w}_dims constants and the
 * GP19_{nb,lognb,Ye,T,w,logw}_axis / GP19_data brace initialisers), read as
 * text at run time; the log axes are optional.  BNSN_ERR_ARG when the file is
 * missing or a declaration is absent or has the wrong length. */
int bnsn_gp19_load_header(const char* path);

/* ======================================================================
 * Part 3: per-point drop-ins, host-buffer batches, utilities
 * ====================================================================== */

/* One point, host structs, synchronous (batch of one on the GPU).  Same
 * arguments and result as ComputeM1Opacities(quad_1d, quad_2d, grey_pars)
 * (m1_opacities.hpp:1306-1313); grey_pars->distr_pars must be filled, as in
 * the reference.  grey_pars is not modified. */
int bnsn_compute_m1_opacities_point(const MyQuadrature* quad_1d,
                                    const MyQuadrature* quad_2d,
                                    const GreyOpacityParams* grey_pars,
                                    int stim_abs, M1Opacities* out);

/* One point; same as CalculateDistrParamsFromM1(m1_pars, eos_pars)
 * (distribution.hpp:323-333, which does not read eos_pars). */
int bnsn_distr_from_m1_point(const M1Quantities* m1, NuDistributionParams* out);

/* One point, one energy; same as ComputeSpectralOpacities{Not,}StimulatedAbs
 * (m1_opacities.hpp:1506-1660). */
int bnsn_compute_spectral_opacities_point(double nu, const MyQuadrature* quad_1d,
                                          const GreyOpacityParams* grey_pars,
                                          int stimulated,
                                          SpectralOpacities* out);

/* bnsn_m1_opacities with every SoA pointer in HOST memory.  The library
 * copies inputs in, computes and copies results out through a staging area
 * on the current device, chunked and overlapped across two streams;
 * returns when the results are in `out`. */
int bnsn_m1_opacities_host(const MyQuadrature* quad_1d,
                           const MyQuadrature* quad_2d,
                           const OpacityFlags* flags,
                           const OpacityParams* params, const bnsn_eos_soa* eos,
                           const bnsn_m1_soa* m1, int stim_abs, int precision,
                           const bnsn_m1_opacities_soa* out, int64_t npts);

/* Fermi-Dirac integrals F_j(x) = int_0^inf t^j / (exp(t - x) + 1) dt of the
 * reference's family (functions.hpp:442-4375), unnormalised as there, for
 * j = twice_order / 2: twice_order -9, -7, -5, -3, -1 replaces FDI_m92 ..
 * FDI_m12 (continued below j = -1 by dF_{j+1}/dx = (j+1) F_j), 0 .. 21
 * replaces FDI_0, FDI_p12, FDI_p1, ..., FDI_p10, FDI_p212.  Integer orders 0..5
 * use the reference's approximations; the others tabulated approximations
 * that agree with the reference's to a few 1e-16 relative.  A NaN argument
 * gives NaN (half-integer orders) or 0 (integer orders), as the reference.
 * bnsn_fdi: x and out are device arrays of n doubles, stream-ordered.
 * bnsn_fdi_host: host arrays, synchronous.  BNSN_ERR_ARG for another order. */
int bnsn_fdi(int twice_order, const double* x, double* out, int64_t n, void* stream);
int bnsn_fdi_host(int twice_order, const double* x, double* out, int64_t n);

/* The mixed path's pair-annihilation integrals at n given (y, z, eta), device
 * arrays, stream-ordered: J_0 = PairPsi(y, z) / (1 - e^{y+z}) and
 * J_1 = PairPsi(z, y) / (1 - e^{y+z}) of kernel_pair.hpp:16-120 (y = omega/T,
 * z = omega'/T, eta = mu_e/T; l = 0), returned as J_l = exp(lscale) * j_l so
 * that values far below the double range stay representable.  The mixed grey
 * path computes them as a positive FP32 integral over the e- energy instead of
 * the reference's cancelling Fermi-integral combination; this entry exposes
 * that integral for testing.  j_l = 0 where the reference zeroes PairPsi
 * (eta - y - z > 200). */
int bnsn_pair_j_mixed(const double* y, const double* z, const double* eta, double* j0,
                      double* j1, double* lscale, int64_t n, void* stream);

/* The mixed path's NES/NPS out-kernel integrals at n given (w, w', eta),
 * device arrays, stream-ordered: MezzacappaIntOut(w, w', b1, b2) of
 * kernel_nes.hpp:50-78 (w = omega/T, w' = omega'/T, eta = mu/T of the lepton;
 * the general branch, not the reference's Taylor expansions for small
 * energies) = exp(lscale) * (b1 m1 + b2 m2).  The mixed grey path computes it
 * as a positive FP32 integral over the lepton energy instead of the
 * reference's cancelling Fermi-integral combination; this entry exposes that
 * integral for testing. */
int bnsn_nes_m_mixed(const double* w, const double* wp, const double* eta, double* m1,
                     double* m2, double* lscale, int64_t n, void* stream);

/* Gauss-Legendre nodes/weights of order quad->nx on [0,1]; replaces
 * GaussLegendre (integration.hpp:28-87), same algorithm. */
int bnsn_gauss_legendre(MyQuadrature* quad);

/* Seeded synthetic thermodynamic points (host, OpenMP): eos[11][npts] in the
 * MyEOSParams field order and m1[12][npts] = n[4], J[4], chi[4].  Point k
 * depends only on (seed, first + k).  rho log-uniform 1e6..1e15 g/cm^3,
 * T log-uniform 0.5..100 MeV, Ye uniform 0.01..0.6; mu_e from an ideal
 * relativistic e+- gas; non-relativistic ideal nucleons with a mean-field
 * shift dU uniform in +-20 MeV; per species T_nu = T U(0.5,1.5), eta_nu
 * U(-5,5), n and J from Fermi-Dirac moments, chi U(1/3,1); anti-nu_x = nu_x. */
int bnsn_synthetic_points(uint64_t seed, int64_t first, int64_t npts,
                          double* eos, double* m1, int nthreads);

/* FP64 fused-multiply-add throughput of the current device in TFLOP/s
 * (independent DFMA chains on every SM, CUDA-event timed): the denominator of
 * the FP64-pipe roofline of the opacity kernels.  A diagnostic with no
 * counterpart in the reference. */
int bnsn_fp64_peak_probe(int64_t iters, double* tflops);
/* The same for FP32 FMA chains (the pipe of the mixed path's double-float
 * arithmetic).  A diagnostic with no counterpart in the reference. */
int bnsn_fp32_peak_probe(int64_t iters, double* tflops);

/* Per-phase device timing of the library's own kernels (diagnostics with no
 * counterpart in the reference).  While enabled, every kernel launch is
 * bracketed by CUDA events on its stream; bnsn_phase_times waits for the
 * recorded events, adds each launch's duration to ms[phase] and its count to
 * launches[phase] (arrays of BNSN_NUM_PHASES entries, accumulated since the
 * previous bnsn_phase_times call), and clears the record.  Phases:
 * 0 grey prelude, 1 pair cells, 2 brem cells, 3 NES/NPS pairs (mixed path:
 * the fast pass), 4 grey assembly, 5 spectral, 6 distribution/equilibrium,
 * 7 mixed NES double-float pass over flagged points, 8 mixed NES FP64 pass
 * over the points flagged again.  Timing one device at a time is
 * supported. */
#define BNSN_NUM_PHASES 9
int bnsn_phase_timing(int enable);
int bnsn_phase_times(double* ms, int64_t* launches);
/* Number of kernels this library has launched in the process. */
int64_t bnsn_kernel_launches(void);
/* Mixed-precision spectral path on the current device since the last reset:
 * counts[0] (point, energy) pairs evaluated, counts[1] pairs recomputed in FP64
 * in some part because the FP32 error guards failed (terms that cancel) or a
 * part could not run in FP32, counts[2] pair + brem recomputations, counts[3]
 * NES recomputations.  reset != 0 zeroes the counters after reading;
 * synchronises the device.  A diagnostic with no counterpart in the
 * reference. */
int bnsn_spectral_mixed_stats(int64_t* counts, int reset);
/* Mixed-precision grey path on the current device since the last reset:
 * counts[0] points evaluated, counts[1] points whose NES/NPS sums went to the
 * double-float pass (their FP32 terms cancel), counts[2] points whose NES sums
 * were computed in FP64 (outside the FP32 range envelope, or cancelling
 * beyond the double-float pass), counts[3] points whose pair sums and
 * counts[4] points whose brem sums were recomputed in FP64 (cancellation
 * against the other reactions).  reset != 0 zeroes the counters after
 * reading; synchronises the device.  A diagnostic with no counterpart in the
 * reference. */
int bnsn_grey_mixed_stats(int64_t* counts, int reset);
/* Outputs holding a NaN or Inf on the current device since the last reset:
 * counts[0] grey points (any of the 20 outputs), counts[1] spectral (point,
 * energy) pairs (any of the 16 outputs).  The kernels never trap: non-finite
 * inputs, or GP19 brem outside its table, propagate into the outputs as in
 * the reference, and these counters let a caller detect it without scanning
 * the outputs.  reset != 0 zeroes the counters after reading; synchronises
 * the device. */
int bnsn_nonfinite_outputs(int64_t* counts, int reset);

const char* bnsn_status_string(int status);
/* Text of the most recent error on the calling thread ("" if none). */
const char* bnsn_last_error(void);
int bnsn_version(void);

#ifdef __cplusplus
}
#endif

#endif /* BNS_NURATES_GB300_H_ */
