// Internal launch descriptors shared by the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bnsn {

constexpr int kMaxQ     = 20;                         // nodes per half-interval
constexpr int kMaxM     = 2 * kMaxQ;                  // energy nodes
constexpr int kMaxCells = kMaxM * (kMaxM + 1) / 2;    // unordered energy pairs

struct Gp19Dev
{
    int d0, d1, d2, d3;
    const double *nb, *ye, *t, *w, *lognb, *logw, *data;
};

// Everything a grey or spectral launch needs, passed by value as a
// __grid_constant__ kernel parameter (no device allocation per call).
struct OpacityLaunch
{
    int64_t npts;
    const int64_t* pidx;   // point q of the launch is pidx[q] (NULL: q itself)
    double grid_scale;     // persistent grid = grid_scale x resident CTAs (0: 1)
    const double* eos[11]; // nb temp ye yp yn mu_p mu_n mu_e mu_mu dU dm_eff
    const double* m1[12];  // n[4] J[4] chi[4]
    const double* distr[28];
    double* out[20];       // grey: eta_0, kappa_0_a, eta, kappa_a, kappa_s
    int has_distr;
    int use_abs_em, use_pair, use_brem, use_inel, use_iso;
    int use_dU, use_dm_eff, use_WM_ab, use_WM_sc, use_decay, brem_impl;
    int use_medium, neglect_blocking;
    int stim;
    int mixed;             // 0: all FP64, 1: mixed precision
    double gamma36;        // GammaStirling(3.6), host libm
    int n1, n2, ncell;
    double x1[kMaxQ], w1[kMaxQ], x2[kMaxQ], w2[kMaxQ];
    double B1[kMaxM];      // 1-D weights: w_i (a < n) or w_i / x_i^2
    double A1[kMaxM];      // 2-D number weights of one energy index
    double A2[kMaxM];      // 2-D energy weights (x t): x_i w_i or w_i / x_i^3
    double wx[kMaxQ];      // NES: w_i x_i
    double wx3[kMaxQ];     // NES: w_i / x_i^3
    double lx2[kMaxQ], l1m[kMaxQ], l1p[kMaxQ]; // NES: log x_i, log(1 - x_i), log(1 + x_i)
    double lx1[kMaxQ];     // spectral: log of the 1-D nodes
    uint32_t cells[kMaxCells]; // a | b << 16, a <= b
    uint16_t nes_order[2 * kMaxQ * kMaxQ]; // NES items (r, i, j) by ascending max(w, w')
    Gp19Dev gp19;
    // spectral launches only
    int n_energies;        // energies of this launch (<= 64)
    int e_stride, e_offset; // output entry p * e_stride + e_offset + e
    double energies[64];
    double* sout[16];      // j, kappa, j_s, kappa_s per species
};

// Multi-group launches of the batched AMR plan: one launch per phase serves
// every configuration group, blockIdx.z selecting the group's descriptor and
// its share of the chunk (points p0 .. p0 + np of its point list, scratch ws).
struct GroupChunk
{
    int64_t p0, np;
    double* ws;
};
struct GroupArgs
{
    const OpacityLaunch* Ls; // per group, device memory
    const GroupChunk* gc;    // per group for the chunk of this launch, device memory
};

// Kernel phases of the timing hooks (bnsn_phase_times).
enum Phase
{
    kPhPrelude = 0,
    kPhPair,
    kPhBrem,
    kPhNeps,
    kPhFinal,
    kPhSpectral,
    kPhAux,
    kPhNepsAccurate, // mixed path: df pass over the points the fast pass flagged
    kPhNepsFp64,     // mixed path: FP64 pass over the points flagged again
    kNumPhases
};

// Records a CUDA event on `stream` before (end = 0) or after (end = 1) a
// launch of `phase` when phase timing is on; always counts launches (end = 1).
void phase_mark(int phase, int end, cudaStream_t stream);

// Grey opacities in chunks of ws_points points; ws holds ws_points per-point
// scratch records of grey_point_scratch_bytes() (= kGreyRecordBytes) each.
// With an auxiliary stream (launch_grey's aux, else nullptr) the chunks are
// ws_points / 2 points, alternating between the two streams.
constexpr size_t kGreyRecordBytes = 800 * sizeof(double);
size_t grey_point_scratch_bytes();

// C-ABI helpers shared by the entry-point translation units (capi.cu).
struct DeviceInfo
{
    int num_sms;
    Gp19Dev gp19;
    bool has_gp19;
};
int capi_fail(int code, const char* msg);              // records the message, returns code
int capi_cuda_fail(cudaError_t e, const char* where);
int capi_fill_launch(const void* quad_1d, const void* quad_2d, const void* flags,
                     const void* params, int stim, OpacityLaunch* L); // MyQuadrature etc.
int capi_device_info(DeviceInfo* info);                // current device (creates its state)

// Static scratch of bnsn_m1_opacities_noalloc: room for kNoAllocPoints grey
// records in a file-scope __device__ array.  noalloc_scratch() looks up its
// address on the current device (cudaGetSymbolAddress, cached per device).
constexpr int64_t kNoAllocPoints = 4096;
cudaError_t noalloc_scratch(int device, double** ptr);
cudaError_t launch_grey(const OpacityLaunch& L, cudaStream_t stream, int num_sms, double* ws,
                        int64_t ws_points, cudaStream_t aux = nullptr);
// The chunk loop of launch_grey without the stream fork and join: chunks of
// `chunk` points, chunk k (the running counter *k, advanced per chunk) on
// stream0 with scratch ws0 when k is even or aux is NULL, else on aux with
// ws1.  The caller orders aux after stream0 before and joins it after.
cudaError_t launch_grey_chunks(const OpacityLaunch& L, cudaStream_t stream0, cudaStream_t aux,
                               int num_sms, double* ws0, double* ws1, int64_t chunk, int64_t* k);
// One multi-group step of the batched plan on `stream`: every phase kernel
// launched once with grid z = groups; group z's descriptor is GA.Ls[z] and
// its share of the step GA.gc[z] (both device memory).  U is a host
// descriptor whose reaction flags are the union of the groups' (the phases
// launched) and whose grid_scale sets the persistent grid; brem_set has bit i
// set when a group uses brem variant i; np_max is the largest share.
cudaError_t launch_grey_multi(const OpacityLaunch& U, unsigned brem_set, const GroupArgs& GA,
                              unsigned groups, int64_t np_max, cudaStream_t stream, int num_sms);
// Spectral opacities (phase kernels over chunks of points).  The scratch of
// one call holds spectral_scratch_bytes(chunk, n_energies) bytes for chunks of
// spectral_chunk_points(n_energies) points (about kSpecChunkRecords
// (point, energy) records of 256 bytes).  With aux and scratch1 (a second
// scratch of the same size) consecutive chunks alternate between stream and
// aux; stream waits for aux at the end.
constexpr int64_t kSpecChunkRecords = 131072;
int64_t spectral_chunk_points(int n_energies);
size_t spectral_scratch_bytes(int64_t chunk_points, int n_energies);
cudaError_t launch_spectral(const OpacityLaunch& L, cudaStream_t stream, int num_sms,
                            void* scratch, int64_t chunk_points, cudaStream_t aux = nullptr,
                            void* scratch1 = nullptr);
cudaError_t spectral_mixed_counts(unsigned long long* counts, bool reset);
// Outputs holding a NaN or Inf since the last reset: grey points, spectral
// (point, energy) pairs (synchronous reads of the current device's counters).
cudaError_t grey_nonfinite_count(unsigned long long* count, bool reset);
cudaError_t grey_mixed_counts(unsigned long long* counts, bool reset);
cudaError_t spectral_nonfinite_count(unsigned long long* count, bool reset);
struct DistrLaunch
{
    int64_t npts;
    const double* m1[12];
    double* out[28];
    double gamma36;
};

struct EquilLaunch
{
    int64_t npts;
    const double* eos[11];
    double* distr[28];
    double* m1[12];
};

cudaError_t launch_distr_from_m1(const DistrLaunch& L, cudaStream_t stream, int num_sms);
// Fermi-Dirac integral F_{k2/2} of n arguments (device arrays).
bool fdi_order_valid(int k2);
cudaError_t launch_nes_m(const double* w, const double* wp, const double* eta, double* m1,
                         double* m2, double* ls, int64_t n, cudaStream_t stream, int num_sms);
cudaError_t launch_pair_j(const double* y, const double* z, const double* eta, double* j0,
                          double* j1, double* ls, int64_t n, cudaStream_t stream, int num_sms);
cudaError_t launch_fdi(int k2, const double* x, double* out, int64_t n, cudaStream_t stream,
                       int num_sms);
cudaError_t launch_nu_equilibrium(const EquilLaunch& L, cudaStream_t stream, int num_sms);

} // namespace bnsn
