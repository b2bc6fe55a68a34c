// C-ABI entry points of the GB300 opacity library (include/bns_nurates_gb300.h).
//
// This layer validates arguments, turns the reference structs
// (MyQuadrature, OpacityFlags, OpacityParams) into a by-value launch
// descriptor and launches on the caller's stream.
//
// Device memory: the grey call takes its per-point scratch records (at most
// kGreyChunk points at a time) from a library-owned stream-ordered memory
// pool, allocated and freed in order on the caller's stream, so calls on
// different streams never share scratch.  The pool keeps its memory after the
// first call.  The per-point drop-ins and the host-buffer batch stage their
// inputs through a per-device buffer allocated on first use.

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bns_nurates_gb300.h"
#include "bnsn_constants.h"
#include "bnsn_internal.h"

using namespace bnsn;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* where)
{
    return fail(BNSN_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Per-device state: SM count, GP19 table and host-API staging buffers.
struct DeviceState
{
    int num_sms  = 0;
    bool gp19    = false;
    Gp19Dev g    = {};
    void* g_buf  = nullptr;
    void* stage  = nullptr; // staging area of the host-buffer APIs
    size_t stage_bytes = 0;
    cudaStream_t streams[2] = {nullptr, nullptr};
    cudaStream_t aux   = nullptr; // second stream of the grey chunk pipeline
    cudaMemPool_t pool = nullptr; // grey scratch records
};

// Points per grey scratch chunk: 8192 records of 6.4 KB (52 MB) stay resident
// in L2 between the phase kernels of a chunk (the batched-blocks autotuner
// picks this size on most configurations).
constexpr int64_t kGreyChunk = 8192;

std::mutex g_mu;
std::map<int, DeviceState> g_dev;

int device_state(DeviceState** out)
{
    int dev = 0, ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(BNSN_ERR_NO_DEVICE, "no CUDA device");
    if ((e = cudaGetDevice(&dev)) != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceState& st = g_dev[dev];
    if (st.num_sms == 0)
    {
        int major = 0, minor = 0;
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
        if (major != 10 || minor != 3)
            return fail(BNSN_ERR_NO_DEVICE, "device is not sm_103 (GB300)");
        if ((e = cudaDeviceGetAttribute(&st.num_sms, cudaDevAttrMultiProcessorCount, dev)) !=
            cudaSuccess)
            return cuda_fail(e, "cudaDeviceGetAttribute");
        cudaMemPoolProps props = {};
        props.allocType     = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id   = dev;
        if ((e = cudaMemPoolCreate(&st.pool, &props)) != cudaSuccess)
        {
            st.num_sms = 0;
            return cuda_fail(e, "cudaMemPoolCreate");
        }
        uint64_t keep = UINT64_MAX;
        if ((e = cudaMemPoolSetAttribute(st.pool, cudaMemPoolAttrReleaseThreshold, &keep)) !=
            cudaSuccess)
        {
            st.num_sms = 0;
            return cuda_fail(e, "cudaMemPoolSetAttribute");
        }
        if ((e = cudaStreamCreateWithFlags(&st.aux, cudaStreamNonBlocking)) != cudaSuccess)
        {
            st.num_sms = 0;
            return cuda_fail(e, "cudaStreamCreateWithFlags");
        }
    }
    *out = &st;
    return BNSN_OK;
}

double gamma_stirling_36()
{
    // GammaStirling(c_f + 3) of functions.hpp:4460-4471 with the host libm
    const double x = k::CF + 3.;
    return sqrt(6.283185307179586 / x) * pow(x / 2.718281828459045235360287471352, x);
}

int check_quad(const MyQuadrature* q)
{
    if (!q)
        return fail(BNSN_ERR_ARG, "quadrature is NULL");
    if (q->nx < 1 || q->nx > BNSN_NQUAD_MAX)
        return fail(BNSN_ERR_NQUAD, "quadrature order nx must be in 1..20");
    for (int i = 0; i < q->nx; ++i)
        if (!(q->points[i] > 0. && q->points[i] < 1.) || !(q->w[i] > 0.))
            return fail(BNSN_ERR_ARG, "quadrature nodes must lie in (0,1) with w > 0");
    return BNSN_OK;
}

// Flags, parameters and quadrature-derived weights of a launch.
int fill_common(const MyQuadrature* q1, const MyQuadrature* q2, const OpacityFlags* fl,
                const OpacityParams* pa, int stim, OpacityLaunch* L)
{
    int rc;
    if ((rc = check_quad(q1)) || (rc = check_quad(q2)))
        return rc;
    if (!fl || !pa)
        return fail(BNSN_ERR_ARG, "flags/params is NULL");
    if ((int)pa->brem_implementation < 0 || (int)pa->brem_implementation > 2)
        return fail(BNSN_ERR_ARG, "unknown brem_implementation");
    if (stim != 0 && stim != 1)
        return fail(BNSN_ERR_ARG, "stim_abs must be 0 or 1");
    L->use_abs_em = fl->use_abs_em != 0;
    L->use_pair   = fl->use_pair != 0;
    L->use_brem   = fl->use_brem != 0;
    L->use_inel   = fl->use_inelastic_scatt != 0;
    L->use_iso    = fl->use_iso != 0;
    L->use_dU     = pa->use_dU;
    L->use_dm_eff = pa->use_dm_eff;
    L->use_WM_ab  = pa->use_WM_ab;
    L->use_WM_sc  = pa->use_WM_sc;
    L->use_decay  = pa->use_decay;
    L->brem_impl  = (int)pa->brem_implementation;
    L->use_medium = pa->use_NN_medium_corr;
    L->neglect_blocking = pa->neglect_blocking;
    L->stim       = stim;
    L->gamma36    = gamma_stirling_36();
    const int n1 = q1->nx, n2 = q2->nx;
    L->n1 = n1;
    L->n2 = n2;
    for (int i = 0; i < kMaxQ; ++i)
    {
        L->x1[i] = i < n1 ? q1->points[i] : 0.5;
        L->w1[i] = i < n1 ? q1->w[i] : 0.;
        L->x2[i] = i < n2 ? q2->points[i] : 0.5;
        L->w2[i] = i < n2 ? q2->w[i] : 0.;
    }
    for (int a = 0; a < kMaxM; ++a)
    {
        L->B1[a] = L->A1[a] = L->A2[a] = 0.;
        if (a < 2 * n1)
        {
            const int i     = a < n1 ? a : a - n1;
            const double x  = q1->points[i];
            L->B1[a]        = a < n1 ? q1->w[i] : q1->w[i] / (x * x);
        }
        if (a < 2 * n2)
        {
            const int i    = a < n2 ? a : a - n2;
            const double x = q2->points[i], w = q2->w[i];
            L->A1[a]       = a < n2 ? w : w / (x * x);
            L->A2[a]       = a < n2 ? w * x : w / (x * x * x);
        }
    }
    for (int i = 0; i < kMaxQ; ++i)
    {
        const double x = L->x2[i], w = L->w2[i];
        L->wx[i]  = w * x;
        L->wx3[i] = w / (x * x * x);
        L->lx2[i] = log(x);
        L->l1m[i] = log1p(-x);
        L->l1p[i] = log1p(x);
        L->lx1[i] = log(L->x1[i]);
    }
    // unordered energy pairs (a <= b), ordered by the sum of the energy
    // factors so that neighbouring lanes see similar Fermi-integral arguments
    const int M = 2 * n2;
    std::vector<std::pair<double, uint32_t>> cells;
    cells.reserve(M * (M + 1) / 2);
    for (int a = 0; a < M; ++a)
        for (int b = a; b < M; ++b)
        {
            const double fa = a < n2 ? q2->points[a] : 1. / q2->points[a - n2];
            const double fb = b < n2 ? q2->points[b] : 1. / q2->points[b - n2];
            cells.push_back({fa + fb, (uint32_t)a | ((uint32_t)b << 16)});
        }
    std::stable_sort(cells.begin(), cells.end(),
                     [](const auto& u, const auto& v) { return u.first < v.first; });
    L->ncell = (int)cells.size();
    for (int c = 0; c < L->ncell; ++c)
        L->cells[c] = cells[c].second;
    // NES items r * n2^2 + i * n2 + j by ascending max(w, w'): the quadrature
    // cost of an item grows with its extent, and a warp's lanes take
    // consecutive items
    std::vector<std::pair<double, uint16_t>> items;
    items.reserve(2 * n2 * n2);
    for (int r = 0; r < 2; ++r)
        for (int i = 0; i < n2; ++i)
            for (int j = 0; j < n2; ++j)
            {
                const double xi = q2->points[i], xj = q2->points[j];
                const double x  = r ? (1. + xj) / xi : xi * (1. + xj);
                items.push_back({x, (uint16_t)((r * n2 + i) * n2 + j)});
            }
    std::stable_sort(items.begin(), items.end(),
                     [](const auto& u, const auto& v) { return u.first < v.first; });
    for (size_t c = 0; c < items.size(); ++c)
        L->nes_order[c] = items[c].second;
    return BNSN_OK;
}

int fill_points(const bnsn_eos_soa* eos, const bnsn_m1_soa* m1, const bnsn_distr_soa* distr,
                bool need_chi, int64_t npts, OpacityLaunch* L)
{
    if (npts < 0)
        return fail(BNSN_ERR_ARG, "npts < 0");
    if (!eos || !m1)
        return fail(BNSN_ERR_ARG, "eos/m1 is NULL");
    const double* e[11] = {eos->nb,   eos->temp, eos->ye,   eos->yp, eos->yn,     eos->mu_p,
                           eos->mu_n, eos->mu_e, eos->mu_mu, eos->dU, eos->dm_eff};
    for (int f = 0; f < 11; ++f)
    {
        if (!e[f] && f != 8 && npts > 0)
            return fail(BNSN_ERR_ARG, "an eos field pointer is NULL");
        L->eos[f] = e[f];
    }
    for (int s = 0; s < 4; ++s)
    {
        L->m1[s]     = m1->n[s];
        L->m1[4 + s] = m1->J[s];
        L->m1[8 + s] = m1->chi[s];
        if (npts > 0 && (!m1->n[s] || !m1->J[s] || (need_chi && !distr && !m1->chi[s])))
            return fail(BNSN_ERR_ARG, "an m1 field pointer is NULL");
    }
    L->has_distr = distr != nullptr;
    if (distr)
    {
        double* const* d[7] = {distr->w_t,   distr->temp_t, distr->eta_t, distr->w_f,
                               distr->temp_f, distr->c_f,    distr->beta_f};
        for (int q = 0; q < 7; ++q)
            for (int s = 0; s < 4; ++s)
            {
                if (npts > 0 && !d[q][s])
                    return fail(BNSN_ERR_ARG, "a distr field pointer is NULL");
                L->distr[q * 4 + s] = d[q][s];
            }
    }
    L->npts = npts;
    return BNSN_OK;
}

// Device-dependent part of a launch: SM count and the GP19 table.
int attach_device(OpacityLaunch* L, DeviceState** st)
{
    int rc = device_state(st);
    if (rc)
        return rc;
    if (L->use_brem && L->brem_impl == BREM_GP19)
    {
        if (!(*st)->gp19)
            return fail(BNSN_ERR_NO_TABLE, "GP19 brem requested but no table loaded");
        L->gp19 = (*st)->g;
    }
    return BNSN_OK;
}

} // namespace

int bnsn::capi_fail(int code, const char* msg) { return fail(code, msg); }
int bnsn::capi_cuda_fail(cudaError_t e, const char* where) { return cuda_fail(e, where); }
int bnsn::capi_fill_launch(const void* q1, const void* q2, const void* fl, const void* pa,
                           int stim, OpacityLaunch* L)
{
    return fill_common((const MyQuadrature*)q1, (const MyQuadrature*)q2, (const OpacityFlags*)fl,
                       (const OpacityParams*)pa, stim, L);
}
int bnsn::capi_device_info(DeviceInfo* info)
{
    DeviceState* st;
    const int rc = device_state(&st);
    if (rc)
        return rc;
    info->num_sms  = st->num_sms;
    info->gp19     = st->g;
    info->has_gp19 = st->gp19;
    return BNSN_OK;
}

// ---------------------------------------------------------------------------
// phase timing and launch counting
// ---------------------------------------------------------------------------
namespace {

std::atomic<int64_t> g_launches{0};
std::atomic<int> g_timing{0};
std::mutex g_timer_mu;
std::vector<cudaEvent_t> g_ev_pool;   // events owned by the timer
std::vector<std::pair<int, size_t>> g_ev_marks; // phase, index of the start event
size_t g_ev_used = 0;

} // namespace

void bnsn::phase_mark(int phase, int end, cudaStream_t stream)
{
    if (end)
        g_launches.fetch_add(1, std::memory_order_relaxed);
    if (!g_timing.load(std::memory_order_relaxed))
        return;
    std::lock_guard<std::mutex> lk(g_timer_mu);
    if (g_ev_used == g_ev_pool.size())
    {
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess)
            return;
        g_ev_pool.push_back(ev);
    }
    if (!end)
        g_ev_marks.push_back({phase, g_ev_used});
    cudaEventRecord(g_ev_pool[g_ev_used++], stream);
}

extern "C" {

int bnsn_phase_timing(int enable)
{
    g_timing.store(enable ? 1 : 0);
    return BNSN_OK;
}

int bnsn_phase_times(double* ms, int64_t* launches)
{
    g_err.clear();
    if (!ms || !launches)
        return fail(BNSN_ERR_ARG, "ms/launches is NULL");
    for (int q = 0; q < BNSN_NUM_PHASES; ++q)
    {
        ms[q]       = 0.;
        launches[q] = 0;
    }
    std::lock_guard<std::mutex> lk(g_timer_mu);
    int rc = BNSN_OK;
    for (const auto& m : g_ev_marks)
    {
        if (m.second + 1 >= g_ev_used)
            break;
        float t = 0.f;
        cudaError_t e = cudaEventSynchronize(g_ev_pool[m.second + 1]);
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&t, g_ev_pool[m.second], g_ev_pool[m.second + 1]);
        if (e != cudaSuccess)
        {
            rc = cuda_fail(e, "phase timing");
            break;
        }
        if (m.first >= 0 && m.first < BNSN_NUM_PHASES)
        {
            ms[m.first] += t;
            launches[m.first] += 1;
        }
    }
    g_ev_marks.clear();
    g_ev_used = 0;
    return rc;
}

int64_t bnsn_kernel_launches(void) { return g_launches.load(); }

int bnsn_spectral_mixed_stats(int64_t* counts, int reset)
{
    g_err.clear();
    if (!counts)
        return fail(BNSN_ERR_ARG, "NULL output");
    unsigned long long c[4] = {0ull, 0ull, 0ull, 0ull};
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = spectral_mixed_counts(c, reset != 0);
    if (e != cudaSuccess)
        return cuda_fail(e, "reading the spectral statistics");
    for (int k = 0; k < 4; ++k)
        counts[k] = (int64_t)c[k];
    return BNSN_OK;
}


int bnsn_grey_mixed_stats(int64_t* counts, int reset)
{
    g_err.clear();
    if (!counts)
        return fail(BNSN_ERR_ARG, "NULL output");
    unsigned long long c[5] = {0ull, 0ull, 0ull, 0ull, 0ull};
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = grey_mixed_counts(c, reset != 0);
    if (e != cudaSuccess)
        return cuda_fail(e, "reading the grey mixed-path statistics");
    for (int k = 0; k < 5; ++k)
        counts[k] = (int64_t)c[k];
    return BNSN_OK;
}

int bnsn_nonfinite_outputs(int64_t* counts, int reset)
{
    g_err.clear();
    if (!counts)
        return fail(BNSN_ERR_ARG, "NULL output");
    unsigned long long g = 0ull, sp = 0ull;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = grey_nonfinite_count(&g, reset != 0);
    if (e == cudaSuccess)
        e = spectral_nonfinite_count(&sp, reset != 0);
    if (e != cudaSuccess)
        return cuda_fail(e, "reading the non-finite output counters");
    counts[0] = (int64_t)g;
    counts[1] = (int64_t)sp;
    return BNSN_OK;
}

int bnsn_version(void) { return 100; }

const char* bnsn_last_error(void) { return g_err.c_str(); }

const char* bnsn_status_string(int status)
{
    switch (status)
    {
    case BNSN_OK: return "ok";
    case BNSN_ERR_ARG: return "invalid argument";
    case BNSN_ERR_NQUAD: return "quadrature order out of range";
    case BNSN_ERR_CUDA: return "CUDA error";
    case BNSN_ERR_NO_TABLE: return "GP19 table not loaded";
    case BNSN_ERR_NO_DEVICE: return "no usable GB300 device";
    default: return "unknown status";
    }
}

int bnsn_m1_opacities(const MyQuadrature* quad_1d, const MyQuadrature* quad_2d,
                      const OpacityFlags* flags, const OpacityParams* params,
                      const bnsn_eos_soa* eos, const bnsn_m1_soa* m1,
                      const bnsn_distr_soa* distr, int stim_abs, int precision,
                      const bnsn_m1_opacities_soa* out, int64_t npts, void* stream)
{
    g_err.clear();
    if (precision != BNSN_FP64 && precision != BNSN_MIXED)
        return fail(BNSN_ERR_ARG, "unknown precision");
    if (!out)
        return fail(BNSN_ERR_ARG, "out is NULL");
    OpacityLaunch L;
    memset(&L, 0, sizeof(L));
    int rc;
    if ((rc = fill_common(quad_1d, quad_2d, flags, params, stim_abs, &L)))
        return rc;
    if ((rc = fill_points(eos, m1, distr, true, npts, &L)))
        return rc;
    double* const* o[5] = {out->eta_0, out->kappa_0_a, out->eta, out->kappa_a, out->kappa_s};
    for (int q = 0; q < 5; ++q)
        for (int s = 0; s < 4; ++s)
        {
            if (npts > 0 && !o[q][s])
                return fail(BNSN_ERR_ARG, "an output pointer is NULL");
            L.out[q * 4 + s] = o[q][s];
        }
    L.mixed = precision == BNSN_MIXED;
    DeviceState* st;
    if ((rc = attach_device(&L, &st)))
        return rc;
    if (npts == 0)
        return BNSN_OK;
    // more than one chunk: two chunks in flight on the caller's stream and aux
    const bool two          = npts > kGreyChunk;
    const int64_t ws_points = two ? 2 * kGreyChunk : npts;
    double* ws = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync((void**)&ws, ws_points * grey_point_scratch_bytes(),
                                           st->pool, (cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "grey scratch allocation");
    e = launch_grey(L, (cudaStream_t)stream, st->num_sms, ws, ws_points,
                    two ? st->aux : nullptr);
    const cudaError_t ef = cudaFreeAsync(ws, (cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "grey kernel launch");
    return ef == cudaSuccess ? BNSN_OK : cuda_fail(ef, "grey scratch release");
}

// Grey opacities with the per-point scratch in a static device array instead
// of the stream-ordered pool: for callers that must not allocate device memory
// inside the call (see the header).  Same arguments and results as
// bnsn_m1_opacities, at most BNSN_NOALLOC_MAX_POINTS points per call.
int bnsn_m1_opacities_noalloc(const MyQuadrature* quad_1d, const MyQuadrature* quad_2d,
                              const OpacityFlags* flags, const OpacityParams* params,
                              const bnsn_eos_soa* eos, const bnsn_m1_soa* m1,
                              const bnsn_distr_soa* distr, int stim_abs, int precision,
                              const bnsn_m1_opacities_soa* out, int64_t npts, void* stream)
{
    static_assert(BNSN_NOALLOC_MAX_POINTS == kNoAllocPoints, "static scratch capacity");
    g_err.clear();
    if (precision != BNSN_FP64 && precision != BNSN_MIXED)
        return fail(BNSN_ERR_ARG, "unknown precision");
    if (!out)
        return fail(BNSN_ERR_ARG, "out is NULL");
    OpacityLaunch L;
    memset(&L, 0, sizeof(L));
    int rc;
    if ((rc = fill_common(quad_1d, quad_2d, flags, params, stim_abs, &L)))
        return rc;
    if ((rc = fill_points(eos, m1, distr, true, npts, &L)))
        return rc;
    if (npts > kNoAllocPoints)
        return fail(BNSN_ERR_ARG, "npts = " + std::to_string(npts) +
                                      " exceeds BNSN_NOALLOC_MAX_POINTS = 4096, the capacity of "
                                      "the static scratch: split the batch, or call "
                                      "bnsn_m1_opacities");
    double* const* o[5] = {out->eta_0, out->kappa_0_a, out->eta, out->kappa_a, out->kappa_s};
    for (int q = 0; q < 5; ++q)
        for (int s = 0; s < 4; ++s)
        {
            if (npts > 0 && !o[q][s])
                return fail(BNSN_ERR_ARG, "an output pointer is NULL");
            L.out[q * 4 + s] = o[q][s];
        }
    L.mixed = precision == BNSN_MIXED;
    // device checks without the per-device state of the pooled calls (whose
    // first use creates the memory pool)
    int dev = 0, ndev = 0, major = 0, minor = 0, sms = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(BNSN_ERR_NO_DEVICE, "no CUDA device");
    if ((e = cudaGetDevice(&dev)) != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3)
        return fail(BNSN_ERR_NO_DEVICE, "device is not sm_103 (GB300)");
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return cuda_fail(e, "cudaDeviceGetAttribute");
    if (L.use_brem && L.brem_impl == BREM_GP19)
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_dev.find(dev);
        if (it == g_dev.end() || !it->second.gp19)
            return fail(BNSN_ERR_NO_TABLE, "GP19 brem requested but no table loaded");
        L.gp19 = it->second.g;
    }
    double* ws = nullptr;
    if ((e = noalloc_scratch(dev, &ws)) != cudaSuccess)
        return cuda_fail(e, "cudaGetSymbolAddress(static grey scratch)");
    if (npts == 0)
        return BNSN_OK;
    e = launch_grey(L, (cudaStream_t)stream, sms, ws, kNoAllocPoints);
    return e == cudaSuccess ? BNSN_OK : cuda_fail(e, "grey kernel launch");
}

int bnsn_spectral_opacities(const MyQuadrature* quad_1d, const OpacityFlags* flags,
                            const OpacityParams* params, const bnsn_eos_soa* eos,
                            const bnsn_m1_soa* m1, const bnsn_distr_soa* distr,
                            const double* energies, int n_energies, int stimulated,
                            int precision, const bnsn_spectral_soa* out, int64_t npts,
                            void* stream)
{
    g_err.clear();
    if (precision != BNSN_FP64 && precision != BNSN_MIXED)
        return fail(BNSN_ERR_ARG, "unknown precision");
    if (!out || (n_energies > 0 && !energies) || n_energies < 0)
        return fail(BNSN_ERR_ARG, "out/energies invalid");
    for (int e = 0; e < n_energies; ++e)
        if (!(energies[e] > 0.))
            return fail(BNSN_ERR_ARG, "energies must be positive");
    OpacityLaunch L;
    memset(&L, 0, sizeof(L));
    int rc;
    if ((rc = fill_common(quad_1d, quad_1d, flags, params, stimulated, &L)))
        return rc;
    if ((rc = fill_points(eos, m1, distr, true, npts, &L)))
        return rc;
    double* const* o[4] = {out->j, out->kappa, out->j_s, out->kappa_s};
    for (int q = 0; q < 4; ++q)
        for (int s = 0; s < 4; ++s)
        {
            if (npts > 0 && n_energies > 0 && !o[q][s])
                return fail(BNSN_ERR_ARG, "an output pointer is NULL");
            L.sout[q * 4 + s] = o[q][s];
        }
    L.mixed = precision == BNSN_MIXED;
    DeviceState* st;
    if ((rc = attach_device(&L, &st)))
        return rc;
    L.e_stride = n_energies;
    if (npts == 0 || n_energies == 0)
        return BNSN_OK;
    const int ne_max     = n_energies < 64 ? n_energies : 64;
    const int64_t chunk  = std::min<int64_t>(npts, spectral_chunk_points(ne_max));
    // more than one chunk: a second scratch, chunks alternating with the aux stream
    const bool two       = npts > chunk && st->aux != nullptr;
    const size_t wbytes  = spectral_scratch_bytes(chunk, ne_max);
    const size_t wpad    = (wbytes + 255) & ~(size_t)255;
    void* ws             = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&ws, two ? wpad + wbytes : wbytes, st->pool,
                                            (cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "spectral scratch allocation");
    void* ws1 = two ? (void*)((char*)ws + wpad) : nullptr;
    for (int e0 = 0; e0 < n_energies && e == cudaSuccess; e0 += 64)
    {
        L.n_energies = (n_energies - e0) < 64 ? (n_energies - e0) : 64;
        L.e_offset   = e0;
        for (int k = 0; k < L.n_energies; ++k)
            L.energies[k] = energies[e0 + k];
        e = launch_spectral(L, (cudaStream_t)stream, st->num_sms, ws, chunk,
                            two ? st->aux : nullptr, ws1);
    }
    const cudaError_t ef = cudaFreeAsync(ws, (cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "spectral kernel launch");
    return ef == cudaSuccess ? BNSN_OK : cuda_fail(ef, "spectral scratch release");
}

int bnsn_distr_from_m1(const bnsn_m1_soa* m1, const bnsn_distr_soa* out, int64_t npts,
                       void* stream)
{
    g_err.clear();
    if (!m1 || !out || npts < 0)
        return fail(BNSN_ERR_ARG, "invalid argument");
    DistrLaunch L;
    memset(&L, 0, sizeof(L));
    L.npts    = npts;
    L.gamma36 = gamma_stirling_36();
    double* const* d[7] = {out->w_t,   out->temp_t, out->eta_t, out->w_f,
                           out->temp_f, out->c_f,    out->beta_f};
    for (int s = 0; s < 4; ++s)
    {
        L.m1[s]     = m1->n[s];
        L.m1[4 + s] = m1->J[s];
        L.m1[8 + s] = m1->chi[s];
        if (npts > 0 && (!m1->n[s] || !m1->J[s] || !m1->chi[s]))
            return fail(BNSN_ERR_ARG, "an m1 field pointer is NULL");
        for (int q = 0; q < 7; ++q)
        {
            if (npts > 0 && !d[q][s])
                return fail(BNSN_ERR_ARG, "a distr field pointer is NULL");
            L.out[q * 4 + s] = d[q][s];
        }
    }
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    cudaError_t e = launch_distr_from_m1(L, (cudaStream_t)stream, st->num_sms);
    return e == cudaSuccess ? BNSN_OK : cuda_fail(e, "distr kernel launch");
}

int bnsn_nu_equilibrium(const bnsn_eos_soa* eos, const bnsn_distr_soa* distr_out,
                        double* const n_out[total_num_species],
                        double* const J_out[total_num_species],
                        double* const chi_out[total_num_species], int64_t npts,
                        void* stream)
{
    g_err.clear();
    if (!eos || !distr_out || !n_out || !J_out || !chi_out || npts < 0)
        return fail(BNSN_ERR_ARG, "invalid argument");
    EquilLaunch L;
    memset(&L, 0, sizeof(L));
    L.npts              = npts;
    const double* e[11] = {eos->nb,   eos->temp, eos->ye,   eos->yp, eos->yn,     eos->mu_p,
                           eos->mu_n, eos->mu_e, eos->mu_mu, eos->dU, eos->dm_eff};
    for (int f = 0; f < 11; ++f)
        L.eos[f] = e[f];
    if (npts > 0 && (!eos->temp || !eos->mu_p || !eos->mu_n || !eos->mu_e))
        return fail(BNSN_ERR_ARG, "eos temp/mu pointers are NULL");
    double* const* d[7] = {distr_out->w_t,   distr_out->temp_t, distr_out->eta_t,
                           distr_out->w_f,   distr_out->temp_f, distr_out->c_f,
                           distr_out->beta_f};
    for (int s = 0; s < 4; ++s)
    {
        for (int q = 0; q < 7; ++q)
            L.distr[q * 4 + s] = d[q][s];
        L.m1[s]     = n_out[s];
        L.m1[4 + s] = J_out[s];
        L.m1[8 + s] = chi_out[s];
    }
    for (int f = 0; f < 28; ++f)
        if (npts > 0 && !L.distr[f])
            return fail(BNSN_ERR_ARG, "a distr output pointer is NULL");
    for (int f = 0; f < 12; ++f)
        if (npts > 0 && !L.m1[f])
            return fail(BNSN_ERR_ARG, "an m1 output pointer is NULL");
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    cudaError_t err = launch_nu_equilibrium(L, (cudaStream_t)stream, st->num_sms);
    return err == cudaSuccess ? BNSN_OK : cuda_fail(err, "equilibrium kernel launch");
}

int bnsn_gp19_set_table(const int dims[4], const double* nb_axis, const double* ye_axis,
                        const double* t_axis, const double* w_axis,
                        const double* lognb_axis, const double* logw_axis,
                        const double* data)
{
    g_err.clear();
    if (!dims || !nb_axis || !ye_axis || !t_axis || !w_axis || !data)
        return fail(BNSN_ERR_ARG, "GP19 table pointer is NULL");
    for (int q = 0; q < 4; ++q)
        if (dims[q] < 2 || dims[q] > (1 << 20))
            return fail(BNSN_ERR_ARG, "GP19 table dimensions must be >= 2");
    const double* axes[4] = {nb_axis, ye_axis, t_axis, w_axis};
    for (int q = 0; q < 4; ++q)
        for (int i = 0; i + 1 < dims[q]; ++i)
            if (!(axes[q][i] < axes[q][i + 1]))
                return fail(BNSN_ERR_ARG, "GP19 axes must be strictly increasing");
    if (!(nb_axis[0] > 0.) || !(w_axis[0] > 0.))
        return fail(BNSN_ERR_ARG, "GP19 nb and w axes must be positive");
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    const size_t nd = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
    const size_t na = (size_t)2 * dims[0] + dims[1] + dims[2] + 2 * dims[3];
    std::vector<double> host(na + nd);
    size_t off = 0;
    auto put   = [&](const double* src, int n) {
        memcpy(&host[off], src, sizeof(double) * n);
        off += n;
    };
    std::vector<double> lnb(dims[0]), lw(dims[3]);
    for (int i = 0; i < dims[0]; ++i)
        lnb[i] = lognb_axis ? lognb_axis[i] : log(nb_axis[i]);
    for (int i = 0; i < dims[3]; ++i)
        lw[i] = logw_axis ? logw_axis[i] : log(w_axis[i]);
    put(nb_axis, dims[0]);
    put(ye_axis, dims[1]);
    put(t_axis, dims[2]);
    put(w_axis, dims[3]);
    put(lnb.data(), dims[0]);
    put(lw.data(), dims[3]);
    put(data, (int)nd);
    std::lock_guard<std::mutex> lk(g_mu);
    if (st->g_buf)
    {
        cudaDeviceSynchronize();
        cudaFree(st->g_buf);
        st->g_buf = nullptr;
        st->gp19  = false;
    }
    cudaError_t e = cudaMalloc(&st->g_buf, sizeof(double) * host.size());
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMalloc(GP19)");
    e = cudaMemcpy(st->g_buf, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(GP19)");
    const double* b = (const double*)st->g_buf;
    st->g.d0    = dims[0];
    st->g.d1    = dims[1];
    st->g.d2    = dims[2];
    st->g.d3    = dims[3];
    st->g.nb    = b;
    st->g.ye    = b + dims[0];
    st->g.t     = b + dims[0] + dims[1];
    st->g.w     = b + dims[0] + dims[1] + dims[2];
    st->g.lognb = st->g.w + dims[3];
    st->g.logw  = st->g.lognb + dims[0];
    st->g.data  = st->g.logw + dims[3];
    st->gp19    = true;
    return BNSN_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Per-point drop-ins and the host-buffer batch: staged through a per-device
// buffer (grown on demand, kept for the process lifetime).
// ---------------------------------------------------------------------------
namespace {

int stage(DeviceState* st, size_t bytes, double** out)
{
    if (st->stage_bytes < bytes)
    {
        if (st->stage)
        {
            cudaDeviceSynchronize();
            cudaFree(st->stage);
            st->stage       = nullptr;
            st->stage_bytes = 0;
        }
        cudaError_t e = cudaMalloc(&st->stage, bytes);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaMalloc(staging)");
        st->stage_bytes = bytes;
    }
    if (!st->streams[0])
    {
        cudaStreamCreateWithFlags(&st->streams[0], cudaStreamNonBlocking);
        cudaStreamCreateWithFlags(&st->streams[1], cudaStreamNonBlocking);
    }
    *out = (double*)st->stage;
    return BNSN_OK;
}

std::mutex g_stage_mu;

} // namespace

extern "C" int bnsn_compute_m1_opacities_point(const MyQuadrature* quad_1d,
                                               const MyQuadrature* quad_2d,
                                               const GreyOpacityParams* gp, int stim_abs,
                                               M1Opacities* out)
{
    g_err.clear();
    if (!gp || !out)
        return fail(BNSN_ERR_ARG, "grey_pars/out is NULL");
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    std::lock_guard<std::mutex> lk(g_stage_mu);
    double* buf;
    if ((rc = stage(st, sizeof(double) * (11 + 12 + 28 + 20), &buf)))
        return rc;
    double h[11 + 12 + 28];
    const MyEOSParams& e = gp->eos_pars;
    const double ev[11]  = {e.nb, e.temp, e.ye, e.yp, e.yn, e.mu_p, e.mu_n, e.mu_e, e.mu_mu,
                           e.dU, e.dm_eff};
    memcpy(h, ev, sizeof(ev));
    for (int s = 0; s < 4; ++s)
    {
        h[11 + s]     = gp->m1_pars.n[s];
        h[11 + 4 + s] = gp->m1_pars.J[s];
        h[11 + 8 + s] = gp->m1_pars.chi[s];
    }
    memcpy(h + 23, &gp->distr_pars, sizeof(double) * 28);
    cudaStream_t s0 = st->streams[0];
    cudaError_t err = cudaMemcpyAsync(buf, h, sizeof(h), cudaMemcpyHostToDevice, s0);
    if (err != cudaSuccess)
        return cuda_fail(err, "cudaMemcpyAsync");
    bnsn_eos_soa E = {buf + 0, buf + 1, buf + 2, buf + 3, buf + 4, buf + 5,
                      buf + 6, buf + 7, buf + 8, buf + 9, buf + 10};
    bnsn_m1_soa Mq;
    bnsn_distr_soa D;
    bnsn_m1_opacities_soa O;
    for (int s = 0; s < 4; ++s)
    {
        Mq.n[s]   = buf + 11 + s;
        Mq.J[s]   = buf + 15 + s;
        Mq.chi[s] = buf + 19 + s;
        double* db = buf + 23;
        D.w_t[s] = db + s;
        D.temp_t[s] = db + 4 + s;
        D.eta_t[s] = db + 8 + s;
        D.w_f[s] = db + 12 + s;
        D.temp_f[s] = db + 16 + s;
        D.c_f[s] = db + 20 + s;
        D.beta_f[s] = db + 24 + s;
        double* ob = buf + 51;
        O.eta_0[s] = ob + s;
        O.kappa_0_a[s] = ob + 4 + s;
        O.eta[s] = ob + 8 + s;
        O.kappa_a[s] = ob + 12 + s;
        O.kappa_s[s] = ob + 16 + s;
    }
    if ((rc = bnsn_m1_opacities(quad_1d, quad_2d, &gp->opacity_flags, &gp->opacity_pars, &E,
                                &Mq, &D, stim_abs, BNSN_FP64, &O, 1, s0)))
        return rc;
    double o[20];
    err = cudaMemcpyAsync(o, buf + 51, sizeof(o), cudaMemcpyDeviceToHost, s0);
    if (err == cudaSuccess)
        err = cudaStreamSynchronize(s0);
    if (err != cudaSuccess)
        return cuda_fail(err, "point result copy");
    memcpy(out, o, sizeof(o));
    return BNSN_OK;
}

extern "C" int bnsn_fdi(int twice_order, const double* x, double* out, int64_t n, void* stream)
{
    g_err.clear();
    if (!fdi_order_valid(twice_order))
        return fail(BNSN_ERR_ARG, "twice_order must be -9, -7, -5, -3, -1 or 0..21");
    if (n < 0 || (n > 0 && (!x || !out)))
        return fail(BNSN_ERR_ARG, "invalid argument");
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    cudaError_t e = launch_fdi(twice_order, x, out, n, (cudaStream_t)stream, st->num_sms);
    return e == cudaSuccess ? BNSN_OK : cuda_fail(e, "fdi kernel launch");
}

extern "C" int bnsn_pair_j_mixed(const double* y, const double* z, const double* eta, double* j0,
                                 double* j1, double* lscale, int64_t n, void* stream)
{
    g_err.clear();
    if (n < 0 || (n > 0 && (!y || !z || !eta || !j0 || !j1 || !lscale)))
        return fail(BNSN_ERR_ARG, "invalid argument");
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    cudaError_t e = launch_pair_j(y, z, eta, j0, j1, lscale, n, (cudaStream_t)stream,
                                  st->num_sms);
    return e == cudaSuccess ? BNSN_OK : cuda_fail(e, "pair integral kernel launch");
}

extern "C" int bnsn_nes_m_mixed(const double* w, const double* wp, const double* eta, double* m1,
                                double* m2, double* lscale, int64_t n, void* stream)
{
    g_err.clear();
    if (n < 0 || (n > 0 && (!w || !wp || !eta || !m1 || !m2 || !lscale)))
        return fail(BNSN_ERR_ARG, "invalid argument");
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    cudaError_t e = launch_nes_m(w, wp, eta, m1, m2, lscale, n, (cudaStream_t)stream,
                                 st->num_sms);
    return e == cudaSuccess ? BNSN_OK : cuda_fail(e, "NES integral kernel launch");
}

extern "C" int bnsn_fdi_host(int twice_order, const double* x, double* out, int64_t n)
{
    g_err.clear();
    if (!fdi_order_valid(twice_order))
        return fail(BNSN_ERR_ARG, "twice_order must be -9, -7, -5, -3, -1 or 0..21");
    if (n < 0 || (n > 0 && (!x || !out)))
        return fail(BNSN_ERR_ARG, "invalid argument");
    if (n == 0)
        return BNSN_OK;
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    const int64_t chunk = std::min<int64_t>(n, (int64_t)1 << 22);
    std::lock_guard<std::mutex> lk(g_stage_mu);
    double* buf;
    if ((rc = stage(st, sizeof(double) * 2 * chunk, &buf)))
        return rc;
    cudaStream_t s0 = st->streams[0];
    for (int64_t p0 = 0; p0 < n; p0 += chunk)
    {
        const int64_t m = std::min<int64_t>(chunk, n - p0);
        cudaError_t err = cudaMemcpyAsync(buf, x + p0, sizeof(double) * m,
                                          cudaMemcpyHostToDevice, s0);
        if (err == cudaSuccess)
            err = launch_fdi(twice_order, buf, buf + chunk, m, s0, st->num_sms);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(out + p0, buf + chunk, sizeof(double) * m,
                                  cudaMemcpyDeviceToHost, s0);
        if (err != cudaSuccess)
            return cuda_fail(err, "fdi host batch");
    }
    cudaError_t err = cudaStreamSynchronize(s0);
    return err == cudaSuccess ? BNSN_OK : cuda_fail(err, "fdi host batch");
}

extern "C" int bnsn_distr_from_m1_point(const M1Quantities* m1, NuDistributionParams* out)
{
    g_err.clear();
    if (!m1 || !out)
        return fail(BNSN_ERR_ARG, "m1/out is NULL");
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    std::lock_guard<std::mutex> lk(g_stage_mu);
    double* buf;
    if ((rc = stage(st, sizeof(double) * (12 + 28), &buf)))
        return rc;
    double h[12];
    for (int s = 0; s < 4; ++s)
    {
        h[s]     = m1->n[s];
        h[4 + s] = m1->J[s];
        h[8 + s] = m1->chi[s];
    }
    cudaStream_t s0 = st->streams[0];
    cudaError_t err = cudaMemcpyAsync(buf, h, sizeof(h), cudaMemcpyHostToDevice, s0);
    if (err != cudaSuccess)
        return cuda_fail(err, "cudaMemcpyAsync");
    bnsn_m1_soa Mq;
    bnsn_distr_soa D;
    double* db = buf + 12; // NuDistributionParams field order, 7 x 4
    for (int s = 0; s < 4; ++s)
    {
        Mq.n[s]     = buf + s;
        Mq.J[s]     = buf + 4 + s;
        Mq.chi[s]   = buf + 8 + s;
        D.w_t[s]    = db + s;
        D.temp_t[s] = db + 4 + s;
        D.eta_t[s]  = db + 8 + s;
        D.w_f[s]    = db + 12 + s;
        D.temp_f[s] = db + 16 + s;
        D.c_f[s]    = db + 20 + s;
        D.beta_f[s] = db + 24 + s;
    }
    if ((rc = bnsn_distr_from_m1(&Mq, &D, 1, s0)))
        return rc;
    double o[28];
    err = cudaMemcpyAsync(o, db, sizeof(o), cudaMemcpyDeviceToHost, s0);
    if (err == cudaSuccess)
        err = cudaStreamSynchronize(s0);
    if (err != cudaSuccess)
        return cuda_fail(err, "point result copy");
    static_assert(sizeof(NuDistributionParams) == sizeof(o), "NuDistributionParams layout");
    memcpy(out, o, sizeof(o));
    return BNSN_OK;
}

extern "C" int bnsn_compute_spectral_opacities_point(double nu, const MyQuadrature* quad_1d,
                                                     const GreyOpacityParams* gp,
                                                     int stimulated, SpectralOpacities* out)
{
    g_err.clear();
    if (!gp || !out)
        return fail(BNSN_ERR_ARG, "grey_pars/out is NULL");
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    std::lock_guard<std::mutex> lk(g_stage_mu);
    double* buf;
    if ((rc = stage(st, sizeof(double) * (11 + 12 + 28 + 16), &buf)))
        return rc;
    double h[11 + 12 + 28];
    const MyEOSParams& e = gp->eos_pars;
    const double ev[11]  = {e.nb, e.temp, e.ye, e.yp, e.yn, e.mu_p, e.mu_n, e.mu_e, e.mu_mu,
                           e.dU, e.dm_eff};
    memcpy(h, ev, sizeof(ev));
    for (int s = 0; s < 4; ++s)
    {
        h[11 + s]     = gp->m1_pars.n[s];
        h[11 + 4 + s] = gp->m1_pars.J[s];
        h[11 + 8 + s] = gp->m1_pars.chi[s];
    }
    memcpy(h + 23, &gp->distr_pars, sizeof(double) * 28);
    cudaStream_t s0 = st->streams[0];
    cudaError_t err = cudaMemcpyAsync(buf, h, sizeof(h), cudaMemcpyHostToDevice, s0);
    if (err != cudaSuccess)
        return cuda_fail(err, "cudaMemcpyAsync");
    bnsn_eos_soa E = {buf + 0, buf + 1, buf + 2, buf + 3, buf + 4, buf + 5,
                      buf + 6, buf + 7, buf + 8, buf + 9, buf + 10};
    bnsn_m1_soa Mq;
    bnsn_distr_soa D;
    bnsn_spectral_soa O;
    for (int s = 0; s < 4; ++s)
    {
        Mq.n[s]     = buf + 11 + s;
        Mq.J[s]     = buf + 15 + s;
        Mq.chi[s]   = buf + 19 + s;
        double* db  = buf + 23;
        D.w_t[s]    = db + s;
        D.temp_t[s] = db + 4 + s;
        D.eta_t[s]  = db + 8 + s;
        D.w_f[s]    = db + 12 + s;
        D.temp_f[s] = db + 16 + s;
        D.c_f[s]    = db + 20 + s;
        D.beta_f[s] = db + 24 + s;
        double* ob  = buf + 51;
        O.j[s]       = ob + s;
        O.kappa[s]   = ob + 4 + s;
        O.j_s[s]     = ob + 8 + s;
        O.kappa_s[s] = ob + 12 + s;
    }
    if ((rc = bnsn_spectral_opacities(quad_1d, &gp->opacity_flags, &gp->opacity_pars, &E, &Mq,
                                      &D, &nu, 1, stimulated, BNSN_FP64, &O, 1, s0)))
        return rc;
    double o[16];
    err = cudaMemcpyAsync(o, buf + 51, sizeof(o), cudaMemcpyDeviceToHost, s0);
    if (err == cudaSuccess)
        err = cudaStreamSynchronize(s0);
    if (err != cudaSuccess)
        return cuda_fail(err, "point result copy");
    memcpy(out, o, sizeof(o));
    return BNSN_OK;
}

extern "C" int bnsn_m1_opacities_host(const MyQuadrature* quad_1d, const MyQuadrature* quad_2d,
                                      const OpacityFlags* flags, const OpacityParams* params,
                                      const bnsn_eos_soa* eos, const bnsn_m1_soa* m1,
                                      int stim_abs, int precision,
                                      const bnsn_m1_opacities_soa* out, int64_t npts)
{
    g_err.clear();
    if (!eos || !m1 || !out || npts < 0)
        return fail(BNSN_ERR_ARG, "invalid argument");
    if (npts == 0)
        return BNSN_OK;
    DeviceState* st;
    int rc = device_state(&st);
    if (rc)
        return rc;
    // 11 eos + 12 m1 inputs and 20 outputs per point, two chunks in flight
    const int64_t chunk = std::min<int64_t>(npts, (int64_t)1 << 20);
    const int nfield    = 11 + 12 + 20;
    std::lock_guard<std::mutex> lk(g_stage_mu);
    double* buf;
    if ((rc = stage(st, sizeof(double) * nfield * chunk * 2, &buf)))
        return rc;
    const double* hin[23] = {eos->nb,   eos->temp, eos->ye,   eos->yp, eos->yn,     eos->mu_p,
                             eos->mu_n, eos->mu_e, eos->mu_mu, eos->dU, eos->dm_eff};
    for (int s = 0; s < 4; ++s)
    {
        hin[11 + s] = m1->n[s];
        hin[15 + s] = m1->J[s];
        hin[19 + s] = m1->chi[s];
    }
    double* const* ho[5] = {out->eta_0, out->kappa_0_a, out->eta, out->kappa_a, out->kappa_s};
    int slot = 0;
    for (int64_t p0 = 0; p0 < npts; p0 += chunk, slot ^= 1)
    {
        const int64_t m  = std::min<int64_t>(chunk, npts - p0);
        cudaStream_t s   = st->streams[slot];
        double* base     = buf + (size_t)slot * nfield * chunk;
        cudaError_t err  = cudaSuccess;
        for (int f = 0; f < 23 && err == cudaSuccess; ++f)
            if (hin[f])
                err = cudaMemcpyAsync(base + (size_t)f * chunk, hin[f] + p0, sizeof(double) * m,
                                      cudaMemcpyHostToDevice, s);
        if (err != cudaSuccess)
            return cuda_fail(err, "input copy");
        bnsn_eos_soa E;
        const double** ef = (const double**)&E;
        for (int f = 0; f < 11; ++f)
            ef[f] = hin[f] ? base + (size_t)f * chunk : nullptr;
        bnsn_m1_soa Mq;
        bnsn_m1_opacities_soa O;
        for (int sp = 0; sp < 4; ++sp)
        {
            Mq.n[sp]   = base + (size_t)(11 + sp) * chunk;
            Mq.J[sp]   = base + (size_t)(15 + sp) * chunk;
            Mq.chi[sp] = base + (size_t)(19 + sp) * chunk;
            double* ob = base + (size_t)23 * chunk;
            O.eta_0[sp]     = ob + (size_t)(0 + sp) * chunk;
            O.kappa_0_a[sp] = ob + (size_t)(4 + sp) * chunk;
            O.eta[sp]       = ob + (size_t)(8 + sp) * chunk;
            O.kappa_a[sp]   = ob + (size_t)(12 + sp) * chunk;
            O.kappa_s[sp]   = ob + (size_t)(16 + sp) * chunk;
        }
        if ((rc = bnsn_m1_opacities(quad_1d, quad_2d, flags, params, &E, &Mq, nullptr, stim_abs,
                                    precision, &O, m, s)))
            return rc;
        for (int q = 0; q < 5 && err == cudaSuccess; ++q)
            for (int sp = 0; sp < 4 && err == cudaSuccess; ++sp)
                err = cudaMemcpyAsync(ho[q][sp] + p0, base + (size_t)(23 + 4 * q + sp) * chunk,
                                      sizeof(double) * m, cudaMemcpyDeviceToHost, s);
        if (err != cudaSuccess)
            return cuda_fail(err, "output copy");
    }
    cudaError_t err = cudaStreamSynchronize(st->streams[0]);
    if (err == cudaSuccess)
        err = cudaStreamSynchronize(st->streams[1]);
    return err == cudaSuccess ? BNSN_OK : cuda_fail(err, "host batch");
}
