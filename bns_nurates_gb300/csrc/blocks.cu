// Batched AMR blocks: many blocks of uneven size, each with its own reaction
// mask, bremsstrahlung variant and quadrature order, in one planned execution.
//
// Plan (bnsn_blocks_plan_create, allocates, synchronous): the blocks are
// grouped by configuration (quadrature order, reactions, brem variant); each
// group gets a device list of its points and a descriptor in device memory.
// The points are split into steps: every step takes the same fraction of
// every group's points (its share), and the steps alternate between two
// streams, each with the scratch records of one step.  The step size (points
// per step over all groups) is the tuner's choice among kStepCandidates, or
// kDefaultStep untuned, or the caller's (bnsn_blocks_set_options); steps are
// made smaller where the scratch limit (a quarter of the free device memory
// by default) needs it.  With tuning on, the step size and the persistent-grid
// scale (points per CTA) are timed on the caller's data -- the first four
// steps of each candidate -- and the fastest kept.
//
// Run (bnsn_blocks_run): per step, every phase kernel is launched once for
// all groups (grid z selects the group; its descriptor and share are read on
// the device), plus one small kernel per run that writes the run's array
// pointers into the descriptors.  A run launches kernels only -- no
// allocation, no host synchronisation, no host-to-device copy -- so it can be
// captured into a CUDA graph and replayed.

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <tuple>
#include <vector>

#include "../../include/bns_nurates_gb300.h"
#include "bnsn_internal.h"

using namespace bnsn;

namespace {

struct Group
{
    OpacityLaunch L;      // flags, params, quadrature and weights of the group
    int64_t* pidx = nullptr;
    int64_t npts  = 0;
    double cost   = 0.;   // relative cost per point (orders the groups in grid z)
};

// Step sizes (points per step over all groups) the tuner times, and the
// untuned default.  Measured on 4M points of the AMR workload (GB300, mixed /
// FP64 points/s): 33k-point steps 1.61M / 504k, 65k 1.62M / 497k, 131k 1.60M
// / 484k, 262k 1.58M / 470k, 524k 1.55M / 458k, 2M 1.52M / 446k -- smaller
// steps keep more of the scratch records the phases pass on in L2.
const int64_t kStepCandidates[] = {16384, 32768, 65536, 131072};
constexpr int64_t kDefaultStep  = 65536;
constexpr int kTrialSteps       = 4; // steps timed per tuner candidate (two per stream)
const double kGrids[]           = {4., 2.};

// Options of plans created afterwards (bnsn_blocks_set_options).
std::atomic<int64_t> g_scratch_limit{0}; // bytes; 0: a quarter of the free memory
std::atomic<int64_t> g_step_points{0};   // points per step; 0: tuned (default untuned)

// The array pointers of a run, written into every group's descriptor.
struct DataPtrs
{
    const double* eos[11];
    const double* m1[12];
    double* out[20];
};

__global__ void __launch_bounds__(64)
    set_data_ptrs_kernel(OpacityLaunch* __restrict__ Ls, int groups, const DataPtrs D)
{
    const int g = blockIdx.x, t = threadIdx.x;
    if (g >= groups)
        return;
    OpacityLaunch& L = Ls[g];
    if (t < 11)
        L.eos[t] = D.eos[t];
    else if (t < 23)
        L.m1[t - 11] = D.m1[t - 11];
    else if (t < 43)
        L.out[t - 23] = D.out[t - 23];
}

// A step layout: every group's points spread evenly over `steps` steps (the
// group's share per step, rounded up), the steps alternating between two
// streams, each stream with the scratch records of one step (half).
struct Layout
{
    int steps = 0;
    std::vector<int64_t> share; // per active group
    int64_t half = 0;           // records of one step
};

Layout make_layout(const std::vector<int64_t>& n, int64_t steps)
{
    Layout Y;
    Y.steps = (int)std::min<int64_t>(std::max<int64_t>(steps, 2), 1 << 30);
    for (int64_t v : n)
    {
        const int64_t c = (v + Y.steps - 1) / Y.steps;
        Y.share.push_back(c);
        Y.half += c;
    }
    return Y;
}

// The layout of steps of about `step_points` points (an even number of
// steps, at least two), with more steps where two steps' records would
// exceed `records` (but at least one record per group).
Layout layout_for(const std::vector<int64_t>& n, int64_t step_points, int64_t records)
{
    int64_t total = 0, maxn = 1;
    for (int64_t v : n)
    {
        total += v;
        maxn = std::max(maxn, v);
    }
    const int64_t G   = (int64_t)n.size();
    const int64_t per = std::max<int64_t>(records / 2, std::max<int64_t>(G, 1));
    const int64_t c   = std::min(std::max<int64_t>(step_points, 1), per);
    // the records of s steps are at most total / s + G: the fewest steps
    // within c records lie between these bounds (they fall as s grows)
    int64_t lo = std::max<int64_t>(2, (total + c - 1) / c);
    int64_t hi = std::max<int64_t>(lo, c > G ? (total + c - G - 1) / (c - G) : maxn);
    auto records_of = [&](int64_t s) {
        int64_t h = 0;
        for (int64_t v : n)
            h += (v + s - 1) / s;
        return h;
    };
    const int64_t cap = std::max(c, G);
    while (lo < hi)
    {
        const int64_t mid = lo + (hi - lo) / 2;
        if (records_of(mid) <= cap)
            hi = mid;
        else
            lo = mid + 1;
    }
    lo += lo % 2; // neither stream runs its last step alone
    return make_layout(n, lo);
}

int fill_points_soa(const bnsn_eos_soa* eos, const bnsn_m1_soa* m1,
                    const bnsn_m1_opacities_soa* out, OpacityLaunch* L)
{
    if (!eos || !m1 || !out)
        return capi_fail(BNSN_ERR_ARG, "eos/m1/out is NULL");
    const double* e[11] = {eos->nb,   eos->temp, eos->ye,    eos->yp, eos->yn,    eos->mu_p,
                           eos->mu_n, eos->mu_e, eos->mu_mu, eos->dU, eos->dm_eff};
    for (int f = 0; f < 11; ++f)
    {
        if (!e[f] && f != 8)
            return capi_fail(BNSN_ERR_ARG, "an eos field pointer is NULL");
        L->eos[f] = e[f];
    }
    for (int s = 0; s < 4; ++s)
    {
        if (!m1->n[s] || !m1->J[s] || !m1->chi[s])
            return capi_fail(BNSN_ERR_ARG, "an m1 field pointer is NULL");
        L->m1[s]     = m1->n[s];
        L->m1[4 + s] = m1->J[s];
        L->m1[8 + s] = m1->chi[s];
    }
    double* const* o[5] = {out->eta_0, out->kappa_0_a, out->eta, out->kappa_a, out->kappa_s};
    for (int q = 0; q < 5; ++q)
        for (int s = 0; s < 4; ++s)
        {
            if (!o[q][s])
                return capi_fail(BNSN_ERR_ARG, "an output pointer is NULL");
            L->out[q * 4 + s] = o[q][s];
        }
    L->has_distr = 0;
    return BNSN_OK;
}

// Step tables of a layout over the active groups: step s, group z gets
// points [s share_z, (s + 1) share_z) of its list (clipped), its records at
// offset off_z of the scratch of stream s % 2.
void step_tables(const Layout& Y, const std::vector<int64_t>& n, double* ws,
                 std::vector<GroupChunk>* gc, std::vector<int64_t>* np_max)
{
    const size_t words = grey_point_scratch_bytes() / sizeof(double);
    const int G        = (int)n.size();
    gc->assign((size_t)Y.steps * G, GroupChunk{0, 0, nullptr});
    np_max->assign(Y.steps, 0);
    for (int s = 0; s < Y.steps; ++s)
    {
        double* half = ws + (int64_t)(s & 1) * Y.half * words;
        int64_t off  = 0;
        for (int z = 0; z < G; ++z)
        {
            const int64_t p0 = (int64_t)s * Y.share[z];
            const int64_t np = std::max<int64_t>(0, std::min<int64_t>(Y.share[z], n[z] - p0));
            (*gc)[(size_t)s * G + z] = GroupChunk{p0, np, half + off * words};
            (*np_max)[s]             = std::max((*np_max)[s], np);
            off += Y.share[z];
        }
    }
}

} // namespace

struct bnsn_blocks_plan
{
    int device  = 0;
    int num_sms = 0;
    bool mixed  = false;
    std::vector<Group> groups; // all configurations, in order of creation
    std::vector<int> active;   // groups with points, by descending cost (grid z)
    std::vector<int64_t> n;    // points of the active groups
    OpacityLaunch* dLs = nullptr; // descriptors of the active groups, device
    GroupChunk* dgc    = nullptr; // steps x active groups shares, device
    int64_t dgc_cap    = 0;
    double* ws         = nullptr; // scratch records of two steps
    int64_t ws_recs    = 0;
    Layout lay;                   // the chosen layout
    std::vector<int64_t> np_max;  // per step, the largest share
    double grid = 4.;             // persistent-grid scale
    cudaStream_t aux  = nullptr;  // the second stream
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

namespace {

// Upload a layout's step tables (synchronous; plan time only).
cudaError_t upload_tables(bnsn_blocks_plan* P, const Layout& Y, std::vector<int64_t>* np_max)
{
    std::vector<GroupChunk> gc;
    step_tables(Y, P->n, P->ws, &gc, np_max);
    cudaError_t e = cudaSuccess;
    if ((int64_t)gc.size() > P->dgc_cap)
    {
        if (P->dgc)
            cudaFree(P->dgc);
        P->dgc     = nullptr;
        P->dgc_cap = 0;
        if ((e = cudaMalloc((void**)&P->dgc, sizeof(GroupChunk) * gc.size())) != cudaSuccess)
            return e;
        P->dgc_cap = (int64_t)gc.size();
    }
    return gc.empty() ? cudaSuccess :
                        cudaMemcpy(P->dgc, gc.data(), sizeof(GroupChunk) * gc.size(),
                                   cudaMemcpyHostToDevice);
}

// The launches of a run over the uploaded tables of layout Y: its first
// `steps` steps (all when steps < 0).
cudaError_t run_steps(bnsn_blocks_plan* P, const Layout& Y, const std::vector<int64_t>& np_max,
                      const DataPtrs& D, cudaStream_t st, int steps = -1)
{
    const unsigned G = (unsigned)P->active.size();
    if (G == 0)
        return cudaSuccess;
    const int S = steps < 0 ? Y.steps : std::min(steps, Y.steps);
    phase_mark(kPhAux, 0, st);
    set_data_ptrs_kernel<<<G, 64, 0, st>>>(P->dLs, (int)G, D);
    phase_mark(kPhAux, 1, st);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaEventRecord(P->ev[0], st);
    if (e == cudaSuccess)
        e = cudaStreamWaitEvent(P->aux, P->ev[0], 0);
    if (e != cudaSuccess)
        return e;
    for (int s = 0; s < S && e == cudaSuccess; ++s)
    {
        // the union of the flags of the groups with points in this step
        OpacityLaunch U = P->groups[P->active[0]].L;
        U.use_abs_em = U.use_pair = U.use_brem = U.use_inel = U.use_iso = 0;
        unsigned brem_set = 0;
        for (unsigned z = 0; z < G; ++z)
        {
            const OpacityLaunch& L = P->groups[P->active[z]].L;
            if ((int64_t)s * Y.share[z] >= P->n[z])
                continue; // no points of the group in this step
            U.use_abs_em |= L.use_abs_em;
            U.use_pair |= L.use_pair;
            U.use_brem |= L.use_brem;
            U.use_inel |= L.use_inel;
            U.use_iso |= L.use_iso;
            if (L.use_brem)
                brem_set |= 1u << L.brem_impl;
        }
        U.mixed            = P->mixed ? 1 : 0;
        U.grid_scale       = P->grid;
        const GroupArgs GA = {P->dLs, P->dgc + (int64_t)s * G};
        e = launch_grey_multi(U, brem_set, GA, G, np_max[s], (s & 1) ? P->aux : st, P->num_sms);
    }
    // join even after an error, so that the caller's stream never runs ahead
    const cudaError_t e1 = cudaEventRecord(P->ev[1], P->aux);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(st, P->ev[1], 0) : e1;
    return e != cudaSuccess ? e : e2;
}

int data_ptrs(const bnsn_eos_soa* eos, const bnsn_m1_soa* m1, const bnsn_m1_opacities_soa* out,
              DataPtrs* D)
{
    OpacityLaunch L;
    const int rc = fill_points_soa(eos, m1, out, &L);
    if (rc)
        return rc;
    memcpy(D->eos, L.eos, sizeof(D->eos));
    memcpy(D->m1, L.m1, sizeof(D->m1));
    memcpy(D->out, L.out, sizeof(D->out));
    return BNSN_OK;
}

int64_t scratch_limit()
{
    const int64_t lim = g_scratch_limit.load();
    if (lim > 0)
        return lim;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess)
        return (int64_t)1 << 30;
    return (int64_t)(fr / 4);
}

} // namespace

extern "C" {

int bnsn_blocks_set_options(int64_t scratch_bytes, int64_t step_points)
{
    if (scratch_bytes < 0 || step_points < 0)
        return capi_fail(BNSN_ERR_ARG, "negative blocks option");
    g_scratch_limit.store(scratch_bytes);
    g_step_points.store(step_points);
    return BNSN_OK;
}

int bnsn_blocks_plan_create(const bnsn_block* blocks, int nblocks, const OpacityParams* params,
                            int stim_abs, int precision, int tune, const bnsn_eos_soa* eos,
                            const bnsn_m1_soa* m1, const bnsn_m1_opacities_soa* out, void* stream,
                            bnsn_blocks_plan_t* plan_out)
{
    if (!plan_out || (nblocks > 0 && !blocks) || nblocks < 0 || !params)
        return capi_fail(BNSN_ERR_ARG, "invalid argument");
    *plan_out = nullptr;
    if (precision != BNSN_FP64 && precision != BNSN_MIXED)
        return capi_fail(BNSN_ERR_ARG, "unknown precision");
    // group the blocks by (nquad, flags, brem)
    std::map<std::tuple<int, int, int>, std::vector<int>> by_cfg;
    int64_t total = 0;
    for (int b = 0; b < nblocks; ++b)
    {
        const bnsn_block& B = blocks[b];
        if (B.first < 0 || B.count < 0)
            return capi_fail(BNSN_ERR_ARG, "block with negative first/count");
        if (B.nquad < 1 || B.nquad > BNSN_NQUAD_MAX)
            return capi_fail(BNSN_ERR_NQUAD, "block quadrature order must be in 1..20");
        if (B.brem_implementation < 0 || B.brem_implementation > 2)
            return capi_fail(BNSN_ERR_ARG, "unknown brem_implementation in a block");
        const OpacityFlags& f = B.flags;
        const int mask = (f.use_abs_em != 0) | (f.use_pair != 0) << 1 | (f.use_brem != 0) << 2 |
                         (f.use_inelastic_scatt != 0) << 3 | (f.use_iso != 0) << 4;
        by_cfg[std::make_tuple(B.nquad, mask, B.brem_implementation)].push_back(b);
        total += B.count;
    }
    DeviceInfo dev;
    int rc = capi_device_info(&dev);
    if (rc)
        return rc;
    bnsn_blocks_plan* P = new bnsn_blocks_plan();
    cudaGetDevice(&P->device);
    P->num_sms = dev.num_sms;
    P->mixed   = precision == BNSN_MIXED;
    auto cleanup = [&](int code) {
        bnsn_blocks_plan_destroy(P);
        return code;
    };
    cudaStream_t st = (cudaStream_t)stream;
    for (auto& kv : by_cfg)
    {
        const int nq = std::get<0>(kv.first), mask = std::get<1>(kv.first);
        const int brem = std::get<2>(kv.first);
        Group G;
        memset(&G.L, 0, sizeof(G.L));
        MyQuadrature q;
        memset(&q, 0, sizeof(q));
        q.nx = nq;
        if ((rc = bnsn_gauss_legendre(&q)))
            return cleanup(rc);
        OpacityFlags fl  = {mask & 1, (mask >> 1) & 1, (mask >> 2) & 1, (mask >> 3) & 1,
                           (mask >> 4) & 1};
        OpacityParams pa = *params;
        pa.brem_implementation = (BremImpl)brem;
        if ((rc = capi_fill_launch(&q, &q, &fl, &pa, stim_abs, &G.L)))
            return cleanup(rc);
        if (fl.use_brem && brem == BREM_GP19)
        {
            if (!dev.has_gp19)
                return cleanup(capi_fail(BNSN_ERR_NO_TABLE, "GP19 brem requested but no table loaded"));
            G.L.gp19 = dev.gp19;
        }
        G.L.mixed = P->mixed ? 1 : 0;
        // relative cost per point: the 2-D cells grow as n^2; NES, pair and
        // brem dominate them
        G.cost = (double)nq * nq * (1. + 2. * fl.use_inelastic_scatt + fl.use_pair + fl.use_brem);
        std::vector<int64_t> idx;
        for (int b : kv.second)
            for (int64_t i = 0; i < blocks[b].count; ++i)
                idx.push_back(blocks[b].first + i);
        G.npts = (int64_t)idx.size();
        if (G.npts > 0)
        {
            cudaError_t e = cudaMalloc((void**)&G.pidx, sizeof(int64_t) * idx.size());
            if (e == cudaSuccess)
                e = cudaMemcpy(G.pidx, idx.data(), sizeof(int64_t) * idx.size(),
                               cudaMemcpyHostToDevice);
            if (e != cudaSuccess)
            {
                P->groups.push_back(G);
                return cleanup(capi_cuda_fail(e, "plan point lists"));
            }
        }
        G.L.pidx = G.pidx;
        G.L.npts = G.npts;
        P->groups.push_back(G);
    }
    // grid z: the active groups, most expensive first (dispatched first)
    for (int g = 0; g < (int)P->groups.size(); ++g)
        if (P->groups[g].npts > 0)
            P->active.push_back(g);
    std::stable_sort(P->active.begin(), P->active.end(), [&](int a, int b) {
        return P->groups[a].cost > P->groups[b].cost;
    });
    const int G = (int)P->active.size();
    P->n.resize(G);
    for (int z = 0; z < G; ++z)
        P->n[z] = P->groups[P->active[z]].npts;
    cudaError_t e = cudaSuccess;
    if (G > 0)
    {
        std::vector<OpacityLaunch> hL(G);
        for (int z = 0; z < G; ++z)
            hL[z] = P->groups[P->active[z]].L;
        e = cudaMalloc((void**)&P->dLs, sizeof(OpacityLaunch) * G);
        if (e == cudaSuccess)
            e = cudaMemcpy(P->dLs, hL.data(), sizeof(OpacityLaunch) * G, cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
            return cleanup(capi_cuda_fail(e, "plan descriptors"));
    }
    if ((e = cudaStreamCreateWithFlags(&P->aux, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&P->ev[0], cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&P->ev[1], cudaEventDisableTiming)) != cudaSuccess)
        return cleanup(capi_cuda_fail(e, "plan stream"));
    // candidate layouts; the scratch holds two steps of the largest
    const int64_t rec     = (int64_t)grey_point_scratch_bytes();
    const int64_t records = scratch_limit() / rec;
    const int64_t fixed   = g_step_points.load();
    std::vector<Layout> cand;
    if (fixed > 0)
        cand.push_back(layout_for(P->n, fixed, records));
    else if (tune && total > 0 && G > 0)
        for (int64_t c : kStepCandidates)
            cand.push_back(layout_for(P->n, c, records));
    else
        cand.push_back(layout_for(P->n, kDefaultStep, records));
    int64_t half = 1;
    for (const Layout& Y : cand)
        half = std::max(half, Y.half);
    P->ws_recs = 2 * half;
    if ((e = cudaMalloc((void**)&P->ws, P->ws_recs * rec)) != cudaSuccess)
        return cleanup(capi_cuda_fail(e, "plan scratch"));
    P->lay  = cand[0];
    P->grid = kGrids[0];
    if (tune && total > 0 && G > 0)
    {
        // each candidate step size at the first grid scale, then the other
        // grid scales at the fastest step size: the first kTrialSteps steps
        // of the layout on the caller's data, after one untimed run of the
        // first candidate (first launches of the kernels)
        DataPtrs D;
        if ((rc = data_ptrs(eos, m1, out, &D)))
            return cleanup(rc);
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        double best = -1.;
        auto trial  = [&](const Layout& Y, double gs, bool timed) {
            std::vector<int64_t> npm;
            if ((e = upload_tables(P, Y, &npm)) != cudaSuccess)
                return;
            const double keep = P->grid;
            P->grid           = gs;
            cudaEventRecord(e0, st);
            e = run_steps(P, Y, npm, D, st, kTrialSteps);
            cudaEventRecord(e1, st);
            P->grid = keep;
            if (e != cudaSuccess || (e = cudaEventSynchronize(e1)) != cudaSuccess || !timed)
                return;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            int64_t pts = 0;
            for (int z = 0; z < G; ++z)
                pts += std::min(P->n[z], kTrialSteps * Y.share[z]);
            const double rate = (double)pts / std::max(1e-3, (double)ms);
            if (rate > best)
            {
                best    = rate;
                P->lay  = Y;
                P->grid = gs;
            }
        };
        trial(cand[0], kGrids[0], false);
        for (size_t c = 0; c < cand.size() && e == cudaSuccess; ++c)
            trial(cand[c], kGrids[0], true);
        const Layout chosen = P->lay;
        for (size_t g = 1; g < sizeof(kGrids) / sizeof(kGrids[0]) && e == cudaSuccess; ++g)
            trial(chosen, kGrids[g], true);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (e != cudaSuccess)
            return cleanup(capi_cuda_fail(e, "plan tuning"));
    }
    if ((e = upload_tables(P, P->lay, &P->np_max)) != cudaSuccess)
        return cleanup(capi_cuda_fail(e, "plan step tables"));
    *plan_out = P;
    return BNSN_OK;
}

int bnsn_blocks_run(bnsn_blocks_plan_t plan, const bnsn_eos_soa* eos, const bnsn_m1_soa* m1,
                    const bnsn_m1_opacities_soa* out, void* stream)
{
    if (!plan)
        return capi_fail(BNSN_ERR_ARG, "plan is NULL");
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != plan->device)
        return capi_fail(BNSN_ERR_ARG, "the plan was made on another device");
    DataPtrs D;
    const int rc = data_ptrs(eos, m1, out, &D);
    if (rc)
        return rc;
    const cudaError_t e = run_steps(plan, plan->lay, plan->np_max, D, (cudaStream_t)stream);
    return e == cudaSuccess ? BNSN_OK : capi_cuda_fail(e, "blocks run");
}

int bnsn_blocks_plan_info(bnsn_blocks_plan_t plan, int group, int* nquad, int* reactions,
                          int* brem, int64_t* npts, int64_t* chunk, double* grid_scale)
{
    if (!plan)
        return capi_fail(BNSN_ERR_ARG, "plan is NULL");
    if (group < 0 || group >= (int)plan->groups.size())
        return capi_fail(BNSN_ERR_ARG, "no such group");
    const Group& G = plan->groups[group];
    int64_t share  = 0;
    for (size_t z = 0; z < plan->active.size(); ++z)
        if (plan->active[z] == group)
            share = plan->lay.share[z];
    if (nquad)
        *nquad = G.L.n2;
    if (reactions)
        *reactions = G.L.use_abs_em | G.L.use_pair << 1 | G.L.use_brem << 2 | G.L.use_inel << 3 |
                     G.L.use_iso << 4;
    if (brem)
        *brem = G.L.brem_impl;
    if (npts)
        *npts = G.npts;
    if (chunk)
        *chunk = share;
    if (grid_scale)
        *grid_scale = plan->grid;
    return BNSN_OK;
}

int bnsn_blocks_plan_layout(bnsn_blocks_plan_t plan, int* steps, int64_t* step_points,
                            int64_t* scratch_bytes)
{
    if (!plan)
        return capi_fail(BNSN_ERR_ARG, "plan is NULL");
    const bool any = !plan->active.empty();
    if (steps)
        *steps = any ? plan->lay.steps : 0;
    if (step_points)
        *step_points = any ? plan->lay.half : 0;
    if (scratch_bytes)
        *scratch_bytes = plan->ws_recs * (int64_t)grey_point_scratch_bytes();
    return BNSN_OK;
}

int bnsn_blocks_plan_groups(bnsn_blocks_plan_t plan)
{
    return plan ? (int)plan->groups.size() : 0;
}

int bnsn_blocks_plan_destroy(bnsn_blocks_plan_t plan)
{
    if (!plan)
        return BNSN_OK;
    for (Group& G : plan->groups)
        if (G.pidx)
            cudaFree(G.pidx);
    if (plan->dLs)
        cudaFree(plan->dLs);
    if (plan->dgc)
        cudaFree(plan->dgc);
    if (plan->ws)
        cudaFree(plan->ws);
    if (plan->aux)
        cudaStreamDestroy(plan->aux);
    for (cudaEvent_t ev : plan->ev)
        if (ev)
            cudaEventDestroy(ev);
    delete plan;
    return BNSN_OK;
}

} // extern "C"
