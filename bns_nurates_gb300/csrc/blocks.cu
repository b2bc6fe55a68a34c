// Batched AMR blocks: many blocks of uneven size, each with its own reaction
// mask, bremsstrahlung variant and quadrature order, in one planned execution.
//
// Plan (bnsn_blocks_plan_create, allocates, synchronous): the blocks are
// grouped by configuration (quadrature order, reactions, brem variant); each
// group gets a device list of its points, and the plan owns the per-point
// scratch records of the largest chunk.  With tuning on, every group's launch
// shape -- points per scratch chunk and the persistent-grid scale -- is timed
// over a set of candidates on the caller's data and the fastest is kept.
//
// Run (bnsn_blocks_run): one grey pipeline (prelude, pair, brem, NES, final)
// per group on the caller's stream, through the point lists.  A run launches
// kernels only -- no allocation, no host synchronisation, no host-to-device
// copy -- so it can be captured into a CUDA graph and replayed.

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
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
    int64_t chunk = 8192; // points per scratch chunk (untuned default)
    double grid   = 4.;   // persistent-grid scale (untuned default)
};

// Candidate launch shapes of the tuner: (points per chunk, grid scale), timed
// on at most kTunePoints points of each group.
const int64_t kChunks[] = {4096, 8192, 16384, 32768};
const double kGrids[]   = {2., 4.};
constexpr int64_t kTunePoints = 65536;

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

} // namespace

struct bnsn_blocks_plan
{
    int device     = 0;
    int num_sms    = 0;
    double* ws     = nullptr; // two halves of ws_pts records, one per stream
    int64_t ws_pts = 0;
    cudaStream_t aux  = nullptr; // second stream of the chunk pipeline
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::vector<Group> groups;
};

extern "C" {

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
        G.L.mixed = precision == BNSN_MIXED;
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
    // scratch for the largest candidate chunk any group can use
    int64_t need = 0;
    for (const Group& G : P->groups)
        need = std::max(need, std::min<int64_t>(G.npts, tune ? kChunks[3] : G.chunk));
    P->ws_pts = std::max<int64_t>(need, 1);
    cudaError_t e = cudaMalloc((void**)&P->ws, 2 * P->ws_pts * grey_point_scratch_bytes());
    if (e != cudaSuccess)
        return cleanup(capi_cuda_fail(e, "plan scratch"));
    if ((e = cudaStreamCreateWithFlags(&P->aux, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&P->ev[0], cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&P->ev[1], cudaEventDisableTiming)) != cudaSuccess)
        return cleanup(capi_cuda_fail(e, "plan stream"));
    if (tune && total > 0)
    {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (Group& G : P->groups)
        {
            if (G.npts == 0)
                continue;
            if ((rc = fill_points_soa(eos, m1, out, &G.L)))
                break;
            G.L.npts = std::min(G.npts, kTunePoints);
            float best = 1e30f;
            int64_t prev = 0;
            for (int64_t ch : kChunks)
            {
                // chunks beyond the group's size or the scratch all run the same
                const int64_t use = std::min(std::min<int64_t>(ch, P->ws_pts), G.L.npts);
                if (use <= prev)
                    continue;
                prev = use;
                for (double gs : kGrids)
                {
                    G.L.grid_scale = gs;
                    cudaEventRecord(e0, st);
                    e = launch_grey(G.L, st, P->num_sms, P->ws, use);
                    cudaEventRecord(e1, st);
                    if (e == cudaSuccess)
                        e = cudaEventSynchronize(e1);
                    if (e != cudaSuccess)
                        break;
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < best)
                    {
                        best    = ms;
                        G.chunk = use;
                        G.grid  = gs;
                    }
                }
                if (e != cudaSuccess)
                    break;
            }
            G.L.npts = G.npts;
            if (e != cudaSuccess)
                break;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc)
            return cleanup(rc);
        if (e != cudaSuccess)
            return cleanup(capi_cuda_fail(e, "plan tuning"));
    }
    else
        for (Group& G : P->groups)
            G.chunk = std::min<int64_t>(G.chunk, P->ws_pts);
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
    // all groups' chunks alternate between the caller's stream and the plan's
    // second stream (the FP64 phases of one chunk beside the FP32 phases of
    // the next), with one fork before the first and one join after the last
    const cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e         = cudaEventRecord(plan->ev[0], st);
    if (e == cudaSuccess)
        e = cudaStreamWaitEvent(plan->aux, plan->ev[0], 0);
    if (e != cudaSuccess)
        return capi_cuda_fail(e, "blocks run");
    int64_t k = 0;
    int rc    = BNSN_OK;
    for (Group& G : plan->groups)
    {
        if (G.npts == 0)
            continue;
        if ((rc = fill_points_soa(eos, m1, out, &G.L)))
            break;
        G.L.grid_scale = G.grid;
        e = launch_grey_chunks(G.L, st, plan->aux, plan->num_sms, plan->ws,
                               plan->ws + plan->ws_pts * (grey_point_scratch_bytes() / sizeof(double)),
                               std::min<int64_t>(G.chunk, plan->ws_pts), &k);
        if (e != cudaSuccess)
            break;
    }
    // join even after an error, so that the caller's stream never runs ahead
    const cudaError_t e1 = cudaEventRecord(plan->ev[1], plan->aux);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(st, plan->ev[1], 0) : e1;
    if (rc)
        return rc;
    if (e != cudaSuccess)
        return capi_cuda_fail(e, "blocks run");
    return e2 == cudaSuccess ? BNSN_OK : capi_cuda_fail(e2, "blocks run");
}

int bnsn_blocks_plan_info(bnsn_blocks_plan_t plan, int group, int* nquad, int* reactions,
                          int* brem, int64_t* npts, int64_t* chunk, double* grid_scale)
{
    if (!plan)
        return capi_fail(BNSN_ERR_ARG, "plan is NULL");
    if (group < 0 || group >= (int)plan->groups.size())
        return capi_fail(BNSN_ERR_ARG, "no such group");
    const Group& G = plan->groups[group];
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
        *chunk = G.chunk;
    if (grid_scale)
        *grid_scale = G.grid;
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
