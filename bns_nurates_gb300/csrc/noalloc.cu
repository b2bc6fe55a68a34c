// Static device scratch of bnsn_m1_opacities_noalloc.
//
// The array below holds kNoAllocPoints = 4096 grey scratch records of
// kGreyRecordBytes = 6,400 bytes (25 MiB in all).  It is part of this
// translation unit's module, so the CUDA driver places it when the module is
// loaded; no call of the library allocates or frees it.  Its address is
// looked up once per device, with that device current, by
// cudaGetSymbolAddress (which may load the module: do it before any stream
// capture).  Nothing in it needs to start at zero: within one call, each
// record field a later phase kernel reads is written first by an earlier one.
// One array per device serves every caller, so two calls in flight at the
// same time on one device (different streams or host threads) race on it.

#include <cuda_runtime.h>

#include <map>
#include <mutex>

#include "bnsn_internal.h"

namespace bnsn {
namespace {

static __device__ __align__(256) double g_grey_static_scratch[kNoAllocPoints * (kGreyRecordBytes /
                                                                               sizeof(double))];

std::mutex g_static_mu;
std::map<int, double*> g_static_addr; // device -> address of the array

} // namespace

cudaError_t noalloc_scratch(int device, double** ptr)
{
    std::lock_guard<std::mutex> lk(g_static_mu);
    auto it = g_static_addr.find(device);
    if (it != g_static_addr.end())
    {
        *ptr = it->second;
        return cudaSuccess;
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_grey_static_scratch);
    if (e != cudaSuccess)
        return e;
    g_static_addr[device] = (double*)p;
    *ptr = (double*)p;
    return cudaSuccess;
}

} // namespace bnsn
