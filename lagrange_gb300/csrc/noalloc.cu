// fwn_query_noalloc: the winding-number query without any device allocation.
//
// Who needs it: callers that must not allocate GPU memory while they run queries — for example
// a voxelizer or renderer that classifies points inside a per-frame loop under a fixed device
// memory budget, or host code that runs where a cudaMalloc/cudaFree could fail under memory
// pressure or would synchronize the device and stall other streams. fwn_query allocates its
// Morton-sort buffers per call (stream-ordered); this entry point uses a fixed region instead.
//
// The region is the file-scope device array below, sized for FWN_NOALLOC_MAX_POINTS points per
// call (about 17.3 MB). Every GPU that loads the library keeps it until the process exits. All
// calls share it, and it keeps whatever the last call left there: the status word is cleared at
// the start of every call; the sort buffers and the histogram are fully rewritten before they
// are read. Two calls whose work overlaps on the GPU (different streams, or different host
// threads) use the same region at the same time and corrupt each other's results: serialize
// them (one stream, or an event between them).
//
// Host code cannot use the array's name as a device address (in host code it names a host-side
// shadow); the first call on each device therefore resolves the address with
// cudaGetSymbolAddress while that device is current, and caches it. Make that first call
// before any stream capture begins.
#include <mutex>
#include <string>

#include "fwn_internal.cuh"

namespace fwn {
namespace {

constexpr int64_t kMaxPoints = FWN_NOALLOC_MAX_POINTS;
// status word (256 B) + four n-entry u32 arrays + sort histogram (256 digits x tiles + totals)
constexpr size_t kScratchBytes =
    256 + 16 * (size_t)kMaxPoints +
    (256 * ((kMaxPoints + kSortTileKeys - 1) / kSortTileKeys) + 256) * 4 + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {};

void* scratch_address(int device) {
    if (device < 0 || device >= kMaxDevices)
        throw Error(FWN_INVALID_ARG, "device ordinal out of range for fwn_query_noalloc");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (err != cudaSuccess || !p)
            throw Error(FWN_CUDA_ERROR, std::string("cudaGetSymbolAddress of the no-alloc scratch "
                                                    "region failed: ") +
                                            cudaGetErrorString(err));
        g_scratch_addr[device] = p;
    }
    return g_scratch_addr[device];
}

}  // namespace
}  // namespace fwn

using namespace fwn;

extern "C" FWN_API fwn_status fwn_query_noalloc(fwn_handle h, const float* d_points, int64_t n,
                                                float* d_omega, uint8_t* d_inside,
                                                void* stream) {
    try {
        if (!h) throw Error(FWN_NOT_BUILT, "null handle (default-constructed or moved-from engine)");
        const Engine& e = *reinterpret_cast<const Engine*>(h);
        if (n < 0) throw Error(FWN_INVALID_ARG, "number of points must be >= 0");
        if (n > kMaxPoints)
            throw Error(FWN_INVALID_ARG,
                        "fwn_query_noalloc takes at most FWN_NOALLOC_MAX_POINTS (" +
                            std::to_string(kMaxPoints) + ") points per call; got " +
                            std::to_string(n) + " (split the batch, or use fwn_query)");
        if (n > 0 && !d_points) throw Error(FWN_INVALID_ARG, "points pointer is null");
        if (e.nmeshes != 1) throw Error(FWN_INVALID_ARG, "forest handle: use fwn_forest_query");
        require_engine_device(e);
        if (n == 0) return FWN_OK;
        void* scratch = scratch_address(e.device);
        const QueryArgs a = resolve_query_args(e, nullptr);
        query_mesh_prealloc(e, 0, a, d_points, n, d_omega, d_inside, scratch, kScratchBytes,
                            static_cast<cudaStream_t>(stream));
        return FWN_OK;
    } catch (const Error& err) {
        set_last_error(err.what());
        return err.status;
    } catch (const std::exception& err) {
        set_last_error(err.what());
        return FWN_INTERNAL;
    } catch (...) {
        set_last_error("unknown error");
        return FWN_INTERNAL;
    }
}
