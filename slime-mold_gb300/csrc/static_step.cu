// static_step.cu - one simulation step over caller-owned device buffers that
// allocates no device memory.
//
// Some callers cannot allocate device memory while they run: a host engine
// that reserves all device memory up front in its own arena and forbids
// allocations afterwards, a real-time display loop where a cudaMalloc (which
// can synchronise the device) would stall a frame, or a process whose device
// memory is already held by another allocator.  For them this file offers
// slime_step_noalloc: the caller passes the agents and both trails as device
// pointers, and the per-cell deposit counts that the agent pass hands to the
// trail pass live in a fixed array compiled into the library
// (slime_noalloc_counts below), so no call allocates.
//
// The array has room for kNoAllocMaxCells cells (1,048,576, e.g. a 1024 x
// 1024 trail; 4 MiB) and every GPU that loads the library keeps it until the
// process exits.  Every call uses the same array: it is cleared at the start
// of each call, and calls whose work overlaps on the GPU (different streams,
// or different host threads on one device) race on it and give wrong counts.
// slime_step_noalloc_scratch takes the counts array from the caller instead
// (width * height 32-bit words of its own device memory): no size limit
// beyond the context's, and calls with separate arrays may overlap.
#include "kernels.h"

namespace {

constexpr uint64_t kNoAllocMaxCells = 1ull << 20;

// The deposit counts of the step in flight.  In host code this name is only a
// host-side stand-in, never a device address: the address is looked up with
// cudaGetSymbolAddress.
static __device__ __align__(256) uint32_t slime_noalloc_counts[kNoAllocMaxCells];

// The array's address on the current device, looked up on every call (the
// lookup allocates nothing).  A cached address would outlive the module it
// belongs to: after a cudaDeviceReset the runtime loads the module again,
// possibly elsewhere.  The first lookup on a device loads the module there.
int counts_address(uint32_t** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, slime_noalloc_counts);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return SLIME_ERR_CUDA;
    }
    *out = (uint32_t*)p;
    return SLIME_OK;
}


// One step with the deposit counts in `counts` (room for `max_cells` cells).
int step_with_counts(const SlimeParams* params, uint32_t width, uint32_t height, uint64_t n_agents, float* d_x,
                     float* d_y, float* d_angle, float* d_speed, const float* d_trail_in, float* d_trail_out,
                     uint32_t* counts, uint64_t max_cells, cudaStream_t s) {
    using namespace slime;
    const size_t cells = (size_t)width * height;
    if (cells > max_cells) return SLIME_ERR_INVALID_ARGUMENT;
    DevParams d;
    const char* why = nullptr;
    if (!make_dev_params(*params, width, height, &d, &why)) return SLIME_ERR_INVALID_ARGUMENT;
    if (cudaMemsetAsync(counts, 0, cells * sizeof(uint32_t), s) != cudaSuccess) {
        cudaGetLastError();
        return SLIME_ERR_CUDA;
    }
    AgentsSoA a;
    a.x = d_x;
    a.y = d_y;
    a.th = d_angle;
    a.v = d_speed;
    a.ids = nullptr;
    a.n = n_agents;
    a.n_pad = n_agents;
    // One agent per thread (scalar loads need no padding or 16-byte
    // alignment of the caller's arrays) and the shared-memory trail tile.
    const int kScalarShape = 2;
    cudaError_t e = launch_agents(d, a, d_trail_in, counts, s, kScalarShape, nullptr);
    if (e == cudaSuccess) e = launch_trail(d, trail_tile_default(), d_trail_in, counts, d_trail_out, nullptr, s, nullptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return SLIME_ERR_CUDA;
    }
    return SLIME_OK;
}

// Argument checks shared by both entry points.
bool valid_step_args(const SlimeParams* params, uint32_t width, uint32_t height, uint64_t n_agents, const float* d_x,
                     const float* d_y, const float* d_angle, const float* d_speed, const float* d_trail_in,
                     const float* d_trail_out) {
    if (!params || !d_trail_in || !d_trail_out || d_trail_in == d_trail_out) return false;
    if (n_agents && (!d_x || !d_y || !d_angle || !d_speed)) return false;
    // The sampler reads up to width + 1 cells past a discarded tap's cell 0,
    // which stays inside the trail only for width, height >= 2.
    return width >= 2 && height >= 2 && (uint64_t)width * height < (1ull << 31) && n_agents < (1ull << 31);
}

} // namespace

extern "C" int slime_step_noalloc(const SlimeParams* params, uint32_t width, uint32_t height, uint64_t n_agents,
                                  float* d_x, float* d_y, float* d_angle, float* d_speed, const float* d_trail_in,
                                  float* d_trail_out, void* stream) {
    if (!valid_step_args(params, width, height, n_agents, d_x, d_y, d_angle, d_speed, d_trail_in, d_trail_out) ||
        (uint64_t)width * height > kNoAllocMaxCells)
        return SLIME_ERR_INVALID_ARGUMENT;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        return SLIME_ERR_NO_DEVICE;
    }
    uint32_t* counts = nullptr;
    int rc = counts_address(&counts);
    if (rc != SLIME_OK) return rc;
    return step_with_counts(params, width, height, n_agents, d_x, d_y, d_angle, d_speed, d_trail_in, d_trail_out,
                            counts, kNoAllocMaxCells, (cudaStream_t)stream);
}

extern "C" int slime_step_noalloc_scratch(const SlimeParams* params, uint32_t width, uint32_t height,
                                          uint64_t n_agents, float* d_x, float* d_y, float* d_angle, float* d_speed,
                                          const float* d_trail_in, float* d_trail_out, uint32_t* d_counts,
                                          void* stream) {
    if (!valid_step_args(params, width, height, n_agents, d_x, d_y, d_angle, d_speed, d_trail_in, d_trail_out) ||
        !d_counts)
        return SLIME_ERR_INVALID_ARGUMENT;
    return step_with_counts(params, width, height, n_agents, d_x, d_y, d_angle, d_speed, d_trail_in, d_trail_out,
                            d_counts, (uint64_t)width * height, (cudaStream_t)stream);
}
