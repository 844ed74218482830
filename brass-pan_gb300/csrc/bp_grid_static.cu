// bp_grid_static.cu -- the hash-grid build for callers that cannot allocate.
//
// Some callers of this library cannot call cudaMalloc at the point where they
// need a grid: code that runs while another component owns the allocator
// (a renderer or physics plug-in inside a host application with its own
// memory pools, or a budgeted real-time loop that forbids allocation after
// start-up), or code that must not synchronise the device, which cudaMalloc /
// cudaFree may do.  bp_grid_build_static gives them the result of
// bp_grid_build without any allocation: the radix sort's scratch lives in the
// fixed device array below, which every GPU that loads the library keeps
// until the process exits.
#include <mutex>
#include <string>

#include "bp_internal.h"

namespace bp {
namespace {

// Largest input: 2^18 particles.  Scratch: two ping-pong key/value pairs of
// that length (grids finer than 64^3 need three or four sort passes) plus the
// per-tile digit histogram and the digit totals -- 4.2 MB.
constexpr int kStaticMaxParticles = 1 << 18;
constexpr size_t kStaticTiles = (kStaticMaxParticles + kSortTile - 1) / kSortTile;
constexpr size_t kStaticBytes = 4 * ((size_t)kStaticMaxParticles * 4 + 256) + (size_t)kRadixBins * kStaticTiles * 4 +
                                256 + (size_t)kRadixBins * 4 + 256;
static_assert(kStaticBytes < (size_t)5 << 20, "fixed grid scratch should stay modest");

static __device__ __align__(256) unsigned char g_grid_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_grid_scratch on the current device.  The host-side
// symbol is only a stand-in; the address must be queried once per device,
// with that device current.  It is kept until the process exits, so it goes
// stale if the caller resets the device (cudaDeviceReset) after the first
// call; the entry point's documentation rules that out.
cudaError_t scratch_address(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_grid_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

bp_status fail(bp_status st, const std::string &msg)
{
    set_last_error(msg.c_str());
    return st;
}

}  // namespace
}  // namespace bp

using namespace bp;

extern "C" bp_status bp_grid_build_static(void *stream, int32_t n, const float *pos, float cell, int32_t D,
                                          int32_t *cell_ids, int32_t *sorted_cell_ids, int32_t *sorted_ids,
                                          int32_t *start, int32_t *end)
{
    if (n < 0 || D < 4 || D > 1024 || (D & (D - 1)) || !(cell > 0.f))
        return fail(BP_ERR_INVALID_ARGUMENT, "bp_grid_build_static: bad argument");
    if (n > kStaticMaxParticles)
        return fail(BP_ERR_CAPACITY,
                    "bp_grid_build_static: at most 262144 particles (fixed device scratch); use bp_grid_build");
    if (n == 0) return BP_OK;
    if (!pos || !cell_ids || !sorted_cell_ids || !sorted_ids || !start || !end)
        return fail(BP_ERR_INVALID_ARGUMENT, "bp_grid_build_static: NULL buffer");
    void *scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess)
        return fail(BP_ERR_CUDA, std::string("bp_grid_build_static: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    // Carved exactly like bp_grid_build's workspace; the array holds the
    // largest carving (n = 2^18 with two ping-pong pairs).  Nothing needs
    // clearing: every word the call reads (histograms, digit totals,
    // ping-pong keys) is written earlier in the same call.
    SortScratch sc;
    sort_scratch_carve(scratch, n, D, &sc);
    cudaStream_t st = (cudaStream_t)stream;
    LaunchLog L;
    L.stream = st;
    launch_hash_f3(st, n, pos, cell, D, cell_ids, sc.hist, &L);
    radix_sort_pairs(st, n, D, cell_ids, nullptr, sorted_cell_ids, sorted_ids, sc, true, &L);
    launch_find_start_end(st, n, sorted_cell_ids, start, end, &L);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(BP_ERR_CUDA, std::string("bp_grid_build_static: ") + cudaGetErrorString(e));
    return BP_OK;
}
