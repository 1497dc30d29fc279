// grid_noalloc.cu -- tss_grid_build_noalloc: the grid build of tss_grid_build with
// its scratch memory in a fixed array compiled into this library, for callers that
// cannot allocate device memory themselves.
//
// Who needs it: code that runs inside a host application's per-frame or per-request
// callback (the reference's display() loop is one) is often not allowed to call
// cudaMalloc/cudaFree -- both can synchronise the whole device and stall every
// other stream -- or runs under a memory manager that owns all device memory and
// hands the plug-in only its input and output buffers.  Such a caller passes its
// particle arrays and output tables; the scratch comes from the array below.
//
// The array costs TSS_GRID_NOALLOC_MAX_BYTES of device memory on every GPU where
// the library's module is loaded, until the process exits.  All calls share it:
// two calls whose work overlaps on the GPU (different streams, or different host
// threads) race on it and both results are undefined.  It keeps the previous
// call's contents; the build clears what must start at zero (its counters) itself.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/tss.h"

namespace {

__device__ __align__(256) unsigned char g_grid_scratch[TSS_GRID_NOALLOC_MAX_BYTES];

// Device address of g_grid_scratch per device.  In host code the name of a
// __device__ array is only a host-side stand-in, never a device address, so it is
// looked up once per device with that device current.
constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

tss_status scratch_for_current_device(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TSS_NO_DEVICE;
    if (dev < 0 || dev >= kMaxDevices) return TSS_INVALID_ARG;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_grid_scratch) != cudaSuccess || !p) return TSS_CUDA_ERROR;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return TSS_OK;
}

}  // namespace

extern "C" tss_status tss_grid_build_noalloc(const float* d_pos, const int32_t* d_id, int n, float origin_x,
                                             float origin_y, float cell_size, int dimx, int dimy, int32_t* d_order,
                                             int32_t* d_cell_off, void* stream) {
    size_t need = 0;
    tss_status st = tss_grid_workspace_size(n, dimx, dimy, &need);
    if (st != TSS_OK) return st;
    if (need > static_cast<size_t>(TSS_GRID_NOALLOC_MAX_BYTES)) return TSS_CAPACITY;
    void* scratch = nullptr;
    if ((st = scratch_for_current_device(&scratch)) != TSS_OK) return st;
    return tss_grid_build(d_pos, d_id, n, origin_x, origin_y, cell_size, dimx, dimy, d_order, d_cell_off, scratch,
                          static_cast<size_t>(TSS_GRID_NOALLOC_MAX_BYTES), stream);
}
