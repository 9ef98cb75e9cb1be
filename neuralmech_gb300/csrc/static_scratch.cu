// Allocation-free forward entry point: wfd_forward_static.
//
// Some callers cannot allocate device memory. A host framework may own every
// byte of the device through its own pool and forbid driver allocations. A
// plugin interface may hand over only input and output buffers, with no
// allocator. A latency-critical loop cannot afford the implicit device
// synchronisation of cudaMalloc/cudaFree. For them, this entry point runs the
// ordinary batched forward (wfd_forward without checkpoints) with its scratch
// (velocity model m, the two wavefield levels, the per-tile point lists and
// the status word) placed in one file-scope device array. The caller still
// passes every input and the traces output.
//
// The array is kStaticScratchBytes (64 MiB). Every GPU that loads this library
// holds it until the process exits. Problems whose forward scratch
// (wfd_workspace_bytes with with_gradient = 0) exceeds it are rejected with
// WFD_ERR_WORKSPACE before any device work.
//
// In host code the array's name is only a host-side stand-in for the symbol,
// not a device address, so the address handed to the kernels comes from
// cudaGetSymbolAddress. That lookup happens once per device, with that device
// current, on the first call of this entry point on it. Make that first call
// before any stream capture.
//
// All calls share the one array and it keeps the last call's contents. The
// forward clears what must start at zero: both wavefield levels, the point
// counters and the status word. Calls that overlap on the GPU (for example on
// two streams at once) race on the array; serialise them.
//
// Device-side errors (a bounded TMA wait that gave up, a source or receiver
// outside the interior) go to the status word at the start of the array, the
// place wfd_status reads in a caller workspace; wfd_forward_static_status
// reads and clears it.
//
// The cached device address belongs to the device's primary context as it was
// at the first call. After cudaDeviceReset (or anything else that destroys
// that context) it no longer names the array: do not call these entry points
// on that device again in the same process.
#include <mutex>

#include "../../include/wavefd.h"
#include "internal.h"

namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_scratch_mutex;
void* g_scratch_address[kMaxDevices] = {};

}  // namespace

// The array's device address on the current device, looked up (and cached)
// on the first use; nullptr with the error recorded when that fails.
static void* scratch_address(int* status) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        *status = wfd::set_error(WFD_ERR_CUDA, "wfd_forward_static: no usable current device");
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_address[dev]) {
        void* addr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&addr, g_static_scratch);
        if (e != cudaSuccess || addr == nullptr) {
            *status = wfd::set_error(WFD_ERR_CUDA, "wfd_forward_static: cudaGetSymbolAddress of the static "
                                                   "scratch failed");
            return nullptr;
        }
        g_scratch_address[dev] = addr;
    }
    *status = WFD_OK;
    return g_scratch_address[dev];
}

extern "C" int wfd_forward_static(const wfd_problem* p, const float* vel, const float* sponge_z,
                                  const float* sponge_y, const float* sponge_x,
                                  const float* wavelet, const int32_t* src, const int32_t* rec,
                                  float* traces, void* stream) {
    size_t need = 0;
    int rc = wfd_workspace_bytes(p, 0, &need);
    if (rc) return rc;
    if (need > kStaticScratchBytes)
        return wfd::set_error(WFD_ERR_WORKSPACE,
                              "wfd_forward_static: the forward scratch of this problem exceeds the "
                              "64 MiB static array; use wfd_forward with a caller workspace");
    void* scratch = scratch_address(&rc);
    if (!scratch) return rc;
    return wfd_forward(p, vel, sponge_z, sponge_y, sponge_x, wavelet, src, rec, traces, 0,
                       scratch, kStaticScratchBytes, stream);
}

extern "C" int wfd_forward_static_status(void* stream) {
    int rc = WFD_OK;
    void* scratch = scratch_address(&rc);
    if (!scratch) return rc;
    return wfd_status(scratch, stream);  // the status word is the array's first bytes
}
