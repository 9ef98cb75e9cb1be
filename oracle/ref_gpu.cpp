// Runs the reference's own GPU step kernels on the GPU, for timing and parity.
//
// TEST AND BENCHMARK INFRASTRUCTURE ONLY. The product library never links or
// loads it.
//
// The kernels are projects/18_simple_wave_fd/step2D_wave.cu (padded_step,
// mixed_step, scaled_step, temporal_step, shared_step, basic_step,
// coalesced_step), compiled from the reference sources by Makefile.ref in
// two forms: with nvcc --use_fast_math, the option the reference's drivers
// hand to NVRTC (2D_wave_cuda_*.py, COMPILER_OPTIONS), for timing; and with
// IEEE division and no contraction into fused multiply-adds (-fmad=false),
// whose results are the reference expression rounded operation by operation,
// for value-for-value parity. That build happens where the reference sources
// are; the module files travel in oracle/_ref/ and are loaded here with the
// CUDA driver API, into the context the caller (PyTorch) made current on its
// thread, in the place of CuPy's RawModule / RawKernel. Launch shapes and
// arguments are the caller's: the drivers' own ones are restated in Python
// next to the calls.
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>

namespace {

constexpr int kMaxModules = 8;

std::mutex g_mu;
CUmodule g_module[kMaxModules] = {};
int g_nmodules = 0;
std::map<std::string, int> g_by_path;
std::map<std::pair<int, std::string>, CUfunction> g_funcs;
char g_err[256] = "";

int fail(const char* what, CUresult r) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::snprintf(g_err, sizeof g_err, "%s: %s (%d)", what, s ? s : "?", (int)r);
    return -1;
}

}  // namespace

extern "C" {

const char* refgpu_error(void) { return g_err; }

// Loads the module file into the current context (made current from the
// primary context of device 0 when the thread has none). Returns a handle
// (>= 0; the same one for a path loaded before) or -1.
int refgpu_load(const char* path) {
    std::lock_guard<std::mutex> lock(g_mu);
    CUresult r = cuInit(0);
    if (r != CUDA_SUCCESS) return fail("cuInit", r);
    CUcontext ctx = nullptr;
    if ((r = cuCtxGetCurrent(&ctx)) != CUDA_SUCCESS) return fail("cuCtxGetCurrent", r);
    if (!ctx) {
        CUdevice dev;
        if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS) return fail("cuDeviceGet", r);
        if ((r = cuDevicePrimaryCtxRetain(&ctx, dev)) != CUDA_SUCCESS) return fail("cuDevicePrimaryCtxRetain", r);
        if ((r = cuCtxSetCurrent(ctx)) != CUDA_SUCCESS) return fail("cuCtxSetCurrent", r);
    }
    auto it = g_by_path.find(path);
    if (it != g_by_path.end()) return it->second;
    if (g_nmodules == kMaxModules) {
        std::snprintf(g_err, sizeof g_err, "refgpu_load: too many modules");
        return -1;
    }
    CUmodule m = nullptr;
    if ((r = cuModuleLoad(&m, path)) != CUDA_SUCCESS) return fail("cuModuleLoad", r);
    g_module[g_nmodules] = m;
    g_by_path[path] = g_nmodules;
    return g_nmodules++;
}

// Launches kernel `name` of module `handle` on grid (gx, gy) x block
// (bx, by) with the argument pointers `args` (one pointer per kernel
// parameter) on `stream` (a CUstream / cudaStream_t as void*). 0 or -1.
int refgpu_launch(int handle, const char* name, unsigned gx, unsigned gy, unsigned bx, unsigned by,
                  void** args, void* stream) {
    CUfunction f = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (handle < 0 || handle >= g_nmodules) {
            std::snprintf(g_err, sizeof g_err, "refgpu_launch: no module %d", handle);
            return -1;
        }
        const auto key = std::make_pair(handle, std::string(name));
        auto it = g_funcs.find(key);
        if (it == g_funcs.end()) {
            CUresult r = cuModuleGetFunction(&f, g_module[handle], name);
            if (r != CUDA_SUCCESS) return fail("cuModuleGetFunction", r);
            g_funcs[key] = f;
        } else {
            f = it->second;
        }
    }
    CUresult r = cuLaunchKernel(f, gx, gy, 1, bx, by, 1, 0, static_cast<CUstream>(stream), args, nullptr);
    if (r != CUDA_SUCCESS) return fail("cuLaunchKernel", r);
    return 0;
}

}  // extern "C"
