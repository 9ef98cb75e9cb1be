// Host shim that lets g++ compile the reference's CUDA C step kernels
// (projects/18_simple_wave_fd/step2D_wave.cu, step1D_wave.cu) as ordinary
// C++ functions, so the reference's own arithmetic runs on the CPU as a
// checker. Test infrastructure only: never linked into the product library.
//
// The kernels that are emulated (basic_step, coalesced_step, padded_step,
// mixed_step, step1D) use only per-thread indices. The ones that need a block
// barrier or warp shuffles (shared_step, temporal_step, scaled_step) still
// compile, but their barrier/shuffle stubs abort, so a call fails loudly.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstdio>

struct ref_index3 {
    unsigned x, y, z;
};

// One set of launch indices per OS thread, written by the launcher in
// ref_launch.cpp before each emulated thread runs.
extern thread_local ref_index3 threadIdx, blockIdx, blockDim, gridDim;

#define __global__
#define __device__
#define __forceinline__ inline
#define __shared__ static

[[noreturn]] inline void ref_unsupported(const char* what) {
    std::fprintf(stderr, "ref_shim: %s cannot be emulated on the host\n", what);
    std::abort();
}

inline void __syncthreads() { ref_unsupported("__syncthreads"); }

template <class T>
inline T __shfl_up_sync(unsigned, T, int) { ref_unsupported("__shfl_up_sync"); }
template <class T>
inline T __shfl_down_sync(unsigned, T, int) { ref_unsupported("__shfl_down_sync"); }
template <class T>
inline T __shfl_xor_sync(unsigned, T, int) { ref_unsupported("__shfl_xor_sync"); }

inline int __float2int_rn(float) { ref_unsupported("__float2int_rn"); }
