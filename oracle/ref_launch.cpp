// Host launcher for the reference's step kernels compiled by g++ through
// ref_shim.h (see Makefile.ref). Each emulated CUDA thread is one call of the
// kernel function with the shim's thread-local indices set. Blocks run in
// parallel under OpenMP; the emulated kernels write disjoint cells, so the
// block order does not change the result.
//
// Test infrastructure only: the CPU twin of the reference kernels, used to
// pin the oracle and to generate golden vectors.
#include "ref_shim.h"
#include <cuda_fp16.h>

thread_local ref_index3 threadIdx, blockIdx, blockDim, gridDim;

extern "C" {
// Declarations of the reference kernels (extern "C" in step2D_wave.cu:3-306
// and step1D_wave.cu:1-19).
void basic_step(const float*, const float*, float*, float, float, float, float, int, int);
void coalesced_step(const float*, const float*, float*, float, float, float, float, int, int);
void padded_step(const float*, const float*, float*, float, float, float, float, int, int, int);
void mixed_step(const __half*, const __half*, __half*, float, float, float, float, int, int, int);
void step1D(const float*, const float*, float*, float, float, float, int);
}

template <class F>
static void emulate(ref_index3 grid, ref_index3 block, F&& body) {
    const long nblocks = (long)grid.x * grid.y * grid.z;
#pragma omp parallel for schedule(static)
    for (long b = 0; b < nblocks; ++b) {
        gridDim = grid;
        blockDim = block;
        blockIdx = {unsigned(b % grid.x), unsigned((b / grid.x) % grid.y),
                    unsigned(b / ((long)grid.x * grid.y))};
        for (unsigned tz = 0; tz < block.z; ++tz)
            for (unsigned ty = 0; ty < block.y; ++ty)
                for (unsigned tx = 0; tx < block.x; ++tx) {
                    threadIdx = {tx, ty, tz};
                    body();
                }
    }
}

static unsigned cdiv(long a, long b) { return unsigned((a + b - 1) / b); }

extern "C" {

// padded_step with the launch shape of 2D_wave_cuda_padding.py:62-75:
// block (128, 4), grid (ceil(M_padded/128), ceil(N/4)).
void ref_padded_step(const float* u0, const float* u1, float* u2, float c, float dt,
                     float dx, float dy, int N, int M, int M_padded) {
    emulate({cdiv(M_padded, 128), cdiv(N, 4), 1}, {128, 4, 1},
            [&] { padded_step(u0, u1, u2, c, dt, dx, dy, N, M, M_padded); });
}

// coalesced_step, block (128, 4) (2D_wave_cuda_coalesced.py:62-67).
void ref_coalesced_step(const float* u0, const float* u1, float* u2, float c, float dt,
                        float dx, float dy, int N, int M) {
    emulate({cdiv(M, 128), cdiv(N, 4), 1}, {128, 4, 1},
            [&] { coalesced_step(u0, u1, u2, c, dt, dx, dy, N, M); });
}

// basic_step, block (4, 128) (2D_wave_cuda_basic.py:58-66).
void ref_basic_step(const float* u0, const float* u1, float* u2, float c, float dt,
                    float dx, float dy, int N, int M) {
    emulate({cdiv(N, 4), cdiv(M, 128), 1}, {4, 128, 1},
            [&] { basic_step(u0, u1, u2, c, dt, dx, dy, N, M); });
}

// mixed_step on FP16 storage (2D_wave_cuda_mixed.py:63-64): two points per
// thread, block (128, 4), grid (ceil(M_padded/2/128), ceil(N/4)). The fields are
// passed as raw 16-bit patterns.
void ref_mixed_step(const unsigned short* u0, const unsigned short* u1, unsigned short* u2,
                    float c, float dt, float dx, float dy, int N, int M, int M_padded) {
    emulate({cdiv(M_padded / 2, 128), cdiv(N, 4), 1}, {128, 4, 1}, [&] {
        mixed_step(reinterpret_cast<const __half*>(u0), reinterpret_cast<const __half*>(u1),
                   reinterpret_cast<__half*>(u2), c, dt, dx, dy, N, M, M_padded);
    });
}

// step1D, 1024 threads per block (1D_wave_cuda_multi_gpu.py:54-61).
void ref_step1d(const float* u0, const float* u1, float* u2, float c, float dt, float dx, int N) {
    emulate({cdiv(N, 1024), 1, 1}, {1024, 1, 1},
            [&] { step1D(u0, u1, u2, c, dt, dx, N); });
}

}  // extern "C"
