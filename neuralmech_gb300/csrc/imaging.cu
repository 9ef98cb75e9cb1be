// Total focusing method on full-matrix-capture traces (sm_103a): the consumer
// of the wave path's traces in projects/18_fwi/2D_tfm.py.
//
// analytic_kernel: the analytic signal h = x + i H[x] of every trace, with H the
// periodic discrete Hilbert transform. The transform is a circular
// convolution with the kernel g (g = ifft(-i sign(k)) with the Nyquist bin
// zeroed for even N, the transform scipy.signal.hilbert applies through its
// FFT). One CTA per trace: the trace and two periods of g sit in shared
// memory, and each thread accumulates its output samples over the N inputs
// (O(N^2) per trace).
//
// tfm_kernel: delay and sum, one thread per pixel:
//   image[p] = | sum_{e <= r} w_er h_er((t0 + tau_e(p) + tau_r(p)) / dt) |,
// tau_e = |p - x_e| / c, w_er = 2 for r > e (reciprocity), linear interpolation
// in time, pairs past the end of the trace skipped
// (projects/18_fwi/tfm.py:12-36). Without reciprocity every ordered pair
// counts once. A pixel's times of flight sit in a shared-memory column of
// its own (any element count up to 256). The complex traces are read through
// the read-only path; they are L2-resident for the array sizes of the
// reference drivers.
#include "common.cuh"
#include "internal.h"

namespace wfd {
namespace {

__global__ void analytic_kernel(const float* __restrict__ x, const float* __restrict__ g, int nt,
                                float2* __restrict__ h) {
    extern __shared__ float sm[];
    float* xs = sm;            // [nt]
    float* gs = sm + nt;       // [2 nt]: g[m mod nt]
    const long long tr = blockIdx.x;
    const float* xt = x + tr * nt;
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        xs[i] = xt[i];
        const float gv = g[i];
        gs[i] = gv;
        gs[i + nt] = gv;
    }
    __syncthreads();
    for (int n = threadIdx.x; n < nt; n += blockDim.x) {
        // H[n] = sum_k x[k] g[(n - k) mod nt] = sum_k x[k] gs[n - k + nt]
        float acc = 0.f;
        const float* gn = gs + n + nt;
        for (int k = 0; k < nt; ++k) acc = fmaf(xs[k], gn[-k], acc);
        h[tr * nt + n] = make_float2(xs[n], acc);
    }
}

constexpr int TFM_THREADS = 128;

__global__ void __launch_bounds__(TFM_THREADS)
    tfm_kernel(const float2* __restrict__ h, int E, const float* __restrict__ xe,
               const float* __restrict__ ye, int nt, float inv_dt, float t0, float inv_c,
               const float* __restrict__ xp, const float* __restrict__ yp, int P, int reciprocity,
               float* __restrict__ image) {
    extern __shared__ float tau_s[];  // [E][TFM_THREADS]: the pixel's times of flight
    const int p = blockIdx.x * TFM_THREADS + threadIdx.x;
    const float px = p < P ? xp[p] : 0.f, py = p < P ? yp[p] : 0.f;
    for (int e = 0; e < E; ++e)
        tau_s[e * TFM_THREADS + threadIdx.x] = hypotf(px - __ldg(xe + e), py - __ldg(ye + e)) * inv_c;
    if (p >= P) return;  // no barrier below: each thread reads only its own column
    float sx = 0.f, sy = 0.f;
    for (int e = 0; e < E; ++e) {
        const float te = t0 + tau_s[e * TFM_THREADS + threadIdx.x];
        const float2* he = h + (long long)e * E * nt;
        for (int r = reciprocity ? e : 0; r < E; ++r) {
            const float t = (te + tau_s[r * TFM_THREADS + threadIdx.x]) * inv_dt;
            const int k = int(t);
            if (k >= nt - 1) continue;
            const float scale = (reciprocity && r > e) ? 2.f : 1.f;
            const float w = (t - float(k)) * scale, v = scale - w;
            const float2* hp = he + (long long)r * nt + k;
            const float2 a = __ldg(hp), b = __ldg(hp + 1);
            sx += v * a.x + w * b.x;
            sy += v * a.y + w * b.y;
        }
    }
    image[p] = hypotf(sx, sy);
}

}  // namespace

cudaError_t launch_analytic(const float* traces, long long ntr, int nt, const float* g, float2* h,
                            cudaStream_t s) {
    const size_t smem = (size_t)3 * nt * sizeof(float);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(analytic_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    analytic_kernel<<<(unsigned)ntr, 256, smem, s>>>(traces, g, nt, h);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_tfm(const float2* h, int E, const float* xe, const float* ye, int nt, float dt,
                       float t0, float c, const float* xp, const float* yp, int P, int reciprocity,
                       float* image, cudaStream_t s) {
    const size_t smem = (size_t)E * TFM_THREADS * sizeof(float);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(tfm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    tfm_kernel<<<(P + TFM_THREADS - 1) / TFM_THREADS, TFM_THREADS, smem, s>>>(
        h, E, xe, ye, nt, 1.f / dt, t0, 1.f / c, xp, yp, P, reciprocity, image);
    count_launch();
    return cudaGetLastError();
}

}  // namespace wfd
