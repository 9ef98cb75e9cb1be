/*
 * wavefd.h - C ABI of the GB300 finite-difference acoustic wave path.
 *
 * Plain pointers and sizes only. Every array argument is a DEVICE pointer
 * owned by the caller (PyTorch tensors on the Python side); the library
 * allocates nothing: all scratch lives in a caller-provided workspace whose
 * size wfd_workspace_bytes() reports. Calls are asynchronous on `stream`
 * (a cudaStream_t passed as void*; NULL = legacy default stream), return 0 or a
 * negative WFD_ERR_* status, never abort, and are reentrant per stream.
 *
 * Grid convention: fields are indexed (z, y, x), x fastest; 2D problems have
 * ny == 1 and y == 0 in every position. The outer ring of R = order/2 cells is
 * held fixed (homogeneous Dirichlet, as padded_step holds its ring of 1); the
 * interior is updated by
 *     u_{n+1} = g (2 u_n + (v dt)^2 L u_n + src_scale * w_n) - g^2 u_{n-1},
 * L the order-`order` central Laplacian, g = sponge_z[z] sponge_y[y] sponge_x[x]
 * (a NULL profile counts as 1). Sources and receivers must lie in the interior.
 * Traces: traces[s][n][r] = u_{n+1}(rec[s][r]), n = 0 .. nt-1.
 */
#ifndef WAVEFD_H
#define WAVEFD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WFD_OK 0
#define WFD_ERR_INVALID (-1)   /* bad argument: shape, order, null pointer, alignment */
#define WFD_ERR_WORKSPACE (-2) /* workspace too small or not 256-byte aligned */
#define WFD_ERR_CUDA (-3)      /* a CUDA runtime / driver call failed */
#define WFD_ERR_UNSTABLE (-4)  /* vmax * dt violates the CFL bound of the stencil */
#define WFD_ERR_POSITION (-5)  /* a source or receiver outside the updated interior */
#define WFD_ERR_TIMEOUT (-6)   /* a kernel gave up waiting for a TMA tile */
#define WFD_ERR_STATE (-7)     /* wfd_backward without a preceding checkpointed forward */

/* Checkpoint snapshot formats (bytes per cell). */
#define WFD_CKPT_FP32 0 /* 4 */
#define WFD_CKPT_BF16 1 /* 2, round to nearest even */
#define WFD_CKPT_I16 2  /* 2 + 4/32: int16 with one FP32 scale per 32 cells (block max / 32767) */

/* Storage of the wavefields (wfd_problem.field_format). Reduced precision is
 * a 2D forward-only mode (no checkpoints, no gradient); arithmetic stays FP32. */
#define WFD_FIELD_FP32 0 /* 4 bytes per cell */
#define WFD_FIELD_FP16 1 /* IEEE binary16, round to nearest even (mixed_step's format) */
#define WFD_FIELD_I16 2  /* int16 with one FP32 scale per 32 cells along x, scale = block
                            max / 32767 (scaled_step's format) */

/* How the adjoint obtains the forward levels u_k (wfd_problem.adjoint_mode). */
#define WFD_ADJOINT_CHECKPOINT 0  /* checkpoints (and kept levels), segments recomputed */
#define WFD_ADJOINT_RECONSTRUCT 1 /* time reversal: u_{k} = 2 u_{k+1} + m L u_{k+1} + s w_{k+1}
                                     - u_{k+2} from the last two levels, exact where the
                                     update is undamped; the damped frame (recon_band cells
                                     along every edge) is restored from per-step copies the
                                     forward saves. No checkpoints (2D, one step per launch,
                                     FP32 fields; the reference's reconstruction_sensitivity,
                                     projects/4_specialized_nns/analog_rnn_train.py:142) */

/* What the checkpointed adjoint keeps of each recomputed step for its imaging
 * term q_{k+1} L u_k. */
#define WFD_LAP_AUTO 0 /* 2D one-step kernel: the level u_k itself (FP32, written by the
                          recompute anyway) and the adjoint forms L u_k; otherwise FP32 L u_k */
#define WFD_LAP_BF16 1 /* L u_k in BF16 */
#define WFD_LAP_FP32 2 /* L u_k in FP32 */

/* How the forward evaluates the update (wfd_problem.update_form). Both forms are
 * the same recursion; they differ in FP32 rounding and memory traffic. */
#define WFD_UPDATE_AUTO 0     /* WFD_UPDATE_SUMMED for a forward that saves the state of a
                                 gradient where that form is available (2D and 3D, FP32
                                 fields, lap_store auto, checkpoint adjoint, not variable
                                 density),
                                 WFD_UPDATE_LEAPFROG otherwise */
#define WFD_UPDATE_LEAPFROG 1 /* u_{n+1} over u_{n-1}: 16 bytes per update */
#define WFD_UPDATE_SUMMED 2   /* the summed (increment) form: the state is (u_n, d_n =
                                 u_n - u_{n-1}), d_{n+1} = g^2 d_n - (1 - g)^2 u_n + g m L u_n,
                                 u_{n+1} = u_n + d_{n+1} (Henrici's summed form of the
                                 two-step recursion). The increment keeps its own FP32
                                 rounding, which cuts the accumulated rounding error of
                                 the traces about 4x and of a gradient from residuals
                                 far smaller than the traces about 9x; 20 bytes per update
                                 (d is read and written, u_{n+1} written), 10 with two steps
                                 per launch in 2D (step_block 2: d_{n+1} stays on chip, d
                                 is double-buffered, one more field). Checkpoints then
                                 hold (d_n, u_n). Forward only: the recompute and the
                                 adjoint stay leapfrog. Only where WFD_UPDATE_AUTO would
                                 choose it; elsewhere WFD_ERR_INVALID */

/* How the forward keeps the levels u_k of the segments the adjoint does not
 * recompute (wfd_problem.level_format; store_levels counts levels in either). */
#define WFD_LEVEL_FP32 0  /* FP32: 4 bytes per cell */
#define WFD_LEVEL_BFP16 1 /* block floating point: 16-bit mantissas and one exponent byte per
                             4 cells along x, u = q 2^(t - 141) with q in [-32767, 32767] (stored
                             as q + 32768) and t the FP32 exponent field of the block's largest
                             magnitude (blocks below 2^-112 kept as 0):
                             2.25 bytes per cell, each value within 2^-15 of its block's
                             largest. About 1.8x the kept levels in the same memory, so fewer
                             segments are recomputed; the forward encodes and the adjoint
                             decodes every kept level in exchange. 2D, two steps per launch,
                             the summed forward (FP32 fields, lap_store auto, checkpoint
                             adjoint) */

typedef struct wfd_problem {
    int32_t ndim;          /* 2 or 3 */
    int32_t order;         /* space order: 2, 4 or 8 */
    int32_t nz, ny, nx;    /* cells per axis; ny = 1 when ndim == 2 */
    int32_t nshot;         /* shots sharing this velocity model */
    int32_t nt;            /* time steps */
    int32_t nsrc, nrec;    /* sources / receivers per shot */
    int32_t ckpt_every;    /* steps between checkpoints; 0 = ceil(sqrt(nt)) */
    int32_t ckpt_format;   /* checkpoint snapshots: WFD_CKPT_FP32, _BF16 or _I16 */
    int32_t lap_store;     /* WFD_LAP_AUTO, _BF16 or _FP32 */
    int32_t shots_per_cta; /* shots one CTA walks through per step; 0 = automatic */
    int32_t group_shots;   /* run the shots in sequential groups of this many, all
                              groups sharing one workspace sized for a group (forward
                              without checkpoints and wfd_misfit_gradient only);
                              0 = all shots at once */
    int32_t tile_rows;     /* 2D tile height: 16 or 32 rows (0 = 32) */
    int32_t step_block;    /* 2D time steps per kernel launch: 1 or 2 (0 = 1); 2 keeps
                              u_{n+1} in shared memory between the two steps. A forward
                              (no gradient) with the leapfrog update and FP32 fields also
                              takes 8 at order 2 and 4 at order 4: a window of 256 x 40
                              cells per CTA stays in registers for the launch's steps */
    int32_t store_levels;  /* WFD_LAP_AUTO path: levels (fields of nshot x cells, in
                              level_format) the workspace may hold. The forward keeps the levels of
                              its last floor((store_levels - 2) / K) segments, K the
                              checkpoint interval, and the adjoint recomputes only
                              the others; 0 (or <= K + 2) = the last segment only */
    int32_t field_format;  /* WFD_FIELD_FP32, _FP16 or _I16 */
    int32_t adjoint_mode;  /* WFD_ADJOINT_CHECKPOINT or WFD_ADJOINT_RECONSTRUCT */
    int32_t recon_band;    /* WFD_ADJOINT_RECONSTRUCT: width in cells of the frame along
                              every edge where the sponge damps (0: no sponge); the
                              forward saves that frame of every level */
    float dt;              /* time step */
    float dz, dy, dx;      /* grid spacing (dy ignored in 2D) */
    float src_scale;       /* factor on every injected wavelet sample */
    float vmax;            /* max velocity for the CFL check; <= 0 skips the check */
    int32_t update_form;   /* WFD_UPDATE_AUTO, _LEAPFROG or _SUMMED */
    int32_t level_format;  /* kept levels: WFD_LEVEL_FP32 or _BFP16 (ABI 3.1) */
} wfd_problem;

/* Human-readable text of a status code. */
const char* wfd_strerror(int status);

/* Detail of the last failure on the calling thread ("" if none). */
const char* wfd_last_error(void);

/* ABI version: (major << 16) | minor. */
int wfd_version(void);

/* Workspace size for wfd_forward (with_gradient = 0) or for the
 * forward + backward pair (with_gradient = 1). Host-only, no CUDA call. */
int wfd_workspace_bytes(const wfd_problem* p, int with_gradient, size_t* bytes);

/*
 * Forward modelling of p->nshot shots through one velocity model.
 * Replaces the reference solver's forward call: cuwave `simulate` /
 * `measure(sim, sources, indicator, sensors)` as driven by
 * projects/18_fwi/plate.py:64 (full matrix capture) and
 * projects/18_fwi/2D_scalar_wave_forward_B_hai.py:30.
 *   vel      [nz][ny][nx] FP32 velocity
 *   sponge_* [nz], [ny], [nx] FP32 damping profiles or NULL
 *   wavelet  [nshot][nt][nsrc] FP32 source samples
 *   src, rec [nshot][nsrc|nrec][3] int32 (z, y, x)
 *   traces   [nshot][nt][nrec] FP32 output (may be NULL)
 *   save_checkpoints: 1 keeps the state wfd_backward needs in the workspace
 *   (which must then be sized with with_gradient = 1).
 */
int wfd_forward(const wfd_problem* p, const float* vel, const float* sponge_z,
                const float* sponge_y, const float* sponge_x, const float* wavelet,
                const int32_t* src, const int32_t* rec, float* traces, int save_checkpoints,
                void* workspace, size_t workspace_bytes, void* stream);

/*
 * wfd_forward without checkpoints that also returns the final wavefield
 * u_final [nshot][nz][ny][nx] (u_nt of every shot, the fixed ring included):
 * cuwave `simulate(sim, source, indicator)` returning the field
 * (projects/18_fwi/2D_scalar_wave_forward_B_hai.py:30). Workspace as for
 * wfd_forward(save_checkpoints = 0); no shot groups.
 */
int wfd_forward_final(const wfd_problem* p, const float* vel, const float* sponge_z,
                      const float* sponge_y, const float* sponge_x, const float* wavelet,
                      const int32_t* src, const int32_t* rec, float* traces, float* u_final,
                      void* workspace, size_t workspace_bytes, void* stream);

/*
 * Adjoint of the forward above for a trace cotangent `dtraces`
 * ([nshot][nt][nrec]): grad_vel [nz][ny][nx] = (dF/dvel)^T dtraces (summed over
 * shots; 0 on the fixed ring) and, when grad_wavelet is not NULL,
 * grad_wavelet [nshot][nt][nsrc] = (dF/dwavelet)^T dtraces. Uses the checkpoints
 * of the preceding wfd_forward(save_checkpoints = 1) on the same workspace and
 * inputs, recomputing the forward per segment; one backward per forward.
 * Together with wfd_forward this is the reference solver's gradient,
 * cuwave `misfit_gradient(sim, sources, gamma, sensors, observed)` as used by
 * projects/18_fwi/2D_fwi.py:40, for a cotangent the caller chooses.
 */
int wfd_backward(const wfd_problem* p, const float* vel, const float* sponge_z,
                 const float* sponge_y, const float* sponge_x, const float* wavelet,
                 const int32_t* src, const int32_t* rec, const float* dtraces, float* grad_vel,
                 float* grad_wavelet, void* workspace, size_t workspace_bytes, void* stream);

/*
 * L2 misfit J = 1/2 sum (d - observed)^2 (accumulated in FP64 into the device
 * double *misfit) and its gradient, in one call: forward with checkpoints,
 * residual, backward. Replaces cuwave `misfit_gradient` -> (cost, gradient),
 * projects/18_fwi/2D_fwi.py:40, and `misfit`, as called by
 * projects/9_structural_optimization/fwi_penalization.py:138-143.
 * traces (optional) receives the modelled traces; grad_wavelet may be NULL.
 */
int wfd_misfit_gradient(const wfd_problem* p, const float* vel, const float* sponge_z,
                        const float* sponge_y, const float* sponge_x, const float* wavelet,
                        const int32_t* src, const int32_t* rec, const float* observed,
                        float* traces, float* grad_vel, float* grad_wavelet, double* misfit,
                        void* workspace, size_t workspace_bytes, void* stream);

/*
 * wfd_misfit_gradient for observed traces that are still arriving: the call
 * makes `stream` wait for `observed_ready` (a cudaEvent_t passed as void*,
 * recorded by the caller after it enqueued the copy of `observed`, e.g. on a
 * second stream) just before its first read of `observed`, which comes after
 * the forward. A host-to-device copy of the observed data then overlaps the
 * forward. No counterpart in the reference.
 */
int wfd_misfit_gradient_overlap(const wfd_problem* p, const float* vel, const float* sponge_z,
                                const float* sponge_y, const float* sponge_x, const float* wavelet,
                                const int32_t* src, const int32_t* rec, const float* observed,
                                void* observed_ready, float* traces, float* grad_vel, float* grad_wavelet,
                                double* misfit, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Allocation-free variant of wfd_forward (no checkpoints): the same forward,
 * with its scratch in a 64 MiB array that the library holds on every device it
 * is loaded on, for callers that cannot allocate device memory (a host
 * framework that owns the device pool, a plugin that receives only input and
 * output buffers, a loop that cannot take cudaMalloc's implicit
 * synchronisation). No counterpart in the reference: an addition of this
 * library. Problems whose forward scratch (wfd_workspace_bytes,
 * with_gradient = 0) exceeds 64 MiB return WFD_ERR_WORKSPACE. The first call on
 * a device looks up the array's device address with cudaGetSymbolAddress; make
 * it before any stream capture. All calls share the array: calls that overlap
 * on the GPU race, so serialise them; each call clears what must start at zero.
 * Device-side errors go to the static array's status word:
 * read them with wfd_forward_static_status.
 */
int wfd_forward_static(const wfd_problem* p, const float* vel, const float* sponge_z,
                       const float* sponge_y, const float* sponge_x, const float* wavelet,
                       const int32_t* src, const int32_t* rec, float* traces, void* stream);

/*
 * Status of wfd_forward_static on the current device: synchronises `stream`,
 * returns the first device-side error that calls of wfd_forward_static have
 * recorded in the static array since the last call of this function
 * (WFD_ERR_TIMEOUT for a TMA wait that gave up, WFD_ERR_POSITION for a source
 * or receiver outside the interior, whose samples are then not written) or 0,
 * and clears it: wfd_status for the static array. The array's device address
 * is cached per device at the first call of either entry point and belongs to
 * that device's context: after cudaDeviceReset, do not call either again in
 * the process. No counterpart in the reference.
 */
int wfd_forward_static_status(void* stream);

/*
 * Analytic signal h = x + i H[x] of `ntraces` traces of `nt` samples each
 * (traces [ntraces][nt] FP32 -> out [ntraces][nt] interleaved (re, im) FP32).
 * H is the periodic discrete Hilbert transform, the one scipy.signal.hilbert
 * applies through its FFT, given as the circular-convolution kernel
 * hilbert_kernel[nt], g = ifft(-i sign(k)) (sign 0 at k = 0 and, for even nt,
 * at nt / 2). Replaces the cupyx.scipy.signal.hilbert call of
 * projects/18_fwi/2D_tfm.py:37 for the delay and sum below. nt <= 18000.
 */
int wfd_analytic_signal(const float* traces, int64_t ntraces, int nt, const float* hilbert_kernel,
                        float* out, void* stream);

/*
 * Total focusing method (projects/18_fwi/tfm.py:12-36, tfm_kernel): for each of
 * npix pixels (xp, yp),
 *   image = | sum_e sum_r h_er((t0 + |p - x_e| / c + |p - x_r| / c) / dt) |,
 * h [E][E][nt] interleaved complex FP32 analytic traces (emitter, receiver,
 * sample), x_e = (xe[e], ye[e]), linear interpolation in time, pairs whose
 * sample index reaches nt - 1 skipped. reciprocity = 1 sums the upper triangle
 * r >= e with weight 2 off the diagonal, as the reference kernel does (valid
 * when h_er = h_re). E <= 256.
 */
int wfd_tfm(const float* h, int E, const float* xe, const float* ye, int nt, float dt, float t0,
            float c, const float* xp, const float* yp, int npix, int reciprocity, float* image,
            void* stream);

/*
 * Batches of independent misfit gradients (several models of different sizes,
 * each with its own shots and workspace) replayed as one CUDA graph: the
 * graph-captured batch of the reference's graph driver
 * (projects/18_simple_wave_fd/2D_wave_cuda_graph.py:73-95) for whole gradients.
 * An item holds the arguments of one wfd_misfit_gradient call (device
 * pointers; the workspace sized with with_gradient = 1).
 *
 * wfd_batch_plan runs every item once on a stream of its own, forked from and
 * joined to `stream` (this checks the arguments and configures the kernels;
 * the outputs hold that run's results), then records the same calls as one
 * CUDA graph with the items on parallel branches. The items and their
 * problem structs are copied; the device buffers they point to must stay
 * valid for the plan's life. wfd_batch_run launches the graph on `stream`:
 * the gradients of the buffers' current contents (write new velocities or
 * observed data into the same buffers between runs). Device-side errors go to
 * each item's workspace (wfd_status). wfd_batch_launches: kernels one run
 * launches. No counterpart in the reference's API beyond the graph driver.
 */
typedef struct wfd_batch_item {
    const wfd_problem* problem;
    const float *vel, *sponge_z, *sponge_y, *sponge_x, *wavelet;
    const int32_t *src, *rec;
    const float* observed;
    float *traces, *grad_vel, *grad_wavelet; /* traces, grad_wavelet may be NULL */
    double* misfit;
    void* workspace;
    size_t workspace_bytes;
} wfd_batch_item;
typedef struct wfd_batch wfd_batch; /* opaque */
int wfd_batch_plan(const wfd_batch_item* items, int count, void* stream, wfd_batch** out);
int wfd_batch_run(wfd_batch* batch, void* stream);
uint64_t wfd_batch_launches(const wfd_batch* batch);
int wfd_batch_free(wfd_batch* batch);

/* Synchronises `stream`, returns the first device-side error recorded in the
 * workspace since the last call (WFD_ERR_TIMEOUT, WFD_ERR_POSITION) or 0, and
 * clears it. */
int wfd_status(void* workspace, void* stream);

/* FP64 sum of squares of n FP32 values, added into the device double *out
 * (gradient norms). */
int wfd_sum_sq(const float* x, int64_t n, double* out, void* stream);

/* Number of kernels this library has launched in this process (monotonic),
 * for launch accounting by benchmarks. */
uint64_t wfd_kernel_launches(void);

/* Device time per phase of the calls made on this thread between
 * wfd_profile_begin() and wfd_profile_end(): CUDA events are recorded on the
 * call's stream around the forward time loop, each recomputed segment and each
 * adjoint segment (NVTX ranges mark the same phases for external profilers).
 * wfd_profile_end synchronises those events and sums them. */
typedef struct wfd_phase_times {
    double ms[3];        /* forward, recompute, adjoint */
    int64_t launches[3]; /* step-kernel launches in each phase */
} wfd_phase_times;
int wfd_profile_begin(void);
int wfd_profile_end(wfd_phase_times* out);

/*
 * One order-2, constant-speed, Dirichlet step with the reference kernel's
 * exact signature and semantics: padded_step, projects/18_simple_wave_fd/
 * step2D_wave.cu:59-65, launched as in 2D_wave_cuda_padding.py:66-76.
 * u0, u1, u2 are [N][M_padded] FP32; rows 1..N-2 and columns 1..M-2 of u2
 * receive -u0 + 2 u1 + dt^2 c^2 (Lap_x/dx^2 + Lap_y/dy^2) (i along N uses dx,
 * j along M uses dy); u2 may alias u0. M_padded must be a multiple of 4 and
 * the pointers 16-byte aligned (the reference pads rows to 32).
 */
int wfd_step2d_order2(const float* u0, const float* u1, float* u2, float wavespeed, float dt,
                      float dx, float dy, int N, int M, int M_padded, void* stream);

/*
 * The same order-2 step evaluated as the reference kernels evaluate it, value
 * for value, for any row stride: padded_step and shared_step
 * (step2D_wave.cu:59-81, 187-240) with M_padded, basic_step and
 * coalesced_step (step2D_wave.cu:8-55, launched as in 2D_wave_cuda_basic.py /
 * 2D_wave_cuda_coalesced.py) with M_padded = M. Each cell follows the
 * kernels' expression in its operation order (IEEE, no contraction); no
 * alignment requirement. u2 may alias u0.
 */
int wfd_step2d_exact(const float* u0, const float* u1, float* u2, float wavespeed, float dt, float dx,
                     float dy, int N, int M, int M_padded, void* stream);

/*
 * Variable density (2D): the conservative acoustic operator
 *     u_{n+1} = g (2 u_n + k Lb u_n + src_scale * w_n) - g^2 u_{n-1},
 *     k = kappa dt^2 / dx^2,  Lb u = Dx^- (b Dx^+ u) + (dx/dz)^2 Dz^- (b Dz^+ u),
 * b = 1 / rho averaged onto the half points, Dx^+ / Dx^- the order-`order`
 * staggered differences on a unit grid (fields and b zero outside the grid);
 * the two-phase medium of cuwave's AcousticWave (projects/8_physics_drivers/
 * waveND.py:52-65), which has no counterpart in this repository's reference
 * kernels. kappa and rho are [nz][nx] FP32 device arrays; the other arguments
 * and the workspace rules are those of wfd_forward / wfd_misfit_gradient
 * (2D, step_block 0/1, lap_store WFD_LAP_AUTO, FP32 fields, no shot groups;
 * store_levels keeps forward levels as in the constant-density path).
 * wfd_vd_misfit_gradient returns dJ/dkappa and dJ/drho, each [nz][nx] and
 * summed over the shots, and optionally dJ/dwavelet.
 * The CFL check reads p->vmax as the operator's speed bound:
 *     vmax^2 >= max_i kappa_i (B_i^z / dz^2 + B_i^x / dx^2) / (2 C (1/dz^2 + 1/dx^2)),
 *     B_i = sum_k |c_k| (b_{i+k-1/2} + b_{i-k+1/2}) along that axis,  C = sum_k |c_k|,
 * the absolute row sums of the operator (Gershgorin). For smooth media that
 * is max kappa / rho; where 1/rho jumps between neighbours (air beside a
 * solid) it is up to ~100x larger, and a vmax of max sqrt(kappa/rho) there
 * lets an unstable dt through. neuralmech_gb300.wavefd.vd_vmax computes it.
 */
int wfd_vd_workspace_bytes(const wfd_problem* p, int with_gradient, size_t* bytes);
int wfd_vd_forward(const wfd_problem* p, const float* kappa, const float* rho, const float* sponge_z,
                   const float* sponge_x, const float* wavelet, const int32_t* src, const int32_t* rec,
                   float* traces, void* workspace, size_t workspace_bytes, void* stream);
/* wfd_vd_forward plus the last field u_nt of every shot, [nshot][nz][nx]
 * (cuwave simulate on an AcousticWave, projects/8_physics_drivers/waveND.py:94
 * with FORMULATION = "acoustic"). */
int wfd_vd_forward_final(const wfd_problem* p, const float* kappa, const float* rho, const float* sponge_z,
                         const float* sponge_x, const float* wavelet, const int32_t* src, const int32_t* rec,
                         float* traces, float* u_final, void* workspace, size_t workspace_bytes, void* stream);
int wfd_vd_misfit_gradient(const wfd_problem* p, const float* kappa, const float* rho, const float* sponge_z,
                           const float* sponge_x, const float* wavelet, const int32_t* src, const int32_t* rec,
                           const float* observed, float* traces, float* grad_kappa, float* grad_rho,
                           float* grad_wavelet, double* misfit, void* workspace, size_t workspace_bytes,
                           void* stream);

/*
 * The same step with the field stored in FP16: mixed_step,
 * projects/18_simple_wave_fd/step2D_wave.cu:85-124, launched as in
 * 2D_wave_cuda_mixed.py. u0, u1, u2 are [N][M_padded] IEEE binary16 (raw
 * 16-bit patterns), M_padded even and > M, pointers 4-byte aligned; FP32
 * arithmetic, round to nearest even on store. u2 may alias u0.
 */
int wfd_step2d_mixed(const void* u0, const void* u1, void* u2, float wavespeed, float dt, float dx,
                     float dy, int N, int M, int M_padded, void* stream);

/*
 * mixed_step's update on FP16 fields with pre-divided weights, cx = k / dx^2
 * and cy = k / dy^2 (k = dt^2 c^2), and fused multiply-adds in FP32, rounded
 * to FP16 once per cell: within an FP16 rounding of the reference kernel as
 * its drivers build it (--use_fast_math, 2D_wave_cuda_mixed.py), not value for
 * value. A thread owns 8 consecutive values (16-byte loads and stores).
 * M_padded a multiple of 8, fields 16-byte aligned; u2 may alias u0.
 */
int wfd_step2d_mixed_fast(const void* u0, const void* u1, void* u2, float wavespeed, float dt, float dx,
                          float dy, int N, int M, int M_padded, void* stream);

/*
 * The same step with the field stored as int16 plus one FP32 scale per block
 * of 32 values along a row, u = s q: scaled_step, step2D_wave.cu:128-183, as
 * driven by 2D_wave_cuda_scaled.py. q* are [N][M_padded] int16 (8-byte
 * aligned), s* are [N][M_padded / 32] FP32, M_padded a multiple of 64. Each
 * new block's scale is its largest magnitude / 32767 and q = rint(u / s).
 * Interior rows are written in full (boundary columns and padding as 0);
 * rows 0 and N - 1 are left untouched. q2/s2 may alias q0/s0.
 */
int wfd_step2d_scaled(const int16_t* q0, const float* s0, const int16_t* q1, const float* s1,
                      int16_t* q2, float* s2, float wavespeed, float dt, float dx, float dy, int N,
                      int M, int M_padded, void* stream);

/*
 * Eight padded_step updates in one launch, with temporal_step's arguments and
 * results: projects/18_simple_wave_fd/step2D_wave.cu:244-304, launched as in
 * 2D_wave_cuda_temporal.py:68-79. u0 = u_{n-1}, u1 = u_n are [N][M_padded]
 * FP32; v0 receives u_{n+7} and v1 u_{n+8} on every cell i < N, j < M (the
 * padding columns are left untouched; boundary cells keep their u0 / u1
 * values). Each cell follows padded_step's expression in its operation order
 * (IEEE, no contraction), so the result equals eight launches of the
 * reference's padded_step source evaluated that way, value for value (the
 * reference states temporal_step is bit-identical to padded_step). v0 and v1 must
 * not overlap each other, u0 or u1; M_padded a multiple of 4, pointers 16-byte
 * aligned.
 */
int wfd_temporal_step(const float* u0, const float* u1, float* v0, float* v1, float wavespeed, float dt,
                      float dx, float dy, int N, int M, int M_padded, void* stream);

/*
 * temporal_step's eight updates (the arguments, cells and level roles of
 * wfd_temporal_step) evaluated as u_{n+1} = (2 u - u_{n-1}) + cx (u_{i-1} -
 * 2u + u_{i+1}) + cy (u_{j-1} - 2u + u_{j+1}) with the weights cx = k / dx^2,
 * cy = k / dy^2 divided once (k = dt^2 c^2) and fused multiply-adds: no
 * division per cell. Within FP32 rounding of the reference expression (1e-5
 * relative L2 over many launches), as the reference's own build with
 * --use_fast_math (2D_wave_cuda_temporal.py, COMPILER_OPTIONS) is, not value
 * for value. The window of each CTA lives in registers. Any M_padded >= M; no
 * alignment requirement. No counterpart beyond temporal_step itself.
 */
int wfd_temporal_step_fast(const float* u0, const float* u1, float* v0, float* v1, float wavespeed, float dt,
                           float dx, float dy, int N, int M, int M_padded, void* stream);

/*
 * The 1D 3-point step: step1D, projects/18_simple_wave_fd/step1D_wave.cu:4-17.
 * u0, u1, u2 are FP32 [N]; cells 1..N-2 of u2 receive
 * -u0 + 2 u1 + dt^2 c^2 (u1[i-1] - 2 u1[i] + u1[i+1]) / dx^2. u2 may alias u0.
 */
int wfd_step1d(const float* u0, const float* u1, float* u2, float wavespeed, float dt, float dx,
               int N, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* WAVEFD_H */
