/*
 * A plain C caller of libwavefd.so, compiled by gcc against include/wavefd.h:
 * the boundary as a foreign-function binding (cgo, JNI, ctypes) sees it, with
 * no C++ and no PyTorch on the caller's side.
 *
 *   check_abi layout  prints sizeof(wfd_problem) and every field's offset, one
 *                     "name offset" line each (wfd_batch_item's as "item.name"),
 *                     for comparison with the ctypes mirrors of the structs;
 *   check_abi host    host-only calls: version, status texts, workspace sizes
 *                     and the argument checks (no CUDA call; runs without a GPU);
 *   check_abi gpu     compute calls on device 0 through the CUDA runtime:
 *                     - wfd_step2d_order2 and wfd_step2d_exact against the
 *                       padded_step update evaluated here in double
 *                       (projects/18_simple_wave_fd/step2D_wave.cu:59-81),
 *                       the boundary ring and the padding columns untouched;
 *                     - wfd_forward, wfd_forward_final and wfd_forward_static
 *                       on one small problem (traces within 1e-6 of each other);
 *                     - wfd_misfit_gradient against zero observed data (J equals
 *                       half the sum of squares of its own traces; the gradient
 *                       is finite, nonzero, and zero on the fixed ring);
 *                     - the same gradient twice in one planned batch (one CUDA
 *                       graph), replayed twice: each item as the single call;
 *                     - a source on the fixed ring reported by wfd_status as
 *                       WFD_ERR_POSITION (the kernel skips that point).
 * Exit status 0 when every check holds; each failed check prints one line.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "wavefd.h"

static int failures = 0;

#define CHECK(cond, ...)                                                  \
    do {                                                                  \
        if (!(cond)) {                                                    \
            fprintf(stderr, "FAIL %s:%d: ", __FILE__, __LINE__);          \
            fprintf(stderr, __VA_ARGS__);                                 \
            fprintf(stderr, " [last error: %s]\n", wfd_last_error());     \
            ++failures;                                                   \
        }                                                                 \
    } while (0)

#define FIELD(name) printf(#name " %zu\n", offsetof(wfd_problem, name))

static int layout(void) {
    printf("sizeof %zu\n", sizeof(wfd_problem));
    FIELD(ndim); FIELD(order); FIELD(nz); FIELD(ny); FIELD(nx); FIELD(nshot); FIELD(nt);
    FIELD(nsrc); FIELD(nrec); FIELD(ckpt_every); FIELD(ckpt_format); FIELD(lap_store);
    FIELD(shots_per_cta); FIELD(group_shots); FIELD(tile_rows); FIELD(step_block);
    FIELD(store_levels); FIELD(field_format); FIELD(adjoint_mode); FIELD(recon_band);
    FIELD(dt); FIELD(dz); FIELD(dy); FIELD(dx); FIELD(src_scale); FIELD(vmax); FIELD(update_form);
    FIELD(level_format);
    printf("item.sizeof %zu\n", sizeof(wfd_batch_item));
#define ITEM(name) printf("item." #name " %zu\n", offsetof(wfd_batch_item, name))
    ITEM(problem); ITEM(vel); ITEM(sponge_z); ITEM(sponge_y); ITEM(sponge_x); ITEM(wavelet); ITEM(src);
    ITEM(rec); ITEM(observed); ITEM(traces); ITEM(grad_vel); ITEM(grad_wavelet); ITEM(misfit);
    ITEM(workspace); ITEM(workspace_bytes);
#undef ITEM
    return 0;
}

/* 2D order-8 problem of 64 x 100 cells, two shots; c = 3000, h = 10, dt = 1e-3. */
static wfd_problem small_problem(void) {
    wfd_problem p;
    memset(&p, 0, sizeof p);
    p.ndim = 2; p.order = 8; p.nz = 64; p.ny = 1; p.nx = 100;
    p.nshot = 2; p.nt = 50; p.nsrc = 1; p.nrec = 5;
    p.ckpt_format = WFD_CKPT_BF16;
    p.dt = 1e-3f; p.dz = 10.0f; p.dy = 1.0f; p.dx = 10.0f;
    p.src_scale = 1.0f; p.vmax = 3000.0f;
    return p;
}

static int expect_invalid(wfd_problem p, int with_gradient, int code) {
    size_t n = 0;
    return wfd_workspace_bytes(&p, with_gradient, &n) == code && wfd_last_error()[0] != '\0';
}

static int host(void) {
    CHECK((wfd_version() >> 16) == 3, "ABI major %d", wfd_version() >> 16);
    const char* seen[8];
    for (int c = 0; c >= -7; --c) {
        const char* s = wfd_strerror(c);
        CHECK(s && s[0], "wfd_strerror(%d) empty", c);
        seen[-c] = s;
        for (int k = 0; k < -c; ++k) CHECK(strcmp(seen[k], s) != 0, "status %d shares a text", c);
    }
    CHECK(strcmp(wfd_strerror(-99), "unknown status") == 0, "wfd_strerror(-99)");
    CHECK(wfd_kernel_launches() == 0, "launches before any call");

    wfd_problem p = small_problem();
    size_t fwd = 0, grad = 0;
    CHECK(wfd_workspace_bytes(&p, 0, &fwd) == WFD_OK && fwd >= (size_t)2 * 2 * 64 * 100 * 4,
          "forward workspace %zu", fwd);
    CHECK(wfd_workspace_bytes(&p, 1, &grad) == WFD_OK && grad > fwd, "gradient workspace %zu", grad);
    CHECK(wfd_workspace_bytes(NULL, 0, &fwd) == WFD_ERR_INVALID, "NULL problem");
    CHECK(wfd_workspace_bytes(&p, 0, NULL) == WFD_ERR_INVALID, "NULL size");

    wfd_problem q;
    q = p; q.order = 6; CHECK(expect_invalid(q, 0, WFD_ERR_INVALID), "order 6");
    q = p; q.ndim = 4; CHECK(expect_invalid(q, 0, WFD_ERR_INVALID), "ndim 4");
    q = p; q.nz = 8; CHECK(expect_invalid(q, 0, WFD_ERR_INVALID), "nz 8 at order 8");
    q = p; q.nt = 0; CHECK(expect_invalid(q, 0, WFD_ERR_INVALID), "nt 0");
    q = p; q.dx = -1.0f; CHECK(expect_invalid(q, 0, WFD_ERR_INVALID), "negative dx");
    q = p; q.update_form = 3; CHECK(expect_invalid(q, 0, WFD_ERR_INVALID), "update_form 3");
    q = p; q.vmax = 1e6f; CHECK(expect_invalid(q, 0, WFD_ERR_UNSTABLE), "CFL");
    /* eight steps per launch: order 2 only, forward only */
    q = p; q.order = 2; q.step_block = 8;
    CHECK(wfd_workspace_bytes(&q, 0, &fwd) == WFD_OK, "order 2, step_block 8 forward");
    CHECK(expect_invalid(q, 1, WFD_ERR_INVALID), "order 2, step_block 8 gradient");
    q.order = 4; CHECK(expect_invalid(q, 0, WFD_ERR_INVALID), "order 4, step_block 8");
    q.step_block = 4; CHECK(wfd_workspace_bytes(&q, 0, &fwd) == WFD_OK, "order 4, step_block 4");
    q.step_block = 3; CHECK(expect_invalid(q, 0, WFD_ERR_INVALID), "step_block 3");

    /* null device pointers are refused before any launch */
    CHECK(wfd_forward(&p, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, 0, NULL, 0, NULL) ==
              WFD_ERR_INVALID, "wfd_forward with NULL arrays");
    CHECK(wfd_step2d_order2(NULL, NULL, NULL, 1.0f, 1.0f, 1.0f, 1.0f, 10, 10, 12, NULL) == WFD_ERR_INVALID,
          "wfd_step2d_order2 with NULL fields");
    CHECK(wfd_status(NULL, NULL) == WFD_ERR_WORKSPACE, "wfd_status without a workspace");
    wfd_batch* none = NULL;
    wfd_batch_item empty[2];
    memset(empty, 0, sizeof empty);
    CHECK(wfd_batch_plan(empty, 2, NULL, &none) == WFD_ERR_INVALID && none == NULL, "batch item without a problem");
    CHECK(wfd_batch_plan(empty, 0, NULL, &none) == WFD_ERR_INVALID, "empty batch");
    CHECK(wfd_kernel_launches() == 0, "a host-only call launched a kernel");
    return failures;
}

/* ---- GPU mode: device memory through the CUDA runtime's C API ---- */
static const enum cudaMemcpyKind H2D = cudaMemcpyHostToDevice, D2H = cudaMemcpyDeviceToHost;

static void* dalloc(size_t n) {
    void* p = NULL;
    if (cudaMalloc(&p, n) != cudaSuccess) {
        fprintf(stderr, "cudaMalloc(%zu) failed\n", n);
        exit(2);
    }
    return p;
}

static void* upload(const void* h, size_t n) {
    void* d = dalloc(n);
    cudaMemcpy(d, h, n, H2D);
    return d;
}

static uint32_t lcg_state = 12345u;
static float uniform(void) { /* in [-1, 1) */
    lcg_state = lcg_state * 1664525u + 1013904223u;
    return (float)((lcg_state >> 8) & 0xffffff) / 8388608.0f - 1.0f;
}

static void check_step(int exact) {
    const int N = 37, M = 70, Mp = 72;
    const float c = 1500.0f, dt = 1e-3f, dx = 5.0f, dy = 4.0f;
    const size_t cells = (size_t)N * Mp, bytes = cells * sizeof(float);
    float* h0 = malloc(bytes); float* h1 = malloc(bytes); float* h2 = malloc(bytes);
    for (size_t k = 0; k < cells; ++k) { h0[k] = uniform(); h1[k] = uniform(); h2[k] = 7.0f; }
    float* u0 = upload(h0, bytes); float* u1 = upload(h1, bytes); float* u2 = upload(h2, bytes);
    int rc = exact ? wfd_step2d_exact(u0, u1, u2, c, dt, dx, dy, N, M, Mp, NULL)
                   : wfd_step2d_order2(u0, u1, u2, c, dt, dx, dy, N, M, Mp, NULL);
    CHECK(rc == WFD_OK, "step (exact %d) status %d", exact, rc);
    cudaMemcpy(h2, u2, bytes, D2H);
    double worst = 0.0;
    int untouched = 1;
    const double k2 = (double)dt * dt * c * c;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < Mp; ++j) {
            const float got = h2[(size_t)i * Mp + j];
            if (i == 0 || i == N - 1 || j == 0 || j >= M - 1) { untouched &= got == 7.0f; continue; }
            const size_t a = (size_t)i * Mp + j;
            const double lx = ((double)h1[a + Mp] - 2.0 * h1[a] + h1[a - Mp]) / ((double)dx * dx);
            const double ly = ((double)h1[a + 1] - 2.0 * h1[a] + h1[a - 1]) / ((double)dy * dy);
            const double want = -(double)h0[a] + 2.0 * h1[a] + k2 * (lx + ly);
            const double e = fabs(got - want) / (1.0 + fabs(want));
            if (e > worst) worst = e;
        }
    CHECK(worst < 1e-5, "step (exact %d) worst error %.3e", exact, worst);
    CHECK(untouched, "step (exact %d) wrote the ring or a padding column", exact);
    cudaFree(u0); cudaFree(u1); cudaFree(u2);
    free(h0); free(h1); free(h2);
}

static double rel_diff(const float* a, const float* b, size_t n) {
    double num = 0.0, den = 0.0;
    for (size_t k = 0; k < n; ++k) {
        num += ((double)a[k] - b[k]) * ((double)a[k] - b[k]);
        den += (double)b[k] * b[k];
    }
    return den > 0.0 ? sqrt(num / den) : (num > 0.0 ? 1.0 : 0.0);
}

static int gpu(void) {
    check_step(0);
    check_step(1);

    wfd_problem p = small_problem();
    const int nz = p.nz, nx = p.nx, ns = p.nshot, nt = p.nt, nr = p.nrec, R = p.order / 2;
    const size_t cells = (size_t)nz * nx, ntr = (size_t)ns * nt * nr;
    float* vel = malloc(cells * sizeof(float));
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nx; ++x) vel[(size_t)z * nx + x] = z < 30 ? 2000.0f : 3000.0f;
    float* wav = malloc((size_t)ns * nt * sizeof(float));
    for (int s = 0; s < ns; ++s)
        for (int n = 0; n < nt; ++n) {
            const double a = 3.14159265358979 * 40.0 * (n * p.dt - 0.03);
            wav[(size_t)s * nt + n] = (float)((1.0 - 2.0 * a * a) * exp(-a * a));
        }
    int32_t src[2][1][3] = {{{6, 0, 30}}, {{6, 0, 70}}};
    int32_t rec[2][5][3];
    for (int s = 0; s < ns; ++s)
        for (int r = 0; r < nr; ++r) { rec[s][r][0] = 5; rec[s][r][1] = 0; rec[s][r][2] = 10 + 20 * r; }

    float* d_vel = upload(vel, cells * sizeof(float));
    float* d_wav = upload(wav, (size_t)ns * nt * sizeof(float));
    int32_t* d_src = upload(src, sizeof src);
    int32_t* d_rec = upload(rec, sizeof rec);
    size_t wsb = 0;
    CHECK(wfd_workspace_bytes(&p, 1, &wsb) == WFD_OK, "workspace");
    void* ws = dalloc(wsb);
    float* d_tr = dalloc(ntr * sizeof(float));
    float* d_fin = dalloc((size_t)ns * cells * sizeof(float));
    float* t_fwd = malloc(ntr * sizeof(float));
    float* t_other = malloc(ntr * sizeof(float));

    const uint64_t launches0 = wfd_kernel_launches();
    CHECK(wfd_profile_begin() == WFD_OK, "wfd_profile_begin");
    CHECK(wfd_forward(&p, d_vel, NULL, NULL, NULL, d_wav, d_src, d_rec, d_tr, 0, ws, wsb, NULL) == WFD_OK,
          "wfd_forward");
    wfd_phase_times ph;
    memset(&ph, 0, sizeof ph);
    CHECK(wfd_profile_end(&ph) == WFD_OK && ph.launches[0] > 0 && ph.ms[0] > 0.0,
          "profile: %lld forward launches, %.3f ms", (long long)ph.launches[0], ph.ms[0]);
    CHECK(wfd_status(ws, NULL) == WFD_OK, "wfd_status after wfd_forward");
    CHECK(wfd_kernel_launches() > launches0, "no launch counted");
    cudaMemcpy(t_fwd, d_tr, ntr * sizeof(float), D2H);
    double peak = 0.0;
    for (size_t k = 0; k < ntr; ++k) {
        CHECK(isfinite(t_fwd[k]), "trace sample %zu not finite", k);
        if (fabs(t_fwd[k]) > peak) peak = fabs(t_fwd[k]);
        if (!isfinite(t_fwd[k])) break;
    }
    CHECK(peak > 0.0, "all traces zero");

    cudaMemset(d_tr, 0, ntr * sizeof(float));
    CHECK(wfd_forward_final(&p, d_vel, NULL, NULL, NULL, d_wav, d_src, d_rec, d_tr, d_fin, ws, wsb, NULL) ==
              WFD_OK, "wfd_forward_final");
    cudaMemcpy(t_other, d_tr, ntr * sizeof(float), D2H);
    CHECK(rel_diff(t_other, t_fwd, ntr) <= 1e-6, "wfd_forward_final traces %.3e", rel_diff(t_other, t_fwd, ntr));
    float* fin = malloc((size_t)ns * cells * sizeof(float));
    cudaMemcpy(fin, d_fin, (size_t)ns * cells * sizeof(float), D2H);
    double ring = 0.0, inner = 0.0;
    for (int s = 0; s < ns; ++s)
        for (int z = 0; z < nz; ++z)
            for (int x = 0; x < nx; ++x) {
                const double v = fabs(fin[((size_t)s * nz + z) * nx + x]);
                if (z < R || z >= nz - R || x < R || x >= nx - R) ring += v; else inner += v;
            }
    CHECK(ring == 0.0 && inner > 0.0, "final field: ring %.3e, interior %.3e", ring, inner);
    free(fin);

    cudaMemset(d_tr, 0, ntr * sizeof(float));
    CHECK(wfd_forward_static(&p, d_vel, NULL, NULL, NULL, d_wav, d_src, d_rec, d_tr, NULL) == WFD_OK,
          "wfd_forward_static");
    CHECK(wfd_forward_static_status(NULL) == WFD_OK, "wfd_forward_static_status");
    cudaMemcpy(t_other, d_tr, ntr * sizeof(float), D2H);
    CHECK(rel_diff(t_other, t_fwd, ntr) <= 1e-6, "wfd_forward_static traces %.3e", rel_diff(t_other, t_fwd, ntr));

    /* misfit against zero data: J = 1/2 sum of its own traces squared */
    float* d_obs = dalloc(ntr * sizeof(float));
    cudaMemset(d_obs, 0, ntr * sizeof(float));
    float* d_g = dalloc(cells * sizeof(float));
    double* d_J = dalloc(sizeof(double));
    cudaMemset(d_J, 0, sizeof(double));
    CHECK(wfd_misfit_gradient(&p, d_vel, NULL, NULL, NULL, d_wav, d_src, d_rec, d_obs, d_tr, d_g, NULL, d_J, ws,
                              wsb, NULL) == WFD_OK, "wfd_misfit_gradient");
    CHECK(wfd_status(ws, NULL) == WFD_OK, "wfd_status after wfd_misfit_gradient");
    double J = 0.0, want = 0.0;
    cudaMemcpy(&J, d_J, sizeof J, D2H);
    cudaMemcpy(t_other, d_tr, ntr * sizeof(float), D2H);
    for (size_t k = 0; k < ntr; ++k) want += 0.5 * (double)t_other[k] * t_other[k];
    CHECK(want > 0.0 && fabs(J - want) <= 1e-6 * want, "misfit %.9e, half sum of squares %.9e", J, want);
    CHECK(rel_diff(t_other, t_fwd, ntr) <= 1e-5, "gradient-call traces %.3e", rel_diff(t_other, t_fwd, ntr));
    float* g = malloc(cells * sizeof(float));
    cudaMemcpy(g, d_g, cells * sizeof(float), D2H);
    ring = 0.0; inner = 0.0;
    int finite = 1;
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nx; ++x) {
            const double v = g[(size_t)z * nx + x];
            finite &= isfinite(v) != 0;
            if (z < R || z >= nz - R || x < R || x >= nx - R) ring += fabs(v); else inner += fabs(v);
        }
    CHECK(finite && ring == 0.0 && inner > 0.0, "gradient: finite %d, ring %.3e, interior %.3e", finite, ring,
          inner);
    free(g);

    /* the same gradient as a two-item batch (one graph): each item against the single call */
    {
        float* d_g2[2];
        double* d_J2[2];
        void* ws2[2];
        wfd_batch_item it[2];
        memset(it, 0, sizeof it);
        for (int i = 0; i < 2; ++i) {
            d_g2[i] = dalloc(cells * sizeof(float));
            d_J2[i] = dalloc(sizeof(double));
            ws2[i] = dalloc(wsb);
            it[i].problem = &p;
            it[i].vel = d_vel; it[i].wavelet = d_wav; it[i].src = d_src; it[i].rec = d_rec;
            it[i].observed = d_obs; it[i].grad_vel = d_g2[i]; it[i].misfit = d_J2[i];
            it[i].workspace = ws2[i]; it[i].workspace_bytes = wsb;
        }
        wfd_batch* bt = NULL;
        CHECK(wfd_batch_plan(it, 2, NULL, &bt) == WFD_OK && bt != NULL, "wfd_batch_plan");
        CHECK(wfd_batch_launches(bt) > 0, "batch graph without kernels");
        float* g1 = malloc(cells * sizeof(float));
        float* g2 = malloc(cells * sizeof(float));
        cudaMemcpy(g1, d_g, cells * sizeof(float), D2H);
        for (int rep = 0; rep < 2; ++rep) {
            for (int i = 0; i < 2; ++i) cudaMemset(d_g2[i], 0, cells * sizeof(float));
            CHECK(wfd_batch_run(bt, NULL) == WFD_OK, "wfd_batch_run");
            for (int i = 0; i < 2; ++i) {
                double Jb = 0.0;
                cudaMemcpy(&Jb, d_J2[i], sizeof Jb, D2H);
                cudaMemcpy(g2, d_g2[i], cells * sizeof(float), D2H);
                CHECK(fabs(Jb - J) <= 1e-9 * J, "batch misfit %.9e against %.9e", Jb, J);
                CHECK(rel_diff(g2, g1, cells) <= 1e-6, "batch gradient %.3e", rel_diff(g2, g1, cells));
                CHECK(wfd_status(ws2[i], NULL) == WFD_OK, "wfd_status of a batch item");
            }
        }
        CHECK(wfd_batch_free(bt) == WFD_OK, "wfd_batch_free");
        for (int i = 0; i < 2; ++i) { cudaFree(d_g2[i]); cudaFree(d_J2[i]); cudaFree(ws2[i]); }
        free(g1); free(g2);
    }

    /* a source on the fixed ring: reported on the device, the point skipped */
    int32_t bad[2][1][3] = {{{1, 0, 30}}, {{6, 0, 70}}};
    cudaMemcpy(d_src, bad, sizeof bad, H2D);
    CHECK(wfd_forward(&p, d_vel, NULL, NULL, NULL, d_wav, d_src, d_rec, d_tr, 0, ws, wsb, NULL) == WFD_OK,
          "wfd_forward with a source on the ring");
    CHECK(wfd_status(ws, NULL) == WFD_ERR_POSITION, "ring source not reported");
    CHECK(wfd_status(ws, NULL) == WFD_OK, "wfd_status did not clear");
    CHECK(cudaDeviceSynchronize() == cudaSuccess, "device error");

    cudaFree(d_vel); cudaFree(d_wav); cudaFree(d_src); cudaFree(d_rec); cudaFree(ws); cudaFree(d_tr);
    cudaFree(d_fin); cudaFree(d_obs); cudaFree(d_g); cudaFree(d_J);
    free(vel); free(wav); free(t_fwd); free(t_other);
    return failures;
}

int main(int argc, char** argv) {
    const char* mode = argc > 1 ? argv[1] : "host";
    int rc;
    if (strcmp(mode, "layout") == 0) rc = layout();
    else if (strcmp(mode, "host") == 0) rc = host();
    else if (strcmp(mode, "gpu") == 0) rc = host() + gpu();
    else {
        fprintf(stderr, "usage: %s layout|host|gpu\n", argv[0]);
        return 2;
    }
    if (rc == 0 && strcmp(mode, "layout") != 0) printf("ok (%s)\n", mode);
    return rc == 0 ? 0 : 1;
}
