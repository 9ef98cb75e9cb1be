// FP64 CPU oracle for the finite-difference acoustic wave path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: the parity tests, the
// smoke check and the CPU baseline of bench.py call it; the product library
// never links, loads or falls back to it.
//
// What it restates:
//  * the explicit 2nd-order-in-time update of projects/18_simple_wave_fd/
//    step2D_wave.cu:59-81 (padded_step) and 2D_wave_cupy.py:54-62 (fd_step):
//    u_new = 2 u - u_old + dt^2 c^2 Lap(u) on the interior, the outer ring held
//    fixed (homogeneous Dirichlet);
//  * generalised to space order 2R (R = 1, 2, 4) with the standard central
//    second-derivative weights, a per-cell velocity, 2D and 3D, and an
//    exponential (Cerjan) sponge applied as a per-cell factor g:
//        u_{n+1} = g (2 u_n + v^2 dt^2 L u_n + s w_n) - g^2 u_{n-1}
//    (damping both stored levels once per step, the classic sponge);
//  * point sources added at their cells (scaled by s and by g) and receivers
//    sampling u_{n+1} at their cells, traces laid out (shot, step, receiver)
//    as the reference's full matrix capture stacks them
//    (projects/18_fwi/plate.py:140-142);
//  * the L2 misfit J = 1/2 sum (d - d_obs)^2 and its exact discrete adjoint
//    gradient with respect to the velocity and to the wavelets, computed with
//    exact FP64 checkpoints and segment recomputation.
//
// All arrays are dense (no row padding), index (z, y, x) with x fastest; 2D
// problems have ny == 1 and no y stencil.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {

struct orc_problem {
    int32_t ndim;    // 2 or 3
    int32_t order;   // 2, 4 or 8
    int32_t nz, ny, nx;
    int32_t nshot, nt, nsrc, nrec;
    int32_t ckpt_every;  // 0: ceil(sqrt(nt))
    double dt, dz, dy, dx;
    double src_scale;
};

// Central second-derivative weights of order 2R on a unit grid:
// a_k = 2 (-1)^(k+1) (R!)^2 / (k^2 (R-k)! (R+k)!), a_0 = -2 sum_k a_k.
int orc_fd_coeffs(int order, double* a) {
    if (order != 2 && order != 4 && order != 6 && order != 8) return -1;
    const int R = order / 2;
    auto fact = [](int n) {
        double f = 1;
        for (int i = 2; i <= n; ++i) f *= i;
        return f;
    };
    double s = 0;
    for (int k = 1; k <= R; ++k) {
        a[k] = 2.0 * ((k % 2) ? 1.0 : -1.0) * fact(R) * fact(R) /
               (double(k) * k * fact(R - k) * fact(R + k));
        s += a[k];
    }
    a[0] = -2.0 * s;
    return 0;
}

}  // extern "C"

namespace {

struct Grid {
    int ndim, R, nz, ny, nx;
    long ncell;
    long sz, sy;  // strides of z and y
    double az[5], ay[5], ax[5];  // per-axis weights a_k / h^2
    double diag;                  // sum of the axis a_0 / h^2
};

Grid make_grid(const orc_problem& p) {
    Grid g{};
    g.ndim = p.ndim;
    g.R = p.order / 2;
    g.nz = p.nz;
    g.ny = p.ndim == 3 ? p.ny : 1;
    g.nx = p.nx;
    g.ncell = (long)g.nz * g.ny * g.nx;
    g.sy = g.nx;
    g.sz = (long)g.ny * g.nx;
    double a[5] = {0, 0, 0, 0, 0};
    orc_fd_coeffs(p.order, a);
    for (int k = 0; k <= g.R; ++k) {
        g.az[k] = a[k] / (p.dz * p.dz);
        g.ax[k] = a[k] / (p.dx * p.dx);
        g.ay[k] = p.ndim == 3 ? a[k] / (p.dy * p.dy) : 0.0;
    }
    g.diag = g.az[0] + g.ax[0] + (p.ndim == 3 ? g.ay[0] : 0.0);
    return g;
}

inline bool interior(const Grid& g, int z, int y, int x) {
    const int R = g.R;
    if (z < R || z >= g.nz - R || x < R || x >= g.nx - R) return false;
    if (g.ndim == 3 && (y < R || y >= g.ny - R)) return false;
    return true;
}

inline double laplacian(const Grid& g, const double* u, long c) {
    double s = g.diag * u[c];
    for (int k = 1; k <= g.R; ++k) {
        s += g.az[k] * (u[c - k * g.sz] + u[c + k * g.sz]);
        s += g.ax[k] * (u[c - k] + u[c + k]);
        if (g.ndim == 3) s += g.ay[k] * (u[c - k * g.sy] + u[c + k * g.sy]);
    }
    return s;
}

// Per-cell sponge factor from the 1D profiles (null profile = 1).
struct Sponge {
    const double *gz, *gy, *gx;
    double at(int z, int y, int x) const {
        double g = 1.0;
        if (gz) g *= gz[z];
        if (gy) g *= gy[y];
        if (gx) g *= gx[x];
        return g;
    }
};

// One interior update: un = g (2 uc + w Lap(uc)) - g^2 uo, w = v^2 dt^2.
// Writes only interior cells; lap_out (optional) receives Lap(uc) there.
void step(const Grid& g, const Sponge& sp, const double* w, const double* uo,
          const double* uc, double* un, double* lap_out) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < g.nz; ++z)
        for (int y = 0; y < g.ny; ++y)
            for (int x = 0; x < g.nx; ++x) {
                if (!interior(g, z, y, x)) continue;
                const long c = z * g.sz + y * g.sy + x;
                const double L = laplacian(g, uc, c);
                const double gg = sp.at(z, y, x);
                un[c] = gg * (2.0 * uc[c] + w[c] * L) - gg * gg * uo[c];
                if (lap_out) lap_out[c] = L;
            }
}

long cell_of(const Grid& g, const int32_t* pos) {
    return (long)pos[0] * g.sz + (long)pos[1] * g.sy + pos[2];
}

bool positions_ok(const Grid& g, const int32_t* pos, long n) {
    for (long i = 0; i < n; ++i) {
        const int32_t* q = pos + 3 * i;
        if (!interior(g, q[0], g.ndim == 3 ? q[1] : g.R, q[2])) return false;
        if (g.ndim == 2 && q[1] != 0) return false;
    }
    return true;
}

}  // namespace

extern "C" {

// One step of the generic update on dense arrays:
// un = g (2 uc + w Lap uc) - g^2 uo on the interior; the ring of un is left
// untouched. w is per cell (v^2 dt^2) when w_field is given, else w_const.
int orc_step(const orc_problem* p, const double* w_field, double w_const, const double* gz,
             const double* gy, const double* gx, const double* uo, const double* uc,
             double* un) {
    const Grid g = make_grid(*p);
    std::vector<double> wc;
    if (!w_field) {
        wc.assign(g.ncell, w_const);
        w_field = wc.data();
    }
    step(g, Sponge{gz, gy, gx}, w_field, uo, uc, un, nullptr);
    return 0;
}

// Forward modelling of nshot shots sharing one velocity model.
// vel[ncell], wavelet[nshot][nt][nsrc], src[nshot][nsrc][3], rec[nshot][nrec][3]
// (z, y, x; y = 0 in 2D) -> traces[nshot][nt][nrec], traces[s][n] = u_{n+1}(rec).
// u_final (optional) receives u_nt of every shot, [nshot][ncell].
int orc_forward(const orc_problem* p, const double* vel, const double* gz, const double* gy,
                const double* gx, const double* wavelet, const int32_t* src,
                const int32_t* rec, double* traces, double* u_final) {
    const Grid g = make_grid(*p);
    if (!positions_ok(g, src, (long)p->nshot * p->nsrc) ||
        !positions_ok(g, rec, (long)p->nshot * p->nrec))
        return -2;
    std::vector<double> w(g.ncell);
    for (long c = 0; c < g.ncell; ++c) w[c] = vel[c] * vel[c] * p->dt * p->dt;
    const Sponge sp{gz, gy, gx};
    std::vector<double> ua(g.ncell), ub(g.ncell);
    for (int s = 0; s < p->nshot; ++s) {
        std::fill(ua.begin(), ua.end(), 0.0);
        std::fill(ub.begin(), ub.end(), 0.0);
        double* uo = ua.data();  // u_{n-1}
        double* uc = ub.data();  // u_n
        const int32_t* sp_pos = src + 3L * s * p->nsrc;
        const int32_t* rp_pos = rec + 3L * s * p->nrec;
        for (int n = 0; n < p->nt; ++n) {
            step(g, sp, w.data(), uo, uc, uo, nullptr);  // uo now holds u_{n+1}
            for (int i = 0; i < p->nsrc; ++i) {
                const int32_t* q = sp_pos + 3 * i;
                const long c = cell_of(g, q);
                uo[c] += sp.at(q[0], q[1], q[2]) * p->src_scale *
                         wavelet[((long)s * p->nt + n) * p->nsrc + i];
            }
            for (int r = 0; r < p->nrec; ++r)
                traces[((long)s * p->nt + n) * p->nrec + r] = uo[cell_of(g, rp_pos + 3 * r)];
            std::swap(uo, uc);
        }
        if (u_final) std::memcpy(u_final + (long)s * g.ncell, uc, sizeof(double) * g.ncell);
    }
    return 0;
}

// Misfit J = 1/2 sum_{s,n,r} (d - d_obs)^2 and its exact discrete gradient.
//
// Adjoint, in the scaled variable q = w g mu (mu the Lagrange multiplier):
//   q_k = g (2 q_{k+1} + w L q_{k+1} + w P^T r_{k-1}) - g^2 q_{k+2},
//   k = nt .. 1, q_{nt+1} = q_{nt+2} = 0, r_n = d_n - d_obs_n,
// which is the forward update itself (L is symmetric on the interior).
//   dJ/dw      = sum_{n=0}^{nt-1} q_{n+1} L u_n / w
//   dJ/dv      = 2 v dt^2 dJ/dw
//   dJ/dwav_n  = s * q_{n+1}(src) / w(src)
// Forward states are recomputed per segment from exact FP64 checkpoints of
// (u_{k-1}, u_k) every ckpt_every steps.
// Outputs: grad_vel[ncell] (summed over shots), grad_wavelet[nshot][nt][nsrc]
// (optional), traces[nshot][nt][nrec] (optional), *misfit.
int orc_gradient(const orc_problem* p, const double* vel, const double* gz, const double* gy,
                 const double* gx, const double* wavelet, const int32_t* src,
                 const int32_t* rec, const double* observed, double* grad_vel,
                 double* grad_wavelet, double* traces, double* misfit) {
    const Grid g = make_grid(*p);
    if (!positions_ok(g, src, (long)p->nshot * p->nsrc) ||
        !positions_ok(g, rec, (long)p->nshot * p->nrec))
        return -2;
    const long N = g.ncell;
    const int nt = p->nt;
    const int K = p->ckpt_every > 0 ? p->ckpt_every : (int)std::ceil(std::sqrt((double)nt));
    const int nseg = (nt + K - 1) / K;
    std::vector<double> w(N);
    for (long c = 0; c < N; ++c) w[c] = vel[c] * vel[c] * p->dt * p->dt;
    const Sponge sp{gz, gy, gx};

    std::vector<double> G(N, 0.0);
    std::vector<double> ua(N), ub(N), qa(N), qb(N);
    std::vector<double> ckpt((size_t)nseg * 2 * N);
    std::vector<double> lap((size_t)K * N);
    std::vector<double> d((size_t)nt * p->nrec), res((size_t)nt * p->nrec);
    double J = 0.0;

    for (int s = 0; s < p->nshot; ++s) {
        const int32_t* sp_pos = src + 3L * s * p->nsrc;
        const int32_t* rp_pos = rec + 3L * s * p->nrec;
        const double* wav = wavelet + (long)s * nt * p->nsrc;
        auto inject = [&](double* u, int n) {
            for (int i = 0; i < p->nsrc; ++i) {
                const int32_t* q = sp_pos + 3 * i;
                u[cell_of(g, q)] += sp.at(q[0], q[1], q[2]) * p->src_scale * wav[n * p->nsrc + i];
            }
        };
        // forward pass with checkpoints of (u_{k-1}, u_k) at k = j K
        std::fill(ua.begin(), ua.end(), 0.0);
        std::fill(ub.begin(), ub.end(), 0.0);
        double* uo = ua.data();
        double* uc = ub.data();
        for (int n = 0; n < nt; ++n) {
            if (n % K == 0) {
                std::memcpy(&ckpt[(size_t)(n / K) * 2 * N], uo, sizeof(double) * N);
                std::memcpy(&ckpt[(size_t)(n / K) * 2 * N + N], uc, sizeof(double) * N);
            }
            step(g, sp, w.data(), uo, uc, uo, nullptr);
            inject(uo, n);
            for (int r = 0; r < p->nrec; ++r) d[(size_t)n * p->nrec + r] = uo[cell_of(g, rp_pos + 3 * r)];
            std::swap(uo, uc);
        }
        const double* obs = observed + (long)s * nt * p->nrec;
        for (size_t i = 0; i < d.size(); ++i) {
            res[i] = d[i] - obs[i];
            J += 0.5 * res[i] * res[i];
        }
        if (traces) std::memcpy(traces + (long)s * nt * p->nrec, d.data(), sizeof(double) * d.size());

        // adjoint pass, segment by segment from the last
        std::fill(qa.begin(), qa.end(), 0.0);
        std::fill(qb.begin(), qb.end(), 0.0);
        double* qo = qa.data();  // q_{k+2}
        double* qc = qb.data();  // q_{k+1}
        auto adjoint_step = [&](int k) {  // produces q_k into qo, then rotates
            step(g, sp, w.data(), qo, qc, qo, nullptr);
            for (int r = 0; r < p->nrec; ++r) {
                const int32_t* q = rp_pos + 3 * r;
                const long c = cell_of(g, q);
                qo[c] += sp.at(q[0], q[1], q[2]) * w[c] * res[(size_t)(k - 1) * p->nrec + r];
            }
            std::swap(qo, qc);  // qc = q_k
        };
        double* gw = grad_wavelet ? grad_wavelet + (long)s * nt * p->nsrc : nullptr;
        auto sample_wavelet_grad = [&](int n, const double* q_np1) {  // q_{n+1}
            if (!gw) return;
            for (int i = 0; i < p->nsrc; ++i) {
                const long c = cell_of(g, sp_pos + 3 * i);
                gw[n * p->nsrc + i] = p->src_scale * q_np1[c] / w[c];
            }
        };
        adjoint_step(nt);  // q_nt (its gradient term pairs q_{nt+1} = 0)
        for (int j = nseg - 1; j >= 0; --j) {
            const int k0 = j * K, k1 = std::min(nt, k0 + K);
            // recompute u_k and L u_k for k in [k0, k1)
            std::memcpy(ua.data(), &ckpt[(size_t)j * 2 * N], sizeof(double) * N);
            std::memcpy(ub.data(), &ckpt[(size_t)j * 2 * N + N], sizeof(double) * N);
            uo = ua.data();
            uc = ub.data();
            for (int k = k0; k < k1; ++k) {
                step(g, sp, w.data(), uo, uc, uo, &lap[(size_t)(k - k0) * N]);
                // lap of the ring is never read: gradient terms are interior only
                inject(uo, k);
                std::swap(uo, uc);
            }
            for (int k = k1 - 1; k >= std::max(k0, 1); --k) {
                // qc = q_{k+1}: gradient term q_{k+1} L u_k, wavelet term n = k
                const double* L = &lap[(size_t)(k - k0) * N];
#pragma omp parallel for schedule(static)
                for (long c = 0; c < N; ++c) G[c] += qc[c] * L[c];
                sample_wavelet_grad(k, qc);
                adjoint_step(k);  // qc = q_k
            }
        }
        sample_wavelet_grad(0, qc);  // qc = q_1
    }
    // G accumulates sum q L u on the interior (ring cells stay 0)
    for (int z = 0; z < g.nz; ++z)
        for (int y = 0; y < g.ny; ++y)
            for (int x = 0; x < g.nx; ++x) {
                const long c = z * g.sz + y * g.sy + x;
                grad_vel[c] = interior(g, z, y, x) ? 2.0 * vel[c] * p->dt * p->dt * G[c] / w[c] : 0.0;
            }
    *misfit = J;
    return 0;
}

}  // extern "C"
