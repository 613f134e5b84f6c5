// vpmc_query.cu -- vorticity queries at arbitrary points, the matrix-free RBF
// SpMV and the CG / MINRES strength solves, all on the evaluation grid of
// vpmc_grid.cu.
#include <cmath>
#include <utility>
#include <vector>

#include "vpmc_grid.cuh"

namespace vpmc {
namespace {

int blocks_for(long n) {
    long b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > 65535L * 8) b = 65535L * 8;
    return int(b);
}

// Queries = the candidates themselves (RBF SpMV): qrec[p] = cand[p], output
// slot = sorted slot (use_perm = 0) or original index (use_perm = 1).
__global__ void k_self_queries(const Cand* __restrict__ cand, const uint32_t* __restrict__ perm,
                               const uint32_t* __restrict__ start, long n, uint32_t nbins, int use_perm,
                               QRec* __restrict__ q) {
    const long nv = start[nbins];
    for (long p = long(blockIdx.x) * blockDim.x + threadIdx.x; p < nv && p < n; p += long(gridDim.x) * blockDim.x) {
        const Cand c = cand[p];
        q[p] = QRec{c.x, c.y, use_perm ? perm[p] : uint32_t(p), (2u) | (2u << 3)};
    }
}

__global__ void k_gather_to_sorted(const float* __restrict__ x, const uint32_t* __restrict__ perm, long n,
                                   double* __restrict__ xs) {
    for (long p = long(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += long(gridDim.x) * blockDim.x)
        xs[p] = double(x[perm[p]]);
}

__global__ void k_gather_to_sorted_d(const double* __restrict__ x, const uint32_t* __restrict__ perm, long n,
                                     double* __restrict__ xs) {
    for (long p = long(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += long(gridDim.x) * blockDim.x)
        xs[p] = x[perm[p]];
}

__global__ void k_scatter_from_sorted(const double* __restrict__ xs, const uint32_t* __restrict__ perm, long n,
                                      float* __restrict__ x) {
    for (long p = long(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += long(gridDim.x) * blockDim.x)
        x[perm[p]] = float(xs[p]);
}

__global__ void k_scale_f32(float* __restrict__ a, long n, float s) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) a[i] *= s;
}

// CG vector updates (FP64).
__global__ void k_cg_init(const double* __restrict__ b, const double* __restrict__ Ax, long n,
                          double* __restrict__ r, double* __restrict__ p) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const double v = b[i] - Ax[i];
        r[i] = v;
        p[i] = v;
    }
}
__global__ void k_cg_xr(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                        const double* __restrict__ Ap, long n, double alpha) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        x[i] += alpha * p[i];
        r[i] -= alpha * Ap[i];
    }
}
__global__ void k_cg_p(double* __restrict__ p, const double* __restrict__ r, long n, double beta) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
        p[i] = r[i] + beta * p[i];
}
__global__ void k_axpby(const double* __restrict__ a, const double* __restrict__ b, long n, double sa, double sb,
                        double* __restrict__ out) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
        out[i] = sa * a[i] + sb * b[i];
}

// MINRES vector steps (FP64).
// u = Av - alpha v - beta v_old  (the next Lanczos vector before normalisation)
// (Av and u may be the same array: each element is read before it is written)
__global__ void k_minres_u(const double* Av, const double* __restrict__ v, const double* __restrict__ v_old, long n,
                           double alpha, double beta, double* u) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
        u[i] = Av[i] - alpha * v[i] - beta * v_old[i];
}
// w_new = (v - rho3 w_old - rho2 w) / rho1 (written over w_old), x += c w_new,
// v_next = u / beta_n (written over v_old)
__global__ void k_minres_step(const double* __restrict__ v, double* __restrict__ w_old, const double* __restrict__ w,
                              double* __restrict__ x, const double* __restrict__ u, double* __restrict__ v_old, long n,
                              double rho1, double rho2, double rho3, double c, double inv_beta_n) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const double wn = (v[i] - rho3 * w_old[i] - rho2 * w[i]) / rho1;
        w_old[i] = wn;
        x[i] += c * wn;
        v_old[i] = u[i] * inv_beta_n;
    }
}

// Working set for one single-instance grid plus self/point queries.
struct Work {
    GridInst plan;
    GridBufs g;
    ItemBufs it;
    QueryBufs q;
    QRec* self = nullptr;
    double* vec[8] = {};
    double* dtmp = nullptr;
};

int setup(vpmc_context* ctx, int slot, long N, float hw, float Lx, float Ly, int periodic, long M, int nvec,
          Work* w, int k = 0, float cover = 1.f, bool deformed = false) {
    InstDesc d{Lx, Ly, hw, periodic, 0, int(N), cover};
    const long nb = grid_plan(&d, 1, k, 1, &w->plan);
    if (nb < 0) return int(-nb);
    const long nq = M > N ? M : N;
    auto carve_all = [&](Carver& c) {
        carve_grid(c, N, nb, 1, &w->g, deformed);
        carve_items(c, nb, nq, &w->it);
        if (M > 0) carve_queries(c, nb, M, &w->q);
        w->self = c.take<QRec>(size_t(N < 1 ? 1 : N));
        for (int i = 0; i < nvec; ++i) w->vec[i] = c.take<double>(size_t(N < 1 ? 1 : N));
        w->dtmp = c.take<double>(dot_tmp_elems(N) + 8);
    };
    Carver dry;
    carve_all(dry);
    char* base = nullptr;
    VPMC_TRY(scratch(ctx, slot, dry.off, &base));
    Carver c{base, 0};
    carve_all(c);
    VPMC_CUDA(cudaMemcpyAsync(w->g.inst, &w->plan, sizeof(GridInst), cudaMemcpyHostToDevice, ctx->stream));
    return VPMC_OK;
}

// y_sorted = A x_sorted (FP64), grid already built, self queries set.
int spmv_sorted(vpmc_context* ctx, Work& w, const double* x_sorted, double* y_sorted, bool precise) {
    // FP64 pairs use W with its sigma; the FP32 form evaluates W / (2 sigma)
    VPMC_TRY(grid_set_weights_sorted(ctx, w.g, x_sorted, precise ? 1.0 : double(w.plan.two_sigma)));
    EvalLaunch L;
    L.mode = precise ? EVAL_SPMV64 : EVAL_SPMV32;
    L.out_f64 = y_sorted;
    VPMC_CUDA(cudaMemsetAsync(w.it.counter, 0, sizeof(uint32_t), ctx->stream));
    return launch_eval(ctx, w.g, w.self, w.it, L);
}

int host_dot(vpmc_context* ctx, Work& w, const double* a, const double* b, long n, double* out) {
    double* d = w.dtmp;
    VPMC_TRY(dot_f64(ctx, a, b, n, d + dot_tmp_elems(n), d));
    VPMC_CUDA(cudaMemcpyAsync(out, d + dot_tmp_elems(n), sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    VPMC_CUDA(cudaStreamSynchronize(ctx->stream));
    return VPMC_OK;
}

}  // namespace
}  // namespace vpmc

using namespace vpmc;

extern "C" {

int vpmc_query_vorticity(vpmc_context* ctx, int N, const float* pos, const float* omega, const float* F, int M,
                         const float* pts, int sign, int use_signed, int exclude_center, float h_w, float Lx,
                         float Ly, int periodic, float* out) {
    if (!ctx || N < 0 || M < 0 || !(h_w > 0.f) || !(Lx > 0.f) || !(Ly > 0.f)) return VPMC_ERR_INVALID;
    if ((N > 0 && (!pos || !omega)) || (M > 0 && (!pts || !out))) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    if (M == 0) return VPMC_OK;
    cudaStream_t st = ctx->stream;
    VPMC_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * size_t(M), st));
    if (N == 0) return vpmc_context_sync(ctx);
    // deformed kernels: the walk must reach sigma_max(F) h_w (at most 2 h_w,
    // the reach of the reference's 3x3 walk of 2 h_w cells)
    float cover = 1.f;
    if (F) {
        char* sb = nullptr;
        VPMC_TRY(scratch(ctx, SLOT_MISC, 64, &sb));
        float sig = 1.f;
        VPMC_TRY(grid_max_sigma(ctx, reinterpret_cast<const float4*>(F), N, reinterpret_cast<unsigned*>(sb), &sig));
        if (!(sig <= 3.0e38f)) return VPMC_ERR_INVALID;   // non-finite F or det F <= 0
        cover = sig > 1.f ? std::min(2.f, std::ceil(sig * 16.f) / 16.f) : 1.f;
    }
    Work w;
    VPMC_TRY(setup(ctx, SLOT_QUERY, N, h_w, Lx, Ly, periodic, M, 0, &w, 0, cover, F != nullptr));
    const int set_mode = sign > 0 ? SET_POS_ONLY
                                   : (sign < 0 ? SET_NEG_ONLY : (use_signed ? SET_ONE_SIGNED : SET_ONE_ABS));
    VPMC_TRY(grid_build(ctx, w.g, reinterpret_cast<const float2*>(pos), omega, set_mode,
                        reinterpret_cast<const float4*>(F)));
    VPMC_TRY(bin_points(ctx, w.g, w.q, reinterpret_cast<const float2*>(pts), M, 0, 0));
    VPMC_TRY(make_items(ctx, w.g, w.q.qstart, w.it, query_chunk(4)));
    EvalLaunch L;
    if (F) L.mode = exclude_center ? EVAL_FIELD_F_EXC : EVAL_FIELD_F;
    else L.mode = exclude_center ? EVAL_FIELD_EXC : EVAL_FIELD;
    L.out_f32 = out;
    VPMC_TRY(launch_eval(ctx, w.g, w.q.qrec, w.it, L));
    if (sign < 0 && use_signed) VPMC_LAUNCH(k_scale_f32, blocks_for(M), 256, 0, st, out, long(M), -1.0f);
    return vpmc_context_sync(ctx);
}

int vpmc_query_vorticity_f64(vpmc_context* ctx, int N, const float* pos, const float* omega, int M, const float* pts,
                             int sign, int use_signed, float h_w, float Lx, float Ly, int periodic, double* out) {
    if (!ctx || N < 0 || M < 0 || !(h_w > 0.f) || !(Lx > 0.f) || !(Ly > 0.f)) return VPMC_ERR_INVALID;
    if ((N > 0 && (!pos || !omega)) || (M > 0 && (!pts || !out))) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    if (M == 0) return VPMC_OK;
    cudaStream_t st = ctx->stream;
    VPMC_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * size_t(M), st));
    if (N == 0) return vpmc_context_sync(ctx);
    Work w;
    VPMC_TRY(setup(ctx, SLOT_QUERY, N, h_w, Lx, Ly, periodic, M, 0, &w));
    const int set_mode = sign > 0 ? SET_POS_ONLY
                                   : (sign < 0 ? SET_NEG_ONLY : (use_signed ? SET_ONE_SIGNED : SET_ONE_ABS));
    VPMC_TRY(grid_build(ctx, w.g, reinterpret_cast<const float2*>(pos), omega, set_mode));
    VPMC_TRY(bin_points(ctx, w.g, w.q, reinterpret_cast<const float2*>(pts), M, 0, 0));
    VPMC_TRY(make_items(ctx, w.g, w.q.qstart, w.it, query_chunk(4)));
    EvalLaunch L;
    L.mode = EVAL_FIELD64;
    L.out_f64 = out;
    VPMC_TRY(launch_eval(ctx, w.g, w.q.qrec, w.it, L));
    if (sign < 0 && use_signed)
        VPMC_LAUNCH(k_axpby, blocks_for(M), 256, 0, st, out, out, long(M), -1.0, 0.0, out);
    return vpmc_context_sync(ctx);
}

int vpmc_rbf_matvec(vpmc_context* ctx, int N, const float* pos, const float* x, float* y, float h_w, float Lx,
                    float Ly, int periodic, int precise) {
    if (!ctx || N < 0 || !(h_w > 0.f) || !(Lx > 0.f) || !(Ly > 0.f)) return VPMC_ERR_INVALID;
    if (N == 0) return VPMC_OK;
    if (!pos || !x || !y) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    Work w;
    VPMC_TRY(setup(ctx, SLOT_CG, N, h_w, Lx, Ly, periodic, 0, 2, &w));
    VPMC_TRY(grid_build(ctx, w.g, reinterpret_cast<const float2*>(pos), nullptr, SET_ONE_SIGNED));
    VPMC_LAUNCH(k_self_queries, blocks_for(N), 256, 0, st, w.g.cand, w.g.perm, w.g.cstart, long(N),
                uint32_t(w.g.nbins), 0, w.self);
    VPMC_TRY(make_items(ctx, w.g, w.g.cstart, w.it, query_chunk(4)));
    VPMC_LAUNCH(k_gather_to_sorted, blocks_for(N), 256, 0, st, x, w.g.perm, long(N), w.vec[0]);
    VPMC_TRY(spmv_sorted(ctx, w, w.vec[0], w.vec[1], precise != 0));
    VPMC_LAUNCH(k_scatter_from_sorted, blocks_for(N), 256, 0, st, w.vec[1], w.g.perm, long(N), y);
    return vpmc_context_sync(ctx);
}

}  // extern "C"

namespace {
int cg_impl(vpmc_context* ctx, int N, const float* pos, const float* b, const double* b64, float* omega_out, float h_w,
            float Lx, float Ly, int periodic, double tol, int max_iter, double* info) {
    if (!ctx || N < 0 || !(h_w > 0.f) || !(Lx > 0.f) || !(Ly > 0.f) || max_iter < 0) return VPMC_ERR_INVALID;
    if (N == 0) {
        if (info) { info[0] = 0; info[1] = 0; info[2] = 0; }
        return VPMC_OK;
    }
    if (!pos || (!b && !b64) || !omega_out) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    Work w;
    VPMC_TRY(setup(ctx, SLOT_CG, N, h_w, Lx, Ly, periodic, 0, 6, &w));
    double *bs = w.vec[0], *x = w.vec[1], *r = w.vec[2], *p = w.vec[3], *Ap = w.vec[4], *tmp = w.vec[5];
    VPMC_TRY(grid_build(ctx, w.g, reinterpret_cast<const float2*>(pos), nullptr, SET_ONE_SIGNED));
    VPMC_LAUNCH(k_self_queries, blocks_for(N), 256, 0, st, w.g.cand, w.g.perm, w.g.cstart, long(N),
                uint32_t(w.g.nbins), 0, w.self);
    VPMC_TRY(make_items(ctx, w.g, w.g.cstart, w.it, query_chunk(4)));
    if (b64) VPMC_LAUNCH(k_gather_to_sorted_d, blocks_for(N), 256, 0, st, b64, w.g.perm, long(N), bs);
    else VPMC_LAUNCH(k_gather_to_sorted, blocks_for(N), 256, 0, st, b, w.g.perm, long(N), bs);
    const double diag = spline_w_d(0.0, double(h_w));   // W(0), the reference's x0 = b / W(0)
    VPMC_LAUNCH(k_axpby, blocks_for(N), 256, 0, st, bs, bs, long(N), 1.0 / diag, 0.0, x);
    VPMC_TRY(spmv_sorted(ctx, w, x, Ap, true));
    VPMC_LAUNCH(k_cg_init, blocks_for(N), 256, 0, st, bs, Ap, long(N), r, p);
    double bb = 0.0, rr = 0.0;
    VPMC_TRY(host_dot(ctx, w, bs, nullptr, N, &bb));
    VPMC_TRY(host_dot(ctx, w, r, nullptr, N, &rr));
    const double bnorm = std::sqrt(bb);
    double res = bnorm > 0 ? std::sqrt(rr) / bnorm : 0.0;
    int it = 0;
    while (it < max_iter && res >= tol && bnorm > 0) {
        VPMC_TRY(spmv_sorted(ctx, w, p, Ap, true));
        double pAp = 0.0;
        VPMC_TRY(host_dot(ctx, w, p, Ap, N, &pAp));
        if (pAp == 0.0 || !std::isfinite(pAp)) break;
        const double alpha = rr / pAp;
        VPMC_LAUNCH(k_cg_xr, blocks_for(N), 256, 0, st, x, r, p, Ap, long(N), alpha);
        double rr_new = 0.0;
        VPMC_TRY(host_dot(ctx, w, r, nullptr, N, &rr_new));
        ++it;
        res = std::sqrt(rr_new) / bnorm;
        if (res < tol) break;
        VPMC_LAUNCH(k_cg_p, blocks_for(N), 256, 0, st, p, r, long(N), rr_new / rr);
        rr = rr_new;
    }
    // true residual with the FP64 SpMV
    VPMC_TRY(spmv_sorted(ctx, w, x, Ap, true));
    VPMC_LAUNCH(k_axpby, blocks_for(N), 256, 0, st, bs, Ap, long(N), 1.0, -1.0, tmp);
    double ee = 0.0;
    VPMC_TRY(host_dot(ctx, w, tmp, nullptr, N, &ee));
    VPMC_LAUNCH(k_scatter_from_sorted, blocks_for(N), 256, 0, st, x, w.g.perm, long(N), omega_out);
    VPMC_TRY(vpmc_context_sync(ctx));
    if (info) {
        info[0] = it;
        info[1] = res;
        info[2] = bnorm > 0 ? std::sqrt(ee) / bnorm : 0.0;
    }
    return res < tol || bnorm == 0 ? VPMC_OK : VPMC_ERR_NOT_CONVERGED;
}
// MINRES (Paige & Saunders, SIAM J. Numer. Anal. 12, 1975) on the same
// system as cg_impl: Lanczos vectors from the FP64 SpMV, Givens rotations on
// the host, residual norm |eta| decreasing monotonically.  Unlike CG it needs
// no definiteness, which the RBF matrix lacks (its spline symbol is negative
// at high wavenumbers, with eigenvalues close to zero on both sides).
int minres_impl(vpmc_context* ctx, int N, const float* pos, const float* b, const double* b64, float* omega_out,
                float h_w, float Lx, float Ly, int periodic, double tol, int max_iter, double* info) {
    if (!ctx || N < 0 || !(h_w > 0.f) || !(Lx > 0.f) || !(Ly > 0.f) || max_iter < 0) return VPMC_ERR_INVALID;
    if (N == 0) {
        if (info) { info[0] = 0; info[1] = 0; info[2] = 0; }
        return VPMC_OK;
    }
    if (!pos || (!b && !b64) || !omega_out) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    Work w;
    VPMC_TRY(setup(ctx, SLOT_CG, N, h_w, Lx, Ly, periodic, 0, 8, &w));
    double *bs = w.vec[0], *x = w.vec[1], *v = w.vec[2], *v_old = w.vec[3], *wv = w.vec[4], *w_old = w.vec[5],
           *u = w.vec[6], *tmp = w.vec[7];
    VPMC_TRY(grid_build(ctx, w.g, reinterpret_cast<const float2*>(pos), nullptr, SET_ONE_SIGNED));
    VPMC_LAUNCH(k_self_queries, blocks_for(N), 256, 0, st, w.g.cand, w.g.perm, w.g.cstart, long(N),
                uint32_t(w.g.nbins), 0, w.self);
    VPMC_TRY(make_items(ctx, w.g, w.g.cstart, w.it, query_chunk(4)));
    if (b64) VPMC_LAUNCH(k_gather_to_sorted_d, blocks_for(N), 256, 0, st, b64, w.g.perm, long(N), bs);
    else VPMC_LAUNCH(k_gather_to_sorted, blocks_for(N), 256, 0, st, b, w.g.perm, long(N), bs);
    const double diag = spline_w_d(0.0, double(h_w));   // the reference's starting point x0 = b / W(0)
    VPMC_LAUNCH(k_axpby, blocks_for(N), 256, 0, st, bs, bs, long(N), 1.0 / diag, 0.0, x);
    VPMC_TRY(spmv_sorted(ctx, w, x, u, true));
    VPMC_LAUNCH(k_axpby, blocks_for(N), 256, 0, st, bs, u, long(N), 1.0, -1.0, tmp);   // r0 = b - A x0
    double bb = 0.0, r0 = 0.0;
    VPMC_TRY(host_dot(ctx, w, bs, nullptr, N, &bb));
    VPMC_TRY(host_dot(ctx, w, tmp, nullptr, N, &r0));
    const double bnorm = std::sqrt(bb);
    double beta = std::sqrt(r0);
    double eta = beta;                                   // |eta| = residual norm of the current iterate
    int it = 0;
    if (bnorm > 0 && beta > 0) {
        VPMC_LAUNCH(k_axpby, blocks_for(N), 256, 0, st, tmp, tmp, long(N), 1.0 / beta, 0.0, v);
        VPMC_CUDA(cudaMemsetAsync(v_old, 0, sizeof(double) * size_t(N), st));
        VPMC_CUDA(cudaMemsetAsync(wv, 0, sizeof(double) * size_t(N), st));
        VPMC_CUDA(cudaMemsetAsync(w_old, 0, sizeof(double) * size_t(N), st));
        double g0 = 1.0, g1 = 1.0, s0 = 0.0, s1 = 0.0;   // the last two Givens rotations (cos, sin)
        while (it < max_iter && std::fabs(eta) >= tol * bnorm) {
            VPMC_TRY(spmv_sorted(ctx, w, v, u, true));
            double alpha = 0.0;
            VPMC_TRY(host_dot(ctx, w, v, u, N, &alpha));
            VPMC_LAUNCH(k_minres_u, blocks_for(N), 256, 0, st, u, v, v_old, long(N), alpha, beta, u);
            double bn2 = 0.0;
            VPMC_TRY(host_dot(ctx, w, u, nullptr, N, &bn2));
            const double beta_n = std::sqrt(bn2);
            // QR of the tridiagonal Lanczos matrix, one column per iteration
            const double delta = g1 * alpha - g0 * s1 * beta;
            const double rho1 = std::hypot(delta, beta_n);
            const double rho2 = s1 * alpha + g0 * g1 * beta;
            const double rho3 = s0 * beta;
            if (!(rho1 > 0.0) || !std::isfinite(rho1)) break;
            g0 = g1;
            s0 = s1;
            g1 = delta / rho1;
            s1 = beta_n / rho1;
            VPMC_LAUNCH(k_minres_step, blocks_for(N), 256, 0, st, v, w_old, wv, x, u, v_old, long(N), rho1, rho2,
                        rho3, g1 * eta, beta_n > 0.0 ? 1.0 / beta_n : 0.0);
            std::swap(w_old, wv);   // w <- w_new, w_old <- w
            std::swap(v_old, v);    // v <- u / beta_n, v_old <- v
            eta = -s1 * eta;
            beta = beta_n;
            ++it;
            if (beta_n == 0.0) break;   // the Krylov space is invariant: x is exact
        }
    }
    // true residual with the FP64 SpMV
    VPMC_TRY(spmv_sorted(ctx, w, x, u, true));
    VPMC_LAUNCH(k_axpby, blocks_for(N), 256, 0, st, bs, u, long(N), 1.0, -1.0, tmp);
    double ee = 0.0;
    VPMC_TRY(host_dot(ctx, w, tmp, nullptr, N, &ee));
    VPMC_LAUNCH(k_scatter_from_sorted, blocks_for(N), 256, 0, st, x, w.g.perm, long(N), omega_out);
    VPMC_TRY(vpmc_context_sync(ctx));
    const double res = bnorm > 0 ? std::fabs(eta) / bnorm : 0.0;
    if (info) {
        info[0] = it;
        info[1] = res;
        info[2] = bnorm > 0 ? std::sqrt(ee) / bnorm : 0.0;
    }
    return res < tol || bnorm == 0 ? VPMC_OK : VPMC_ERR_NOT_CONVERGED;
}
}  // namespace

extern "C" {

int vpmc_minres_rbf(vpmc_context* ctx, int N, const float* pos, const float* b, float* omega_out, float h_w,
                    float Lx, float Ly, int periodic, double tol, int max_iter, double* info) {
    if (!b && N > 0) return VPMC_ERR_INVALID;
    return minres_impl(ctx, N, pos, b, nullptr, omega_out, h_w, Lx, Ly, periodic, tol, max_iter, info);
}

int vpmc_minres_rbf_f64rhs(vpmc_context* ctx, int N, const float* pos, const double* b, float* omega_out, float h_w,
                           float Lx, float Ly, int periodic, double tol, int max_iter, double* info) {
    if (!b && N > 0) return VPMC_ERR_INVALID;
    return minres_impl(ctx, N, pos, nullptr, b, omega_out, h_w, Lx, Ly, periodic, tol, max_iter, info);
}

int vpmc_cg_rbf(vpmc_context* ctx, int N, const float* pos, const float* b, float* omega_out, float h_w, float Lx,
                float Ly, int periodic, double tol, int max_iter, double* info) {
    if (!b && N > 0) return VPMC_ERR_INVALID;
    return cg_impl(ctx, N, pos, b, nullptr, omega_out, h_w, Lx, Ly, periodic, tol, max_iter, info);
}

int vpmc_cg_rbf_f64rhs(vpmc_context* ctx, int N, const float* pos, const double* b, float* omega_out, float h_w,
                       float Lx, float Ly, int periodic, double tol, int max_iter, double* info) {
    if (!b && N > 0) return VPMC_ERR_INVALID;
    return cg_impl(ctx, N, pos, nullptr, b, omega_out, h_w, Lx, Ly, periodic, tol, max_iter, info);
}



}  // extern "C"
