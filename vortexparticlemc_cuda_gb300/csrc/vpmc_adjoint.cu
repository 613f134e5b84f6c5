// vpmc_adjoint.cu -- the adjoint of the plain MIS step (no counterpart in
// the reference): checkpointed forward record, segment recompute, and per
// step the value/gradient field sums at the samples, the per-sample
// derivatives of the MIS term and the transposed field sum at the particles,
// each term in the forward's precision and every sum in FP64.
#include <algorithm>
#include <type_traits>
#include <vector>

#include "vpmc_sim.cuh"

namespace vpmc {
namespace {

using namespace sim;

// ------------------------------------------------------------------ adjoint
// The adjoint of one plain MIS step X' = X + dt U(X, omega) with the step's
// Philox samples held fixed (common random numbers; the discrete CDF index
// and image-tile choices are constants of the pathwise derivative).  With
// lambda' = dL/dX' and v_t = dt lambda'_t (+-1/Q per sign), each MIS term
// T(x_t, y, f(y), Omega) contributes c = v_t . T and
//   dL/dx_t   += dc/dx                       (and dc/dy for disk samples, y = x_t + offset)
//   dL/dx_I   += dc/dy                       (branch-1 samples, y = x_I + shift + F r)
//   dc/dy      = -dc/dx|_f + dc/df grad f(y)
//   dL/domega_J, dL/dx_J through f(y) = sum_J |omega_J| W(|y - x_J|):
//              sgn(omega_J) G(x_J) and |omega_J| grad G(x_J), G(q) = sum_s dc_s/df W(|q - y_s|)
//              (the transposed field sum, evaluated with queries and candidates swapped)
//   dL/domega_J through Omega: sgn(omega_J) (9 if periodic) sum_s dc_s/dOmega.

// d(v . T)/d{x, f, Omega} of one MIS term (mis_term64's arithmetic), in R
// arithmetic: FP64 on the FP64 path, FP32 on the FP32 path (each term is then
// as precise as the forward's FP32 term; the caller accumulates in FP64).
// The factor 1 - (w1 f / cum) / D of df/f is written as the disk term's share
// w2 p2 / D, which equals it and has no cancellation when branch 1 dominates.
template <typename R_>
__device__ __forceinline__ void mis_term_adj(int law, float2 xf, float2 yf, R_ f, R_ w1, R_ w2, R_ cum, R_ alpha,
                                             R_ R, const InstMC& I, R_ vx, R_ vy, R_& gxx, R_& gxy, R_& df, R_& dc,
                                             R_& cval) {
    gxx = gxy = df = dc = cval = R_(0);
    if (!(f > R_(0))) return;
    const R_ rx = R_(xf.x) - R_(yf.x), ry = R_(xf.y) - R_(yf.y);
    const R_ P = vy * rx - vx * ry;   // v . perp(r)
    const R_ two_pi = R_(2.0 * kPiD);
    if (law == VPMC_LAW_REFERENCE) {
        R_ wx = rx, wy = ry;
        if (I.periodic) {
            wx = rx - round(rx / R_(I.Lx)) * R_(I.Lx);
            wy = ry - round(ry / R_(I.Ly)) * R_(I.Ly);
        }
        const R_ wn = sqrt(wx * wx + wy * wy);
        const R_ rn = fmax(wn, R_(1e-6));
        const R_ inv = R_(1) / (rx * rx + ry * ry + R_(1e-8));
        const R_ K = inv / two_pi;
        const R_ b2 = w2 * alpha / rn;   // the disk term of the denominator
        const R_ denom = w1 * f / cum + b2;
        const R_ sc = f / denom;
        const R_ drx = wn > R_(1e-6) ? wx / wn : R_(0), dry = wn > R_(1e-6) ? wy / wn : R_(0);   // d rn / d r
        const R_ g = sc / denom * (b2 / rn);                                                       // d sc / d rn
        cval = sc * K * P;
        gxx = sc * K * vy - R_(2) * rx * inv * K * sc * P + K * P * g * drx;
        gxy = -sc * K * vx - R_(2) * ry * inv * K * sc * P + K * P * g * dry;
        df = K * P * (b2 / denom) / denom;
        dc = K * P * sc * (w1 * f / (cum * cum * denom));
        return;
    }
    const R_ r2 = rx * rx + ry * ry;
    if (!(r2 > R_(0))) return;
    const R_ rn = sqrt(r2);
    const bool in = rn < R;
    const R_ p2 = in ? alpha / rn : R_(0);
    const R_ D = w1 * f / cum + w2 * p2;
    const R_ sc = f / (D * two_pi * r2);
    const R_ ex = (in ? -w2 * alpha / (rn * r2) : R_(0)) / D + R_(2) / r2;   // -(d sc / d r) / (sc r)
    cval = sc * P;
    gxx = sc * vy - P * sc * ex * rx;
    gxy = -sc * vx - P * sc * ex * ry;
    df = P * (w2 * p2 / D) / (two_pi * r2 * D);
    dc = P * sc * (w1 * f / (cum * cum * D));
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct AdjArgs {
    const InstMC* mc;
    int n_inst;
    const float2* pos;
    const float2* ys;
    const double* fg;       // 3 per sample: f, df/dx, df/dy
    const int* src;
    const double* cum64;    // 2 per instance (x9 when periodic)
    long t0, nt;
    int N1, N2;
    const double* lam_next;
    double* lam;
    double* as;             // per sample: dc/df
    double* dcum;           // 2 per instance
    double* gsc;            // score-function term: per particle, sum of c over the samples that drew it
    double* csum;           // 2 per instance: sum of c over branch-1 samples
};

// One warp per target: the MIS-term derivatives of all its samples, each in
// FP32 (F32: the FP32 path) or FP64, every sum and atomic in FP64.
template <bool F32>
__global__ void __launch_bounds__(256) k_adj_terms(AdjArgs a) {
    using R_ = typename std::conditional<F32, float, double>::type;
    const int lane = threadIdx.x & 31;
    const long warp = (long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const long nwarps = (long(gridDim.x) * blockDim.x) >> 5;
    const int Q = a.N1 + a.N2;
    const double w1 = double(a.N1) / Q, w2 = double(a.N2) / Q, inv = 1.0 / Q;
    for (long tl = warp; tl < a.nt; tl += nwarps) {
        const long t = a.t0 + tl;
        const int ii = inst_of(a.mc, a.n_inst, t);
        const InstMC& I = a.mc[ii];
        const float2 x = a.pos[t];
        const double R = sqrt(double(I.Lx) * I.Lx + double(I.Ly) * I.Ly);   // as the FP64 path
        const double alpha = 1.0 / (2.0 * kPiD * R);
        const double mux = double(I.dt) * a.lam_next[2 * t], muy = double(I.dt) * a.lam_next[2 * t + 1];
        double ltx = 0.0, lty = 0.0;
        for (int s = 0; s < 2; ++s) {
            const double sg = (s == 0 ? inv : -inv);
            const double vx = mux * sg, vy = muy * sg;
            const double cum = a.cum64[2 * ii + s];
            const long base = (tl * 2 + s) * Q;
            double dca = 0.0, csa = 0.0;
            for (int j = lane; j < Q; j += 32) {
                const long sid = base + j;
                R_ gxr, gyr, dfr, dcr, cvr;
                mis_term_adj<R_>(I.law, x, a.ys[sid], R_(a.fg[3 * sid]), R_(w1), R_(w2), R_(cum), R_(alpha), R_(R), I,
                                 R_(vx), R_(vy), gxr, gyr, dfr, dcr, cvr);
                const double gxx = gxr, gxy = gyr, df = dfr, dc = dcr, cv = cvr;
                ltx += gxx;
                lty += gxy;
                const double dyx = -gxx + double(dfr * R_(a.fg[3 * sid + 1]));
                const double dyy = -gxy + double(dfr * R_(a.fg[3 * sid + 2]));
                if (j >= a.N1) {
                    ltx += dyx;
                    lty += dyy;
                } else {
                    const int p = a.src[sid];
                    if (p >= 0 && (dyx != 0.0 || dyy != 0.0)) {
                        atomicAdd(&a.lam[2 * p], dyx);
                        atomicAdd(&a.lam[2 * p + 1], dyy);
                    }
                    if (a.gsc && p >= 0 && cv != 0.0) {
                        atomicAdd(&a.gsc[p], cv);
                        csa += cv;
                    }
                }
                a.as[sid] = df;
                dca += dc;
            }
            dca = warp_sum_d(dca);
            if (lane == 0 && dca != 0.0) atomicAdd(&a.dcum[2 * ii + s], dca);
            if (a.gsc) {
                csa = warp_sum_d(csa);
                if (lane == 0 && csa != 0.0) atomicAdd(&a.csum[2 * ii + s], csa);
            }
        }
        ltx = warp_sum_d(ltx);
        lty = warp_sum_d(lty);
        if (lane == 0) {
            atomicAdd(&a.lam[2 * t], ltx);
            atomicAdd(&a.lam[2 * t + 1], lty);
        }
    }
}

// The transposed sums (by grid slot) onto the particles: dL/domega through the
// strength, lambda through the position (the weight |omega| of each particle's
// kernel).  Each particle holds at most one slot (sign-split sets).
__global__ void k_adj_sources(const float* __restrict__ omega, const uint32_t* __restrict__ perm,
                              const uint32_t* __restrict__ cstart, uint32_t nbins, long n,
                              const double* __restrict__ dual, double* __restrict__ lam, double* __restrict__ gom) {
    const long nv = min(long(cstart[nbins]), n);
    for (long p = long(blockIdx.x) * blockDim.x + threadIdx.x; p < nv; p += long(gridDim.x) * blockDim.x) {
        const uint32_t i = perm[p];
        const float w = omega[i];
        if (w == 0.f) continue;
        const double aw = fabs(double(w));
        gom[i] += (w > 0.f ? 1.0 : -1.0) * dual[3 * p];
        lam[2 * i] += aw * dual[3 * p + 1];
        lam[2 * i + 1] += aw * dual[3 * p + 2];
    }
}

// Omega terms, and (score) the score-function term of the discrete branch-1
// draw P(I = J) = |omega_J| / Omega_s: d log P(I)/d omega_J =
// sgn(omega_J) (delta_IJ / |omega_J| - 1 / Omega_s), weighted by each sample's c.
__global__ void k_adj_cum(const InstMC* __restrict__ mc, int n_inst, const float* __restrict__ omega, long n,
                          const double* __restrict__ dcum, const double* __restrict__ cum64,
                          const double* __restrict__ gsc, const double* __restrict__ csum,
                          double* __restrict__ gom) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const float w = omega[i];
        if (w == 0.f) continue;
        const int ii = inst_of(mc, n_inst, i);
        const int s = w > 0.f ? 0 : 1;
        const double sg = w > 0.f ? 1.0 : -1.0;
        const double f9 = mc[ii].periodic ? 9.0 : 1.0;
        double g = f9 * dcum[2 * ii + s];
        if (gsc) g += gsc[i] / fabs(double(w)) - csum[2 * ii + s] / (cum64[2 * ii + s] / f9);
        gom[i] += sg * g;
    }
}

// Adjoint working set (allocated on first use): per chunk of samples the
// source index, FP64 value + gradient and dc/df; per particle the transposed
// sums (by grid slot), two lambda buffers and dL/domega.
struct AdjBufs {
    int* src;
    double* fg;
    double* as;
    double* dual_out;
    double* lam[2];
    double* gom;
    double* dcum;
    double* gsc;
    double* csum;
};

int adj_bufs(vpmc_sim* s, AdjBufs* A) {
    const long ns = s->chunk_targets * 2 * samples_per(s);
    auto carve = [&](Carver& c) {
        A->src = c.take<int>(size_t(ns));
        A->fg = c.take<double>(3 * size_t(ns));
        A->as = c.take<double>(size_t(ns));
        A->dual_out = c.take<double>(3 * size_t(s->N));
        A->lam[0] = c.take<double>(2 * size_t(s->N));
        A->lam[1] = c.take<double>(2 * size_t(s->N));
        A->gom = c.take<double>(size_t(s->N));
        A->dcum = c.take<double>(2 * size_t(s->n_inst));
        A->gsc = c.take<double>(size_t(s->N));
        A->csum = c.take<double>(2 * size_t(s->n_inst));
    };
    Carver dry;
    carve(dry);
    VPMC_TRY(s->adj.reserve(dry.off));
    Carver c{static_cast<char*>(s->adj.p), 0};
    carve(c);
    return VPMC_OK;
}

// lam_out = lam_in + (dX'/dX)^T lam_in; gom += (dX'/domega)^T lam_in, at the
// state in s->pos with the step counter already on the device.
int adjoint_step(vpmc_sim* s, AdjBufs& A, const double* lam_in, double* lam_out, bool score) {
    vpmc_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    VPMC_TRY(grid_build(ctx, s->g, s->pos, s->omega, SET_SIGN_SPLIT));
    VPMC_CUDA(cudaMemcpyAsync(lam_out, lam_in, 2 * sizeof(double) * size_t(s->N), cudaMemcpyDeviceToDevice, st));
    VPMC_CUDA(cudaMemsetAsync(A.dcum, 0, 2 * sizeof(double) * size_t(s->n_inst), st));
    if (score) {
        VPMC_CUDA(cudaMemsetAsync(A.gsc, 0, sizeof(double) * size_t(s->N), st));
        VPMC_CUDA(cudaMemsetAsync(A.csum, 0, 2 * sizeof(double) * size_t(s->n_inst), st));
    }
    const bool unb = s->mc[0].law == VPMC_LAW_UNBIASED;
    const long Q = samples_per(s);
    for (long t0 = 0; t0 < s->N; t0 += s->chunk_targets) {
        const long nt = std::min(s->chunk_targets, s->N - t0);
        const long ns = nt * 2 * Q;
        VPMC_CUDA(cudaMemsetAsync(s->q.qcount, 0, sizeof(uint32_t) * size_t(s->g.nbins + 1), st));
        GenArgs ga{s->d_mc, s->n_inst, s->g.inst, s->pos, nullptr, nullptr, s->sub, s->cdf, s->guide, s->jit, s->d_step, t0,
                   nt, s->N1, s->N2, 1, A.src, s->ys, s->q.qbin, s->q.qcount, s->q.tmp ? nullptr : s->q.qrank};
        VPMC_LAUNCH(k_gen, blocks_for(ns), 256, 0, st, ga);
        VPMC_TRY(scatter_ranked(ctx, s->g, s->q, s->ys, ns));
        // f and grad f at every sample (FP64)
        VPMC_TRY(make_items(ctx, s->g, s->q.qstart, s->it, query_chunk(4)));
        VPMC_CUDA(cudaMemsetAsync(A.fg, 0, 3 * sizeof(double) * size_t(ns), st));
        EvalLaunch L;
        // field values and gradients at the samples: the FP32 path's adjoint sums
        // its pairs in FP32 (into FP64 run sums; the candidates are the particles
        // in grid order, so the sums are fixed-order), the FP64 path's in FP64
        const bool f32 = s->precision == 32;
        L.mode = unb ? (f32 ? EVAL_GRAD9_32 : EVAL_GRAD9_64) : (f32 ? EVAL_GRAD32 : EVAL_GRAD64);
        L.qpt = 4;
        L.out_f64 = A.fg;
        VPMC_TRY(launch_eval(ctx, s->g, s->q.qrec, s->it, L));
        AdjArgs aa{s->d_mc, s->n_inst, s->pos, s->ys, A.fg, A.src, s->cum64, t0, nt, s->N1, s->N2, lam_in, lam_out,
                   A.as, A.dcum, score ? A.gsc : nullptr, A.csum};
        if (f32) VPMC_LAUNCH(k_adj_terms<true>, blocks_for(nt * 32), 256, 0, st, aa);
        else VPMC_LAUNCH(k_adj_terms<false>, blocks_for(nt * 32), 256, 0, st, aa);
        // transposed sums from the sample side: the same items, each sample
        // weighted by its dc/df, every in-support (sample, particle) pair adding
        // a_s W and a_s dW/dx_p to the particle's slot
        VPMC_TRY(make_items(ctx, s->g, s->q.qstart, s->it, query_chunk(4)));
        VPMC_CUDA(cudaMemsetAsync(A.dual_out, 0, 3 * sizeof(double) * size_t(s->N), st));
        EvalLaunch D;
        D.mode = unb ? (f32 ? EVAL_SCAT9_32 : EVAL_SCAT9_64) : (f32 ? EVAL_SCAT32 : EVAL_SCAT64);
        D.qpt = 4;
        D.out_f64 = A.dual_out;
        D.qweight = A.as;
        VPMC_TRY(launch_eval(ctx, s->g, s->q.qrec, s->it, D));
        VPMC_LAUNCH(k_adj_sources, blocks_for(s->N), 256, 0, st, s->omega, s->g.perm, s->g.cstart,
                    uint32_t(s->g.nbins), s->N, A.dual_out, lam_out, A.gom);
    }
    VPMC_LAUNCH(k_adj_cum, blocks_for(s->N), 256, 0, st, s->d_mc, s->n_inst, s->omega, s->N, A.dcum, s->cum64,
                score ? A.gsc : nullptr, A.csum, A.gom);
    return VPMC_OK;
}

}  // namespace
}  // namespace vpmc

using namespace vpmc;
using namespace vpmc::sim;

extern "C" {

int vpmc_sim_record(vpmc_sim* s, int nsteps, int k_ckpt) {
    if (!s || nsteps < 1 || k_ckpt < 1) return VPMC_ERR_INVALID;
    if (s->deform) return VPMC_ERR_UNSUPPORTED;   // the adjoint covers the plain method
    if (s->t_begin != 0 || s->t_end != s->N) return VPMC_ERR_UNSUPPORTED;   // and whole simulations, not shards
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    if (!s->prepared) VPMC_TRY(vpmc_sim_prepare(s));
    cudaStream_t st = s->ctx->stream;
    const long nck = (nsteps + k_ckpt - 1) / k_ckpt + 1;   // X_0, X_k, ..., and X_T
    VPMC_TRY(s->ckpt.reserve(sizeof(float2) * size_t(s->N) * size_t(nck)));
    float2* ck = static_cast<float2*>(s->ckpt.p);
    s->rec_steps = nsteps;
    s->rec_k = k_ckpt;
    s->rec_step0 = s->step;
    for (int n = 0; n < nsteps; ++n) {
        if (n % k_ckpt == 0)
            VPMC_CUDA(cudaMemcpyAsync(ck + size_t(n / k_ckpt) * s->N, s->pos, sizeof(float2) * size_t(s->N),
                                      cudaMemcpyDeviceToDevice, st));
        VPMC_TRY(run_pass(s, true, 1));
    }
    VPMC_CUDA(cudaMemcpyAsync(ck + size_t(nck - 1) * s->N, s->pos, sizeof(float2) * size_t(s->N),
                              cudaMemcpyDeviceToDevice, st));
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_adjoint(vpmc_sim* s, const double* dL_dXT, double* dL_dX0, double* dL_domega, int flags) {
    if (!s || !dL_dXT || !dL_dX0 || !dL_domega) return VPMC_ERR_INVALID;
    if (s->rec_steps < 1) return VPMC_ERR_INVALID;   // vpmc_sim_record first
    if (s->deform || s->t_begin != 0 || s->t_end != s->N) return VPMC_ERR_UNSUPPORTED;
    vpmc_context* ctx = s->ctx;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    s->ys_t0 = -1;   // the adjoint redraws samples into the sample buffer
    s->ys_nt = 0;
    AdjBufs A;
    VPMC_TRY(adj_bufs(s, &A));
    const int T = s->rec_steps, k = s->rec_k;
    const long nck = (T + k - 1) / k + 1;
    float2* ck = static_cast<float2*>(s->ckpt.p);
    VPMC_TRY(s->seg.reserve(sizeof(float2) * size_t(s->N) * size_t(k)));
    float2* seg = static_cast<float2*>(s->seg.p);
    VPMC_CUDA(cudaMemcpyAsync(A.lam[0], dL_dXT, 2 * sizeof(double) * size_t(s->N), cudaMemcpyDeviceToDevice, st));
    VPMC_CUDA(cudaMemsetAsync(A.gom, 0, sizeof(double) * size_t(s->N), st));
    int cur = 0;
    for (long sg = nck - 2; sg >= 0; --sg) {
        const int n0 = int(sg) * k, n1 = std::min(T, n0 + k);
        // recompute the segment's states from its checkpoint (bitwise the forward's)
        VPMC_CUDA(cudaMemcpyAsync(s->pos, ck + size_t(sg) * s->N, sizeof(float2) * size_t(s->N),
                                  cudaMemcpyDeviceToDevice, st));
        VPMC_TRY(set_step_counter(s, s->rec_step0 + uint64_t(n0)));
        for (int n = n0; n < n1; ++n) {
            VPMC_CUDA(cudaMemcpyAsync(seg + size_t(n - n0) * s->N, s->pos, sizeof(float2) * size_t(s->N),
                                      cudaMemcpyDeviceToDevice, st));
            if (n + 1 < n1) VPMC_TRY(run_pass(s, true, 1));
        }
        for (int n = n1 - 1; n >= n0; --n) {
            VPMC_CUDA(cudaMemcpyAsync(s->pos, seg + size_t(n - n0) * s->N, sizeof(float2) * size_t(s->N),
                                      cudaMemcpyDeviceToDevice, st));
            VPMC_TRY(set_step_counter(s, s->rec_step0 + uint64_t(n)));
            VPMC_TRY(adjoint_step(s, A, A.lam[cur], A.lam[cur ^ 1], (flags & VPMC_ADJ_SCORE) != 0));
            cur ^= 1;
        }
    }
    VPMC_CUDA(cudaMemcpyAsync(dL_dX0, A.lam[cur], 2 * sizeof(double) * size_t(s->N), cudaMemcpyDeviceToDevice, st));
    VPMC_CUDA(cudaMemcpyAsync(dL_domega, A.gom, sizeof(double) * size_t(s->N), cudaMemcpyDeviceToDevice, st));
    // back to the recorded final state
    VPMC_CUDA(cudaMemcpyAsync(s->pos, ck + size_t(nck - 1) * s->N, sizeof(float2) * size_t(s->N),
                              cudaMemcpyDeviceToDevice, st));
    VPMC_TRY(set_step_counter(s, s->rec_step0 + uint64_t(T)));
    return vpmc_context_sync(ctx);
}

}  // extern "C"
