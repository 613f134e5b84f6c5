// vpmc_sim.cu -- the simulation handle: MIS Monte-Carlo Biot-Savart velocity
// with advection (Simulation::step_cuda, src/cuda/simulation_step.cu:9-90;
// monte_carlo_bs_kernel_safe, src/cuda/monte_carlo_bs.cu:144-271), batched
// over instances (ensembles), captured as one CUDA graph per step.
//
// Per step:
//   1. grid: particles -> bins (instance, sign, cell), stable sort, candidate
//      runs {x, y, |omega| 2 sigma} (vpmc_grid.cu);
//   2. per chunk of targets:
//      gen     one thread per (target, sign, sample): Philox4x32-10 keyed by
//              (seed, instance) with counter (sample|sign, target, step) ->
//              branch 1: |omega| CDF (FP64, guide table + binary search),
//              image tile, kernel jitter; branch 2: disk draw.  Writes the
//              sample point and its bin;
//      bin     counts -> scan -> scatter into per-bin query records;
//      eval    field value at every sample (vpmc_grid.cu k_eval);
//      accum   one warp per target: MIS terms, Kahan-compensated FP32 sums in
//              a fixed order, u = u(+) - u(-), x += dt u with an FP64 wrap.
//   Results do not depend on scheduling: each sample's field value is a fixed
//   ordered sum and every reduction has a fixed tree.
//
// Deformation mode (the reference's step_cuda, which always runs with
// aux = 1): every particle carries F (row-major float4); kernels are
// W(|F^-1 d|), branch-1 jitter is F r, each target has four auxiliary points
// x -/+ dx e_x, x +/- dx e_y (dx = h_w / 2) with their own disk samples and a
// share of the branch-1 samples, and after the step F = renorm_det1(I + dt
// grad u) from central differences of the auxiliary velocities
// (update_jacobian_from5, src/cuda/monte_carlo_bs.cu:274-288).
//
// The adjoint of the step is in vpmc_adjoint.cu; state shared with it is in
// vpmc_sim.cuh.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include "vpmc_sim.cuh"

namespace vpmc {

using namespace sim;

int build_subsets_dev(vpmc_context* ctx, long N, const float* omega, int* sub_pos, int* sub_neg, double* cdf_pos,
                      double* cdf_neg, float* c32p, float* c32n, int* cnt, double* cum);

namespace {

// update_jacobian_from5 + renorm_det1 (src/cuda/monte_carlo_bs.cu:274-288,
// include/monte_carlo_bs.cuh:140-144) for callers that hold the five velocity
// arrays themselves; the same FP32 steps as the deformation step.
__global__ void k_jacobian5(long n, float dt, float dx, const float2* __restrict__ vC, const float2* __restrict__ vL,
                            const float2* __restrict__ vR, const float2* __restrict__ vT,
                            const float2* __restrict__ vB, float4* __restrict__ F) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        (void)vC;
        const float c = 0.5f * dt / dx;
        float4 f;
        f.x = 1.f + (vR[i].x - vL[i].x) * c;
        f.y = (vT[i].x - vB[i].x) * c;
        f.z = (vR[i].y - vL[i].y) * c;
        f.w = 1.f + (vT[i].y - vB[i].y) * c;
        const float det = f.x * f.w - f.y * f.z;
        const float sc = rsqrtf(fmaxf(det, 1e-12f));
        F[i] = make_float4(f.x * sc, f.y * sc, f.z * sc, f.w * sc);
    }
}

// Cell-centred lattice, ix-major: x = (ix + 1/2) / Nx * Lx in FP64, rounded once.
__global__ void k_lattice(float2* __restrict__ pos, int Nx, int Ny, float Lx, float Ly) {
    const long n = long(Nx) * Ny;
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const long ix = i / Ny, iy = i - ix * Ny;
        pos[i] = make_float2(float((double(ix) + 0.5) / double(Nx) * double(Lx)),
                             float((double(iy) + 0.5) / double(Ny) * double(Ly)));
    }
}

__global__ void k_identity(float4* __restrict__ F, long n) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
        F[i] = make_float4(1.f, 0.f, 0.f, 1.f);
}

// upper_bound(cdf[0..n), u) bracketed by a guide table of G = n entries:
// guide(j) = upper_bound(j / G), guide(G) = n; result clamped to n-1 as the
// reference does.  Slot k of the table holds the bracket
// (guide(max(k - 1, 0)), guide(min(k + 2, G))): one 8-byte load.
// u = u01d(r) = (2 r + 1) 2^-33 exactly.  The search runs on integers: for
// non-negative doubles the IEEE bit patterns order as the values do, so
// cdf[i] > u compares the 64-bit patterns (no FP64 instruction, the same index).
// The guide slot is floor((2 r + 1) n / 2^33) in exact integer arithmetic; the
// one-slot margin on both sides of the bracket covers the rounding of the
// guide's own k / G.
__device__ __forceinline__ unsigned long long u01d_bits(uint32_t r) {
    const unsigned long long m = 2ull * r + 1ull;                 // 1 .. 2^33 - 1
    const int p = 63 - __clzll(static_cast<long long>(m));        // leading bit
    return (static_cast<unsigned long long>(1023 + p - 33) << 52) | ((m << (52 - p)) & ((1ull << 52) - 1ull));
}
__device__ __forceinline__ int sample_cdf(const double* __restrict__ cdf, const uint2* __restrict__ bracket, int n,
                                          uint32_t r) {
    const int G = n;
    const unsigned long long ub = u01d_bits(r);
    int k = int(((2ull * r + 1ull) * static_cast<unsigned long long>(G)) >> 33);
    k = min(max(k, 0), G - 1);
    const uint2 b = bracket[k];
    int lo = int(b.x), hi = int(b.y);
    const unsigned long long* cb = reinterpret_cast<const unsigned long long*>(cdf);
    // first index in [lo, hi) with cdf > u
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cb[mid] > ub) hi = mid; else lo = mid + 1;
    }
    return min(lo, n - 1);
}

__device__ __forceinline__ int guide_at(const double* __restrict__ cdf, int n, long j) {
    if (j >= n) return n;
    const double v = double(j) / double(n);
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cdf[mid] > v) hi = mid; else lo = mid + 1;
    }
    return lo;
}

__global__ void k_guide(const double* __restrict__ cdf, int n, uint2* __restrict__ bracket) {
    for (long k = long(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += long(gridDim.x) * blockDim.x)
        bracket[k] = make_uint2(uint32_t(guide_at(cdf, n, k > 0 ? k - 1 : 0)), uint32_t(guide_at(cdf, n, k + 2)));
}

// Positions in subset order (plain method): pos_sub[e] = pos of subset entry e,
// so a branch-1 draw reads its source in one load.  Entries past a subset's
// count are left alone.
__global__ void k_sub_pos(const InstMC* __restrict__ mc, int n_inst, const int* __restrict__ sub,
                          const float2* __restrict__ pos, long n2, float2* __restrict__ pos_sub) {
    for (long e = long(blockIdx.x) * blockDim.x + threadIdx.x; e < n2; e += long(gridDim.x) * blockDim.x) {
        const InstMC& I = mc[inst_of(mc, n_inst, e >> 1)];
        const bool in0 = e >= I.off[0] && e - I.off[0] < I.cnt[0];
        const bool in1 = e >= I.off[1] && e - I.off[1] < I.cnt[1];
        if (in0 || in1) pos_sub[e] = pos[sub[e] + I.p_begin];
    }
}

}  // namespace

namespace sim {

// Auxiliary point a of target x: C, L, R, T, B as monte_carlo_bs_kernel_safe
// forms them (src/cuda/monte_carlo_bs.cu:163-167).
__device__ __forceinline__ float2 aux_point(float2 x, int a, float dx) {
    switch (a) {
        case 1: return make_float2(x.x - dx, x.y);
        case 2: return make_float2(x.x + dx, x.y);
        case 3: return make_float2(x.x, x.y + dx);
        case 4: return make_float2(x.x, x.y - dx);
        default: return x;
    }
}

__global__ void __launch_bounds__(256) k_gen(GenArgs a) {
    const int Q = a.N1 + a.naux * a.N2;
    const uint32_t Q2 = uint32_t(2 * Q);
    const uint32_t total = uint32_t(a.nt) * Q2;   // samples of one chunk (< 2^31)
    const unsigned long long step = *a.step;
    // sample sid = (target tl, sign s, sample j): decomposed once, then advanced
    // by the grid stride without dividing again
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t dtl = stride / Q2, drem = stride - dtl * Q2;
    uint32_t sid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t tl = sid / Q2, rem = sid - tl * Q2;
    for (; sid < total; sid += stride) {
        const int s = rem >= uint32_t(Q) ? 1 : 0, j = int(rem) - s * Q;
        const long t = a.t0 + long(tl);
        tl += dtl;
        rem += drem;
        if (rem >= Q2) { rem -= Q2; ++tl; }
        const int ii = inst_of(a.mc, a.n_inst, t);
        const InstMC& I = a.mc[ii];
        const GridInst& G = a.gi[ii];
        const float2 x = a.pos[t];
        // counter = (sample | sign, instance-local target, step): an ensemble
        // member draws exactly what a standalone run with its seed draws
        const U4 r = philox4x32_10(U4{uint32_t(j) | (uint32_t(s) << 31), uint32_t(t - I.p_begin), uint32_t(step),
                                      uint32_t(step >> 32)},
                                   I.key0, I.key1);
        float2 y = x;
        bool valid = true;
        int src = -1;
        if (j < a.N1) {
            const int n = I.cnt[s];
            if (n == 0) {
                valid = false;
            } else {
                const int idx = sample_cdf(a.cdf + I.off[s], a.guide + I.goff[s], n, r.x);
                int p = -1;
                if (a.pos_sub) {
                    y = a.pos_sub[I.off[s] + idx];
                } else {
                    p = a.sub[I.off[s] + idx] + I.p_begin;   // subsets hold instance-local indices
                    src = p;
                    y = a.pos[p];
                }
                if (I.periodic) {
                    const int m9 = min(int(u01(r.y) * 9.f), 8);
                    y.x += float(m9 / 3 - 1) * I.Lx;
                    y.y += float(m9 % 3 - 1) * I.Ly;
                }
                float rr;
                const float ur = u01(r.z);
                if (I.law == VPMC_LAW_REFERENCE) {
                    // sample_kernel_radius (include/monte_carlo_bs.cuh:78-88): the
                    // table already holds h_w and is scaled by h_w once more
                    const float f = ur * (kIcdfRef - 1);
                    const int i0 = int(f), i1 = min(i0 + 1, kIcdfRef - 1);
                    const float tt = f - i0;
                    rr = (I.icdf[i0] * (1.f - tt) + I.icdf[i1] * tt) * I.hw;
                } else {
                    const float f = ur * kJitTab;
                    const int i0 = min(int(f), kJitTab - 1);
                    const float tt = f - i0;
                    const float2 jt = a.jit[i0];   // (table[i0], table[i0 + 1])
                    rr = (jt.x * (1.f - tt) + jt.y * tt) * I.hw;
                }
                float sn, cs;
                sincospif(2.f * u01(r.w), &sn, &cs);   // angle 2 pi u
                const float jx = rr * cs, jy = rr * sn;
                if (a.F) {
                    // mul_mat2(F, r) (include/monte_carlo_bs.cuh:99-103)
                    const float4 f = a.F[p];
                    y.x += f.x * jx + f.y * jy;
                    y.y += f.z * jx + f.w * jy;
                } else {
                    y.x += jx;
                    y.y += jy;
                }
            }
        } else {
            const int ax = a.naux > 1 ? (j - a.N1) / a.N2 : 0;
            const float2 xa = aux_point(x, ax, I.dx);
            const float R = disk_radius(xa, I.periodic != 0, I.Lx, I.Ly);
            const float ur = u01(r.y);
            const float rr = I.law == VPMC_LAW_REFERENCE ? R * sqrtf(ur) : R * ur;
            float sn, cs;
            sincospif(2.f * u01(r.x), &sn, &cs);   // angle 2 pi u
            y.x = xa.x + rr * cs;
            y.y = xa.y + rr * sn;
        }
        uint32_t b = kNoBin;
        if (valid) {
            float px = y.x, py = y.y;
            bool ok = true;
            if (I.periodic) {
                const float kx = floorf(px / I.Lx), ky = floorf(py / I.Ly);
                if (I.law == VPMC_LAW_UNBIASED && (fabsf(kx) > 2.f || fabsf(ky) > 2.f)) ok = false;
                px -= kx * I.Lx;
                py -= ky * I.Ly;
            } else {
                ok = !(px < 0.f || px > I.Lx || py < 0.f || py > I.Ly);
            }
            if (ok) {
                const int cx = min(max(floor_int(px * G.inv_sx), 0), G.gx - 1);
                const int cy = min(max(floor_int(py * G.inv_sy), 0), G.gy - 1);
                b = uint32_t(G.bin_base) + uint32_t(s) * uint32_t(G.gx * G.gy) + uint32_t(cx * G.gy + cy);
                if (a.qrank) a.qrank[sid] = atomicAdd(&a.qcount[b], 1u);   // rank in its bin
                else atomicAdd(&a.qcount[b], 1u);                            // count only
            }
        }
        a.ys[sid] = y;
        a.qbin[sid] = b;
        if (a.src) a.src[sid] = src;
    }
}

}  // namespace sim

namespace {

using namespace sim;

struct AccArgs {
    const InstMC* mc;
    int n_inst;
    const float2* pos;
    const float2* ys;
    const float* fv;       // field value per sample
    long t0, nt;
    int N1, N2;
    int advect;
    float2* vel;
    float2* pos_out;
};

// mis_contrib_dev (src/cuda/monte_carlo_bs.cu:35-51) for the reference law;
// the balance-heuristic estimator with the true sampling densities for the
// unbiased law.
__device__ __forceinline__ float2 mis_term(int law, float2 x, float2 y, float f, float w1, float w2, float cum,
                                           float alpha, float R, const InstMC& I) {
    if (!(f > 0.f)) return make_float2(0.f, 0.f);
    const float rx = x.x - y.x, ry = x.y - y.y;
    if (law == VPMC_LAW_REFERENCE) {
        float wx = rx, wy = ry;
        if (I.periodic) {
            wx = rx - roundf(rx / I.Lx) * I.Lx;
            wy = ry - roundf(ry / I.Ly) * I.Ly;
        }
        const float rn = fmaxf(sqrtf(wx * wx + wy * wy), 1e-6f);
        const float inv_r2 = 1.f / (rx * rx + ry * ry + 1e-8f);
        const float kx = -ry * inv_r2 / (2 * kPiF), ky = rx * inv_r2 / (2 * kPiF);
        const float denom = w1 * f / cum + w2 * alpha / rn;
        const float sc = f / denom;
        return make_float2(kx * sc, ky * sc);
    }
    const float r2 = rx * rx + ry * ry;
    if (!(r2 > 0.f)) return make_float2(0.f, 0.f);
    // K(x - y) f / (w1 f / cum + w2 p2(|x - y|)), p2 = alpha / r inside the disk:
    // multiplied through by cum r, one division per term (the fast form, a
    // reciprocal and a product: ~2 ulp, far below the estimator's noise)
    //   sc = f cum r / ((w1 f r + w2 alpha cum) 2 pi r^2)   (inside)
    //   sc = cum / (w1 2 pi r^2)                             (outside)
    const float rn = sqrtf(r2);
    const float tpr2 = 2.f * kPiF * r2;
    const float sc = rn < R ? __fdividef(f * cum * rn, fmaf(w1 * f, rn, w2 * alpha * cum) * tpr2)
                            : __fdividef(cum, w1 * tpr2);
    return make_float2(-ry * sc, rx * sc);
}

// Plain method: 8 lanes per target, 4 targets per warp.  Each lane sums its
// samples j = l, l + 8, ... (four loads in flight before their terms are
// added), then the 8 lanes combine their compensated sums in a fixed tree.
constexpr int kAccLanes = 8;

__global__ void __launch_bounds__(256) k_accum(AccArgs a) {
    const int lane = threadIdx.x & 31, sub = lane & (kAccLanes - 1), grp = lane / kAccLanes;
    constexpr int kPerWarp = 32 / kAccLanes;
    const long warp = (long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const long nwarps = (long(gridDim.x) * blockDim.x) >> 5;
    const int Q = a.N1 + a.N2;
    const float w1 = float(a.N1) / float(Q), w2 = float(a.N2) / float(Q);
    const float inv = 1.f / float(Q);
    // the loop runs the same trips in every lane of a warp (the group sums shuffle)
    for (long tw = warp * kPerWarp; tw < a.nt; tw += nwarps * kPerWarp) {
        const long tl = tw + grp;
        const bool live = tl < a.nt;
        const long t = a.t0 + (live ? tl : tw);
        const InstMC& I = a.mc[inst_of(a.mc, a.n_inst, t)];
        const float2 x = a.pos[t];
        const float R = disk_radius(x, I.periodic != 0, I.Lx, I.Ly);
        const float alpha = 1.f / (2.f * kPiF * R);
        float u[2][2], uc[2][2];
        for (int s = 0; s < 2; ++s) {
            KSum sx, sy;
            const long base = (tl * 2 + s) * Q;
            for (int j0 = sub; j0 < Q; j0 += 4 * kAccLanes) {
                float2 y[4];
                float f[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const int j = j0 + kAccLanes * v;
                    y[v] = live && j < Q ? a.ys[base + j] : make_float2(0.f, 0.f);
                    f[v] = live && j < Q ? a.fv[base + j] : 0.f;
                }
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    if (j0 + kAccLanes * v >= Q) break;
                    const float2 c = mis_term(I.law, x, y[v], f[v], w1, w2, I.cum9[s], alpha, R, I);
                    sx.add(c.x);
                    sy.add(c.y);
                }
            }
            group_sum_comp_pair<kAccLanes>(sx.s, sx.c);
            group_sum_comp_pair<kAccLanes>(sy.s, sy.c);
            u[s][0] = sx.s;
            u[s][1] = sy.s;
            uc[s][0] = sx.c;
            uc[s][1] = sy.c;
        }
        if (live && sub == 0) {
            // u(+) - u(-) with the leading parts subtracted exactly: a near-singular
            // sample makes both sign sums large, their difference small
            const float vx = comp_diff(u[0][0], uc[0][0], u[1][0], uc[1][0]) * inv;
            const float vy = comp_diff(u[0][1], uc[0][1], u[1][1], uc[1][1]) * inv;
            a.vel[t] = make_float2(vx, vy);
            if (a.advect) {
                double nx = double(x.x) + double(I.dt) * double(vx);
                double ny = double(x.y) + double(I.dt) * double(vy);
                float ox, oy;
                if (I.periodic) {
                    nx -= floor(nx / double(I.Lx)) * double(I.Lx);
                    ny -= floor(ny / double(I.Ly)) * double(I.Ly);
                    ox = float(nx);
                    oy = float(ny);
                    if (ox >= I.Lx) ox = 0.f;
                    if (oy >= I.Ly) oy = 0.f;
                } else {
                    ox = float(nx);
                    oy = float(ny);
                }
                a.pos_out[t] = make_float2(ox, oy);
            }
        }
    }
}

// Deformation mode: one warp per target, five estimates (C, L, R, T, B).
// Branch-1 samples serve all five points, disk samples j in
// [N1 + a N2, N1 + (a+1) N2) serve point a; the normalisation is 1/(N1+N2)
// for each.  Lane 0 writes u = u(+) - u(-) at C (and the four auxiliary
// velocities), advects, and forms F_next = renorm_det1(I + dt grad u).
struct Acc5Args {
    const InstMC* mc;
    int n_inst;
    const float2* pos;
    const float2* ys;
    const float* fv;
    long t0, nt;
    int N1, N2;
    int advect;
    float2* vel;
    float2* vel5;          // 5 per target
    float2* pos_out;
    float4* F_out;
    unsigned* sig;         // [0] = max sigma_max(F_out) (float bits), [1] = targets with sigma_max > cap
    float cap;
};

__global__ void __launch_bounds__(256) k_accum5(Acc5Args a) {
    const int lane = threadIdx.x & 31;
    const long warp = (long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const long nwarps = (long(gridDim.x) * blockDim.x) >> 5;
    const int Q = a.N1 + 5 * a.N2;
    const float w1 = float(a.N1) / float(a.N1 + a.N2), w2 = float(a.N2) / float(a.N1 + a.N2);
    const float inv = 1.f / float(a.N1 + a.N2);
    for (long tl = warp; tl < a.nt; tl += nwarps) {
        const long t = a.t0 + tl;
        const InstMC& I = a.mc[inst_of(a.mc, a.n_inst, t)];
        const float2 x = a.pos[t];
        float2 xa[5];
        float R[5], alpha[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            xa[k] = aux_point(x, k, I.dx);
            R[k] = disk_radius(xa[k], I.periodic != 0, I.Lx, I.Ly);
            alpha[k] = 1.f / (2.f * kPiF * R[k]);
        }
        float u[5][2], su[2][5][2], cu[2][5][2];
        for (int s = 0; s < 2; ++s) {
            KSum sx[5], sy[5];
            const long base = (tl * 2 + s) * Q;
            for (int j = lane; j < a.N1; j += 32) {
                const float2 y = a.ys[base + j];
                const float f = a.fv[base + j];
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    const float2 c = mis_term(I.law, xa[k], y, f, w1, w2, I.cum9[s], alpha[k], R[k], I);
                    sx[k].add(c.x);
                    sy[k].add(c.y);
                }
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                const long b0 = base + a.N1 + long(k) * a.N2;
                for (int j = lane; j < a.N2; j += 32) {
                    const float2 c = mis_term(I.law, xa[k], a.ys[b0 + j], a.fv[b0 + j], w1, w2, I.cum9[s], alpha[k],
                                              R[k], I);
                    sx[k].add(c.x);
                    sy[k].add(c.y);
                }
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                group_sum_comp_pair<32>(sx[k].s, sx[k].c);
                group_sum_comp_pair<32>(sy[k].s, sy[k].c);
                su[s][k][0] = sx[k].s;
                cu[s][k][0] = sx[k].c;
                su[s][k][1] = sy[k].s;
                cu[s][k][1] = sy[k].c;
            }
        }
#pragma unroll
        for (int k = 0; k < 5; ++k)
#pragma unroll
            for (int d = 0; d < 2; ++d) u[k][d] = comp_diff(su[0][k][d], cu[0][k][d], su[1][k][d], cu[1][k][d]) * inv;
        if (lane == 0) {
            const float vx = u[0][0], vy = u[0][1];
            a.vel[t] = make_float2(vx, vy);
#pragma unroll
            for (int k = 0; k < 5; ++k) a.vel5[5 * t + k] = make_float2(u[k][0], u[k][1]);
            if (a.advect) {
                double nx = double(x.x) + double(I.dt) * double(vx);
                double ny = double(x.y) + double(I.dt) * double(vy);
                float ox, oy;
                if (I.periodic) {
                    nx -= floor(nx / double(I.Lx)) * double(I.Lx);
                    ny -= floor(ny / double(I.Ly)) * double(I.Ly);
                    ox = float(nx);
                    oy = float(ny);
                    if (ox >= I.Lx) ox = 0.f;
                    if (oy >= I.Ly) oy = 0.f;
                } else {
                    ox = float(nx);
                    oy = float(ny);
                }
                a.pos_out[t] = make_float2(ox, oy);
                // update_jacobian_from5 + renorm_det1 (src/cuda/monte_carlo_bs.cu:274-288,
                // include/monte_carlo_bs.cuh:140-144), FP32 as there
                const float c = 0.5f * I.dt / I.dx;
                float4 F;
                F.x = 1.f + (u[2][0] - u[1][0]) * c;
                F.y = (u[3][0] - u[4][0]) * c;
                F.z = (u[2][1] - u[1][1]) * c;
                F.w = 1.f + (u[3][1] - u[4][1]) * c;
                const float det = F.x * F.w - F.y * F.z;
                const float sc = rsqrtf(fmaxf(det, 1e-12f));
                F.x *= sc;
                F.y *= sc;
                F.z *= sc;
                F.w *= sc;
                a.F_out[t] = F;
                const float sm = sigma_max(F);
                atomicMax(&a.sig[0], __float_as_uint(sm));   // non-negative floats order as their bits
                if (!(sm <= a.cap)) atomicAdd(&a.sig[1], 1u);
            }
        }
    }
}

// The plain FP64 path of the same estimator: field values, MIS terms, sums
// and the Euler update in FP64 (sample points are drawn as in FP32 mode).
__device__ __forceinline__ double2 mis_term64(int law, float2 xf, float2 yf, double f, double w1, double w2,
                                              double cum, double alpha, double R, const InstMC& I) {
    if (!(f > 0.0)) return make_double2(0.0, 0.0);
    const double rx = double(xf.x) - double(yf.x), ry = double(xf.y) - double(yf.y);
    if (law == VPMC_LAW_REFERENCE) {
        double wx = rx, wy = ry;
        if (I.periodic) {
            wx = rx - round(rx / I.Lx) * I.Lx;
            wy = ry - round(ry / I.Ly) * I.Ly;
        }
        const double rn = fmax(sqrt(wx * wx + wy * wy), 1e-6);
        const double inv_r2 = 1.0 / (rx * rx + ry * ry + 1e-8);
        const double denom = w1 * f / cum + w2 * alpha / rn;
        const double sc = f / denom * inv_r2 / (2.0 * kPiD);
        return make_double2(-ry * sc, rx * sc);
    }
    const double r2 = rx * rx + ry * ry;
    if (!(r2 > 0.0)) return make_double2(0.0, 0.0);
    const double rn = sqrt(r2);
    const double p2 = rn < R ? alpha / rn : 0.0;
    const double sc = f / ((w1 * f / cum + w2 * p2) * (2.0 * kPiD * r2));
    return make_double2(-ry * sc, rx * sc);
}

struct AccArgs64 {
    const InstMC* mc;
    int n_inst;
    const float2* pos;
    const float2* ys;
    const double* fv;
    const double* cum64;   // per instance: Omega_+, Omega_- (x9 when periodic), FP64
    long t0, nt;
    int N1, N2;
    int advect;
    float2* vel;
    float2* pos_out;
};

__global__ void __launch_bounds__(256) k_accum64(AccArgs64 a) {
    const int lane = threadIdx.x & 31;
    const long warp = (long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const long nwarps = (long(gridDim.x) * blockDim.x) >> 5;
    const int Q = a.N1 + a.N2;
    const double w1 = double(a.N1) / Q, w2 = double(a.N2) / Q;
    for (long tl = warp; tl < a.nt; tl += nwarps) {
        const long t = a.t0 + tl;
        const int ii = inst_of(a.mc, a.n_inst, t);
        const InstMC& I = a.mc[ii];
        const float2 x = a.pos[t];
        const double R = sqrt(double(I.Lx) * I.Lx + double(I.Ly) * I.Ly);
        const double alpha = 1.0 / (2.0 * kPiD * R);
        double u[2][2];
        for (int s = 0; s < 2; ++s) {
            double sx = 0.0, sy = 0.0;
            const long base = (tl * 2 + s) * Q;
            for (int j = lane; j < Q; j += 32) {
                const double2 c = mis_term64(I.law, x, a.ys[base + j], a.fv[base + j], w1, w2, a.cum64[2 * ii + s],
                                             alpha, R, I);
                sx += c.x;
                sy += c.y;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {   // fixed butterfly, identical on every lane
                const double ox = __shfl_xor_sync(0xffffffffu, sx, o), oy = __shfl_xor_sync(0xffffffffu, sy, o);
                const bool lo = (lane & o) == 0;
                sx = lo ? sx + ox : ox + sx;
                sy = lo ? sy + oy : oy + sy;
            }
            u[s][0] = sx / Q;
            u[s][1] = sy / Q;
        }
        if (lane == 0) {
            const double vx = u[0][0] - u[1][0], vy = u[0][1] - u[1][1];
            a.vel[t] = make_float2(float(vx), float(vy));
            if (a.advect) {
                double nx = double(x.x) + double(I.dt) * vx, ny = double(x.y) + double(I.dt) * vy;
                float ox, oy;
                if (I.periodic) {
                    nx -= floor(nx / double(I.Lx)) * double(I.Lx);
                    ny -= floor(ny / double(I.Ly)) * double(I.Ly);
                    ox = float(nx);
                    oy = float(ny);
                    if (ox >= I.Lx) ox = 0.f;
                    if (oy >= I.Ly) oy = 0.f;
                } else {
                    ox = float(nx);
                    oy = float(ny);
                }
                a.pos_out[t] = make_float2(ox, oy);
            }
        }
    }
}

__global__ void k_inc_step(unsigned long long* s) { *s += 1ull; }

// sum over targets of |u|^2 in FP64 (one atomic per warp)
__global__ void k_vel_sumsq(const float2* __restrict__ v, long n, double* __restrict__ out) {
    double acc = 0.0;
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
        acc += double(v[i].x) * double(v[i].x) + double(v[i].y) * double(v[i].y);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// taylor_green_vorticity (include/analytical_flow.hpp:24-28) evaluated in
// FP64: on a lattice the FP64 field is an exact eigenvector of the RBF matrix,
// which an FP32-rounded copy is not (its rounding spreads over eigenvalues
// near zero and stalls CG near 1e-6 at 2048^2).
__global__ void k_taylor_green(const float2* __restrict__ pos, long n, double* __restrict__ b) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const double x = pos[i].x, y = pos[i].y;
        b[i] = 4.0 * kPiD * sin(2.0 * kPiD * x) * sin(2.0 * kPiD * y);
    }
}

__global__ void k_advect(float2* __restrict__ pos, const float2* __restrict__ vel, const double* __restrict__ vel64,
                         long n, float dt, float Lx, float Ly, int periodic) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const float2 x = pos[i];
        const double vx = vel64 ? vel64[2 * i] : double(vel[i].x);
        const double vy = vel64 ? vel64[2 * i + 1] : double(vel[i].y);
        double nx = double(x.x) + double(dt) * vx, ny = double(x.y) + double(dt) * vy;
        float ox, oy;
        if (periodic) {
            nx -= floor(nx / double(Lx)) * double(Lx);
            ny -= floor(ny / double(Ly)) * double(Ly);
            ox = float(nx);
            oy = float(ny);
            if (ox >= Lx) ox = 0.f;
            if (oy >= Ly) oy = 0.f;
        } else {
            ox = float(nx);
            oy = float(ny);
        }
        pos[i] = make_float2(ox, oy);
    }
}

__global__ void k_check_finite(const float2* __restrict__ p, long n, unsigned* flags) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const float2 v = p[i];
        if (!isfinite(v.x) || !isfinite(v.y)) atomicOr(flags, FLAG_NONFINITE);
    }
}


// Inverse of the radial mass C(q) of the cubic spline (2 pi r W(r) dr, h_w = 1)
// tabulated at u = i / T by bisection in FP64; the unbiased branch-1 jitter
// radius is h_w * interp(u).
void build_jitter_table(std::vector<float>& t) {
    t.resize(kJitTab + 1);
    for (int i = 0; i <= kJitTab; ++i) {
        const double u = double(i) / kJitTab;
        double lo = 0.0, hi = 1.0;
        for (int it = 0; it < 80; ++it) {
            const double mid = 0.5 * (lo + hi);
            if (spline_mass_d(mid) < u) lo = mid; else hi = mid;
        }
        t[i] = float(0.5 * (lo + hi));
    }
    t[0] = 0.f;
    t[kJitTab] = 1.f;
}

}  // namespace
}  // namespace vpmc

using namespace vpmc;


namespace {

constexpr float kCoverCap = 2.f;   // the reference's 3x3 walk of 2 h_w cells reaches 2 h_w


// Cover level for a stretch sigma: 1, else the next multiple of 1/16, at most kCoverCap.
float cover_for(float sigma) {
    if (!(sigma > 1.f)) return 1.f;
    return std::min(kCoverCap, std::ceil(sigma * 16.f) / 16.f);
}

void drop_graphs(vpmc_sim* s) {
    if (s->graph_step) cudaGraphExecDestroy(s->graph_step);
    if (s->graph_vel) cudaGraphExecDestroy(s->graph_vel);
    s->graph_step = s->graph_vel = nullptr;
}

uint32_t mix32(uint64_t v) {
    v ^= v >> 33;
    v *= 0xff51afd7ed558ccdULL;
    v ^= v >> 33;
    v *= 0xc4ceb9fe1a85ec53ULL;
    v ^= v >> 33;
    return uint32_t(v);
}

// Philox key of an instance = its own 64-bit seed (scrambled so that small
// seeds give unrelated keys); nothing else enters the key.
void set_keys(vpmc_sim* s) {
    for (int i = 0; i < s->n_inst; ++i) {
        const uint64_t seed = s->prm[i].seed;
        s->mc[i].key0 = mix32(seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL);
        s->mc[i].key1 = mix32(seed ^ 0xA4093822299F31D0ULL);
        s->mc[i].law = s->prm[i].law;
    }
}

int upload_mc(vpmc_sim* s) {
    VPMC_CUDA(cudaMemcpyAsync(s->d_mc, s->mc.data(), sizeof(InstMC) * s->mc.size(), cudaMemcpyHostToDevice,
                              s->ctx->stream));
    return VPMC_OK;
}

// Working set sized for the largest chunk (samples <= max_samples).
int alloc_work(vpmc_sim* s) {
    vpmc_context* ctx = s->ctx;
    std::vector<InstDesc> d(s->n_inst);
    for (int i = 0; i < s->n_inst; ++i)
        d[i] = InstDesc{s->prm[i].Lx, s->prm[i].Ly, s->mc[i].hw, s->prm[i].periodic, int(s->begin[i]),
                        int(s->begin[i] + s->counts[i]), s->deform ? s->cover : 1.f};
    s->plan.resize(s->n_inst);
    const long nb = grid_plan(d.data(), s->n_inst, s->k_walk, 2, s->plan.data());
    if (nb < 0) return int(-nb);
    const long Q2 = 2L * samples_per(s);
    long per_chunk = s->max_samples / Q2;
    if (per_chunk < 1) per_chunk = 1;
    if (per_chunk > s->N) per_chunk = s->N;
    s->chunk_targets = per_chunk;
    const long ns = per_chunk * Q2;
    const size_t nchunks = size_t((s->N + per_chunk - 1) / per_chunk);
    for (auto e : s->chunk_ev) cudaEventDestroy(e);
    s->chunk_ev.assign(2 * nchunks, nullptr);
    for (auto& e : s->chunk_ev) VPMC_CUDA(cudaEventCreate(&e));
    auto carve_all = [&](Carver& c) {
        carve_grid(c, s->N, nb, s->n_inst, &s->g, s->deform != 0, s->rows);
        carve_items(c, nb, ns, &s->it);
        carve_queries(c, nb, ns, &s->q, true);
        s->ys = c.take<float2>(size_t(ns));
        s->ys_t0 = -1;
        s->ys_nt = 0;
        s->fv = c.take<float>(size_t(ns));
        s->fv64 = s->precision == 64 ? c.take<double>(size_t(ns)) : nullptr;
        s->cum64 = c.take<double>(2 * size_t(s->n_inst));
    };
    Carver dry;
    carve_all(dry);
    drop_graphs(s);
    VPMC_TRY(s->work.reserve(dry.off));
    Carver c{static_cast<char*>(s->work.p), 0};
    carve_all(c);
    VPMC_CUDA(cudaMemcpyAsync(s->g.inst, s->plan.data(), sizeof(GridInst) * s->plan.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
    if (!s->cum64_h.empty())
        VPMC_CUDA(cudaMemcpyAsync(s->cum64, s->cum64_h.data(), sizeof(double) * s->cum64_h.size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
    return VPMC_OK;
}

// Deformation mode: read sigma_max of F (after a step from its F update,
// else by a reduction over F) and re-plan the grid when the walk must reach
// further.  reset = set the cover to what F needs (also lower); otherwise it
// only grows.  Kernels stretched beyond kCoverCap are counted, not covered.
// realloc: re-carve the working set even if the cover stays (mode switch).
int refresh_cover(vpmc_sim* s, bool from_step, bool reset, bool realloc = false) {
    cudaStream_t st = s->ctx->stream;
    float sig = 1.f;
    if (!from_step) {
        VPMC_TRY(grid_max_sigma(s->ctx, s->F, s->N, s->d_sig, &sig));
    } else {
        unsigned h[2] = {0u, 0u};
        VPMC_CUDA(cudaMemcpyAsync(h, s->d_sig, sizeof(h), cudaMemcpyDeviceToHost, st));
        VPMC_CUDA(cudaStreamSynchronize(st));
        std::memcpy(&sig, &h[0], sizeof(sig));
        s->over_cap += h[1];
    }
    s->sigma = sig;
    if (!s->deform) {
        s->cover = 1.f;
        if (realloc) VPMC_TRY(alloc_work(s));
        return VPMC_OK;
    }
    const float need = std::max(s->min_cover, cover_for(sig));
    const bool changed = reset ? need != s->cover : need > s->cover;
    if (changed) s->cover = need;
    if (changed || realloc) VPMC_TRY(alloc_work(s));
    return VPMC_OK;
}

// The sample buffer holds the last chunk's samples after a pass.
void mark_samples(vpmc_sim* s) {
    s->ys_t0 = s->t_begin + ((s->t_end - s->t_begin - 1) / s->chunk_targets) * s->chunk_targets;
    s->ys_nt = s->t_end - s->ys_t0;
}

// Issue one MIS pass over all targets (advect: positions -> pos_next, then
// copied back, step counter incremented).  No host synchronisation inside, so
// it can be captured.  Returns launches issued.
int issue_pass(vpmc_sim* s, bool advect, bool timed, int* nlaunch) {
    vpmc_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const uint64_t l0 = vpmc_kernel_launch_count();
    // inside stream capture the timing events must become graph event nodes
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    VPMC_CUDA(cudaStreamIsCapturing(st, &cap));
    const unsigned ev_flags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    const bool def = s->deform != 0;
    VPMC_TRY(grid_build(ctx, s->g, s->pos, s->omega, SET_SIGN_SPLIT, def ? s->F : nullptr));
    if (def && advect) VPMC_CUDA(cudaMemsetAsync(s->d_sig, 0, 2 * sizeof(unsigned), st));
    const long Q = samples_per(s);
    if (!def) VPMC_LAUNCH(k_sub_pos, blocks_for(2 * s->N), 256, 0, st, s->d_mc, s->n_inst, s->sub, s->pos, 2 * s->N,
                          s->pos_sub);
    for (long t0 = s->t_begin; t0 < s->t_end; t0 += s->chunk_targets) {
        const long nt = std::min(s->chunk_targets, s->t_end - t0);
        const long ns = nt * 2 * Q;
        VPMC_CUDA(cudaMemsetAsync(s->q.qcount, 0, sizeof(uint32_t) * size_t(s->g.nbins + 1), st));
        GenArgs ga{s->d_mc, s->n_inst, s->g.inst, s->pos, def ? s->F : nullptr, def ? nullptr : s->pos_sub, s->sub,
                   s->cdf, s->guide, s->jit,
                   s->d_step, t0, nt, s->N1, s->N2, def ? 5 : 1, nullptr, s->ys, s->q.qbin, s->q.qcount,
                   s->q.tmp ? nullptr : s->q.qrank};
        VPMC_LAUNCH(k_gen, blocks_for(ns), 256, 0, st, ga);
        VPMC_TRY(scatter_ranked(ctx, s->g, s->q, s->ys, ns));
        VPMC_TRY(make_items(ctx, s->g, s->q.qstart, s->it, query_chunk(s->precision == 64 ? 4 : s->qpt)));
        const bool f64 = s->precision == 64;
        if (f64) VPMC_CUDA(cudaMemsetAsync(s->fv64, 0, sizeof(double) * size_t(ns), st));
        else VPMC_CUDA(cudaMemsetAsync(s->fv, 0, sizeof(float) * size_t(ns), st));
        EvalLaunch L;
        const bool unb = s->mc[0].law == VPMC_LAW_UNBIASED;
        L.mode = f64 ? (unb ? EVAL_FIELD9_64 : EVAL_FIELD64)
                     : (def ? (unb ? EVAL_FIELD9_F : EVAL_FIELD_F) : (unb ? EVAL_FIELD9 : EVAL_FIELD));
        L.qpt = f64 ? 4 : s->qpt;
        L.out_f32 = s->fv;
        L.out_f64 = s->fv64;
        const size_t ci = size_t((t0 - s->t_begin) / s->chunk_targets);
        if (timed) VPMC_CUDA(cudaEventRecordWithFlags(s->chunk_ev[2 * ci], st, ev_flags));
        VPMC_TRY(launch_eval(ctx, s->g, s->q.qrec, s->it, L));
        if (timed) VPMC_CUDA(cudaEventRecordWithFlags(s->chunk_ev[2 * ci + 1], st, ev_flags));
        if (def) {
            Acc5Args aa{s->d_mc, s->n_inst, s->pos, s->ys, s->fv, t0, nt, s->N1, s->N2, advect ? 1 : 0, s->vel,
                        s->vel5, s->pos_next, s->F_next, s->d_sig, kCoverCap};
            VPMC_LAUNCH(k_accum5, blocks_for(nt * 32), 256, 0, st, aa);
        } else if (f64) {
            AccArgs64 aa{s->d_mc, s->n_inst, s->pos, s->ys, s->fv64, s->cum64, t0, nt, s->N1, s->N2, advect ? 1 : 0,
                         s->vel, s->pos_next};
            VPMC_LAUNCH(k_accum64, blocks_for(nt * 32), 256, 0, st, aa);
        } else {
            AccArgs aa{s->d_mc, s->n_inst, s->pos, s->ys, s->fv, t0, nt, s->N1, s->N2, advect ? 1 : 0, s->vel,
                       s->pos_next};
            VPMC_LAUNCH(k_accum, blocks_for(nt * kAccLanes), 256, 0, st, aa);
        }
    }
    mark_samples(s);
    if (advect) {
        // only the pass's targets moved (a shard leaves the others to the exchange)
        const size_t tb = size_t(s->t_begin), tn = size_t(s->t_end - s->t_begin);
        VPMC_CUDA(cudaMemcpyAsync(s->pos + tb, s->pos_next + tb, sizeof(float2) * tn, cudaMemcpyDeviceToDevice, st));
        if (def)
            VPMC_CUDA(cudaMemcpyAsync(s->F + tb, s->F_next + tb, sizeof(float4) * tn, cudaMemcpyDeviceToDevice, st));
        VPMC_LAUNCH(k_inc_step, 1, 1, 0, st, s->d_step);
    }
    *nlaunch = int(vpmc_kernel_launch_count() - l0);
    return VPMC_OK;
}

// Device time of the eval launches of the last completed pass (call after a sync).
int collect_eval_time(vpmc_sim* s) {
    const long nchunks = (s->t_end - s->t_begin + s->chunk_targets - 1) / s->chunk_targets;
    float tot = 0.f;
    for (long c = 0; c < nchunks; ++c) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, s->chunk_ev[2 * c], s->chunk_ev[2 * c + 1]) != cudaSuccess) {
            (void)cudaGetLastError();
            return VPMC_OK;   // events not recorded (no timed pass yet)
        }
        tot += ms;
    }
    s->eval_ms = tot;
    s->eval_launches = int(nchunks);
    return VPMC_OK;
}

}  // namespace

int sim::run_pass(vpmc_sim* s, bool advect, int use_graph) {
    vpmc_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    if (!s->prepared) VPMC_TRY(vpmc_sim_prepare(s));
    if (s->mc[0].law == VPMC_LAW_UNBIASED)
        for (auto& m : s->mc) if (m.law != VPMC_LAW_UNBIASED) return VPMC_ERR_INVALID;
    cudaGraphExec_t* gx = advect ? &s->graph_step : &s->graph_vel;
    if (!use_graph) {
        int nl = 0;
        VPMC_TRY(issue_pass(s, advect, true, &nl));
        s->launches_per_step = nl;
        if (advect) s->step += 1;
        return VPMC_OK;
    }
    if (!*gx) {
        // eager pass first (sets kernel attributes, sizes the eval grid), then capture
        int nl = 0;
        VPMC_TRY(issue_pass(s, advect, true, &nl));
        VPMC_CUDA(cudaStreamSynchronize(st));
        if (advect) s->step += 1;
        cudaGraph_t graph = nullptr;
        VPMC_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int rc = issue_pass(s, advect, true, &nl);
        const cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (rc != VPMC_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
        VPMC_CUDA(ce);
        const cudaError_t ie = cudaGraphInstantiate(gx, graph, 0);
        cudaGraphDestroy(graph);
        VPMC_CUDA(ie);
        s->launches_per_step = nl;
        if (advect) return VPMC_OK;   // the eager pass was this call's step
    }
    VPMC_CUDA(cudaGraphLaunch(*gx, st));
    mark_samples(s);
    if (advect) s->step += 1;
    return VPMC_OK;
}


int sim::set_step_counter(vpmc_sim* s, uint64_t step) {
    s->step = step;
    unsigned long long v = step;
    VPMC_CUDA(cudaMemcpyAsync(s->d_step, &v, sizeof(v), cudaMemcpyHostToDevice, s->ctx->stream));
    VPMC_CUDA(cudaStreamSynchronize(s->ctx->stream));   // v lives on this stack frame
    return VPMC_OK;
}

extern "C" {

int vpmc_sim_create(vpmc_context* ctx, int n_inst, const vpmc_sim_params* prms, const int* counts, vpmc_sim** out) {
    if (!ctx || n_inst < 1 || !prms || !counts || !out) return VPMC_ERR_INVALID;
    *out = nullptr;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    long N = 0;
    for (int i = 0; i < n_inst; ++i) {
        const vpmc_sim_params& p = prms[i];
        if (counts[i] < 0 || p.Nx < 1 || !(p.hwr > 0.f) || !(p.Lx > 0.f) || !(p.Ly > 0.f)) return VPMC_ERR_INVALID;
        if (p.N1 < 0 || p.N2 < 0 || p.N1 + p.N2 < 1 || p.N1 != prms[0].N1 || p.N2 != prms[0].N2) return VPMC_ERR_INVALID;
        if (p.law != VPMC_LAW_REFERENCE && p.law != VPMC_LAW_UNBIASED) return VPMC_ERR_INVALID;
        if (p.law != prms[0].law) return VPMC_ERR_INVALID;
        N += counts[i];
    }
    if (N >= (1L << 31) || N < 1) return N < 1 ? VPMC_ERR_INVALID : VPMC_ERR_CAPACITY;
    auto* s = new (std::nothrow) vpmc_sim();
    if (!s) return VPMC_ERR_NOMEM;
    s->ctx = ctx;
    ctx->refs.fetch_add(1);   // released by vpmc_sim_destroy
    s->n_inst = n_inst;
    s->prm.assign(prms, prms + n_inst);
    s->counts.assign(counts, counts + n_inst);
    s->begin.resize(n_inst);
    s->N = N;
    s->t_begin = 0;
    s->t_end = N;
    s->N1 = prms[0].N1;
    s->N2 = prms[0].N2;
    s->max_samples = 1L << 30;   // samples per chunk (~52 B of records each): fuller bins, fewer passes
    long b = 0;
    s->mc.resize(n_inst);
    for (int i = 0; i < n_inst; ++i) {
        s->begin[i] = b;
        const vpmc_sim_params& p = prms[i];
        InstMC m{};
        // SimParam (include/vortex_particle_mc.hpp:119-133): h = Lx/Nx, h_w = h*hwr
        const float h = p.Lx / float(p.Nx);
        m.hw = h * p.hwr;
        m.dx = 0.5f * m.hw;
        m.Lx = p.Lx;
        m.Ly = p.Ly;
        m.dt = p.dt;
        m.periodic = p.periodic;
        m.law = p.law;
        m.p_begin = int(b);
        m.p_end = int(b + counts[i]);
        float cdf[kIcdfRef];
        vpmc_kernel_icdf_table(m.hw, kIcdfRef, cdf, m.icdf);
        s->mc[i] = m;
        b += counts[i];
    }
    set_keys(s);
    // particle + subset memory
    Carver dry;
    auto carve_state = [&](Carver& c) {
        s->pos = c.take<float2>(size_t(N));
        s->pos_next = c.take<float2>(size_t(N));
        s->vel = c.take<float2>(size_t(N));
        s->omega = c.take<float>(size_t(N));
        s->sub = c.take<int>(2 * size_t(N) + 2);
        s->cdf = c.take<double>(2 * size_t(N) + 2);
        s->guide = c.take<uint2>(size_t(N) + 4 * size_t(n_inst) + 4);
        s->jit = c.take<float2>(kJitTab + 1);
        s->pos_sub = c.take<float2>(2 * size_t(N) + 2);
        s->d_mc = c.take<InstMC>(size_t(n_inst));
        s->d_step = c.take<unsigned long long>(1);
        s->F = c.take<float4>(size_t(N));
        s->F_next = c.take<float4>(size_t(N));
        s->d_sig = c.take<unsigned>(2);
        s->d_check = c.take<double>(1);
    };
    carve_state(dry);
    int rc = s->mem.reserve(dry.off);
    if (rc != VPMC_OK) { vpmc_sim_destroy(s); return rc; }
    Carver c{static_cast<char*>(s->mem.p), 0};
    carve_state(c);
    std::vector<float> jt;
    build_jitter_table(jt);
    cudaStream_t st = ctx->stream;
    cudaMemsetAsync(s->mem.p, 0, s->mem.bytes, st);
    std::vector<float2> jt2(kJitTab);
    for (int i = 0; i < kJitTab; ++i) jt2[i] = make_float2(jt[i], jt[i + 1]);
    cudaMemcpyAsync(s->jit, jt2.data(), sizeof(float2) * jt2.size(), cudaMemcpyHostToDevice, st);
    unsigned long long zero = 0;
    cudaMemcpyAsync(s->d_step, &zero, sizeof(zero), cudaMemcpyHostToDevice, st);
    k_identity<<<blocks_for(N), 256, 0, st>>>(s->F, N);
    if (cudaEventCreate(&s->ev[0]) != cudaSuccess || cudaEventCreate(&s->ev[1]) != cudaSuccess) {
        vpmc_sim_destroy(s);
        return VPMC_ERR_CUDA;
    }
    rc = upload_mc(s);
    if (rc == VPMC_OK) rc = alloc_work(s);
    if (rc == VPMC_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = VPMC_ERR_CUDA;
    if (rc != VPMC_OK) { vpmc_sim_destroy(s); return rc; }
    *out = s;
    return VPMC_OK;
}

int vpmc_sim_destroy(vpmc_sim* s) {
    if (!s) return VPMC_ERR_INVALID;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    drop_graphs(s);
    for (auto& e : s->ev) if (e) cudaEventDestroy(e);
    for (auto e : s->chunk_ev) if (e) cudaEventDestroy(e);
    s->mem.release();
    s->work.release();
    s->aux.release();
    s->ckpt.release();
    s->seg.release();
    s->adj.release();
    vpmc_context* ctx = s->ctx;
    delete s;
    return context_release(ctx);
}

int vpmc_sim_num_particles(vpmc_sim* s) { return s ? int(s->N) : -1; }

int vpmc_advect(vpmc_context* ctx, int N, float* pos, const float* vel, const double* vel64, float dt, float Lx,
                float Ly, int periodic) {
    if (!ctx || N < 0 || (N > 0 && (!pos || (!vel && !vel64))) || !(Lx > 0.f) || !(Ly > 0.f)) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    if (N > 0)
        VPMC_LAUNCH(k_advect, blocks_for(N), 256, 0, ctx->stream, reinterpret_cast<float2*>(pos),
                    reinterpret_cast<const float2*>(vel), vel64, long(N), dt, Lx, Ly, periodic);
    return vpmc_context_sync(ctx);
}

int vpmc_sim_set_particles(vpmc_sim* s, const float* pos, const float* omega, int is_host) {
    if (!s) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    cudaStream_t st = s->ctx->stream;
    const cudaMemcpyKind k = is_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (pos) {
        VPMC_CUDA(cudaMemcpyAsync(s->pos, pos, sizeof(float2) * size_t(s->N), k, st));
        VPMC_LAUNCH(k_check_finite, blocks_for(s->N), 256, 0, st, s->pos, s->N, s->ctx->d_flags);
    }
    if (omega) {
        VPMC_CUDA(cudaMemcpyAsync(s->omega, omega, sizeof(float) * size_t(s->N), k, st));
        s->prepared = false;
    }
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_get_particles(vpmc_sim* s, float* pos, float* omega, float* vel, int is_host) {
    if (!s) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    cudaStream_t st = s->ctx->stream;
    const cudaMemcpyKind k = is_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (pos) VPMC_CUDA(cudaMemcpyAsync(pos, s->pos, sizeof(float2) * size_t(s->N), k, st));
    if (omega) VPMC_CUDA(cudaMemcpyAsync(omega, s->omega, sizeof(float) * size_t(s->N), k, st));
    if (vel) VPMC_CUDA(cudaMemcpyAsync(vel, s->vel, sizeof(float2) * size_t(s->N), k, st));
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_prepare(vpmc_sim* s) {
    if (!s) return VPMC_ERR_INVALID;
    vpmc_context* ctx = s->ctx;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    long goff = 0;
    std::vector<double> cum64_h;
    for (int i = 0; i < s->n_inst; ++i) {
        const long b = s->begin[i], n = s->counts[i];
        InstMC& m = s->mc[i];
        int cnt[2] = {0, 0};
        double cum[2] = {0, 0};
        if (n > 0 && s->frozen && s->prepared_once) {
            // sampling frozen: subsets, CDF and guide stay; only Omega follows omega
            // (built into scratch; the sign pattern must not change)
            DevBuf tmp;
            VPMC_TRY(tmp.reserve((2 * sizeof(int) + 2 * sizeof(double)) * size_t(n) + 1024));
            Carver c{static_cast<char*>(tmp.p), 0};
            int* sp = c.take<int>(size_t(n));
            int* sn = c.take<int>(size_t(n));
            double* cp = c.take<double>(size_t(n));
            double* cn = c.take<double>(size_t(n));
            const int rc = build_subsets_dev(ctx, n, s->omega + b, sp, sn, cp, cn, nullptr, nullptr, cnt, cum);
            tmp.release();
            if (rc != VPMC_OK) return rc;
            if (cnt[0] != m.cnt[0] || cnt[1] != m.cnt[1]) return VPMC_ERR_INVALID;
        } else if (n > 0) {
            VPMC_TRY(build_subsets_dev(ctx, n, s->omega + b, s->sub + 2 * b, s->sub + 2 * b + n, s->cdf + 2 * b,
                                       s->cdf + 2 * b + n, nullptr, nullptr, cnt, cum));
        }
        m.cnt[0] = cnt[0];
        m.cnt[1] = cnt[1];
        m.off[0] = 2 * b;
        m.off[1] = 2 * b + n;
        const float f9 = m.periodic ? 9.f : 1.f;
        m.cum9[0] = float(cum[0]) * f9;
        m.cum9[1] = float(cum[1]) * f9;
        cum64_h.push_back(cum[0] * (m.periodic ? 9.0 : 1.0));
        cum64_h.push_back(cum[1] * (m.periodic ? 9.0 : 1.0));
        for (int sg = 0; sg < 2; ++sg) {
            m.goff[sg] = goff;
            if (cnt[sg] > 0 && !(s->frozen && s->prepared_once))
                VPMC_LAUNCH(k_guide, blocks_for(cnt[sg]), 256, 0, st, s->cdf + m.off[sg], cnt[sg], s->guide + goff);
            goff += cnt[sg] + 2;
        }
    }
    VPMC_TRY(upload_mc(s));
    s->cum64_h = cum64_h;
    VPMC_CUDA(cudaMemcpyAsync(s->cum64, cum64_h.data(), sizeof(double) * cum64_h.size(), cudaMemcpyHostToDevice, st));
    VPMC_CUDA(cudaStreamSynchronize(st));
    drop_graphs(s);
    s->prepared = true;
    s->prepared_once = true;
    return vpmc_context_sync(ctx);
}

int vpmc_sim_init_strengths(vpmc_sim* s, const float* omega_field, double tol, int max_iter, double* info) {
    if (!s) return VPMC_ERR_INVALID;
    vpmc_context* ctx = s->ctx;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    double* b = nullptr;
    if (!omega_field) {
        // reuse the sample-position scratch for the FP64 right-hand side
        b = reinterpret_cast<double*>(s->ys);
        s->ys_t0 = -1;
        s->ys_nt = 0;
        if (s->chunk_targets * 2L * (s->N1 + s->N2) < s->N) return VPMC_ERR_CAPACITY;
        VPMC_LAUNCH(k_taylor_green, blocks_for(s->N), 256, 0, st, s->pos, s->N, b);
    }
    int worst = VPMC_OK;
    for (int i = 0; i < s->n_inst; ++i) {
        const long off = s->begin[i];
        const vpmc_sim_params& p = s->prm[i];
        double inf[3] = {0, 0, 0};
        const bool mr = s->rbf_solver == VPMC_RBF_MINRES;
        const float* pi = reinterpret_cast<const float*>(s->pos + off);
        const int rc = omega_field
                           ? (mr ? vpmc_minres_rbf : vpmc_cg_rbf)(ctx, s->counts[i], pi, omega_field + off,
                                                                 s->omega + off, s->mc[i].hw, p.Lx, p.Ly, p.periodic,
                                                                 tol, max_iter, inf)
                           : (mr ? vpmc_minres_rbf_f64rhs : vpmc_cg_rbf_f64rhs)(ctx, s->counts[i], pi, b + off,
                                                                               s->omega + off, s->mc[i].hw, p.Lx,
                                                                               p.Ly, p.periodic, tol, max_iter, inf);
        if (rc != VPMC_OK && rc != VPMC_ERR_NOT_CONVERGED) return rc;
        if (rc != VPMC_OK) worst = rc;
        if (info) { info[3 * i] = inf[0]; info[3 * i + 1] = inf[1]; info[3 * i + 2] = inf[2]; }
    }
    s->prepared = false;
    VPMC_TRY(vpmc_sim_prepare(s));
    return worst;
}

int vpmc_sim_step(vpmc_sim* s, int nsteps, int use_graph) {
    if (!s || nsteps < 0) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    for (int k = 0; k < nsteps; ++k) {
        VPMC_TRY(run_pass(s, true, use_graph));
        if (s->deform) VPMC_TRY(refresh_cover(s, true, false));
    }
    VPMC_TRY(vpmc_context_sync(s->ctx));
    return collect_eval_time(s);
}

int vpmc_sim_velocity(vpmc_sim* s, uint64_t step, float* vel) {
    if (!s || !vel) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    cudaStream_t st = s->ctx->stream;
    unsigned long long v = step;
    VPMC_CUDA(cudaMemcpyAsync(s->d_step, &v, sizeof(v), cudaMemcpyHostToDevice, st));
    VPMC_TRY(run_pass(s, false, 0));
    VPMC_CUDA(cudaMemcpyAsync(vel, s->vel, sizeof(float2) * size_t(s->N), cudaMemcpyDeviceToDevice, st));
    unsigned long long cur = s->step;
    VPMC_CUDA(cudaMemcpyAsync(s->d_step, &cur, sizeof(cur), cudaMemcpyHostToDevice, st));
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_step_host(vpmc_sim* s, const float* pos_in, float* pos_out, float* vel_out) {
    if (!s) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    cudaStream_t st = s->ctx->stream;
    if (pos_in) VPMC_CUDA(cudaMemcpyAsync(s->pos, pos_in, sizeof(float2) * size_t(s->N), cudaMemcpyHostToDevice, st));
    VPMC_TRY(run_pass(s, true, 1));
    if (s->deform) VPMC_TRY(refresh_cover(s, true, false));
    if (pos_out) VPMC_CUDA(cudaMemcpyAsync(pos_out, s->pos, sizeof(float2) * size_t(s->N), cudaMemcpyDeviceToHost, st));
    if (vel_out) VPMC_CUDA(cudaMemcpyAsync(vel_out, s->vel, sizeof(float2) * size_t(s->N), cudaMemcpyDeviceToHost, st));
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_set_law(vpmc_sim* s, int law) {
    if (!s || (law != VPMC_LAW_REFERENCE && law != VPMC_LAW_UNBIASED)) return VPMC_ERR_INVALID;
    for (auto& p : s->prm) p.law = law;
    set_keys(s);
    VPMC_TRY(upload_mc(s));
    drop_graphs(s);
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_set_seed(vpmc_sim* s, uint64_t seed) {
    if (!s) return VPMC_ERR_INVALID;
    for (auto& p : s->prm) p.seed = seed;
    set_keys(s);
    VPMC_TRY(upload_mc(s));
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_set_step(vpmc_sim* s, uint64_t step) {
    if (!s) return VPMC_ERR_INVALID;
    s->step = step;
    unsigned long long v = step;
    VPMC_CUDA(cudaMemcpyAsync(s->d_step, &v, sizeof(v), cudaMemcpyHostToDevice, s->ctx->stream));
    return vpmc_context_sync(s->ctx);
}

uint64_t vpmc_sim_get_step(vpmc_sim* s) { return s ? s->step : 0; }

int vpmc_sim_set_precision(vpmc_sim* s, int bits) {
    if (!s || (bits != 32 && bits != 64)) return VPMC_ERR_INVALID;
    if (bits == 64 && s->deform) return VPMC_ERR_UNSUPPORTED;   // deformed kernels run in FP32 only
    if (bits == s->precision) return VPMC_OK;
    s->precision = bits;
    VPMC_TRY(alloc_work(s));
    if (s->prepared) {   // the FP64 totals live in the re-carved working set
        s->prepared = false;
        VPMC_TRY(vpmc_sim_prepare(s));
    }
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_set_target_range(vpmc_sim* s, long long begin, long long end) {
    if (!s || begin < 0 || end > s->N || begin >= end) return VPMC_ERR_INVALID;
    if (s->deform && (begin != 0 || end != s->N)) return VPMC_ERR_UNSUPPORTED;
    s->t_begin = long(begin);
    s->t_end = long(end);
    s->ys_t0 = -1;
    s->ys_nt = 0;
    drop_graphs(s);   // the captured passes cover the old range (the chunk events cover all N)
    return VPMC_OK;
}

int vpmc_sim_get_target_range(vpmc_sim* s, long long* begin, long long* end) {
    if (!s) return VPMC_ERR_INVALID;
    if (begin) *begin = s->t_begin;
    if (end) *end = s->t_end;
    return VPMC_OK;
}

int vpmc_sim_set_rbf_solver(vpmc_sim* s, int solver) {
    if (!s || (solver != VPMC_RBF_CG && solver != VPMC_RBF_MINRES)) return VPMC_ERR_INVALID;
    s->rbf_solver = solver;
    return VPMC_OK;
}

int vpmc_sim_set_tuning(vpmc_sim* s, int k_walk, int qpt) {
    if (!s || k_walk < 0 || k_walk > 8 || !(qpt == 0 || qpt == 1 || qpt == 4 || qpt == 6 || qpt == 8))
        return VPMC_ERR_INVALID;
    s->k_walk = k_walk;
    s->qpt = qpt == 0 ? 4 : qpt;
    VPMC_TRY(alloc_work(s));
    return vpmc_context_sync(s->ctx);
}

// Autotuner: time one full velocity pass (gen + bin + eval + accumulate) for
// each candidate (cells per h_w, queries per thread) and keep the fastest.
// Results are cached in-process by (hwr, samples per target, particles per
// h_w^2 of instance 0), so a second simulation of the same shape reuses them.
namespace {
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, std::pair<int, int>> g_tune_cache;
}  // namespace

int vpmc_sim_autotune(vpmc_sim* s, int* k_out, int* qpt_out, float* best_ms) {
    if (!s) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    if (!s->prepared) VPMC_TRY(vpmc_sim_prepare(s));
    const vpmc_sim_params& p = s->prm[0];
    const double density = double(s->counts[0]) / (double(p.Lx) * p.Ly) * double(s->mc[0].hw) * s->mc[0].hw;
    const auto key = std::make_tuple(int(std::lround(p.hwr * 16 * (s->deform ? s->cover : 1.f))),
                                     int(samples_per(s)) * (s->deform ? -1 : 1), int(std::lround(density)));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            VPMC_TRY(vpmc_sim_set_tuning(s, it->second.first, it->second.second));
            if (k_out) *k_out = s->plan[0].k;
            if (qpt_out) *qpt_out = s->qpt;
            if (best_ms) *best_ms = -1.f;
            return VPMC_OK;
        }
    }
    cudaStream_t st = s->ctx->stream;
    // queries per thread 4, 6, 8: the one-warp CUDA-core evaluation; 1: the
    // tensor-core evaluation (plain kernels only: deformed ones run the former)
    const int cands[][2] = {{2, 4}, {3, 4}, {4, 4}, {5, 4}, {6, 4}, {7, 4}, {8, 4}, {3, 6}, {4, 6}, {6, 6},
                            {8, 6}, {2, 8}, {3, 8}, {4, 8}, {6, 8}, {8, 8}, {3, 1}, {4, 1}, {5, 1}, {6, 1},
                            {7, 1}, {8, 1}};
    struct Trial { int k, q; float ms; double check; };
    std::vector<Trial> tr;
    for (const auto& c : cands) {
        if (c[1] == 1 && s->deform) continue;
        if (vpmc_sim_set_tuning(s, c[0], c[1]) != VPMC_OK) continue;
        if (s->plan[0].k != c[0]) continue;   // geometry clamped k: skip duplicates
        int nl = 0;
        VPMC_TRY(issue_pass(s, false, false, &nl));   // warm (kernel attributes, caches)
        VPMC_CUDA(cudaEventRecord(s->ev[0], st));
        VPMC_TRY(issue_pass(s, false, false, &nl));
        VPMC_CUDA(cudaEventRecord(s->ev[1], st));
        // the same samples every pass (the step counter does not move): the
        // velocities agree up to rounding of the field sums
        VPMC_CUDA(cudaMemsetAsync(s->d_check, 0, sizeof(double), st));
        VPMC_LAUNCH(k_vel_sumsq, std::min(blocks_for(s->N), 4 * s->ctx->sm_count), 256, 0, st, s->vel, s->N,
                    s->d_check);
        double chk = 0.0;
        VPMC_CUDA(cudaMemcpyAsync(&chk, s->d_check, sizeof(double), cudaMemcpyDeviceToHost, st));
        VPMC_CUDA(cudaStreamSynchronize(st));
        float ms = 0.f;
        VPMC_CUDA(cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]));
        tr.push_back({c[0], c[1], ms, chk});
    }
    if (tr.empty()) return VPMC_ERR_GEOMETRY;
    std::vector<double> chks;
    for (const Trial& t : tr) chks.push_back(t.check);
    std::nth_element(chks.begin(), chks.begin() + chks.size() / 2, chks.end());
    const double med = chks[chks.size() / 2];
    float best = 1e30f;
    int bk = 0, bq = 4;
    for (const Trial& t : tr) {
        if (!(std::fabs(t.check - med) <= 1e-4 * std::fabs(med))) return VPMC_ERR_DEVICE;
        if (t.ms < best) { best = t.ms; bk = t.k; bq = t.q; }
    }
    VPMC_TRY(vpmc_sim_set_tuning(s, bk, bq));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = {bk, bq};
    }
    if (k_out) *k_out = s->plan[0].k;
    if (qpt_out) *qpt_out = s->qpt;
    if (best_ms) *best_ms = best;
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_get_tuning(vpmc_sim* s, int* k_walk, int* qpt) {
    if (!s) return VPMC_ERR_INVALID;
    if (k_walk) *k_walk = s->plan.empty() ? 0 : s->plan[0].k;
    if (qpt) *qpt = s->qpt;
    return VPMC_OK;
}

int vpmc_sim_last_stats(vpmc_sim* s, int* launches_per_step, float* eval_ms) {
    if (!s) return VPMC_ERR_INVALID;
    if (launches_per_step) *launches_per_step = s->launches_per_step;
    if (eval_ms) *eval_ms = s->eval_ms;
    return VPMC_OK;
}

int vpmc_sim_read_samples(vpmc_sim* s, long long first, long long count, long long* t0, float* xy) {
    if (!s || first < 0 || count < 0 || (count > 0 && !xy)) return VPMC_ERR_INVALID;
    if (s->ys_t0 < 0) return VPMC_ERR_INVALID;   // no pass has drawn samples into the current buffer
    if (t0) *t0 = s->ys_t0;
    if (first + count > s->ys_nt * 2LL * samples_per(s)) return VPMC_ERR_INVALID;
    if (count == 0) return VPMC_OK;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    VPMC_CUDA(cudaMemcpyAsync(xy, s->ys + first, sizeof(float2) * size_t(count), cudaMemcpyDeviceToHost,
                              s->ctx->stream));
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_read_field(vpmc_sim* s, long long first, long long count, long long* t0, double* f) {
    if (!s || first < 0 || count < 0 || (count > 0 && !f)) return VPMC_ERR_INVALID;
    if (s->ys_t0 < 0) return VPMC_ERR_INVALID;   // no pass has evaluated samples into the current buffer
    if (t0) *t0 = s->ys_t0;
    if (first + count > s->ys_nt * 2LL * samples_per(s)) return VPMC_ERR_INVALID;
    if (count == 0) return VPMC_OK;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    cudaStream_t st = s->ctx->stream;
    if (s->precision == 64) {
        VPMC_CUDA(cudaMemcpyAsync(f, s->fv64 + first, sizeof(double) * size_t(count), cudaMemcpyDeviceToHost, st));
        return vpmc_context_sync(s->ctx);
    }
    std::vector<float> tmp(static_cast<size_t>(count));
    VPMC_CUDA(cudaMemcpyAsync(tmp.data(), s->fv + first, sizeof(float) * size_t(count), cudaMemcpyDeviceToHost, st));
    VPMC_TRY(vpmc_context_sync(s->ctx));
    for (size_t i = 0; i < tmp.size(); ++i) f[i] = double(tmp[i]);
    return VPMC_OK;
}

int vpmc_sim_geometry(vpmc_sim* s, long long* info) {
    if (!s || !info) return VPMC_ERR_INVALID;
    info[0] = s->N;
    info[1] = s->chunk_targets;
    info[2] = (s->t_end - s->t_begin + s->chunk_targets - 1) / s->chunk_targets;
    info[3] = s->g.nbins;
    info[4] = s->plan.empty() ? 0 : s->plan[0].gx;
    info[5] = s->plan.empty() ? 0 : s->plan[0].k;
    info[6] = 2LL * samples_per(s);
    info[7] = s->eval_launches;
    return VPMC_OK;
}

int vpmc_update_jacobian_from5(vpmc_context* ctx, int N, float dt, float dx, const float* velC, const float* velL,
                                const float* velR, const float* velT, const float* velB, float* F_out) {
    if (!ctx || N < 0 || !(dx > 0.f)) return VPMC_ERR_INVALID;
    if (N == 0) return VPMC_OK;
    if (!velL || !velR || !velT || !velB || !F_out) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    VPMC_LAUNCH(k_jacobian5, blocks_for(N), 256, 0, ctx->stream, long(N), dt, dx,
                reinterpret_cast<const float2*>(velC), reinterpret_cast<const float2*>(velL),
                reinterpret_cast<const float2*>(velR), reinterpret_cast<const float2*>(velT),
                reinterpret_cast<const float2*>(velB), reinterpret_cast<float4*>(F_out));
    return vpmc_context_sync(ctx);
}

int vpmc_sim_reinit(vpmc_sim* s, double tol, int max_iter, double* info) {
    if (!s || max_iter < 0) return VPMC_ERR_INVALID;
    vpmc_context* ctx = s->ctx;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    for (int i = 0; i < s->n_inst; ++i) {
        const vpmc_sim_params& p = s->prm[i];
        // SimParam (include/vortex_particle_mc.hpp:119-133): Ny = round(Ly / h), h = Lx / Nx in FP32
        const float h = p.Lx / float(p.Nx);
        int Ny = int(std::round(p.Ly / h));
        if (Ny == 0) Ny = 1;
        if (long(p.Nx) * Ny != s->counts[i]) return VPMC_ERR_INVALID;
    }
    if (!s->prepared) VPMC_TRY(vpmc_sim_prepare(s));
    s->ys_t0 = -1;   // the field values of the last pass are overwritten below
    s->ys_nt = 0;
    int worst = VPMC_OK;
    for (int i = 0; i < s->n_inst; ++i) {
        const vpmc_sim_params& p = s->prm[i];
        const long b = s->begin[i], n = s->counts[i];
        if (n == 0) continue;
        const float h = p.Lx / float(p.Nx);
        const int Ny = std::max(1, int(std::round(p.Ly / h)));
        // 1. the current field (signed, deformed kernels in deformation mode) at the new lattice
        VPMC_LAUNCH(k_lattice, blocks_for(n), 256, 0, st, s->pos_next + b, p.Nx, Ny, p.Lx, p.Ly);
        VPMC_TRY(vpmc_query_vorticity(ctx, int(n), reinterpret_cast<const float*>(s->pos + b), s->omega + b,
                                      s->deform ? reinterpret_cast<const float*>(s->F + b) : nullptr, int(n),
                                      reinterpret_cast<const float*>(s->pos_next + b), 0, 1, 0, s->mc[i].hw, p.Lx,
                                      p.Ly, p.periodic, s->fv));
        // 2. positions to the lattice, F to the identity
        VPMC_CUDA(cudaMemcpyAsync(s->pos + b, s->pos_next + b, sizeof(float2) * size_t(n), cudaMemcpyDeviceToDevice,
                                  st));
        VPMC_LAUNCH(k_identity, blocks_for(n), 256, 0, st, s->F + b, n);
        // 3. strengths re-fitted by CG-RBF
        double inf[3] = {0, 0, 0};
        const int rc = (s->rbf_solver == VPMC_RBF_MINRES ? vpmc_minres_rbf : vpmc_cg_rbf)(
            ctx, int(n), reinterpret_cast<const float*>(s->pos + b), s->fv, s->omega + b, s->mc[i].hw, p.Lx, p.Ly,
            p.periodic, tol, max_iter, inf);
        if (rc != VPMC_OK && rc != VPMC_ERR_NOT_CONVERGED) return rc;
        if (rc != VPMC_OK) worst = rc;
        if (info) { info[3 * i] = inf[0]; info[3 * i + 1] = inf[1]; info[3 * i + 2] = inf[2]; }
    }
    s->prepared = false;
    VPMC_TRY(vpmc_sim_prepare(s));
    if (s->deform) VPMC_TRY(refresh_cover(s, false, true));
    VPMC_TRY(vpmc_context_sync(ctx));
    return worst;
}

int vpmc_sim_vorticity_grid(vpmc_sim* s, int inst, int res_x, int res_y, int sign, float* out) {
    if (!s || inst < 0 || inst >= s->n_inst || res_x < 1 || res_y < 1 || !out) return VPMC_ERR_INVALID;
    if (long(res_x) * res_y > (1L << 28)) return VPMC_ERR_CAPACITY;
    vpmc_context* ctx = s->ctx;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    const vpmc_sim_params& p = s->prm[inst];
    const long b = s->begin[inst], n = s->counts[inst], m = long(res_x) * res_y;
    char* base = nullptr;
    VPMC_TRY(scratch(ctx, SLOT_DIRECT, sizeof(float2) * size_t(m) + 256, &base));
    float2* pts = reinterpret_cast<float2*>(base);
    VPMC_LAUNCH(k_lattice, blocks_for(m), 256, 0, ctx->stream, pts, res_x, res_y, p.Lx, p.Ly);
    return vpmc_query_vorticity(ctx, int(n), reinterpret_cast<const float*>(s->pos + b), s->omega + b,
                                s->deform ? reinterpret_cast<const float*>(s->F + b) : nullptr, int(m),
                                reinterpret_cast<const float*>(pts), sign, sign == 0 ? 1 : 0, 0, s->mc[inst].hw,
                                p.Lx, p.Ly, p.periodic, out);
}

int vpmc_sim_freeze_sampling(vpmc_sim* s, int on) {
    if (!s) return VPMC_ERR_INVALID;
    if (on && !s->prepared) VPMC_TRY(vpmc_sim_prepare(s));
    s->frozen = on != 0;
    return VPMC_OK;
}

int vpmc_sim_set_deformation(vpmc_sim* s, int on, float min_cover) {
    if (!s || !(min_cover <= kCoverCap)) return VPMC_ERR_INVALID;
    if (on && s->precision == 64) return VPMC_ERR_UNSUPPORTED;
    if (on && (s->t_begin != 0 || s->t_end != s->N)) return VPMC_ERR_UNSUPPORTED;   // no F exchange for shards
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    if (on && !s->vel5) {
        VPMC_TRY(s->aux.reserve(5 * sizeof(float2) * size_t(s->N)));
        s->vel5 = static_cast<float2*>(s->aux.p);
        VPMC_CUDA(cudaMemsetAsync(s->vel5, 0, 5 * sizeof(float2) * size_t(s->N), s->ctx->stream));
    }
    s->deform = on ? 1 : 0;
    s->min_cover = std::max(1.f, min_cover);
    if (!s->deform) s->cover = 1.f;
    VPMC_TRY(refresh_cover(s, false, true, true));
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_set_F(vpmc_sim* s, const float* F, int is_host) {
    if (!s || !F) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    VPMC_CUDA(cudaMemcpyAsync(s->F, F, sizeof(float4) * size_t(s->N),
                              is_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s->ctx->stream));
    VPMC_TRY(refresh_cover(s, false, s->deform != 0));
    if (!std::isfinite(s->sigma)) return VPMC_ERR_INVALID;   // non-finite or det <= 0 somewhere
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_get_F(vpmc_sim* s, float* F, int is_host) {
    if (!s || !F) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    VPMC_CUDA(cudaMemcpyAsync(F, s->F, sizeof(float4) * size_t(s->N),
                              is_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s->ctx->stream));
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_get_aux_velocities(vpmc_sim* s, float* vel5, int is_host) {
    if (!s || !vel5) return VPMC_ERR_INVALID;
    if (!s->deform || !s->vel5) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(s->ctx->device));
    VPMC_CUDA(cudaMemcpyAsync(vel5, s->vel5, 5 * sizeof(float2) * size_t(s->N),
                              is_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s->ctx->stream));
    return vpmc_context_sync(s->ctx);
}

int vpmc_sim_deform_info(vpmc_sim* s, double* info) {
    if (!s || !info) return VPMC_ERR_INVALID;
    info[0] = s->sigma;
    info[1] = s->deform ? s->cover : 1.0;
    info[2] = double(s->over_cap);
    info[3] = s->deform;
    return VPMC_OK;
}

}  // extern "C"
