// vpmc_direct.cu -- FP64 direct Biot-Savart sums (the accuracy oracle on the
// GPU and the "plain FP64" comparison path).
//
// Targets x sources is tiled two ways: a block owns 256 targets and one chunk
// of the sources, stages the chunk through shared memory, and writes a partial
// (u, v) per target; a second kernel adds the chunk partials in chunk order,
// so the result does not depend on scheduling.
#include "vpmc_internal.cuh"

namespace vpmc {
namespace {

constexpr int kDT = 256;        // targets per block
constexpr int kTileSrc = 256;   // sources staged per step

template <int KERNEL>
__global__ void __launch_bounds__(kDT) k_direct(const float2* __restrict__ pos, const float* __restrict__ om,
                                                 long N, const float2* __restrict__ pts,
                                                 const int* __restrict__ tidx, long M, double param, double Lx,
                                                 double Ly, int periodic, long chunk, double2* __restrict__ part) {
    __shared__ double sx[kTileSrc], sy[kTileSrc], sw[kTileSrc];
    __shared__ int sj[kTileSrc];
    const long m = long(blockIdx.x) * kDT + threadIdx.x;
    const long c = blockIdx.y;
    const long s0 = c * chunk, s1 = min(N, s0 + chunk);
    double px = 0.0, py = 0.0;
    long self = -1;
    if (m < M) {
        if (KERNEL == VPMC_DIRECT_PLUMMER) {
            self = tidx[m];
            px = pos[self].x;
            py = pos[self].y;
        } else {
            px = pts[m].x;
            py = pts[m].y;
        }
    }
    const double e2 = param * param;
    const double inv2pi = 1.0 / (2.0 * kPiD);
    double u = 0.0, v = 0.0;
    for (long t0 = s0; t0 < s1; t0 += kTileSrc) {
        __syncthreads();
        const long j = t0 + threadIdx.x;
        if (threadIdx.x < kTileSrc) {
            if (j < s1) {
                sx[threadIdx.x] = pos[j].x;
                sy[threadIdx.x] = pos[j].y;
                sw[threadIdx.x] = om[j];
                sj[threadIdx.x] = int(j);
            } else {
                sw[threadIdx.x] = 0.0;
                sj[threadIdx.x] = -2;
            }
        }
        __syncthreads();
        const int cnt = int(min(long(kTileSrc), s1 - t0));
        for (int q = 0; q < cnt; ++q) {
            const double w = sw[q];
            if (w == 0.0) continue;
            if (KERNEL == VPMC_DIRECT_PLUMMER) {
                if (sj[q] == self) continue;
                double dx = px - sx[q], dy = py - sy[q];
                if (periodic) {
                    dx -= Lx * rint(dx / Lx);
                    dy -= Ly * rint(dy / Ly);
                }
                const double k = w * inv2pi / (dx * dx + dy * dy + e2);
                u -= dy * k;
                v += dx * k;
            } else {
                const int lo = periodic ? -1 : 0, hi = periodic ? 1 : 0;
                for (int ix = lo; ix <= hi; ++ix)
                    for (int iy = lo; iy <= hi; ++iy) {
                        const double dx = px - (sx[q] + ix * Lx);
                        const double dy = py - (sy[q] + iy * Ly);
                        const double r2 = dx * dx + dy * dy;
                        if (r2 == 0.0) continue;
                        double k = w * inv2pi / r2;
                        if (r2 < param * param) k *= spline_mass_d(sqrt(r2) / param);
                        u -= dy * k;
                        v += dx * k;
                    }
            }
        }
    }
    if (m < M) part[c * M + m] = make_double2(u, v);
}

// FP32 tiles: the deterministic "P" particle method of the reference
// (biot_savart_naive_kernel, src/cuda/naive_biot_savart.cu:15-40, is FP32).
__device__ __forceinline__ float spline_mass_f(float q) {
    if (q >= 1.f) return 1.f;
    const float c = 80.f / 7.f, q2 = q * q;
    if (q <= 0.5f) return c * q2 * fmaf(q2, fmaf(1.2f, q, -1.5f), 0.5f);
    const float g = q2 * fmaf(q2, fmaf(-0.4f, q, 1.5f), fmaf(-2.f, q, 1.f));
    return c * (0.06875f + g - 0.08125f);
}

template <int KERNEL>
__global__ void __launch_bounds__(kDT) k_direct_f32(const float2* __restrict__ pos, const float* __restrict__ om,
                                                     long N, const float2* __restrict__ pts,
                                                     const int* __restrict__ tidx, long M, float param, float Lx,
                                                     float Ly, int periodic, long chunk, float2* __restrict__ part) {
    __shared__ float2 sp[kTileSrc];
    __shared__ float sw[kTileSrc];
    __shared__ int sj[kTileSrc];
    const long m = long(blockIdx.x) * kDT + threadIdx.x;
    const long c = blockIdx.y;
    const long s0 = c * chunk, s1 = min(N, s0 + chunk);
    float2 x = make_float2(0.f, 0.f);
    long self = -1;
    if (m < M) {
        if (KERNEL == VPMC_DIRECT_PLUMMER) { self = tidx[m]; x = pos[self]; }
        else x = pts[m];
    }
    const float e2 = param * param, inv2pi = 1.f / (2.f * kPiF), ih = 1.f / param;
    float u = 0.f, v = 0.f;
    for (long t0 = s0; t0 < s1; t0 += kTileSrc) {
        __syncthreads();
        const long j = t0 + threadIdx.x;
        if (threadIdx.x < kTileSrc) {
            sp[threadIdx.x] = j < s1 ? pos[j] : make_float2(0.f, 0.f);
            sw[threadIdx.x] = j < s1 ? om[j] : 0.f;
            sj[threadIdx.x] = j < s1 ? int(j) : -2;
        }
        __syncthreads();
        const int cnt = int(min(long(kTileSrc), s1 - t0));
        for (int q = 0; q < cnt; ++q) {
            const float w = sw[q];
            if (KERNEL == VPMC_DIRECT_PLUMMER) {
                if (sj[q] == self) continue;
                float dx = x.x - sp[q].x, dy = x.y - sp[q].y;
                if (periodic) {   // wrap_min_image (include/monte_carlo_bs.cuh:140-143)
                    dx -= rintf(dx / Lx) * Lx;
                    dy -= rintf(dy / Ly) * Ly;
                }
                const float k = w * inv2pi / (dx * dx + dy * dy + e2);
                u -= dy * k;
                v += dx * k;
            } else {
                const int lo = periodic ? -1 : 0, hi = periodic ? 1 : 0;
                for (int ix = lo; ix <= hi; ++ix)
                    for (int iy = lo; iy <= hi; ++iy) {
                        const float dx = x.x - (sp[q].x + ix * Lx), dy = x.y - (sp[q].y + iy * Ly);
                        const float r2 = dx * dx + dy * dy;
                        if (r2 == 0.f) continue;
                        float k = w * inv2pi / r2;
                        if (r2 < e2) k *= spline_mass_f(sqrtf(r2) * ih);
                        u -= dy * k;
                        v += dx * k;
                    }
            }
        }
    }
    if (m < M) part[c * M + m] = make_float2(u, v);
}

__global__ void k_direct_reduce_f32(const float2* __restrict__ part, long M, int nchunk, float* __restrict__ out) {
    for (long m = long(blockIdx.x) * blockDim.x + threadIdx.x; m < M; m += long(gridDim.x) * blockDim.x) {
        float u = 0.f, v = 0.f;
        for (int c = 0; c < nchunk; ++c) {
            const float2 p = part[long(c) * M + m];
            u += p.x;
            v += p.y;
        }
        out[2 * m] = u;
        out[2 * m + 1] = v;
    }
}

__global__ void k_direct_reduce(const double2* __restrict__ part, long M, int nchunk, double* __restrict__ out) {
    for (long m = long(blockIdx.x) * blockDim.x + threadIdx.x; m < M; m += long(gridDim.x) * blockDim.x) {
        double u = 0.0, v = 0.0;
        for (int c = 0; c < nchunk; ++c) {
            const double2 p = part[long(c) * M + m];
            u += p.x;
            v += p.y;
        }
        out[2 * m] = u;
        out[2 * m + 1] = v;
    }
}

}  // namespace
}  // namespace vpmc

using namespace vpmc;

extern "C" int vpmc_direct_velocity_f64(vpmc_context* ctx, int kernel, int N, const float* pos, const float* omega,
                                        int M, const float* pts, const int* tidx, double param, double Lx, double Ly,
                                        int periodic, double* out_uv) {
    if (!ctx || N < 0 || M < 0 || !(Lx > 0) || !(Ly > 0)) return VPMC_ERR_INVALID;
    if (kernel != VPMC_DIRECT_MOLLIFIED && kernel != VPMC_DIRECT_PLUMMER) return VPMC_ERR_INVALID;
    if (M == 0) return VPMC_OK;
    if (!out_uv || (N > 0 && (!pos || !omega))) return VPMC_ERR_INVALID;
    if (kernel == VPMC_DIRECT_PLUMMER ? !tidx : !pts) return VPMC_ERR_INVALID;
    if (kernel == VPMC_DIRECT_MOLLIFIED && !(param > 0)) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const long tblocks = (long(M) + kDT - 1) / kDT;
    // enough blocks to fill the GPU several times over
    long nchunk = (8L * ctx->sm_count + tblocks - 1) / tblocks;
    if (nchunk < 1) nchunk = 1;
    if (nchunk > 4096) nchunk = 4096;
    long chunk = (long(N) + nchunk - 1) / nchunk;
    if (chunk < kTileSrc) chunk = kTileSrc;
    nchunk = N > 0 ? (long(N) + chunk - 1) / chunk : 1;
    char* base = nullptr;
    VPMC_TRY(scratch(ctx, SLOT_DIRECT, sizeof(double2) * size_t(nchunk) * size_t(M) + 256, &base));
    double2* part = reinterpret_cast<double2*>(base);
    if (N == 0) {
        VPMC_CUDA(cudaMemsetAsync(part, 0, sizeof(double2) * size_t(M), st));
    } else {
        const dim3 grid{static_cast<unsigned>(tblocks), static_cast<unsigned>(nchunk), 1u};
        if (kernel == VPMC_DIRECT_PLUMMER)
            VPMC_LAUNCH(k_direct<VPMC_DIRECT_PLUMMER>, grid, kDT, 0, st, reinterpret_cast<const float2*>(pos), omega,
                        long(N), nullptr, tidx, long(M), param, Lx, Ly, periodic, chunk, part);
        else
            VPMC_LAUNCH(k_direct<VPMC_DIRECT_MOLLIFIED>, grid, kDT, 0, st, reinterpret_cast<const float2*>(pos),
                        omega, long(N), reinterpret_cast<const float2*>(pts), nullptr, long(M), param, Lx, Ly,
                        periodic, chunk, part);
    }
    VPMC_LAUNCH(k_direct_reduce, unsigned((M + 255) / 256), 256, 0, st, part, long(M), int(nchunk), out_uv);
    return vpmc_context_sync(ctx);
}

extern "C" int vpmc_direct_velocity_f32(vpmc_context* ctx, int kernel, int N, const float* pos, const float* omega,
                                        int M, const float* pts, const int* tidx, float param, float Lx, float Ly,
                                        int periodic, float* out_uv) {
    if (!ctx || N < 0 || M < 0 || !(Lx > 0.f) || !(Ly > 0.f)) return VPMC_ERR_INVALID;
    if (kernel != VPMC_DIRECT_MOLLIFIED && kernel != VPMC_DIRECT_PLUMMER) return VPMC_ERR_INVALID;
    if (M == 0) return VPMC_OK;
    if (!out_uv || (N > 0 && (!pos || !omega))) return VPMC_ERR_INVALID;
    if (kernel == VPMC_DIRECT_PLUMMER ? !tidx : !pts) return VPMC_ERR_INVALID;
    if (kernel == VPMC_DIRECT_MOLLIFIED && !(param > 0.f)) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const long tblocks = (long(M) + kDT - 1) / kDT;
    long nchunk = (8L * ctx->sm_count + tblocks - 1) / tblocks;
    if (nchunk < 1) nchunk = 1;
    if (nchunk > 4096) nchunk = 4096;
    long chunk = (long(N) + nchunk - 1) / nchunk;
    if (chunk < kTileSrc) chunk = kTileSrc;
    nchunk = N > 0 ? (long(N) + chunk - 1) / chunk : 1;
    char* base = nullptr;
    VPMC_TRY(scratch(ctx, SLOT_DIRECT, sizeof(float2) * size_t(nchunk) * size_t(M) + 256, &base));
    float2* part = reinterpret_cast<float2*>(base);
    if (N == 0) {
        VPMC_CUDA(cudaMemsetAsync(part, 0, sizeof(float2) * size_t(M), st));
    } else {
        const dim3 grid{static_cast<unsigned>(tblocks), static_cast<unsigned>(nchunk), 1u};
        if (kernel == VPMC_DIRECT_PLUMMER)
            VPMC_LAUNCH(k_direct_f32<VPMC_DIRECT_PLUMMER>, grid, kDT, 0, st, reinterpret_cast<const float2*>(pos),
                        omega, long(N), nullptr, tidx, long(M), param, Lx, Ly, periodic, chunk, part);
        else
            VPMC_LAUNCH(k_direct_f32<VPMC_DIRECT_MOLLIFIED>, grid, kDT, 0, st, reinterpret_cast<const float2*>(pos),
                        omega, long(N), reinterpret_cast<const float2*>(pts), nullptr, long(M), param, Lx, Ly,
                        periodic, chunk, part);
    }
    VPMC_LAUNCH(k_direct_reduce_f32, unsigned((M + 255) / 256), 256, 0, st, part, long(M), int(nchunk), out_uv);
    return vpmc_context_sync(ctx);
}
