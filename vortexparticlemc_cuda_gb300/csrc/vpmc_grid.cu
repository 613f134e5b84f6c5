// vpmc_grid.cu -- evaluation grid: planning, stable build, query binning and
// the field-evaluation kernel (the hot loop of queries, MIS samples and SpMV).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "vpmc_grid.cuh"

namespace vpmc {

namespace {

constexpr int kEvalThreads = 32;
constexpr int kMaxK = 8;
constexpr int kMaxPieces = 2 * (2 * kMaxK + 1);
constexpr int kCandCap = 208;                  // candidates staged per batch (6.5 KB: 24 one-warp CTAs fill an SM's shared memory)
constexpr uint32_t kWaitLimit = VPMC_WAIT_LIMIT_DEFAULT;   // drain wait of an aborted CTA (always the full cap)

__device__ __forceinline__ int inst_of_particle(const GridInst* inst, int n_inst, long i) {
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].p_begin <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int inst_of_bin(const GridInst* inst, int n_inst, uint32_t b) {
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (uint32_t(inst[mid].bin_base) <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Wrap into [0, L) the way the reference does (p - floor(p/L)*L).
__device__ __forceinline__ float wrapf(float p, float L) { return p - floorf(p / L) * L; }

__global__ void k_grid_keys(const float2* __restrict__ pos, const float* __restrict__ omega, long n,
                            const GridInst* __restrict__ inst, int n_inst, int set_mode, uint32_t nbins, int rows,
                            uint32_t* __restrict__ keys, uint32_t* __restrict__ count) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const GridInst G = inst[inst_of_particle(inst, n_inst, i)];
        const float w = omega ? omega[i] : 1.f;
        int set = 0;
        bool use = true;
        switch (set_mode) {
            case SET_SIGN_SPLIT: set = w > 0.f ? 0 : 1; use = w != 0.f; break;
            case SET_POS_ONLY: use = w > 0.f; break;
            case SET_NEG_ONLY: use = w < 0.f; break;
            default: break;
        }
        uint32_t key = nbins * uint32_t(rows);
        if (use) {
            float2 p = pos[i];
            if (G.periodic) { p.x = wrapf(p.x, G.Lx); p.y = wrapf(p.y, G.Ly); }
            const int cx = min(max(floor_int(p.x * G.inv_sx), 0), G.gx - 1);
            const int cy = min(max(floor_int(p.y * G.inv_sy), 0), G.gy - 1);
            const uint32_t bin = uint32_t(G.bin_base) + uint32_t(set) * uint32_t(G.gx * G.gy) + uint32_t(cx * G.gy + cy);
            // sub-row of the cell (nested: clamped into the cell's own rows)
            const int r = min(max(floor_int(p.y * G.inv_sy * float(rows)) - cy * rows, 0), rows - 1);
            key = bin * uint32_t(rows) + uint32_t(r);
            atomicAdd(&count[key], 1u);
        }
        keys[i] = key;
    }
}

__global__ void k_grid_gather(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ start, long n,
                              uint32_t nbins, const float2* __restrict__ pos, const float* __restrict__ omega,
                              const GridInst* __restrict__ inst, int n_inst, int set_mode,
                              Cand* __restrict__ cand) {
    const long nv = start[nbins];
    for (long p = long(blockIdx.x) * blockDim.x + threadIdx.x; p < nv && p < n; p += long(gridDim.x) * blockDim.x) {
        const uint32_t i = perm[p];
        const GridInst G = inst[inst_of_particle(inst, n_inst, i)];
        float2 q = pos[i];
        if (G.periodic) { q.x = wrapf(q.x, G.Lx); q.y = wrapf(q.y, G.Ly); }
        const float w = omega ? omega[i] : 1.f;
        // weight 2 sigma |omega| (or 2 sigma omega), FP32 hi part + remainder
        const double wd = double(set_mode == SET_ONE_SIGNED ? w : fabsf(w)) * (80.0 / (7.0 * kPiD * double(G.hw) * G.hw));
        const float wt = float(wd);
        cand[p] = Cand{q.x, q.x, q.y, q.y, wt, wt, float(wd - double(wt)), 0.f};
    }
}

// Deformed records: metric G = F^-T F^-1 of F = [[F.x, F.y], [F.z, F.w]]
// (the inverse the reference applies, include/vorticity_query.cuh:52-63,
// divides the adjugate by det F), formed in FP64.
__global__ void k_grid_gather_f(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ start, long n,
                                uint32_t nbins, const float2* __restrict__ pos, const float* __restrict__ omega,
                                const float4* __restrict__ F, const GridInst* __restrict__ inst, int n_inst,
                                int set_mode, CandF* __restrict__ cand) {
    const long nv = start[nbins];
    for (long p = long(blockIdx.x) * blockDim.x + threadIdx.x; p < nv && p < n; p += long(gridDim.x) * blockDim.x) {
        const uint32_t i = perm[p];
        const GridInst G = inst[inst_of_particle(inst, n_inst, i)];
        float2 q = pos[i];
        if (G.periodic) { q.x = wrapf(q.x, G.Lx); q.y = wrapf(q.y, G.Ly); }
        const float w = omega ? omega[i] : 1.f;
        const double wd = double(set_mode == SET_ONE_SIGNED ? w : fabsf(w)) * (80.0 / (7.0 * kPiD * double(G.hw) * G.hw));
        const float wt = float(wd);
        const float4 f = F[i];
        const double det = double(f.x) * f.w - double(f.y) * f.z;
        const double id2 = 1.0 / (det * det);
        CandF r;
        r.f[0] = q.x;
        r.f[1] = q.y;
        r.f[2] = float((double(f.w) * f.w + double(f.z) * f.z) * id2);
        r.f[3] = float(-(double(f.w) * f.y + double(f.z) * f.x) * id2);
        r.f[4] = float((double(f.y) * f.y + double(f.x) * f.x) * id2);
        r.f[5] = wt;
        r.f[6] = float(wd - double(wt));
#pragma unroll
        for (int k = 7; k < 16; ++k) r.f[k] = 0.f;
        cand[p] = r;
    }
}

__global__ void k_sigma(const float4* __restrict__ F, long n, unsigned* __restrict__ out) {
    unsigned m = 0u;
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const float4 f = F[i];
        const float sm = sigma_max(f);
        const float det = f.x * f.w - f.y * f.z;
        // non-negative floats order as their bit patterns; degenerate F -> +inf
        m = max(m, (sm == sm && sm <= 3.0e38f && det > 0.f) ? __float_as_uint(sm) : 0x7f800000u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void k_coarse_starts(const uint32_t* __restrict__ start, long nbins, int rows,
                                uint32_t* __restrict__ cstart) {
    for (long b = long(blockIdx.x) * blockDim.x + threadIdx.x; b <= nbins; b += long(gridDim.x) * blockDim.x)
        cstart[b] = start[b * rows];
}

__global__ void k_grid_weights(const double* __restrict__ x, long n, double scale, Cand* __restrict__ cand) {
    for (long p = long(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += long(gridDim.x) * blockDim.x) {
        const double v = x[p] * scale;
        const float hi = float(v);
        cand[p].w = hi;
        cand[p].w2 = hi;
        cand[p].wl = float(v - double(hi));
    }
}

__global__ void k_bin_points(const float2* __restrict__ pts, long M, const GridInst* __restrict__ inst,
                             int set, int field9, uint32_t* __restrict__ qbin, uint32_t* __restrict__ qcount) {
    for (long m = long(blockIdx.x) * blockDim.x + threadIdx.x; m < M; m += long(gridDim.x) * blockDim.x) {
        const GridInst G = inst[0];
        float2 p = pts[m];
        uint32_t b = kNoBin;
        bool ok = p.x == p.x && p.y == p.y;
        if (ok && G.periodic) {
            const float kx = floorf(p.x / G.Lx), ky = floorf(p.y / G.Ly);
            if (field9 && (fabsf(kx) > 2.f || fabsf(ky) > 2.f)) ok = false;
            p.x = p.x - kx * G.Lx;
            p.y = p.y - ky * G.Ly;
        } else if (ok) {
            ok = !(p.x < 0.f || p.x > G.Lx || p.y < 0.f || p.y > G.Ly);
        }
        if (ok) {
            const int cx = min(max(floor_int(p.x * G.inv_sx), 0), G.gx - 1);
            const int cy = min(max(floor_int(p.y * G.inv_sy), 0), G.gy - 1);
            b = uint32_t(G.bin_base) + uint32_t(set) * uint32_t(G.gx * G.gy) + uint32_t(cx * G.gy + cy);
            atomicAdd(&qcount[b], 1u);
        }
        qbin[m] = b;
    }
}

__global__ void k_scatter_points(const float2* __restrict__ pts, long M, const GridInst* __restrict__ inst,
                                 int n_inst, const uint32_t* __restrict__ qbin, const uint32_t* __restrict__ qstart,
                                 uint32_t* __restrict__ qfill, QRec* __restrict__ qrec) {
    for (long m = long(blockIdx.x) * blockDim.x + threadIdx.x; m < M; m += long(gridDim.x) * blockDim.x) {
        const uint32_t b = qbin[m];
        if (b == kNoBin) continue;
        const GridInst G = inst[inst_of_bin(inst, n_inst, b)];
        float2 p = pts[m];
        uint32_t fl = (2u) | (2u << 3);
        if (G.periodic) {
            const float kx = floorf(p.x / G.Lx), ky = floorf(p.y / G.Ly);
            p.x = p.x - kx * G.Lx;
            p.y = p.y - ky * G.Ly;
            const int ikx = min(max(int(kx), -2), 2), iky = min(max(int(ky), -2), 2);
            fl = uint32_t(ikx + 2) | (uint32_t(iky + 2) << 3);
        }
        const uint32_t slot = atomicAdd(&qfill[b], 1u);
        qrec[qstart[b] + slot] = QRec{p.x, p.y, uint32_t(m), fl};
    }
}

// Scatter with precomputed in-bin ranks: slot = qstart[bin] + rank.
__global__ void k_scatter_ranked(const float2* __restrict__ pts, long M, const GridInst* __restrict__ inst,
                                 int n_inst, const uint32_t* __restrict__ qbin, const uint32_t* __restrict__ qrank,
                                 const uint32_t* __restrict__ qstart, QRec* __restrict__ qrec) {
    for (long m = long(blockIdx.x) * blockDim.x + threadIdx.x; m < M; m += long(gridDim.x) * blockDim.x) {
        const uint32_t b = qbin[m];
        if (b == kNoBin) continue;
        const GridInst& G = inst[inst_of_bin(inst, n_inst, b)];
        float2 p = pts[m];
        uint32_t fl = (2u) | (2u << 3);
        if (G.periodic) {
            const float kx = floorf(p.x / G.Lx), ky = floorf(p.y / G.Ly);
            p.x = p.x - kx * G.Lx;
            p.y = p.y - ky * G.Ly;
            const int ikx = min(max(int(kx), -2), 2), iky = min(max(int(ky), -2), 2);
            fl = uint32_t(ikx + 2) | (uint32_t(iky + 2) << 3);
        }
        qrec[qstart[b] + qrank[m]] = QRec{p.x, p.y, uint32_t(m), fl};
    }
}

// Placement of binned samples (three streaming passes).  Writing a 16-byte
// record straight to its final slot touches a different DRAM sector per
// sample (the bins of consecutive samples are unrelated).  Instead:
//   pass 1 (k_scatter_coarse): each CTA moves its tile of samples into runs
//     per super-bin (2^S consecutive bins; one global atomic per CTA and
//     super-bin) as {unwrapped point, sample id, bin};
//   pass 2 (k_scatter_window): the super-bin segments into runs per window
//     (2^W consecutive bins, ~1-2k samples), placed at the window's first
//     slot qstart[w << W];
//   pass 3 (k_scatter_assemble): one CTA per window gives every record its
//     slot from shared-memory counters started at qstart of its bin, builds
//     the window in shared memory (wrapping the point, deriving its image
//     flags) and writes it out as one contiguous block.
// The order of queries inside a bin is not fixed by this; no result depends
// on it (each query's field value is its own fixed-order sum).
constexpr int kPlaceThreads = 512;
constexpr int kPlaceTile = 8;                                // records per thread per tile
constexpr int kTileRecs = kPlaceThreads * kPlaceTile;        // 4096 records = 64 KB staged per tile
constexpr int kTargetSuper = 512;                            // super-bins per grid
constexpr int kWinMax = 2048;                                // windows one tile may sort in shared memory
constexpr int kWinCap = 4096;                                // records a window assembles in shared memory
constexpr int kAsmThreads = 512;                             // window assembly: 2 CTAs per SM
constexpr int kWinBinsMax = 256;                             // bins per window at most

// Exclusive prefix sum of v[0..n) in place (shared memory, n small), block
// of kPlaceThreads; returns the total.
__device__ __forceinline__ uint32_t block_scan_excl(uint32_t* v, int n, uint32_t* s_warp) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int per = (n + kPlaceThreads - 1) / kPlaceThreads;
    const int b = min(n, tid * per), e = min(n, b + per);
    uint32_t sum = 0;
    for (int i = b; i < e; ++i) sum += v[i];
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < kPlaceThreads / 32 ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kPlaceThreads / 32) s_warp[lane] = t;
    }
    __syncthreads();
    uint32_t run = (x - sum) + (wid > 0 ? s_warp[wid - 1] : 0u);
    for (int i = b; i < e; ++i) {
        const uint32_t c = v[i];
        v[i] = run;
        run += c;
    }
    const uint32_t total = s_warp[kPlaceThreads / 32 - 1];
    __syncthreads();
    return total;
}

// Pass 1: each tile of samples counting-sorted by super-bin in shared memory,
// one global reservation per (tile, super-bin), then written out as
// contiguous runs (coalesced stores).
__global__ void __launch_bounds__(kPlaceThreads) k_scatter_coarse(const float2* __restrict__ pts, long M,
                                                                 const uint32_t* __restrict__ qbin,
                                                                 const uint32_t* __restrict__ qstart, int shift,
                                                                 int nsuper, uint32_t* __restrict__ super_fill,
                                                                 uint4* __restrict__ tmp) {
    extern __shared__ __align__(16) uint4 srec[];   // kTileRecs
    __shared__ uint32_t hist[kTargetSuper], loff[kTargetSuper], s_warp[32];
    __shared__ long long goff[kTargetSuper];
    // the tile's bins and points are loaded one tile ahead (while the previous
    // tile is written out)
    uint32_t bb[kPlaceTile], lr[kPlaceTile];
    float2 pp[kPlaceTile];
    auto load_tile = [&](long t) {
#pragma unroll
        for (int j = 0; j < kPlaceTile; ++j) {
            const long m = t + long(j) * kPlaceThreads + threadIdx.x;
            bb[j] = m < M ? qbin[m] : kNoBin;
            pp[j] = m < M ? pts[m] : make_float2(0.f, 0.f);   // unwrapped: pass 3 wraps it
        }
    };
    long t0 = long(blockIdx.x) * kTileRecs;
    if (t0 >= M) return;
    load_tile(t0);
    for (;;) {
        for (int k = threadIdx.x; k < nsuper; k += kPlaceThreads) hist[k] = 0u;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kPlaceTile; ++j)
            if (bb[j] != kNoBin) lr[j] = atomicAdd(&hist[bb[j] >> shift], 1u);
        __syncthreads();
        for (int k = threadIdx.x; k < nsuper; k += kPlaceThreads) loff[k] = hist[k];
        __syncthreads();
        const uint32_t ntile = block_scan_excl(loff, nsuper, s_warp);
        for (int k = threadIdx.x; k < nsuper; k += kPlaceThreads) {
            const uint32_t c = hist[k];
            goff[k] = c ? (long long)(qstart[uint32_t(k) << shift] + atomicAdd(&super_fill[k], c)) - loff[k] : 0;
        }
#pragma unroll
        for (int j = 0; j < kPlaceTile; ++j) {
            if (bb[j] == kNoBin) continue;
            const long m = t0 + long(j) * kPlaceThreads + threadIdx.x;
            srec[loff[bb[j] >> shift] + lr[j]] = make_uint4(__float_as_uint(pp[j].x), __float_as_uint(pp[j].y),
                                                            uint32_t(m), bb[j]);
        }
        __syncthreads();
        const long tn = t0 + long(gridDim.x) * kTileRecs;
        if (tn < M) load_tile(tn);
        for (uint32_t i = threadIdx.x; i < ntile; i += kPlaceThreads) {
            const uint4 r = srec[i];
            tmp[goff[r.w >> shift] + i] = r;
        }
        __syncthreads();
        if (tn >= M) break;
        t0 = tn;
    }
}

// Query record of a placed sample: wrapped point and image flags.
__device__ __forceinline__ QRec make_qrec(uint4 r, const GridInst* __restrict__ inst, int n_inst) {
    const GridInst& G = inst[n_inst == 1 ? 0 : inst_of_bin(inst, n_inst, r.w)];
    float2 p = make_float2(__uint_as_float(r.x), __uint_as_float(r.y));
    uint32_t fl = (2u) | (2u << 3);
    if (G.periodic) {
        const float kx = floorf(p.x / G.Lx), ky = floorf(p.y / G.Ly);
        p.x = p.x - kx * G.Lx;
        p.y = p.y - ky * G.Ly;
        const int ikx = min(max(int(kx), -2), 2), iky = min(max(int(ky), -2), 2);
        fl = uint32_t(ikx + 2) | (uint32_t(iky + 2) << 3);
    }
    return QRec{p.x, p.y, r.z, fl};
}

// Sub-cell of a query (wrapped point p in the cell of its bin): 4 x 4
// sub-cells in serpentine order (rows of sub-cells, alternate rows reversed),
// so that any run of consecutive keys covers a compact part of the cell.
// c = {cx, cy, gx / Lx, gy / Ly} of the bin's cell.
constexpr int kSubCells = 16;
__device__ __forceinline__ uint32_t subcell_key(float px, float py, float4 c) {
    const int ix = min(max(int((px * c.z - c.x) * 4.f), 0), 3);
    const int iy = min(max(int((py * c.w - c.y) * 4.f), 0), 3);
    return uint32_t(iy * 4 + ((iy & 1) ? 3 - ix : ix));
}

// Pass 2: the same per tile of the super-bin-grouped records, by window
// (2^W consecutive bins), placed from the window's first slot qstart[w << W].
// A tile spanning more windows than the shared-memory counters hold (one
// across many sparse super-bins) reserves per record instead.
__global__ void __launch_bounds__(kPlaceThreads) k_scatter_window(const uint4* __restrict__ tmp,
                                                                 const uint32_t* __restrict__ total, long M,
                                                                 int wshift, const uint32_t* __restrict__ qstart,
                                                                 uint32_t* __restrict__ win_fill,
                                                                 uint4* __restrict__ tmp2) {
    extern __shared__ __align__(16) uint4 srec[];   // kTileRecs
    __shared__ uint32_t hist[kWinMax], loff[kWinMax], s_warp[32];
    __shared__ long long goff[kWinMax];
    __shared__ uint32_t s_lo, s_hi;
    const long n = min(long(*total), M);
    // records loaded one tile ahead (while the previous tile is written out)
    uint4 r[kPlaceTile];
    auto load_tile = [&](long t) {
#pragma unroll
        for (int j = 0; j < kPlaceTile; ++j) {
            const long i = t + long(j) * kPlaceThreads + threadIdx.x;
            r[j] = i < n ? tmp[i] : make_uint4(0u, 0u, 0u, kNoBin);
        }
    };
    long t0 = long(blockIdx.x) * kTileRecs;
    if (t0 >= n) return;
    if (threadIdx.x == 0) { s_lo = 0xffffffffu; s_hi = 0u; }
    load_tile(t0);
    __syncthreads();
    for (;;) {
        uint32_t lo = 0xffffffffu, hi = 0u;
#pragma unroll
        for (int j = 0; j < kPlaceTile; ++j)
            if (r[j].w != kNoBin) { lo = min(lo, r[j].w >> wshift); hi = max(hi, r[j].w >> wshift); }
        atomicMin(&s_lo, lo);
        atomicMax(&s_hi, hi);
        __syncthreads();
        const uint32_t wlo = s_lo, span = s_hi >= s_lo ? s_hi - s_lo + 1u : 0u;
        const long tn = t0 + long(gridDim.x) * kTileRecs;
        if (span > uint32_t(kWinMax)) {
#pragma unroll
            for (int j = 0; j < kPlaceTile; ++j) {
                if (r[j].w == kNoBin) continue;
                const uint32_t w = r[j].w >> wshift;
                tmp2[qstart[w << wshift] + atomicAdd(&win_fill[w], 1u)] = r[j];
            }
            __syncthreads();
            if (threadIdx.x == 0) { s_lo = 0xffffffffu; s_hi = 0u; }
            if (tn < n) load_tile(tn);
            __syncthreads();
            if (tn >= n) break;
            t0 = tn;
            continue;
        }
        for (uint32_t k = threadIdx.x; k < span; k += kPlaceThreads) hist[k] = 0u;
        __syncthreads();
        uint32_t lr[kPlaceTile];
#pragma unroll
        for (int j = 0; j < kPlaceTile; ++j)
            if (r[j].w != kNoBin) lr[j] = atomicAdd(&hist[(r[j].w >> wshift) - wlo], 1u);
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < span; k += kPlaceThreads) loff[k] = hist[k];
        __syncthreads();
        const uint32_t ntile = block_scan_excl(loff, int(span), s_warp);
        for (uint32_t k = threadIdx.x; k < span; k += kPlaceThreads) {
            const uint32_t c = hist[k];
            goff[k] = c ? (long long)(qstart[(wlo + k) << wshift] + atomicAdd(&win_fill[wlo + k], c)) - loff[k] : 0;
        }
#pragma unroll
        for (int j = 0; j < kPlaceTile; ++j)
            if (r[j].w != kNoBin) srec[loff[(r[j].w >> wshift) - wlo] + lr[j]] = r[j];
        __syncthreads();
        if (threadIdx.x == 0) { s_lo = 0xffffffffu; s_hi = 0u; }
        if (tn < n) load_tile(tn);
        for (uint32_t i = threadIdx.x; i < ntile; i += kPlaceThreads) {
            const uint4 q = srec[i];
            tmp2[goff[(q.w >> wshift) - wlo] + i] = q;
        }
        __syncthreads();
        if (tn >= n) break;
        t0 = tn;
    }
}

// Pass 3: one window per CTA: every record gets its slot from shared-memory
// counters started at qstart of its bin, the window is built in shared memory
// and written out as one contiguous block (an over-full window stores
// directly).
__global__ void __launch_bounds__(kAsmThreads, 2) k_scatter_assemble(const uint4* __restrict__ tmp2, long nbins, int wshift,
                                                            const uint32_t* __restrict__ qstart,
                                                            const GridInst* __restrict__ inst, int n_inst,
                                                            QRec* __restrict__ qrec) {
    constexpr int kPer = kWinCap / kAsmThreads;     // records per thread of a window that fits
    extern __shared__ __align__(16) QRec buf[];   // kWinCap records
    __shared__ uint32_t cnt[kWinBinsMax];
    __shared__ uint32_t sub[kSubCells * kWinBinsMax];   // per (sub-cell, bin of the window): count, then first slot
    __shared__ float4 corg[kWinBinsMax];                 // per bin of the window: its cell, for subcell_key
    const long nwin = ((nbins - 1) >> wshift) + 1;
    long w = blockIdx.x;
    if (w >= nwin) return;
    // window w's bounds and (when it fits) its records: loaded one window ahead,
    // so the loads overlap the previous window's write-out
    long b0 = w << wshift, b1 = min(nbins, b0 + (1L << wshift));
    uint32_t start = qstart[b0], nw = qstart[b1] - start;
    uint4 r[kPer];
    auto load_records = [&](uint32_t st, uint32_t n) {
        if (n > uint32_t(kWinCap)) return;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t k = threadIdx.x + uint32_t(j) * uint32_t(kAsmThreads);
            r[j] = k < n ? tmp2[st + k] : make_uint4(0u, 0u, 0u, 0u);
        }
    };
    load_records(start, nw);
    for (;;) {
        const bool fits = nw <= uint32_t(kWinCap);
        const uint32_t nb = uint32_t(b1 - b0);
        for (long b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
            cnt[b - b0] = qstart[b];
            const GridInst& G = inst[n_inst == 1 ? 0 : inst_of_bin(inst, n_inst, uint32_t(b))];
            const uint32_t cell = (uint32_t(b) - uint32_t(G.bin_base)) % uint32_t(G.gx * G.gy);
            corg[b - b0] = make_float4(float(int(cell) / G.gy), float(int(cell) % G.gy), G.inv_sx, G.inv_sy);
        }
        for (uint32_t i = threadIdx.x; i < uint32_t(kSubCells) * nb; i += blockDim.x) sub[i] = 0u;
        __syncthreads();
        if (fits) {
            // inside each bin the records are ordered by sub-cell, so that
            // consecutive queries of a bin lie close together
            uint32_t kr[kPer];   // bin in the window | sub-cell << 8 | rank within (sub-cell, bin) << 12
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const uint32_t k = threadIdx.x + uint32_t(j) * uint32_t(kAsmThreads);
                if (k >= nw) break;
                const uint32_t bl = r[j].w - uint32_t(b0);
                const QRec q = make_qrec(r[j], inst, n_inst);
                const uint32_t key = subcell_key(q.x, q.y, corg[bl]);
                kr[j] = bl | (key << 8) | (atomicAdd(&sub[key * nb + bl], 1u) << 12);
                r[j] = make_uint4(__float_as_uint(q.x), __float_as_uint(q.y), q.id, q.flags);
            }
            __syncthreads();
            // each bin's 16 sub-cell counters -> first slots, by warp 0: two bins
            // per pass, one counter per lane, a scan inside each 16-lane half
            if (threadIdx.x < 32) {
                const uint32_t lane = threadIdx.x, c = lane & 15u;
                for (uint32_t b = lane >> 4; b < ((nb + 1u) & ~1u); b += 2u) {
                    const bool live = b < nb;
                    const uint32_t n = live ? sub[c * nb + b] : 0u;
                    uint32_t incl = n;
#pragma unroll
                    for (int o = 1; o < 16; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o, 16);
                        if (c >= uint32_t(o)) incl += y;
                    }
                    if (live) sub[c * nb + b] = cnt[b] + incl - n;
                }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const uint32_t k = threadIdx.x + uint32_t(j) * uint32_t(kAsmThreads);
                if (k >= nw) break;
                const uint32_t slot = sub[((kr[j] >> 8) & 15u) * nb + (kr[j] & 255u)] + (kr[j] >> 12);
                buf[slot - start] = QRec{__uint_as_float(r[j].x), __uint_as_float(r[j].y), r[j].z, r[j].w};
            }
        } else {
            for (uint32_t k = threadIdx.x; k < nw; k += blockDim.x) {
                const uint4 rr = tmp2[start + k];
                const uint32_t slot = atomicAdd(&cnt[rr.w - uint32_t(b0)], 1u);
                qrec[slot] = make_qrec(rr, inst, n_inst);
            }
        }
        __syncthreads();
        // the next window's bounds and records go out before this one is written
        const long wn = w + gridDim.x;
        long nb0 = 0, nb1 = 0;
        uint32_t nstart = 0, nnw = 0;
        if (wn < nwin) {
            nb0 = wn << wshift;
            nb1 = min(nbins, nb0 + (1L << wshift));
            nstart = qstart[nb0];
            nnw = qstart[nb1] - nstart;
            load_records(nstart, nnw);
        }
        if (fits)
            for (uint32_t k = threadIdx.x; k < nw; k += blockDim.x) qrec[start + k] = buf[k];
        __syncthreads();
        if (wn >= nwin) break;
        w = wn;
        b0 = nb0;
        b1 = nb1;
        start = nstart;
        nw = nnw;
    }
}

__global__ void k_items_count(const uint32_t* __restrict__ qstart, long nbins, int chunk,
                              uint32_t* __restrict__ per_bin) {
    for (long b = long(blockIdx.x) * blockDim.x + threadIdx.x; b < nbins; b += long(gridDim.x) * blockDim.x) {
        const uint32_t c = qstart[b + 1] - qstart[b];
        per_bin[b] = (c + chunk - 1) / chunk;
    }
}

__global__ void k_items_fill(const uint32_t* __restrict__ qstart, long nbins, int chunk,
                             const uint32_t* __restrict__ item_start, const GridInst* __restrict__ inst,
                             int n_inst, Item* __restrict__ items, uint32_t* __restrict__ n_items,
                             uint32_t* __restrict__ counter, long max_items) {
    for (long b = long(blockIdx.x) * blockDim.x + threadIdx.x; b < nbins; b += long(gridDim.x) * blockDim.x) {
        const uint32_t q0 = qstart[b], c = qstart[b + 1] - q0;
        uint32_t it = item_start[b];
        const uint32_t ib = uint32_t(inst_of_bin(inst, n_inst, uint32_t(b)));
        for (uint32_t o = 0; o < c; o += chunk, ++it)
            if (it < max_items) items[it] = Item{uint32_t(b), q0 + o, min(uint32_t(chunk), c - o), ib};
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint32_t t = item_start[nbins];
        *n_items = t < max_items ? t : uint32_t(max_items);
        *counter = 0;
    }
}

// ---------------------------------------------------------------- eval kernel
struct Piece {
    uint32_t gstart, cnt;   // candidate run in global memory
    float qdx, qdy;         // offset added to the query point (folds the periodic image)
    uint32_t b0;            // index into the sub-row starts of the run's first sub-row
    float x0, y0;           // bin-local left edge of the run's column, lower edge of its first sub-row
    int16_t nr;             // sub-rows in the run
    int8_t mx, my;          // image index of the run (for FIELD9)
};
struct BatchPiece {
    uint32_t soff, cnt, gstart;
    int piece;
};

struct EvalArgs {
    const GridInst* inst;
    const uint32_t* cstart;   // candidate range per sub-row (rows per cell: `rows`)
    int rows;
    const Cand* cand;
    const CandF* candf;
    const QRec* qrec;
    const Item* items;
    const uint32_t* n_items;
    uint32_t* counter;
    float* out_f32;
    double* out_f64;
    unsigned* flags;
    uint32_t wait_limit;      // polls of a staging wait before the kernel gives up
    const double* qweight;    // SCAT modes: the weight of each query (by id)
};

// Sum over one staged run of candidates for NPR packed query pairs, in
// bin-local coordinates, every squared distance pre-scaled by kappa = -3/h^2:
// candidates hold (x, y) relative to the bin centre and kappa c2; queries
// enter as -2 kappa q and kappa |q|^2, so
//   s2 = kappa c2 + kappa q2 - 2 kappa c.q = -3 (r/h)^2,   sqrt(|s2|) = sqrt(3) r/h
//   t  = saturate(1 - sqrt(|s2|)/sqrt(3))                  (= max(1 - r/h, 0))
//   P += w * min(0.5 + s2 t, t^3)                          (= w W / 2 sigma)
// because the spline's inner branch 1/2 - 3 q^2 + 3 q^3 is 1/2 - 3 q^2 (1 - q),
// and beyond the support t = 0 leaves min(1/2, 0) = 0.
// Per pair of queries: 7 packed FMA-pipe operations + 2 saturating scalar FMAs,
// 2 square roots on the XU and 2 min on the ALU.  The candidate loop is unrolled
// eight times (independent chains across candidates, 80 registers; at tg2048
// 257.7 ms per evaluation against 261.1 unrolled four times, 274.4 twice,
// 272.5 twelve times, 258.4 sixteen times).
template <int NPR, int NPMAX>
__device__ __forceinline__ void packed_run(const Cand* __restrict__ cs, int cnt, const f2x (&QX)[NPMAX],
                                           const f2x (&QY)[NPMAX], const f2x (&Q2)[NPMAX], f2x (&P)[NPMAX]) {
    const f2x HALF = pk2(0.5f, 0.5f);
#pragma unroll 8
    for (int c = 0; c < cnt; ++c) {
        const ulonglong2 XY = *reinterpret_cast<const ulonglong2*>(&cs[c].x);
        const ulonglong2 WC = *reinterpret_cast<const ulonglong2*>(&cs[c].w);   // (w, w), (kappa c2, kappa c2)
#pragma unroll
        for (int pr = 0; pr < NPR; ++pr) {
            const f2x s = add2(WC.y, Q2[pr]);
            const f2x s2 = fma2(XY.y, QY[pr], fma2(XY.x, QX[pr], s));
            float ra, rb;
            up2(s2, ra, rb);
            // rounding can leave s2 a hair above 0 when c ~ q: take sqrt(|s2|)
            const float sa = sqrt_approx(fabsf(ra)), sb = sqrt_approx(fabsf(rb));
            const f2x t = pk2(__saturatef(fmaf(-kInvSqrt3, sa, 1.f)), __saturatef(fmaf(-kInvSqrt3, sb, 1.f)));
            const f2x in = fma2(s2, t, HALF);
            const f2x t3 = mul2(mul2(t, t), t);
            float ia, ib, ta, tb;
            up2(in, ia, ib);
            up2(t3, ta, tb);
            P[pr] = fma2(WC.x, pk2(fminf(ia, ta), fminf(ib, tb)), P[pr]);
        }
    }
}

// The same sum for deformed kernels: s2 from the expanded metric form, its
// coefficients pre-scaled by kappa (5 packed FMAs instead of 3), the spline as above.
template <int NPR, int NPMAX>
__device__ __forceinline__ void packed_run_f(const CandF* __restrict__ cs, int cnt, const f2x (&QXX)[NPMAX],
                                             const f2x (&QXY)[NPMAX], const f2x (&QYY)[NPMAX],
                                             const f2x (&QX)[NPMAX], const f2x (&QY)[NPMAX], f2x (&P)[NPMAX]) {
    const f2x HALF = pk2(0.5f, 0.5f);
#pragma unroll 2
    for (int c = 0; c < cnt; ++c) {
        const ulonglong2* rec = reinterpret_cast<const ulonglong2*>(cs[c].f);
        const ulonglong2 R0 = rec[0];   // kappa (g11), kappa (2 g12)
        const ulonglong2 R1 = rec[1];   // kappa (g22), kappa (a)
        const ulonglong2 R2 = rec[2];   // kappa (b), kappa (e)
        const ulonglong2 R3 = rec[3];   // (w), (0)
#pragma unroll
        for (int pr = 0; pr < NPR; ++pr) {
            f2x s2 = fma2(R0.x, QXX[pr], R2.y);
            s2 = fma2(R0.y, QXY[pr], s2);
            s2 = fma2(R1.x, QYY[pr], s2);
            s2 = fma2(R1.y, QX[pr], s2);
            s2 = fma2(R2.x, QY[pr], s2);
            float ra, rb;
            up2(s2, ra, rb);
            const float sa = sqrt_approx(fabsf(ra)), sb = sqrt_approx(fabsf(rb));
            const f2x t = pk2(__saturatef(fmaf(-kInvSqrt3, sa, 1.f)), __saturatef(fmaf(-kInvSqrt3, sb, 1.f)));
            const f2x in = fma2(s2, t, HALF);
            const f2x t3 = mul2(mul2(t, t), t);
            float ia, ib, ta, tb;
            up2(in, ia, ib);
            up2(t3, ta, tb);
            P[pr] = fma2(R3.x, pk2(fminf(ia, ta), fminf(ib, tb)), P[pr]);
        }
    }
}

// s + e += x with s the running sum and e the running sum of its rounding errors
// (Knuth's TwoSum; the products are formed with __fmul_rn so no FMA contraction
// can fold them into the sum and break the exact error term).
__device__ __forceinline__ void two_sum_acc(float& s, float& e, float x) {
    const float t = __fadd_rn(s, x);
    const float bp = __fsub_rn(t, s);
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp)));
    s = t;
}

// W / 2 sigma of the cubic spline and its r-derivative over r, for FP32 pairs
// without a branch: one reciprocal square root gives r and 1/r, the inner and
// outer pieces are selected, and beyond the support t = (1 - r/h)+ = 0 makes
// both exactly zero (r > h/2 there).  r2 is floored at 1e-30, where the inner
// piece gives v = 1/2 and a zero gradient term (dx = dy = 0).
__device__ __forceinline__ void spline_vdr_f32(float r2, float hw, float ih, float A, float B, float& v, float& dr) {
    r2 = fmaxf(r2, 1e-30f);
    const float rs = rsqrtf(r2);
    const float r = r2 * rs;
    const float t = fmaxf(fmaf(-ih, r, 1.f), 0.f);
    const bool inner = r <= 0.5f * hw;
    v = inner ? fmaf(r2, fmaf(A, r, B), 0.5f) : t * t * t;
    dr = inner ? fmaf(3.f * A, r, 2.f * B) : -3.f * ih * (t * t) * rs;
}

// Images a sample may pair through (unbiased law): bit (sx + 1) * 3 + (sy + 1)
// is set when a run shifted by image (sx, sy) pairs the sample in unwrapped tile
// k with source image k + s inside {-1, 0, 1}^2 (flags: bits 0-2 kx + 2, 3-5 ky + 2).
__device__ __forceinline__ uint32_t image_mask9(uint32_t flags) {
    const int kx = int(flags & 7u) - 2, ky = int((flags >> 3) & 7u) - 2;
    uint32_t m = 0u;
#pragma unroll
    for (int sx = -1; sx <= 1; ++sx)
#pragma unroll
        for (int sy = -1; sy <= 1; ++sy)
            if (kx + sx >= -1 && kx + sx <= 1 && ky + sy >= -1 && ky + sy <= 1) m |= 1u << ((sx + 1) * 3 + (sy + 1));
    return m;
}

// The transposed sums of one staged batch, from the sample side (SCAT modes).
// The item's samples sit in s_sq (x, y, weight hi, weight lo; image masks in
// s_sqm); the batch's particles are staged back to back in s_cand.  Lane l
// takes staged particles l, l + 32, ... (whatever run each lies in), sums over
// all the item's samples the terms a_s W(|x_p - y_s|) and a_s dW/dx_p in the
// pair's image, and adds them to out[3 slot + {0, 1, 2}] with one FP64 atomic
// each, slot = the particle's candidate index.  The pair is the one the GRAD
// modes form with the roles of query and candidate swapped: the sample seen
// through the run's image is y + qdx, so x_p - y_s = (c - qdx) - q.
template <typename ST, bool K9>
__device__ __forceinline__ void scat_batch(const Cand* __restrict__ s_cand, const BatchPiece* s_bp,
                                           const Piece* s_pc, int nbp, uint32_t btot, const float4* s_sq,
                                           const uint16_t* s_sqm, int nq, const GridInst& G,
                                           double* __restrict__ out) {
    constexpr bool k32 = std::is_same<ST, float>::value;
    const int lane = threadIdx.x & 31;
    const ST hw = ST(G.hw), ih = ST(1) / hw;
    const ST A = ST(3) * ih * ih * ih, B = ST(-3) * ih * ih;
    int b = 0;
    for (uint32_t i = uint32_t(lane); i < btot; i += 32u) {
        while (b + 1 < nbp && s_bp[b + 1].soff <= i) ++b;
        const BatchPiece bp = s_bp[b];
        const Piece pc = s_pc[bp.piece];
        const Cand cv = s_cand[i];
        const uint32_t pbit = uint32_t((pc.mx + 1) * 3 + (pc.my + 1));
        const ST cx = ST(cv.x) - ST(pc.qdx), cy = ST(cv.y) - ST(pc.qdy);
        ST sv = ST(0), sgx = ST(0), sgy = ST(0);
        float ev = 0.f, egx = 0.f, egy = 0.f;   // FP32 pairs: the sums' error terms
        if constexpr (k32) {
            // branch-free: a pair outside the support or the sample's images adds
            // exact zeros, which leave the compensated sums unchanged
            for (int j = 0; j < nq; ++j) {
                const float4 q = s_sq[j];
                float w = q.z;
                if (K9) w = ((uint32_t(s_sqm[j]) >> pbit) & 1u) ? w : 0.f;
                const float dx = cx - q.x, dy = cy - q.y;   // x_p - y_s
                float v, dr;
                spline_vdr_f32(fmaf(dx, dx, dy * dy), hw, ih, A, B, v, dr);
                const float wdr = __fmul_rn(w, dr);
                two_sum_acc(sv, ev, __fmul_rn(w, v));
                two_sum_acc(sgx, egx, __fmul_rn(wdr, dx));
                two_sum_acc(sgy, egy, __fmul_rn(wdr, dy));
            }
        } else {
            for (int j = 0; j < nq; ++j) {
                if (K9 && !((uint32_t(s_sqm[j]) >> pbit) & 1u)) continue;
                const float4 q = s_sq[j];
                const double dx = cx - double(q.x), dy = cy - double(q.y);   // x_p - y_s
                const double r2 = dx * dx + dy * dy;
                const double r = sqrt(r2);
                if (r >= hw) continue;
                const double t = 1.0 - ih * r;
                double v, dr;   // W / 2 sigma and its r-derivative over r
                if (r <= 0.5 * hw) {
                    v = 0.5 + r2 * (A * r + B);
                    dr = 3.0 * A * r + 2.0 * B;
                } else {
                    v = t * t * t;
                    dr = -3.0 * t * t * ih / r;
                }
                const double w = double(q.z) + double(q.w);
                sv += w * v;
                sgx += w * dr * dx;
                sgy += w * dr * dy;
            }
        }
        const double gv = double(sv) + double(ev), ggx = double(sgx) + double(egx), ggy = double(sgy) + double(egy);
        if (gv != 0.0 || ggx != 0.0 || ggy != 0.0) {
            double* o = out + 3 * (size_t(bp.gstart) + size_t(i - bp.soff));
            atomicAdd(o, gv);
            atomicAdd(o + 1, ggx);
            atomicAdd(o + 2, ggy);
        }
    }
}

// The packed FP32 kernels run one-warp CTAs, 24 per SM (their 6.5 KB staging
// buffers fit 24 times in shared memory; 85 registers a thread at most) with 4
// queries per thread, 16 per SM with 6 and 12 with 8.  One warp per CTA: no warp of an item
// waits at a barrier for another.
constexpr int eval_min_blocks(int mode, int qpt) {
    return (mode == EVAL_FIELD || mode == EVAL_FIELD9 || mode == EVAL_FIELD_F || mode == EVAL_FIELD9_F)
               ? (qpt == 4 ? 24 : qpt == 6 ? 16 : 12) : 1;
}

template <int MODE, int QPT>
__global__ void __launch_bounds__(kEvalThreads, eval_min_blocks(MODE, QPT)) k_eval(EvalArgs a) {
    extern __shared__ __align__(128) Cand s_cand[];
    __shared__ Piece s_pc[kMaxPieces];
    __shared__ BatchPiece s_bp[kMaxPieces + 2];
    __shared__ uint2 s_rng[kEvalThreads / 32][kMaxPieces + 2];   // per warp: its part of each batch piece
    __shared__ float4 s_wb[kEvalThreads / 32];                    // per warp: query bounding box (x0, x1, y0, y1)
    __shared__ int s_np, s_nbp, s_cur_piece, s_abort, s_pre;
    __shared__ uint32_t s_cur_off, s_btot, s_item;
    __shared__ float s_ox, s_oy;
    __shared__ __align__(8) uint64_t s_bar;
    constexpr bool kScat = eval_scat(MODE);
    constexpr int kScatQ = kScat ? kEvalThreads * QPT : 1;   // an item's queries (make_items' chunk)
    __shared__ float4 s_sq[kScatQ];
    __shared__ uint16_t s_sqm[kScatQ];

    constexpr bool kF64 = MODE == EVAL_SPMV64;
    constexpr bool kComp = MODE == EVAL_SPMV32;
    constexpr bool kField64 = MODE == EVAL_FIELD64 || MODE == EVAL_FIELD9_64;
    constexpr bool kGrad = eval_grad(MODE);
    constexpr bool kGrad32 = MODE == EVAL_GRAD32 || MODE == EVAL_GRAD9_32;
    constexpr bool kGrad9 = MODE == EVAL_GRAD9_64 || MODE == EVAL_GRAD9_32;
    constexpr bool kScat9 = MODE == EVAL_SCAT9_64 || MODE == EVAL_SCAT9_32;
    using ST = typename std::conditional<MODE == EVAL_SCAT32 || MODE == EVAL_SCAT9_32, float, double>::type;
    using GT = typename std::conditional<kGrad32, float, double>::type;
    constexpr bool kDef = eval_deformed(MODE);
    constexpr bool kDefExc = MODE == EVAL_FIELD_F_EXC;
    constexpr bool kPacked = MODE == EVAL_FIELD || MODE == EVAL_FIELD9 || MODE == EVAL_FIELD_F || MODE == EVAL_FIELD9_F;
    constexpr bool kField9 = MODE == EVAL_FIELD9 || MODE == EVAL_FIELD9_64 || MODE == EVAL_FIELD9_F;
    constexpr uint32_t kRec = kDef ? uint32_t(sizeof(CandF)) : uint32_t(sizeof(Cand));
    constexpr int kCap = kDef ? kCandCap / 2 : kCandCap;   // records per staged batch
    CandF* const s_candf = reinterpret_cast<CandF*>(s_cand);
    constexpr int NP = QPT / 2;   // packed query pairs
    static_assert(!kPacked || (QPT % 2 == 0), "packed path needs an even query count");
    using Acc = typename std::conditional<kF64 || kField64 || kGrad, double, float>::type;

    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&s_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
        s_item = atomicAdd(a.counter, 1u);
    }
    __syncthreads();
    uint32_t phase = 0;

    for (;;) {
        const uint32_t item = s_item;
        if (item >= *a.n_items) break;
        // claim the next item now: the atomic's round trip hides behind this one
        uint32_t next_item = 0;
        if (tid == 0) next_item = atomicAdd(a.counter, 1u);
        const Item it = a.items[item];
        const GridInst G = a.inst[it.inst];
        // the item's queries form units of 64 (one packed pair per lane); the warps
        // take consecutive units, as evenly as the count allows (a partly filled
        // item leaves no warp idle while another holds two units more), and a
        // warp runs only the pairs it holds: npw = its units (warp-uniform)
        constexpr int kWarps = kEvalThreads / 32;
        const int nunits = (int(it.qcnt) + 63) >> 6;   // <= kWarps * QPT / 2
        const int u0 = ((tid >> 5) * nunits) / kWarps;
        const int npw = (((tid >> 5) + 1) * nunits) / kWarps - u0;

        if (tid < 32) {
            // the walk, one column per lane of warp 0 (2 k + 1 <= 17 columns): each
            // column gives up to two runs (a periodic column wrapping in y splits),
            // emitted in column order as a serial walk would
            const int lane = tid;
            const uint32_t local = it.bin - uint32_t(G.bin_base);
            const uint32_t ncell = uint32_t(G.gx * G.gy);
            const uint32_t set = local / ncell, cell = local % ncell;
            const int cx = int(cell) / G.gy, cy = int(cell) % G.gy;
            const int R = a.rows, gyR = G.gy * R;
            const uint32_t colbase = (uint32_t(G.bin_base) + set * ncell) * uint32_t(R);
            int gxx, sxi, r0[2], r1[2], syi[2];
            walk_column(G, cx, cy, R, lane, gxx, sxi, r0, r1, syi);
            uint32_t rs[2] = {0u, 0u}, re[2] = {0u, 0u};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (r0[h] <= r1[h]) {
                    const uint32_t b0 = colbase + uint32_t(gxx * gyR + r0[h]);
                    rs[h] = a.cstart[b0];
                    re[h] = a.cstart[b0 + uint32_t(r1[h] - r0[h]) + 1];
                }
            }
            const bool v0 = re[0] > rs[0], v1 = re[1] > rs[1];
            const unsigned m0 = __ballot_sync(0xffffffffu, v0), m1 = __ballot_sync(0xffffffffu, v1);
            const unsigned lt = (1u << lane) - 1u;
            const int pos = __popc(m0 & lt) + __popc(m1 & lt);   // <= 2 (2 k + 1) = kMaxPieces
            // bin centre (wrapped coordinates): origin of the local frame
            const float ocx = (float(cx) + 0.5f) / G.inv_sx, ocy = (float(cy) + 0.5f) / G.inv_sy;
            const float srow = 1.f / (G.inv_sy * float(R));
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (!(h == 0 ? v0 : v1)) continue;
                Piece pc;
                pc.gstart = rs[h];
                pc.cnt = re[h] - rs[h];
                pc.qdx = -float(sxi) * G.Lx;
                pc.qdy = -float(syi[h]) * G.Ly;
                pc.b0 = colbase + uint32_t(gxx * gyR + r0[h]);
                pc.x0 = float(gxx) / G.inv_sx - ocx - pc.qdx;
                pc.y0 = float(r0[h]) * srow - ocy - pc.qdy;
                pc.nr = int16_t(r1[h] - r0[h] + 1);
                pc.mx = int8_t(sxi);
                pc.my = int8_t(syi[h]);
                s_pc[pos + (h == 1 && v0 ? 1 : 0)] = pc;
            }
            // a walk that fits one batch is planned and its bulk copies issued here,
            // by the lanes that hold its runs (the previous item's reads of the
            // staging buffer ended at the item's closing barrier)
            const uint32_t c0 = v0 ? re[0] - rs[0] : 0u, c1 = v1 ? re[1] - rs[1] : 0u;
            uint32_t incl = c0 + c1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const uint32_t tot_all = __shfl_sync(0xffffffffu, incl, 31);
            const uint32_t ex = incl - c0 - c1;   // staging offset of this lane's first run
            const bool one = tot_all > 0u && tot_all <= uint32_t(kCap);
            const int np = __popc(m0) + __popc(m1);
            if (one) {
                if (v0) s_bp[pos] = BatchPiece{ex, c0, rs[0], pos};
                if (v1) s_bp[pos + (v0 ? 1 : 0)] = BatchPiece{ex + c0, c1, rs[1], pos + (v0 ? 1 : 0)};
                if (lane == 0) {
                    fence_proxy_async_smem();
                    mbar_arrive_expect_tx(&s_bar, tot_all * kRec);
                }
                __syncwarp();
                fence_proxy_async_smem();
                const char* gsrc = kDef ? reinterpret_cast<const char*>(a.candf) : reinterpret_cast<const char*>(a.cand);
                if (v0)
                    bulk_g2s(reinterpret_cast<char*>(s_cand) + size_t(ex) * kRec, gsrc + size_t(rs[0]) * kRec,
                             c0 * kRec, &s_bar);
                if (v1)
                    bulk_g2s(reinterpret_cast<char*>(s_cand) + size_t(ex + c0) * kRec, gsrc + size_t(rs[1]) * kRec,
                             c1 * kRec, &s_bar);
            }
            if (lane == 0) {
                s_np = np;
                s_cur_piece = one ? np : 0;
                s_cur_off = 0;
                s_pre = one ? 1 : 0;
                s_nbp = one ? np : 0;
                s_btot = one ? tot_all : 0u;
                s_ox = ocx;
                s_oy = ocy;
            }
        }

        // this thread's queries
        float qx[QPT], qy[QPT];
        uint32_t qid[QPT];
        // image flags of the queries, 6 bits each (FIELD9)
        using QFlags = typename std::conditional<(6 * QPT > 32), unsigned long long, uint32_t>::type;
        QFlags qfl = 0;
        bool qv[QPT];
        Acc acc[QPT];
        float acc_c[QPT];
        double accg[kGrad ? QPT : 1][2];
#pragma unroll
        for (int j = 0; j < QPT; ++j) {
            const uint32_t idx = uint32_t((u0 + (j >> 1)) * 64 + (j & 1) * 32 + (tid & 31));
            qv[j] = (j >> 1) < npw && idx < it.qcnt;
            QRec r = qv[j] ? a.qrec[it.qbeg + idx] : QRec{0.f, 0.f, 0u, (2u) | (2u << 3)};
            qx[j] = r.x;
            qy[j] = r.y;
            qid[j] = r.id;
            qfl |= QFlags(r.flags & 63u) << (6 * j);
            acc[j] = Acc(0);
            acc_c[j] = 0.f;
            if constexpr (kGrad) accg[j][0] = accg[j][1] = 0.0;
        }
        if constexpr (kScat) {
            // the item's samples with their weights a_s 2 sigma (FP32 hi + lo)
            const double sig2 = 80.0 / (7.0 * kPiD * double(G.hw) * double(G.hw));
            for (uint32_t k = uint32_t(tid); k < it.qcnt && k < uint32_t(kScatQ); k += kEvalThreads) {
                const QRec r = a.qrec[it.qbeg + k];
                const double w = a.qweight[r.id] * sig2;
                const float wh = float(w);
                s_sq[k] = make_float4(r.x, r.y, wh, float(w - double(wh)));
                s_sqm[k] = uint16_t(image_mask9(r.flags));
            }
            if (tid == 0 && it.qcnt > uint32_t(kScatQ)) atomicOr(a.flags, FLAG_CAPACITY);
        }
        __syncthreads();
        if constexpr (kPacked) {
            // bounding box of this warp's queries in the bin's frame
            float bx0 = INFINITY, bx1 = -INFINITY, by0 = INFINITY, by1 = -INFINITY;
#pragma unroll
            for (int j = 0; j < QPT; ++j) {
                if (!qv[j]) continue;
                bx0 = fminf(bx0, qx[j]);
                bx1 = fmaxf(bx1, qx[j]);
                by0 = fminf(by0, qy[j]);
                by1 = fmaxf(by1, qy[j]);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
                bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
                by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
                by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
            }
            if ((tid & 31) == 0) s_wb[tid >> 5] = make_float4(bx0 - s_ox, bx1 - s_ox, by0 - s_oy, by1 - s_oy);
            // the warp's lanes read the box below, possibly before any CTA barrier
            // (a first batch issued with the walk skips the planning barrier)
            __syncwarp();
        }

        for (;;) {
            // s_pre: this batch was planned and issued with the walk (read after a
            // barrier, cleared by thread 0 once every thread is past the next one)
            if (!s_pre) {
            if (tid == 0) {
                // next batch: whole or partial pieces up to the staging capacity
                int pc = s_cur_piece;
                uint32_t po = s_cur_off, tot = 0;
                int nb = 0;
                while (pc < s_np && tot < uint32_t(kCap) && nb < kMaxPieces + 2) {
                    const uint32_t rem = s_pc[pc].cnt - po;
                    const uint32_t take = min(rem, uint32_t(kCap) - tot);
                    s_bp[nb++] = BatchPiece{tot, take, s_pc[pc].gstart + po, pc};
                    tot += take;
                    po += take;
                    if (po == s_pc[pc].cnt) { ++pc; po = 0; }
                }
                s_cur_piece = pc;
                s_cur_off = po;
                s_nbp = nb;
                s_btot = tot;
                if (tot > 0) {
                    fence_proxy_async_smem();
                    mbar_arrive_expect_tx(&s_bar, tot * kRec);
                    const char* gsrc = kDef ? reinterpret_cast<const char*>(a.candf)
                                            : reinterpret_cast<const char*>(a.cand);
                    for (int b = 0; b < nb; ++b)
                        bulk_g2s(reinterpret_cast<char*>(s_cand) + size_t(s_bp[b].soff) * kRec,
                                 gsrc + size_t(s_bp[b].gstart) * kRec, s_bp[b].cnt * kRec, &s_bar);
                }
            }
            __syncthreads();
            }
            if (s_btot == 0) break;
            if constexpr (kPacked) {
                // this warp's part of each staged run: the sub-rows within reach of
                // its queries' bounding box (reach widened by 0.1%, sub-row bounds by
                // 1% of a sub-row, so no pair with a non-zero term is dropped: the
                // sums equal those over the whole runs).  The sub-row starts are read
                // while the bulk copy is in flight.
                if (npw > 0) {
                    const int wid = tid >> 5;
                    const float4 bb = s_wb[wid];
                    const float sxw = 1.f / G.inv_sx, inv_srow = G.inv_sy * float(a.rows);
                    const float rm = G.reach * 1.001f;
                    for (int b = tid & 31; b < s_nbp; b += 32) {
                        const BatchPiece bp = s_bp[b];
                        const Piece pc = s_pc[bp.piece];
                        uint32_t lo = 0u, hi = 0u;
                        const float dxw = fmaxf(0.f, fmaxf(pc.x0 - bb.y, bb.x - (pc.x0 + sxw)));
                        if (dxw < rm) {
                            const float dy = sqrtf(fmaf(rm, rm, -dxw * dxw));
                            const int ilo = max(int(floorf(fmaf(bb.z - dy - pc.y0, inv_srow, -0.01f))), 0);
                            const int ihi = min(int(floorf(fmaf(bb.w + dy - pc.y0, inv_srow, 0.01f))), int(pc.nr) - 1);
                            if (ilo <= ihi) {
                                const uint32_t t0 = a.cstart[pc.b0 + uint32_t(ilo)];
                                const uint32_t t1 = a.cstart[pc.b0 + uint32_t(ihi) + 1u];
                                const uint32_t g0 = bp.gstart, g1 = bp.gstart + bp.cnt;
                                lo = min(max(t0, g0), g1) - g0;
                                hi = max(min(max(t1, g0), g1) - g0, lo);
                            }
                        }
                        s_rng[wid][b] = make_uint2(lo, hi);
                    }
                }
            }
            // each thread sees the copied bytes once its own wait completes; the
            // packed modes rewrite them first, so their barrier follows that pass
            if (!mbar_wait_bounded(&s_bar, phase, a.wait_limit)) atomicOr(&s_abort, 1);
            phase ^= 1u;
            if constexpr (!kPacked) {
                __syncthreads();
                if (tid == 0) s_pre = 0;
                if (s_abort) break;
            }

            const int nbp = s_nbp;
            if constexpr (kScat)
                scat_batch<ST, kScat9>(s_cand, s_bp, s_pc, nbp, s_btot, s_sq, s_sqm,
                                       min(int(it.qcnt), kScatQ), G, a.out_f64);
            if constexpr (kPacked) {
                // staged candidates -> image-shifted, bin-local coordinates + kappa c2
                // (kappa = -3/h^2 scales every squared distance, see packed_run)
                const float kap = G.B;
                for (int b = 0; b < nbp; ++b) {
                    const BatchPiece bp = s_bp[b];
                    const Piece pc = s_pc[bp.piece];
                    const float ox = s_ox + pc.qdx, oy = s_oy + pc.qdy;
                    for (uint32_t c = threadIdx.x; c < bp.cnt; c += kEvalThreads) {
                        if constexpr (kDef) {
                            float* f = s_candf[bp.soff + c].f;
                            const float lx = f[0] - ox, ly = f[1] - oy;
                            const float g11 = f[2], g12 = f[3], g22 = f[4], w = f[5];
                            const float gx = fmaf(g11, lx, g12 * ly), gy = fmaf(g12, lx, g22 * ly);
                            const float e = kap * fmaf(lx, gx, ly * gy);
                            f[0] = kap * g11; f[1] = f[0];
                            f[2] = kap * (2.f * g12); f[3] = f[2];
                            f[4] = kap * g22; f[5] = f[4];
                            f[6] = kap * (-2.f * gx); f[7] = f[6];
                            f[8] = kap * (-2.f * gy); f[9] = f[8];
                            f[10] = e; f[11] = e;
                            f[12] = w; f[13] = w;
                            f[14] = 0.f; f[15] = 0.f;
                        } else {
                            Cand& cd = s_cand[bp.soff + c];
                            const float lx = cd.x - ox, ly = cd.y - oy;
                            const float c2 = kap * fmaf(lx, lx, ly * ly);
                            cd.x = lx;
                            cd.x2 = lx;
                            cd.y = ly;
                            cd.y2 = ly;
                            cd.wl = c2;
                            cd.pad = c2;
                        }
                    }
                }
                __syncthreads();
                if (tid == 0) s_pre = 0;
                if (s_abort) break;   // (a thread whose wait expired rewrote stale bytes: unused)
            }
            for (int b = 0; b < (kScat ? 0 : nbp); ++b) {
                const BatchPiece bp = s_bp[b];
                const Piece pc = s_pc[bp.piece];
                int cnt = int(bp.cnt);
                const int bfirst = b;
                if constexpr (kPacked) {
                    // staged runs sit back to back in shared memory, already in the
                    // bin's frame: consecutive runs under the same image mask are one
                    // sweep (each warp visits its own part of each run, in run order)
                    while (b + 1 < nbp) {
                        const Piece nx = s_pc[s_bp[b + 1].piece];
                        if (kField9 && (nx.mx != pc.mx || nx.my != pc.my)) break;
                        cnt += int(s_bp[b + 1].cnt);
                        ++b;
                    }
                }
                const Cand* cs = s_cand + bp.soff;
                Acc part[QPT];
                if constexpr (kPacked && kDef) {
                    // queries in the local frame: the monomials of the expanded metric form
                    f2x QXX[NP], QXY[NP], QYY[NP], QX[NP], QY[NP], P[NP];
#pragma unroll
                    for (int pr = 0; pr < NP; ++pr) {
                        const float ax = qx[2 * pr] - s_ox, bx = qx[2 * pr + 1] - s_ox;
                        const float ay = qy[2 * pr] - s_oy, by = qy[2 * pr + 1] - s_oy;
                        QXX[pr] = pk2(ax * ax, bx * bx);
                        QXY[pr] = pk2(ax * ay, bx * by);
                        QYY[pr] = pk2(ay * ay, by * by);
                        QX[pr] = pk2(ax, bx);
                        QY[pr] = pk2(ay, by);
                        P[pr] = pk2(0.f, 0.f);
                    }
                    for (int gb = bfirst; gb <= b && npw > 0; ++gb) {
                        const uint2 rg = s_rng[tid >> 5][gb];
                        const int n = int(rg.y) - int(rg.x);
                        if (n <= 0) continue;
                        const CandF* csf = s_candf + s_bp[gb].soff + rg.x;
                        if (npw == 1) packed_run_f<1, NP>(csf, n, QXX, QXY, QYY, QX, QY, P);
                        else if (NP >= 2 && npw == 2)
                            packed_run_f<(NP >= 2 ? 2 : 1), NP>(csf, n, QXX, QXY, QYY, QX, QY, P);
                        else packed_run_f<NP, NP>(csf, n, QXX, QXY, QYY, QX, QY, P);
                    }
#pragma unroll
                    for (int pr = 0; pr < NP; ++pr) {
                        float lo, hi;
                        up2(P[pr], lo, hi);
                        part[2 * pr] = lo;
                        part[2 * pr + 1] = hi;
                    }
                } else if constexpr (kPacked) {
                    // queries in the same local frame: -2 kappa q and kappa |q|^2
                    f2x QX[NP], QY[NP], Q2[NP], P[NP];
                    const float kap = G.B, m2k = -2.f * G.B;
#pragma unroll
                    for (int pr = 0; pr < NP; ++pr) {
                        const float ax = qx[2 * pr] - s_ox, bx = qx[2 * pr + 1] - s_ox;
                        const float ay = qy[2 * pr] - s_oy, by = qy[2 * pr + 1] - s_oy;
                        QX[pr] = pk2(m2k * ax, m2k * bx);
                        QY[pr] = pk2(m2k * ay, m2k * by);
                        Q2[pr] = pk2(kap * fmaf(ax, ax, ay * ay), kap * fmaf(bx, bx, by * by));
                        P[pr] = pk2(0.f, 0.f);
                    }
                    // a warp with few queries runs fewer pairs (none when it holds no query)
                    for (int gb = bfirst; gb <= b && npw > 0; ++gb) {
                        const uint2 rg = s_rng[tid >> 5][gb];
                        const int n = int(rg.y) - int(rg.x);
                        if (n <= 0) continue;
                        const Cand* c0 = s_cand + s_bp[gb].soff + rg.x;
                        if (npw == 1) packed_run<1, NP>(c0, n, QX, QY, Q2, P);
                        else if (NP >= 2 && npw == 2) packed_run<(NP >= 2 ? 2 : 1), NP>(c0, n, QX, QY, Q2, P);
                        else packed_run<NP, NP>(c0, n, QX, QY, Q2, P);
                    }
#pragma unroll
                    for (int pr = 0; pr < NP; ++pr) {
                        float lo, hi;
                        up2(P[pr], lo, hi);
                        part[2 * pr] = lo;
                        part[2 * pr + 1] = hi;
                    }
                } else if constexpr (kDefExc) {
                    // deformed kernels, differences taken directly (an exact zero
                    // for coincident points, so the centre test is reliable)
                    float px[QPT], py[QPT];
#pragma unroll
                    for (int j = 0; j < QPT; ++j) {
                        px[j] = qx[j] + pc.qdx;
                        py[j] = qy[j] + pc.qdy;
                        part[j] = Acc(0);
                    }
                    const float A = G.A, B = G.B, ih = G.inv_hw;
                    const CandF* csf = s_candf + bp.soff;
                    for (int c = 0; c < cnt; ++c) {
                        const float cx = csf[c].f[0], cy = csf[c].f[1];
                        const float g11 = csf[c].f[2], g12 = csf[c].f[3], g22 = csf[c].f[4], cw = csf[c].f[5];
#pragma unroll
                        for (int j = 0; j < QPT; ++j) {
                            const float dx = cx - px[j], dy = cy - py[j];
                            const float r2 = fmaf(g11 * dx, dx, fmaf(2.f * g12 * dx, dy, g22 * dy * dy));
                            const float r = sqrtf(fmaxf(r2, 0.f));
                            const float inner = fmaf(r2, fmaf(A, r, B), 0.5f);
                            const float t = fmaf(-ih, r, 1.0f);
                            float v = fmaxf(fminf(inner, t * t * t), 0.0f);
                            if (r < 1e-6f) v = 0.f;
                            part[j] = fmaf(cw, v, part[j]);
                        }
                    }
                } else if constexpr (kGrad) {
                    // value and gradient in q of sum w W(|q - c|), pair by pair in GT
                    // (FP64, or FP32 for the FP32 path's adjoint; run sums into FP64):
                    // dW/dr / r = 2 sigma (3 A r + 2 B) for r < h/2, -6 sigma t^2/(h r) below h
                    const GT hw = GT(G.hw), ih = GT(1) / hw;
                    const GT A = GT(3) * ih * ih * ih, B = GT(-3) * ih * ih;
                    GT px[QPT], py[QPT], pv[QPT], pgx[QPT], pgy[QPT];
                    bool use[QPT];
#pragma unroll
                    for (int j = 0; j < QPT; ++j) {
                        px[j] = GT(qx[j]) + GT(pc.qdx);
                        py[j] = GT(qy[j]) + GT(pc.qdy);
                        pv[j] = pgx[j] = pgy[j] = GT(0);
                        use[j] = true;
                        if (kGrad9) {
                            const int mx = int(uint32_t(qfl >> (6 * j)) & 7u) - 2 + pc.mx;
                            const int my = int(uint32_t(qfl >> (6 * j + 3)) & 7u) - 2 + pc.my;
                            use[j] = mx >= -1 && mx <= 1 && my >= -1 && my <= 1;
                        }
                    }
                    for (int c = 0; c < cnt; ++c) {
                        const Cand cv = cs[c];
                        const GT cxd = cv.x, cyd = cv.y;
                        const GT wd = kGrad32 ? GT(cv.w) : GT(double(cv.w) + double(cv.wl));
#pragma unroll
                        for (int j = 0; j < QPT; ++j) {
                            const GT dx = px[j] - cxd, dy = py[j] - cyd;   // q - c
                            if constexpr (kGrad32) {
                                // FP32 pairs without a branch (zeros outside the support)
                                float v, dr;
                                spline_vdr_f32(fmaf(dx, dx, dy * dy), hw, ih, A, B, v, dr);
                                const float wdr = wd * dr;
                                pv[j] = fmaf(wd, v, pv[j]);
                                pgx[j] = fmaf(wdr, dx, pgx[j]);
                                pgy[j] = fmaf(wdr, dy, pgy[j]);
                                continue;
                            }
                            const GT r2 = dx * dx + dy * dy;
                            const GT r = sqrt(r2);
                            if (r >= hw) continue;
                            const GT t = GT(1) - ih * r;
                            GT v, dr;   // W / 2 sigma and its r-derivative over r
                            if (r <= GT(0.5) * hw) {
                                v = GT(0.5) + r2 * (A * r + B);
                                dr = GT(3) * A * r + GT(2) * B;
                            } else {
                                v = t * t * t;
                                dr = GT(-3) * t * t * ih / r;
                            }
                            pv[j] += wd * v;
                            pgx[j] += wd * dr * dx;
                            pgy[j] += wd * dr * dy;
                        }
                    }
#pragma unroll
                    for (int j = 0; j < QPT; ++j) {
                        if (!use[j]) continue;
                        acc[j] += double(pv[j]);
                        accg[j][0] += double(pgx[j]);
                        accg[j][1] += double(pgy[j]);
                        part[j] = 0.0;
                    }
                } else if constexpr (kField64) {
                    // the plain FP64 path: every pair and the sum in FP64
                    const double hw = double(G.hw), ih = 1.0 / hw;
                    const double A = 3.0 * ih * ih * ih, B = -3.0 * ih * ih;
                    double px[QPT], py[QPT];
#pragma unroll
                    for (int j = 0; j < QPT; ++j) {
                        px[j] = double(qx[j]) + double(pc.qdx);
                        py[j] = double(qy[j]) + double(pc.qdy);
                        part[j] = 0.0;
                    }
                    for (int c = 0; c < cnt; ++c) {
                        const Cand cv = cs[c];
                        const double cxd = cv.x, cyd = cv.y, wd = double(cv.w) + double(cv.wl);
#pragma unroll
                        for (int j = 0; j < QPT; ++j) {
                            const double dx = cxd - px[j], dy = cyd - py[j];
                            const double r2 = dx * dx + dy * dy;
                            const double r = sqrt(r2);
                            const double inner = 0.5 + r2 * (A * r + B);
                            const double t = 1.0 - ih * r;
                            const double v = fmax(fmin(inner, t * t * t), 0.0);
                            part[j] += wd * v;
                        }
                    }
                } else if constexpr (kF64) {
                    float px[QPT], py[QPT];
#pragma unroll
                    for (int j = 0; j < QPT; ++j) {
                        px[j] = qx[j] + pc.qdx;
                        py[j] = qy[j] + pc.qdy;
                        part[j] = Acc(0);
                    }
                    const double hw = double(G.hw);
                    const float lim = G.hw * G.hw * 1.0001f;
#pragma unroll 2
                    for (int c = 0; c < cnt; ++c) {
                        const Cand cv = cs[c];
#pragma unroll
                        for (int j = 0; j < QPT; ++j) {
                            const float dx = cv.x - px[j], dy = cv.y - py[j];
                            if (dx * dx + dy * dy < lim) {
                                const double ddx = double(cv.x) - (double(qx[j]) + double(pc.qdx));
                                const double ddy = double(cv.y) - (double(qy[j]) + double(pc.qdy));
                                const double r = sqrt(ddx * ddx + ddy * ddy);
                                part[j] += (double(cv.w) + double(cv.wl)) * spline_w_d(r, hw);
                            }
                        }
                    }
                } else {
                    float px[QPT], py[QPT];
#pragma unroll
                    for (int j = 0; j < QPT; ++j) {
                        px[j] = qx[j] + pc.qdx;
                        py[j] = qy[j] + pc.qdy;
                        part[j] = Acc(0);
                    }
                    const float A = G.A, B = G.B, ih = G.inv_hw;
#pragma unroll 4
                    for (int c = 0; c < cnt; ++c) {
                        const float cx = cs[c].x, cy = cs[c].y, cw = cs[c].w;
#pragma unroll
                        for (int j = 0; j < QPT; ++j) {
                            const float dx = cx - px[j], dy = cy - py[j];
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, 1e-30f));
                            const float r = r2 * rsqrtf(r2);
                            const float inner = fmaf(r2, fmaf(A, r, B), 0.5f);
                            const float t = fmaf(-ih, r, 1.0f);
                            float v = fmaxf(fminf(inner, t * t * t), 0.0f);
                            if (MODE == EVAL_FIELD_EXC && r2 < 1e-12f) v = 0.f;
                            part[j] = fmaf(cw, v, part[j]);
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < QPT && !kGrad; ++j) {
                    bool use = true;
                    if (kField9) {
                        const int mx = int(uint32_t(qfl >> (6 * j)) & 7u) - 2 + pc.mx;
                        const int my = int(uint32_t(qfl >> (6 * j + 3)) & 7u) - 2 + pc.my;
                        use = mx >= -1 && mx <= 1 && my >= -1 && my <= 1;
                    }
                    if (use) {
                        if constexpr (kComp) {
                            // compensated accumulation of the per-run partial sums
                            const float y = float(part[j]) - acc_c[j];
                            const float tt = float(acc[j]) + y;
                            acc_c[j] = (tt - float(acc[j])) - y;
                            acc[j] = tt;
                        } else {
                            acc[j] += part[j];
                        }
                    }
                }
            }
            // no further batch in this item: the item's closing barrier guards the
            // staging buffer (the cursor only moves in the next planning step)
            if (s_cur_piece >= s_np) break;
            __syncthreads();   // all reads of s_cand done before the next batch overwrites it
        }
        if (s_abort) break;
#pragma unroll
        for (int j = 0; j < QPT && !kScat; ++j) {
            if (!qv[j]) continue;
            if constexpr (kGrad) {
                a.out_f64[3 * size_t(qid[j])] = acc[j];
                a.out_f64[3 * size_t(qid[j]) + 1] = accg[j][0];
                a.out_f64[3 * size_t(qid[j]) + 2] = accg[j][1];
            } else if constexpr (kF64 || kField64) a.out_f64[qid[j]] = acc[j];
            else if constexpr (kComp) a.out_f64[qid[j]] = double(acc[j]) - double(acc_c[j]);
            else a.out_f32[qid[j]] = acc[j];
        }
        if (tid == 0) s_item = next_item;
        __syncthreads();
    }
    if (s_abort) {
        if (tid == 0) {
            atomicOr(a.flags, FLAG_TIMEOUT);
            (void)mbar_wait_bounded(&s_bar, phase ^ 1u, kWaitLimit);   // let an in-flight copy land
        }
    }
}

template <int MODE, int QPT>
int launch_eval_t(vpmc_context* ctx, const EvalArgs& a) {
    const size_t smem = size_t(kCandCap) * sizeof(Cand);
    static bool configured[64] = {};
    const int dev = ctx->device;
    if (dev < 64 && !configured[dev]) {
        VPMC_CUDA(cudaFuncSetAttribute(k_eval<MODE, QPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        configured[dev] = true;
    }
    int per_sm = 0;
    VPMC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eval<MODE, QPT>, kEvalThreads, smem));
    if (per_sm < 1) per_sm = 1;
    const int grid = ctx->sm_count * per_sm;
    VPMC_LAUNCH((k_eval<MODE, QPT>), grid, kEvalThreads, smem, ctx->stream, a);
    return VPMC_OK;
}

int blocks_for(long n, int threads = 256) {
    long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 65535L * 16) b = 65535L * 16;
    return int(b);
}

}  // namespace

int default_k() { return 2; }

int query_chunk(int qpt) { return (qpt == 8 ? 8 : qpt == 6 ? 6 : 4) * kEvalThreads; }   // qpt 1 (tensor cores): 128

long grid_plan(const InstDesc* in, int n, int k, int nsets, GridInst* out) {
    if (k <= 0) k = default_k();
    if (k > kMaxK) k = kMaxK;
    long base = 0;
    for (int i = 0; i < n; ++i) {
        const InstDesc& d = in[i];
        if (!(d.hw > 0.f) || !(d.Lx > 0.f) || !(d.Ly > 0.f)) return -VPMC_ERR_INVALID;
        if (!(d.cover >= 1.f)) return -VPMC_ERR_INVALID;
        const double reach = double(d.hw) * double(d.cover);   // physical support radius to cover
        int kk = k, gx = 0, gy = 0;
        for (; kk >= 1; --kk) {
            gx = int(std::floor(double(kk) * double(d.Lx) / reach + 1e-9));
            gy = int(std::floor(double(kk) * double(d.Ly) / reach + 1e-9));
            if (!d.periodic || (gx >= 2 * kk + 1 && gy >= 2 * kk + 1)) break;
        }
        if (kk < 1 || gx < 1 || gy < 1) return -VPMC_ERR_GEOMETRY;
        if (long(gx) * gy > (1L << 24)) return -VPMC_ERR_CAPACITY;
        GridInst g{};
        g.Lx = d.Lx;
        g.Ly = d.Ly;
        g.gx = gx;
        g.gy = gy;
        g.inv_sx = float(gx) / d.Lx;
        g.inv_sy = float(gy) / d.Ly;
        g.k = kk;
        g.bin_base = int(base);
        g.nsets = nsets;
        g.periodic = d.periodic;
        g.hw = d.hw;
        g.reach = float(reach);
        const double h = d.hw;
        g.inv_hw = float(1.0 / h);
        g.A = float(3.0 / (h * h * h));
        g.B = float(-3.0 / (h * h));
        g.two_sigma = float(2.0 * 40.0 / (7.0 * kPiD * h * h));
        g.p_begin = d.p_begin;
        g.p_end = d.p_end;
        out[i] = g;
        base += long(nsets) * gx * gy;
        if (base >= (1L << 31)) return -VPMC_ERR_CAPACITY;
    }
    return base;
}

void carve_grid(Carver& c, long n, long nbins, int n_inst, GridBufs* g, bool deformed, int rows) {
    g->inst = c.take<GridInst>(size_t(n_inst));
    g->n_inst = n_inst;
    g->nbins = nbins;
    g->rows = rows < 1 ? 1 : rows;
    g->n = n;
    const long nsub = nbins * g->rows;
    g->keys = c.take<uint32_t>(size_t(n < 1 ? 1 : n));
    g->count = c.take<uint32_t>(size_t(nsub + 1));
    g->start = c.take<uint32_t>(size_t(nsub + 1));
    g->cstart = g->rows > 1 ? c.take<uint32_t>(size_t(nbins + 1)) : g->start;
    g->cand = c.take<Cand>(size_t(n < 1 ? 1 : n));
    g->candf = deformed ? c.take<CandF>(size_t(n < 1 ? 1 : n)) : nullptr;
    carve_radix(c, n, &g->rs);
    // the bin scan reuses the radix scan scratch when it is large enough
    const size_t need = scan_tmp_elems(nsub + 1);
    if (need > scan_tmp_elems(long(radix_counts_elems(n)))) g->rs.scan_tmp = c.take<uint32_t>(need + 1);
}

int grid_build(vpmc_context* ctx, GridBufs& g, const float2* pos, const float* omega, int set_mode,
               const float4* F) {
    if (F && !g.candf) return VPMC_ERR_INVALID;
    cudaStream_t st = ctx->stream;
    const long nsub = g.nbins * g.rows;
    VPMC_CUDA(cudaMemsetAsync(g.count, 0, sizeof(uint32_t) * size_t(nsub + 1), st));
    VPMC_LAUNCH(k_grid_keys, blocks_for(g.n), 256, 0, st, pos, omega, g.n, g.inst, g.n_inst, set_mode,
                uint32_t(g.nbins), g.rows, g.keys, g.count);
    VPMC_TRY(exclusive_scan(ctx, g.count, g.start, nsub, g.rs.scan_tmp, true));
    uint32_t *ks = nullptr, *vs = nullptr;
    VPMC_TRY(radix_sort(ctx, g.keys, nullptr, g.n, bits_for(uint64_t(nsub) + 1), g.rs, &ks, &vs));
    g.perm = vs;
    if (F)
        VPMC_LAUNCH(k_grid_gather_f, blocks_for(g.n), 256, 0, st, vs, g.start, g.n, uint32_t(nsub), pos, omega, F,
                    g.inst, g.n_inst, set_mode, g.candf);
    else
        VPMC_LAUNCH(k_grid_gather, blocks_for(g.n), 256, 0, st, vs, g.start, g.n, uint32_t(nsub), pos, omega,
                    g.inst, g.n_inst, set_mode, g.cand);
    if (g.rows > 1)
        VPMC_LAUNCH(k_coarse_starts, blocks_for(g.nbins + 1), 256, 0, st, g.start, g.nbins, g.rows, g.cstart);
    return VPMC_OK;
}

int grid_set_weights_sorted(vpmc_context* ctx, GridBufs& g, const double* x_sorted, double scale) {
    VPMC_LAUNCH(k_grid_weights, blocks_for(g.n), 256, 0, ctx->stream, x_sorted, g.n, scale, g.cand);
    return VPMC_OK;
}

int grid_max_sigma(vpmc_context* ctx, const float4* F, long n, unsigned* d_words, float* sigma) {
    cudaStream_t st = ctx->stream;
    VPMC_CUDA(cudaMemsetAsync(d_words, 0, 2 * sizeof(unsigned), st));
    if (n > 0)
        VPMC_LAUNCH(k_sigma, std::min(blocks_for(n), 4 * ctx->sm_count), 256, 0, st, F, n, d_words);
    unsigned h = 0u;
    VPMC_CUDA(cudaMemcpyAsync(&h, d_words, sizeof(h), cudaMemcpyDeviceToHost, st));
    VPMC_CUDA(cudaStreamSynchronize(st));
    float v;
    memcpy(&v, &h, sizeof(v));
    *sigma = n > 0 ? v : 1.f;
    return VPMC_OK;
}

void carve_items(Carver& c, long nbins, long max_queries, ItemBufs* it) {
    it->max_items = max_queries / query_chunk(1) + nbins + 1;
    it->items = c.take<Item>(size_t(it->max_items));
    it->n_items = c.take<uint32_t>(1);
    it->counter = c.take<uint32_t>(1);
    it->per_bin = c.take<uint32_t>(size_t(nbins + 1));
    it->item_start = c.take<uint32_t>(size_t(nbins + 1));
    it->scan_tmp = c.take<uint32_t>(scan_tmp_elems(nbins + 1) + 1);
}

int make_items(vpmc_context* ctx, const GridBufs& g, const uint32_t* qstart, ItemBufs& it, int chunk) {
    cudaStream_t st = ctx->stream;
    VPMC_LAUNCH(k_items_count, blocks_for(g.nbins), 256, 0, st, qstart, g.nbins, chunk, it.per_bin);
    VPMC_TRY(exclusive_scan(ctx, it.per_bin, it.item_start, g.nbins, it.scan_tmp, true));
    VPMC_LAUNCH(k_items_fill, blocks_for(g.nbins), 256, 0, st, qstart, g.nbins, chunk, it.item_start, g.inst,
                g.n_inst, it.items, it.n_items, it.counter, it.max_items);
    return VPMC_OK;
}

void carve_queries(Carver& c, long nbins, long max_points, QueryBufs* q, bool two_pass) {
    const size_t m = size_t(max_points < 1 ? 1 : max_points);
    q->qbin = c.take<uint32_t>(m);
    q->qcount = c.take<uint32_t>(size_t(nbins + 1));
    q->qstart = c.take<uint32_t>(size_t(nbins + 1));
    q->qfill = c.take<uint32_t>(size_t(nbins + 1));
    q->qrank = two_pass ? nullptr : c.take<uint32_t>(m);   // ranks are only needed without the staged placement
    q->qrec = c.take<QRec>(m);
    q->tmp = two_pass ? c.take<uint4>(m) : nullptr;
    q->tmp2 = two_pass ? c.take<uint4>(m) : nullptr;
    q->super_fill = two_pass ? c.take<uint32_t>(kTargetSuper + 1) : nullptr;
    q->win_fill = two_pass ? c.take<uint32_t>(size_t(nbins + 1)) : nullptr;
    q->scan_tmp = c.take<uint32_t>(scan_tmp_elems(nbins + 1) + 1);
}

int scatter_points(vpmc_context* ctx, const GridBufs& g, QueryBufs& q, const float2* pts, long M, int field9) {
    (void)field9;
    cudaStream_t st = ctx->stream;
    VPMC_TRY(exclusive_scan(ctx, q.qcount, q.qstart, g.nbins, q.scan_tmp, true));
    VPMC_CUDA(cudaMemsetAsync(q.qfill, 0, sizeof(uint32_t) * size_t(g.nbins + 1), st));
    VPMC_LAUNCH(k_scatter_points, blocks_for(M), 256, 0, st, pts, M, g.inst, g.n_inst, q.qbin, q.qstart, q.qfill,
                q.qrec);
    return VPMC_OK;
}

int scatter_ranked(vpmc_context* ctx, const GridBufs& g, QueryBufs& q, const float2* pts, long M) {
    VPMC_TRY(exclusive_scan(ctx, q.qcount, q.qstart, g.nbins, q.scan_tmp, true));
    cudaStream_t st = ctx->stream;
    if (q.tmp) {
        int shift = 0;
        while (((g.nbins - 1) >> shift) + 1 > kTargetSuper) ++shift;
        const int nsuper = int(((g.nbins - 1) >> shift) + 1);
        // windows of 2^W bins holding about half the assembly capacity on average
        const double per_bin = double(M) / double(std::max<long>(g.nbins, 1));
        int wshift = 0;
        while ((1 << (wshift + 1)) <= kWinBinsMax && per_bin * double(2L << wshift) <= 0.5 * kWinCap) ++wshift;
        const long nwin = ((g.nbins - 1) >> wshift) + 1;
        VPMC_CUDA(cudaMemsetAsync(q.super_fill, 0, sizeof(uint32_t) * size_t(nsuper), st));
        VPMC_CUDA(cudaMemsetAsync(q.win_fill, 0, sizeof(uint32_t) * size_t(nwin), st));
        static bool configured[64] = {};
        const size_t tile_smem = sizeof(uint4) * size_t(kTileRecs), win_smem = sizeof(QRec) * size_t(kWinCap);
        if (ctx->device < 64 && !configured[ctx->device]) {
            VPMC_CUDA(cudaFuncSetAttribute(k_scatter_coarse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           int(tile_smem)));
            VPMC_CUDA(cudaFuncSetAttribute(k_scatter_window, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           int(tile_smem)));
            VPMC_CUDA(cudaFuncSetAttribute(k_scatter_assemble, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           int(win_smem)));
            configured[ctx->device] = true;
        }
        const long tiles = (M + kTileRecs - 1) / kTileRecs;
        const int tgrid = int(std::max<long>(1, std::min<long>(tiles, 2L * ctx->sm_count)));
        VPMC_LAUNCH(k_scatter_coarse, tgrid, kPlaceThreads, tile_smem, st, pts, M, q.qbin, q.qstart, shift, nsuper,
                    q.super_fill, q.tmp);
        VPMC_LAUNCH(k_scatter_window, tgrid, kPlaceThreads, tile_smem, st, q.tmp, q.qstart + g.nbins, M, wshift,
                    q.qstart, q.win_fill, q.tmp2);
        VPMC_LAUNCH(k_scatter_assemble, int(std::max<long>(1, std::min<long>(nwin, 2L * ctx->sm_count))), kAsmThreads, win_smem,
                    st, q.tmp2, g.nbins, wshift, q.qstart, g.inst, g.n_inst, q.qrec);
        return VPMC_OK;
    }
    VPMC_LAUNCH(k_scatter_ranked, blocks_for(M), 256, 0, st, pts, M, g.inst, g.n_inst, q.qbin, q.qrank, q.qstart,
                q.qrec);
    return VPMC_OK;
}

int bin_points(vpmc_context* ctx, const GridBufs& g, QueryBufs& q, const float2* pts, long M, int set, int field9) {
    cudaStream_t st = ctx->stream;
    VPMC_CUDA(cudaMemsetAsync(q.qcount, 0, sizeof(uint32_t) * size_t(g.nbins + 1), st));
    VPMC_LAUNCH(k_bin_points, blocks_for(M), 256, 0, st, pts, M, g.inst, set, field9, q.qbin, q.qcount);
    return scatter_points(ctx, g, q, pts, M, field9);
}

int launch_eval(vpmc_context* ctx, const GridBufs& g, const QRec* qrec, ItemBufs& it, const EvalLaunch& L) {
    if (eval_deformed(L.mode) && !g.candf) return VPMC_ERR_INVALID;
    if (eval_scat(L.mode) && (!L.qweight || !L.out_f64 || L.qpt != 4)) return VPMC_ERR_INVALID;
    if (L.qpt == 1 && (L.mode == EVAL_FIELD || L.mode == EVAL_FIELD9)) {
        const EvalTcArgs t{g.inst, g.start, L.rows > 0 ? L.rows : g.rows, g.cand, qrec, it.items, it.n_items,
                           it.counter, L.out_f32, ctx->d_flags, ctx->wait_limit};
        return launch_eval_tc(ctx, t, L.mode == EVAL_FIELD9);
    }
    EvalArgs a{g.inst, g.start, L.rows > 0 ? L.rows : g.rows, g.cand, g.candf, qrec, it.items, it.n_items, it.counter,
               L.out_f32, L.out_f64, ctx->d_flags, ctx->wait_limit, L.qweight};
    switch (L.mode) {
        case EVAL_FIELD:
            if (L.qpt == 8) return launch_eval_t<EVAL_FIELD, 8>(ctx, a);
            if (L.qpt == 6) return launch_eval_t<EVAL_FIELD, 6>(ctx, a);
            return launch_eval_t<EVAL_FIELD, 4>(ctx, a);
        case EVAL_FIELD9:
            if (L.qpt == 8) return launch_eval_t<EVAL_FIELD9, 8>(ctx, a);
            if (L.qpt == 6) return launch_eval_t<EVAL_FIELD9, 6>(ctx, a);
            return launch_eval_t<EVAL_FIELD9, 4>(ctx, a);
        case EVAL_FIELD_EXC:
            if (L.qpt != 4) return VPMC_ERR_INVALID;
            return launch_eval_t<EVAL_FIELD_EXC, 4>(ctx, a);
        case EVAL_SPMV64:
            if (L.qpt != 4) return VPMC_ERR_INVALID;
            return launch_eval_t<EVAL_SPMV64, 4>(ctx, a);
        case EVAL_SPMV32:
            if (L.qpt != 4) return VPMC_ERR_INVALID;
            return launch_eval_t<EVAL_SPMV32, 4>(ctx, a);
        case EVAL_FIELD_F:
            if (L.qpt == 8) return launch_eval_t<EVAL_FIELD_F, 8>(ctx, a);
            if (L.qpt == 6) return launch_eval_t<EVAL_FIELD_F, 6>(ctx, a);
            return launch_eval_t<EVAL_FIELD_F, 4>(ctx, a);
        case EVAL_FIELD9_F:
            if (L.qpt == 8) return launch_eval_t<EVAL_FIELD9_F, 8>(ctx, a);
            if (L.qpt == 6) return launch_eval_t<EVAL_FIELD9_F, 6>(ctx, a);
            return launch_eval_t<EVAL_FIELD9_F, 4>(ctx, a);
        case EVAL_FIELD_F_EXC:
            if (L.qpt != 4) return VPMC_ERR_INVALID;
            return launch_eval_t<EVAL_FIELD_F_EXC, 4>(ctx, a);
        case EVAL_GRAD64: return launch_eval_t<EVAL_GRAD64, 4>(ctx, a);
        case EVAL_GRAD9_64: return launch_eval_t<EVAL_GRAD9_64, 4>(ctx, a);
        case EVAL_GRAD32: return launch_eval_t<EVAL_GRAD32, 4>(ctx, a);
        case EVAL_GRAD9_32: return launch_eval_t<EVAL_GRAD9_32, 4>(ctx, a);
        case EVAL_SCAT64: return launch_eval_t<EVAL_SCAT64, 4>(ctx, a);
        case EVAL_SCAT9_64: return launch_eval_t<EVAL_SCAT9_64, 4>(ctx, a);
        case EVAL_SCAT32: return launch_eval_t<EVAL_SCAT32, 4>(ctx, a);
        case EVAL_SCAT9_32: return launch_eval_t<EVAL_SCAT9_32, 4>(ctx, a);
        case EVAL_FIELD64: return launch_eval_t<EVAL_FIELD64, 4>(ctx, a);
        case EVAL_FIELD9_64: return launch_eval_t<EVAL_FIELD9_64, 4>(ctx, a);
        default: return VPMC_ERR_INVALID;
    }
}

}  // namespace vpmc
