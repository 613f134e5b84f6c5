// vpmc_sort.cu -- exclusive scan, stable LSD radix sort, deterministic FP64 dot.
//
// Design: reduce-then-scan everywhere (no inter-block spin waits).  The radix
// sort is the classic three-kernel pass (tile digit histograms, one scan of the
// [digit][tile] count matrix, stable scatter); within a tile, ranks come from
// __match_any_sync over 32 consecutive keys, warp-private digit counters and a
// cross-warp prefix, so equal keys keep their input order.  Stability is what
// makes the spatial hash bit-identical to the reference's sequential counting
// sort (src/cpu/hash.cpp:36-48).
#include "vpmc_internal.cuh"

namespace vpmc {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;   // 4096

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;                          // per thread
constexpr int kSortTile = kSortThreads * kSortItems;    // 4096
constexpr int kWarpSpan = 32 * kSortItems;              // 512 consecutive keys per warp

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix, *total receives the block sum.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* warp_tot, uint32_t* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t w = lane < nw ? warp_tot[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nw) warp_tot[lane] = wi - w;
        if (lane == nw - 1) warp_tot[32] = wi;
    }
    __syncthreads();
    const uint32_t res = warp_tot[wid] + inc - v;
    *total = warp_tot[32];
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t* __restrict__ in, long n,
                                                              uint32_t* __restrict__ sums) {
    __shared__ uint32_t wt[33];
    const long base = long(blockIdx.x) * kScanTile;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long e = base + long(i) * kScanThreads + threadIdx.x;
        if (e < n) s += in[e];
    }
    uint32_t tot;
    (void)block_exclusive(s, wt, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const uint32_t* in, uint32_t* out, long n,
                                                             const uint32_t* __restrict__ offs,
                                                             int write_total) {
    __shared__ uint32_t wt[33];
    const long base = long(blockIdx.x) * kScanTile + long(threadIdx.x) * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long e = base + i;
        v[i] = e < n ? in[e] : 0u;
        s += v[i];
    }
    uint32_t tot;
    uint32_t run = block_exclusive(s, wt, &tot) + (offs ? offs[blockIdx.x] : 0u);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long e = base + i;
        if (e < n) out[e] = run;
        run += v[i];
        if (write_total && e == n - 1) out[n] = run;
    }
}

__global__ void __launch_bounds__(kSortThreads) k_radix_upsweep(const uint32_t* __restrict__ keys, long n,
                                                                int shift, uint32_t mask,
                                                                uint32_t* __restrict__ counts, int ntiles) {
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const long base = long(blockIdx.x) * kSortTile;
#pragma unroll 4
    for (int i = 0; i < kSortItems; ++i) {
        const long e = base + long(i) * kSortThreads + threadIdx.x;
        if (e < n) atomicAdd(&hist[(keys[e] >> shift) & mask], 1u);
    }
    __syncthreads();
    if (threadIdx.x <= mask) counts[long(threadIdx.x) * ntiles + blockIdx.x] = hist[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) k_radix_downsweep(
    const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
    uint32_t* __restrict__ vout, long n, int shift, uint32_t mask, const uint32_t* __restrict__ offs,
    int ntiles) {
    __shared__ uint32_t wh[kSortWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortThreads) (&wh[0][0])[i] = 0;
    __syncthreads();
    const long base = long(blockIdx.x) * kSortTile + long(w) * kWarpSpan;
    const uint32_t lt = lanemask_lt();
    uint32_t k[kSortItems], v[kSortItems], lr[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const long e = base + long(r) * 32 + lane;
        const bool valid = e < n;
        k[r] = valid ? kin[e] : 0u;
        v[r] = valid ? (vin ? vin[e] : uint32_t(e)) : 0u;
        const uint32_t d = (k[r] >> shift) & mask;
        const uint32_t act = __ballot_sync(0xffffffffu, valid);
        uint32_t peers = 0, rank = 0, b = 0;
        if (valid) {
            peers = __match_any_sync(act, d);
            rank = __popc(peers & lt);
            b = wh[w][d];
        }
        __syncwarp();
        if (valid && rank == 0) wh[w][d] = b + __popc(peers);
        __syncwarp();
        lr[r] = b + rank;
    }
    __syncthreads();
    if (threadIdx.x <= mask) {
        uint32_t run = offs[long(threadIdx.x) * ntiles + blockIdx.x];
#pragma unroll
        for (int q = 0; q < kSortWarps; ++q) {
            const uint32_t c = wh[q][threadIdx.x];
            wh[q][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const long e = base + long(r) * 32 + lane;
        if (e < n) {
            const uint32_t p = wh[w][(k[r] >> shift) & mask] + lr[r];
            kout[p] = k[r];
            vout[p] = v[r];
        }
    }
}

constexpr int kDotThreads = 256;
constexpr int kDotMaxBlocks = 1024;

__global__ void __launch_bounds__(kDotThreads) k_dot_partial(const double* __restrict__ a,
                                                             const double* __restrict__ b, long n,
                                                             double* __restrict__ part) {
    __shared__ double sh[kDotThreads];
    double s = 0.0;
    for (long i = long(blockIdx.x) * kDotThreads + threadIdx.x; i < n; i += long(gridDim.x) * kDotThreads)
        s += b ? a[i] * b[i] : a[i] * a[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = kDotThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kDotMaxBlocks) k_dot_final(const double* __restrict__ part, int nb,
                                                             double* __restrict__ out) {
    __shared__ double sh[kDotMaxBlocks];
    sh[threadIdx.x] = threadIdx.x < nb ? part[threadIdx.x] : 0.0;
    __syncthreads();
    for (int o = kDotMaxBlocks / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = sh[0];
}

int dot_blocks(long n) {
    long b = (n + 4 * kDotThreads - 1) / (4 * kDotThreads);
    return int(b < 1 ? 1 : (b > kDotMaxBlocks ? kDotMaxBlocks : b));
}

}  // namespace

size_t scan_tmp_elems(long n) {
    const long nb = (n + kScanTile - 1) / kScanTile;
    if (nb <= 1) return 0;
    return size_t(2 * nb) + scan_tmp_elems(nb) + 64;
}

int exclusive_scan(vpmc_context* ctx, const uint32_t* in, uint32_t* out, long n, uint32_t* tmp,
                   bool write_total) {
    if (n <= 0) {
        if (write_total) VPMC_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), ctx->stream));
        return VPMC_OK;
    }
    const long nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        VPMC_LAUNCH(k_scan_apply, 1, kScanThreads, 0, ctx->stream, in, out, n, nullptr, write_total ? 1 : 0);
        return VPMC_OK;
    }
    uint32_t* sums = tmp;
    uint32_t* offs = tmp + nb;
    VPMC_LAUNCH(k_scan_reduce, unsigned(nb), kScanThreads, 0, ctx->stream, in, n, sums);
    VPMC_TRY(exclusive_scan(ctx, sums, offs, nb, tmp + 2 * nb, false));
    VPMC_LAUNCH(k_scan_apply, unsigned(nb), kScanThreads, 0, ctx->stream, in, out, n, offs,
                write_total ? 1 : 0);
    return VPMC_OK;
}

size_t radix_counts_elems(long n) {
    const long t = (n + kSortTile - 1) / kSortTile;
    return size_t(256) * size_t(t < 1 ? 1 : t);
}

void carve_radix(Carver& c, long n, RadixScratch* rs) {
    const size_t m = size_t(n < 1 ? 1 : n);
    rs->kbuf[0] = c.take<uint32_t>(m);
    rs->kbuf[1] = c.take<uint32_t>(m);
    rs->vbuf[0] = c.take<uint32_t>(m);
    rs->vbuf[1] = c.take<uint32_t>(m);
    const size_t ce = radix_counts_elems(n);
    rs->counts = c.take<uint32_t>(ce);
    rs->scan_tmp = c.take<uint32_t>(scan_tmp_elems(long(ce)) + 1);
}

int radix_sort(vpmc_context* ctx, const uint32_t* keys_in, const uint32_t* vals_in, long n, int key_bits,
               const RadixScratch& rs, uint32_t** keys_out, uint32_t** vals_out) {
    if (key_bits < 1) key_bits = 1;
    if (key_bits > 32) return VPMC_ERR_INVALID;
    const int passes = (key_bits + 7) / 8;
    const int dbits = (key_bits + passes - 1) / passes;
    const uint32_t mask = (dbits >= 32) ? 0xffffffffu : ((1u << dbits) - 1u);
    const long ntiles = (n + kSortTile - 1) / kSortTile;
    const uint32_t* kc = keys_in;
    const uint32_t* vc = vals_in;
    *keys_out = rs.kbuf[0];
    *vals_out = rs.vbuf[0];
    if (n <= 0) return VPMC_OK;
    for (int p = 0; p < passes; ++p) {
        const int shift = p * dbits;
        VPMC_LAUNCH(k_radix_upsweep, unsigned(ntiles), kSortThreads, 0, ctx->stream, kc, n, shift, mask,
                    rs.counts, int(ntiles));
        const long ce = long(mask + 1) * ntiles;
        VPMC_TRY(exclusive_scan(ctx, rs.counts, rs.counts, ce, rs.scan_tmp, false));
        uint32_t* ko = rs.kbuf[p & 1];
        uint32_t* vo = rs.vbuf[p & 1];
        VPMC_LAUNCH(k_radix_downsweep, unsigned(ntiles), kSortThreads, 0, ctx->stream, kc, vc, ko, vo, n, shift,
                    mask, rs.counts, int(ntiles));
        kc = ko;
        vc = vo;
    }
    *keys_out = const_cast<uint32_t*>(kc);
    *vals_out = const_cast<uint32_t*>(vc);
    return VPMC_OK;
}

size_t dot_tmp_elems(long n) { return size_t(dot_blocks(n)) + 1; }

int dot_f64(vpmc_context* ctx, const double* a, const double* b, long n, double* out_dev, double* tmp) {
    const int nb = dot_blocks(n);
    VPMC_LAUNCH(k_dot_partial, nb, kDotThreads, 0, ctx->stream, a, b, n, tmp);
    VPMC_LAUNCH(k_dot_final, 1, kDotMaxBlocks, 0, ctx->stream, tmp, nb, out_dev);
    return VPMC_OK;
}

}  // namespace vpmc
