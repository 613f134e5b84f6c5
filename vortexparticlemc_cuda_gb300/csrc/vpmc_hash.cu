// vpmc_hash.cu -- the reference-shaped spatial hash (FillCells / CountingSort)
// and the sign subsets with their FP64 |omega| CDFs.
//
// Hash: one key kernel (cell of sub[i], histogram into cell_num), an exclusive
// scan (cell_acc), and a stable radix sort of (cell, local index) pairs, whose
// values are vp_sort.  The result equals the reference's sequential counting
// sort (src/cpu/hash.cpp:36-48) bit for bit: members of a cell ascend by local
// index.  The reference's CUDA scatter (src/cuda/hash.cu:27-39) uses atomicSub
// and is order-nondeterministic; this one is deterministic.
#include <vector>

#include "vpmc_internal.cuh"

namespace vpmc {
namespace {

constexpr int kHashThreads = 256;
constexpr int kPrivCells = 4096;   // histogram privatised in shared memory up to this many cells

int blocks_for(long n) {
    long b = (n + kHashThreads - 1) / kHashThreads;
    if (b < 1) b = 1;
    if (b > 65535L * 8) b = 65535L * 8;
    return int(b);
}

// FillCells_kernel equivalent (src/cuda/hash.cu:6-25): same FP32 cell formula
// as FillCells_cpu (floor(x * (rshx/Lx)), clamp), histogram privatised per
// block when the grid is small.
__global__ void __launch_bounds__(kHashThreads) k_fill_cells(int rshx, int rshy, float inv_hx, float inv_hy,
                                                             const int* __restrict__ sub,
                                                             const float2* __restrict__ pos, long N,
                                                             int* __restrict__ cell_num,
                                                             int* __restrict__ vp_cell) {
    __shared__ int hist[kPrivCells];
    const int ncell = rshx * rshy;
    const bool priv = ncell <= kPrivCells;
    if (priv) {
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) hist[c] = 0;
        __syncthreads();
    }
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += long(gridDim.x) * blockDim.x) {
        const float2 p = pos[sub ? sub[i] : int(i)];
        const int ix = min(max(floor_int(p.x * inv_hx), 0), rshx - 1);
        const int iy = min(max(floor_int(p.y * inv_hy), 0), rshy - 1);
        const int c = ix * rshy + iy;
        vp_cell[i] = c;
        if (priv) atomicAdd(&hist[c], 1);
        else atomicAdd(&cell_num[c], 1);
    }
    if (priv) {
        __syncthreads();
        for (int c = threadIdx.x; c < ncell; c += blockDim.x)
            if (hist[c]) atomicAdd(&cell_num[c], hist[c]);
    }
}

__global__ void k_max_key(const int* __restrict__ keys, long n, int* __restrict__ out) {
    int m = -1;
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
        m = max(m, keys[i]);
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void k_check_keys(const int* __restrict__ keys, long n, int ncell, unsigned* flags) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
        if (keys[i] < 0 || keys[i] >= ncell) atomicOr(flags, FLAG_INTERNAL);
}

// ---- subsets: sign flags, stable compaction, FP64 prefix sums ----
__global__ void k_sign_flags(const float* __restrict__ om, long N, uint32_t* __restrict__ fpos,
                             uint32_t* __restrict__ fneg) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += long(gridDim.x) * blockDim.x) {
        const float w = om[i];
        fpos[i] = w > 0.f;
        fneg[i] = w < 0.f;
    }
}

__global__ void k_compact(const float* __restrict__ om, long N, const uint32_t* __restrict__ spos,
                          const uint32_t* __restrict__ sneg, int* __restrict__ sub_pos, int* __restrict__ sub_neg,
                          double* __restrict__ apos, double* __restrict__ aneg) {
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += long(gridDim.x) * blockDim.x) {
        const float w = om[i];
        if (w > 0.f) { sub_pos[spos[i]] = int(i); apos[spos[i]] = double(w); }
        else if (w < 0.f) { sub_neg[sneg[i]] = int(i); aneg[sneg[i]] = -double(w); }
    }
}

// Inclusive FP64 scan, deterministic: block partial sums (fixed partition) ->
// scan of block sums in one block -> per-block scan with offset.
constexpr int kD = 256, kDItems = 8, kDTile = kD * kDItems;

__global__ void __launch_bounds__(kD) k_dscan_reduce(const double* __restrict__ a, long n, double* __restrict__ bs) {
    __shared__ double sh[kD];
    const long base = long(blockIdx.x) * kDTile + long(threadIdx.x) * kDItems;
    double s = 0.0;
    for (int i = 0; i < kDItems; ++i) if (base + i < n) s += a[base + i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = kD / 2; o; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) bs[blockIdx.x] = sh[0];
}

__device__ double block_dscan_excl(double v, double* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    // Hillis-Steele inclusive in shared memory (fixed order, deterministic)
    for (int o = 1; o < kD; o <<= 1) {
        const double t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0.0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    const double inc = sh[threadIdx.x];
    __syncthreads();
    return inc - v;
}

__global__ void __launch_bounds__(kD) k_dscan_apply(const double* in, double* out, long n,
                                                    const double* __restrict__ offs, int inclusive) {
    __shared__ double sh[kD];
    const long base = long(blockIdx.x) * kDTile + long(threadIdx.x) * kDItems;
    double v[kDItems], s = 0.0;
    for (int i = 0; i < kDItems; ++i) { v[i] = base + i < n ? in[base + i] : 0.0; s += v[i]; }
    double run = block_dscan_excl(s, sh) + (offs ? offs[blockIdx.x] : 0.0);
    for (int i = 0; i < kDItems; ++i) {
        const double ex = run;
        run += v[i];
        if (base + i < n) out[base + i] = inclusive ? run : ex;
    }
}

__global__ void k_normalise(double* __restrict__ c, long n, const double* __restrict__ total,
                            float* __restrict__ c32) {
    const double t = *total;
    for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
        const double v = t > 0.0 ? c[i] / t : 0.0;
        c[i] = (i == n - 1 && t > 0.0) ? 1.0 : v;
        if (c32) c32[i] = float(c[i]);
    }
}

// Deterministic FP64 scan (fixed partition and tree): in-place allowed.
int dscan(vpmc_context* ctx, const double* in, double* out, long n, double* tmp, bool inclusive) {
    if (n <= 0) return VPMC_OK;
    const long nb = (n + kDTile - 1) / kDTile;
    if (nb == 1) {
        VPMC_LAUNCH(k_dscan_apply, 1, kD, 0, ctx->stream, in, out, n, nullptr, inclusive ? 1 : 0);
        return VPMC_OK;
    }
    double* sums = tmp;
    double* offs = tmp + nb;
    VPMC_LAUNCH(k_dscan_reduce, unsigned(nb), kD, 0, ctx->stream, in, n, sums);
    VPMC_TRY(dscan(ctx, sums, offs, nb, tmp + 2 * nb, false));
    VPMC_LAUNCH(k_dscan_apply, unsigned(nb), kD, 0, ctx->stream, in, out, n, offs, inclusive ? 1 : 0);
    return VPMC_OK;
}

size_t dscan_tmp_elems(long n) {
    const long nb = (n + kDTile - 1) / kDTile;
    if (nb <= 1) return 8;
    return size_t(2 * nb) + dscan_tmp_elems(nb) + 8;
}

}  // namespace

// FillCells kernel on a caller-given stream, no context and no allocation
// (used by the allocation-free hash entry point).  cell_num must be zeroed.
int launch_fill_cells(cudaStream_t st, int rshx, int rshy, float inv_hx, float inv_hy, const int* sub,
                      const float2* pos, long N, int* cell_num, int* vp_cell) {
    if (N <= 0) return VPMC_OK;
    VPMC_LAUNCH(k_fill_cells, blocks_for(N), kHashThreads, 0, st, rshx, rshy, inv_hx, inv_hy, sub, pos, N, cell_num,
                vp_cell);
    return VPMC_OK;
}

// Subset build shared with the simulation: writes sub/abs values, returns
// counts and totals (host), CDF normalised in place.  Device scratch from `c`.
int build_subsets_dev(vpmc_context* ctx, long N, const float* omega, int* sub_pos, int* sub_neg, double* cdf_pos,
                      double* cdf_neg, float* c32p, float* c32n, int* cnt, double* cum) {
    Carver dry;
    uint32_t* f[4];
    for (auto& p : f) p = dry.take<uint32_t>(size_t(N + 1));
    dry.take<uint32_t>(scan_tmp_elems(N + 1) + 1);
    dry.take<double>(dscan_tmp_elems(N) + 8);
    dry.take<double>(4);
    char* base = nullptr;
    VPMC_TRY(scratch(ctx, SLOT_MISC, dry.off, &base));
    Carver c{base, 0};
    for (auto& p : f) p = c.take<uint32_t>(size_t(N + 1));
    uint32_t* stmp = c.take<uint32_t>(scan_tmp_elems(N + 1) + 1);
    double* dtmp = c.take<double>(dscan_tmp_elems(N) + 8);
    double* tot = c.take<double>(4);
    cudaStream_t st = ctx->stream;
    VPMC_LAUNCH(k_sign_flags, blocks_for(N), kHashThreads, 0, st, omega, N, f[0], f[1]);
    VPMC_TRY(exclusive_scan(ctx, f[0], f[2], N, stmp, true));
    VPMC_TRY(exclusive_scan(ctx, f[1], f[3], N, stmp, true));
    uint32_t counts[2];
    VPMC_CUDA(cudaMemcpyAsync(&counts[0], f[2] + N, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    VPMC_CUDA(cudaMemcpyAsync(&counts[1], f[3] + N, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    VPMC_LAUNCH(k_compact, blocks_for(N), kHashThreads, 0, st, omega, N, f[2], f[3], sub_pos, sub_neg, cdf_pos,
                cdf_neg);
    VPMC_CUDA(cudaStreamSynchronize(st));
    cnt[0] = int(counts[0]);
    cnt[1] = int(counts[1]);
    double* cdfs[2] = {cdf_pos, cdf_neg};
    float* c32[2] = {c32p, c32n};
    for (int s = 0; s < 2; ++s) {
        const long n = cnt[s];
        if (n == 0) { cum[s] = 0.0; continue; }
        VPMC_TRY(dscan(ctx, cdfs[s], cdfs[s], n, dtmp, true));
        VPMC_CUDA(cudaMemcpyAsync(tot + s, cdfs[s] + n - 1, sizeof(double), cudaMemcpyDeviceToDevice, st));
        VPMC_LAUNCH(k_normalise, blocks_for(n), kHashThreads, 0, st, cdfs[s], n, tot + s, c32[s]);
    }
    double h[2] = {0.0, 0.0};
    VPMC_CUDA(cudaMemcpyAsync(h, tot, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
    VPMC_CUDA(cudaStreamSynchronize(st));
    for (int s = 0; s < 2; ++s) if (cnt[s] > 0) cum[s] = h[s];
    return VPMC_OK;
}

}  // namespace vpmc

using namespace vpmc;

namespace {

struct HashScratch {
    RadixScratch rs;
    uint32_t* cellacc_u = nullptr;
    int* maxkey = nullptr;
};

int hash_scratch(vpmc_context* ctx, long N, HashScratch* h) {
    Carver dry;
    carve_radix(dry, N, &h->rs);
    dry.take<int>(4);
    char* base = nullptr;
    VPMC_TRY(scratch(ctx, SLOT_HASH, dry.off, &base));
    Carver c{base, 0};
    carve_radix(c, N, &h->rs);
    h->maxkey = c.take<int>(4);
    return VPMC_OK;
}

int sort_cells(vpmc_context* ctx, long N, int ncell, const int* vp_cell, int* vp_sort) {
    HashScratch h;
    VPMC_TRY(hash_scratch(ctx, N, &h));
    uint32_t *ks = nullptr, *vs = nullptr;
    VPMC_TRY(radix_sort(ctx, reinterpret_cast<const uint32_t*>(vp_cell), nullptr, N, bits_for(uint64_t(ncell)), h.rs,
                        &ks, &vs));
    VPMC_CUDA(cudaMemcpyAsync(vp_sort, vs, sizeof(int) * size_t(N), cudaMemcpyDeviceToDevice, ctx->stream));
    return VPMC_OK;
}

}  // namespace

extern "C" {

int vpmc_fill_cells(vpmc_context* ctx, int rshx, int rshy, float Lx, float Ly, int N, const int* sub,
                    const float* pos, int* cell_num, int* cell_acc, int* vp_cell) {
    if (!ctx || rshx < 1 || rshy < 1 || N < 0 || !(Lx > 0.f) || !(Ly > 0.f)) return VPMC_ERR_INVALID;
    if ((N > 0 && (!pos || !vp_cell)) || !cell_num || !cell_acc) return VPMC_ERR_INVALID;
    if (long(rshx) * rshy > (1L << 30)) return VPMC_ERR_CAPACITY;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    const int ncell = rshx * rshy;
    cudaStream_t st = ctx->stream;
    VPMC_CUDA(cudaMemsetAsync(cell_num, 0, sizeof(int) * size_t(ncell), st));
    const float inv_hx = rshx / Lx;   // same FP32 expressions as the reference
    const float inv_hy = rshy / Ly;
    if (N > 0)
        VPMC_LAUNCH(k_fill_cells, blocks_for(N), kHashThreads, 0, st, rshx, rshy, inv_hx, inv_hy, sub,
                    reinterpret_cast<const float2*>(pos), long(N), cell_num, vp_cell);
    Carver dry;
    dry.take<uint32_t>(scan_tmp_elems(ncell) + 1);
    char* base = nullptr;
    VPMC_TRY(scratch(ctx, SLOT_MISC, dry.off, &base));
    VPMC_TRY(exclusive_scan(ctx, reinterpret_cast<const uint32_t*>(cell_num), reinterpret_cast<uint32_t*>(cell_acc),
                            ncell, reinterpret_cast<uint32_t*>(base), false));
    VPMC_CUDA(cudaStreamSynchronize(st));
    return collect_flags(ctx);
}

int vpmc_counting_sort(vpmc_context* ctx, int N, int ncell, int* cell_num, const int* cell_acc, const int* vp_cell,
                       int* vp_sort) {
    if (!ctx || N < 0 || (N > 0 && (!vp_cell || !vp_sort))) return VPMC_ERR_INVALID;
    (void)cell_acc;   // offsets are implied by the stable sort
    VPMC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    if (N == 0) return VPMC_OK;
    if (ncell <= 0) {
        HashScratch h;
        VPMC_TRY(hash_scratch(ctx, N, &h));
        int init = -1, mk = -1;
        VPMC_CUDA(cudaMemcpyAsync(h.maxkey, &init, sizeof(int), cudaMemcpyHostToDevice, st));
        VPMC_LAUNCH(k_max_key, blocks_for(N), kHashThreads, 0, st, vp_cell, long(N), h.maxkey);
        VPMC_CUDA(cudaMemcpyAsync(&mk, h.maxkey, sizeof(int), cudaMemcpyDeviceToHost, st));
        VPMC_CUDA(cudaStreamSynchronize(st));
        if (mk < 0) return VPMC_ERR_INVALID;
        ncell = mk + 1;
    } else {
        VPMC_LAUNCH(k_check_keys, blocks_for(N), kHashThreads, 0, st, vp_cell, long(N), ncell, ctx->d_flags);
    }
    VPMC_TRY(sort_cells(ctx, N, ncell, vp_cell, vp_sort));
    if (cell_num) VPMC_CUDA(cudaMemsetAsync(cell_num, 0, sizeof(int) * size_t(ncell), st));
    VPMC_CUDA(cudaStreamSynchronize(st));
    return collect_flags(ctx);
}

int vpmc_hash_build(vpmc_context* ctx, int rshx, int rshy, float Lx, float Ly, int N, const int* sub,
                    const float* pos, int* cell_num, int* cell_acc, int* vp_cell, int* vp_sort) {
    if (!ctx || rshx < 1 || rshy < 1 || N < 0 || !cell_acc || (N > 0 && (!pos || !vp_cell || !vp_sort)))
        return VPMC_ERR_INVALID;
    if (!(Lx > 0.f) || !(Ly > 0.f)) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    const int ncell = rshx * rshy;
    int* cn = cell_num;
    if (!cn) {
        // borrow scratch for the counts when the caller does not want them
        char* base = nullptr;
        VPMC_TRY(scratch(ctx, SLOT_QUERY, sizeof(int) * size_t(ncell) + 256, &base));
        cn = reinterpret_cast<int*>(base);
    }
    VPMC_TRY(vpmc_fill_cells(ctx, rshx, rshy, Lx, Ly, N, sub, pos, cn, cell_acc, vp_cell));
    if (N > 0) VPMC_TRY(sort_cells(ctx, N, ncell, vp_cell, vp_sort));
    VPMC_CUDA(cudaMemsetAsync(cn, 0, sizeof(int) * size_t(ncell), ctx->stream));
    VPMC_CUDA(cudaStreamSynchronize(ctx->stream));
    return collect_flags(ctx);
}

int vpmc_hash_build_host(vpmc_context* ctx, int rshx, int rshy, float Lx, float Ly, int N, int n_pos,
                         const int* sub, const float* pos, int* cell_num, int* cell_acc, int* vp_cell,
                         int* vp_sort) {
    if (!ctx || N < 0 || n_pos < 0 || rshx < 1 || rshy < 1 || !cell_acc) return VPMC_ERR_INVALID;
    if (N > 0 && (!pos || !vp_cell || !vp_sort)) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    const int ncell = rshx * rshy;
    void* d = nullptr;
    const size_t bytes = sizeof(float) * 2 * size_t(n_pos) + sizeof(int) * (size_t(N) * 3 + size_t(ncell) * 2) + 1024;
    VPMC_CUDA(cudaMalloc(&d, bytes));
    char* p = static_cast<char*>(d);
    auto take = [&](size_t b) { char* r = p; p += (b + 255) & ~size_t(255); return r; };
    float* dpos = reinterpret_cast<float*>(take(sizeof(float) * 2 * size_t(n_pos)));
    int* dsub = sub ? reinterpret_cast<int*>(take(sizeof(int) * size_t(N))) : nullptr;
    int* dcn = reinterpret_cast<int*>(take(sizeof(int) * size_t(ncell)));
    int* dca = reinterpret_cast<int*>(take(sizeof(int) * size_t(ncell)));
    int* dvc = reinterpret_cast<int*>(take(sizeof(int) * size_t(N)));
    int* dvs = reinterpret_cast<int*>(take(sizeof(int) * size_t(N)));
    cudaStream_t st = ctx->stream;
    int rc = VPMC_OK;
    if (n_pos > 0 && cudaMemcpyAsync(dpos, pos, sizeof(float) * 2 * size_t(n_pos), cudaMemcpyHostToDevice, st) != cudaSuccess) rc = VPMC_ERR_CUDA;
    if (rc == VPMC_OK && dsub && N > 0 && cudaMemcpyAsync(dsub, sub, sizeof(int) * size_t(N), cudaMemcpyHostToDevice, st) != cudaSuccess) rc = VPMC_ERR_CUDA;
    if (rc == VPMC_OK) rc = vpmc_hash_build(ctx, rshx, rshy, Lx, Ly, N, dsub, dpos, dcn, dca, dvc, dvs);
    if (rc == VPMC_OK) {
        if (cell_num) cudaMemcpyAsync(cell_num, dcn, sizeof(int) * size_t(ncell), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(cell_acc, dca, sizeof(int) * size_t(ncell), cudaMemcpyDeviceToHost, st);
        if (N > 0) {
            cudaMemcpyAsync(vp_cell, dvc, sizeof(int) * size_t(N), cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(vp_sort, dvs, sizeof(int) * size_t(N), cudaMemcpyDeviceToHost, st);
        }
        if (cudaStreamSynchronize(st) != cudaSuccess) rc = VPMC_ERR_CUDA;
    }
    cudaFree(d);
    return rc;
}

int vpmc_build_subsets(vpmc_context* ctx, int N, const float* omega, int* sub_pos, int* sub_neg, double* cdf_pos,
                       double* cdf_neg, float* cdf32_pos, float* cdf32_neg, int* cnt, double* cum) {
    if (!ctx || N < 0 || !cnt || !cum || (N > 0 && (!omega || !sub_pos || !sub_neg || !cdf_pos || !cdf_neg)))
        return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(ctx->device));
    if (N == 0) { cnt[0] = cnt[1] = 0; cum[0] = cum[1] = 0.0; return VPMC_OK; }
    VPMC_TRY(build_subsets_dev(ctx, N, omega, sub_pos, sub_neg, cdf_pos, cdf_neg, cdf32_pos, cdf32_neg, cnt, cum));
    return collect_flags(ctx);
}

}  // extern "C"
