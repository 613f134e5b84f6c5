// vpmc_internal.cuh -- shared internals of the sm_103a vortex-particle MC library.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdint>

#include "vpmc.h"

// ---------------------------------------------------------------- error plumbing
#define VPMC_CUDA(call)                                                        \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            vpmc::record_cuda_error(e_, #call, __FILE__, __LINE__);            \
            return e_ == cudaErrorMemoryAllocation ? VPMC_ERR_NOMEM            \
                                                   : VPMC_ERR_CUDA;            \
        }                                                                      \
    } while (0)

#define VPMC_TRY(call)                                                         \
    do {                                                                       \
        int s_ = (call);                                                       \
        if (s_ != VPMC_OK) return s_;                                          \
    } while (0)

// Every kernel launch in the library goes through this: counts it and checks
// the launch error.
#define VPMC_LAUNCH(kernel, grid, block, smem, stream, ...)                    \
    do {                                                                       \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);            \
        vpmc::count_launch();                                                  \
        VPMC_CUDA(cudaGetLastError());                                         \
    } while (0)

namespace vpmc {

void record_cuda_error(cudaError_t e, const char* what, const char* file, int line);
void count_launch();

// Device-side error flag bits (context flag word).
enum : unsigned {
    FLAG_TIMEOUT = 1u << 0,   // a bounded mbarrier wait expired
    FLAG_CAPACITY = 1u << 1,  // more data than a fixed buffer holds
    FLAG_INTERNAL = 1u << 2,  // an index check failed
    FLAG_NONFINITE = 1u << 3,
};

// Growable device buffer (cudaMalloc; freed on growth / destruction).
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    int reserve(size_t b);
    void release();
};

// Bump allocator over one DevBuf: a dry run (base == nullptr) sizes it.
struct Carver {
    char* base = nullptr;
    size_t off = 0;
    template <class T>
    T* take(size_t n) {
        off = (off + 255) & ~size_t(255);
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += n * sizeof(T) + 16;
        return p;
    }
};

constexpr int kScratchSlots = 8;
enum ScratchSlot { SLOT_HASH = 0, SLOT_QUERY = 1, SLOT_CG = 2, SLOT_DIRECT = 3, SLOT_MISC = 4 };

}  // namespace vpmc

struct vpmc_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sm_count = 0;
    size_t smem_optin = 0;
    vpmc::DevBuf scratch[vpmc::kScratchSlots];
    unsigned* d_flags = nullptr;   // device error flags
    unsigned* h_flags = nullptr;   // pinned mirror
    uint32_t wait_limit = VPMC_WAIT_LIMIT_DEFAULT;   // polls of a staging wait before it gives up
    // holders: the creator plus every simulation bound to the context; the
    // context is freed when the last one lets go (so destroying a context
    // before its simulations, as a garbage collector may, stays safe)
    std::atomic<int> refs{1};
};

namespace vpmc {

// Drop one holder of the context; the last one frees it.
int context_release(vpmc_context* ctx);
// Read and clear the device flag word (synchronises the stream).
int collect_flags(vpmc_context* ctx);
// Reserve a scratch slot of at least `bytes` and return its base.
int scratch(vpmc_context* ctx, int slot, size_t bytes, char** base);

// ----------------------------------------------------------------- sort / scan
// Stable LSD radix sort of (key, value) pairs by key, key < 2^key_bits.
// vals_in == nullptr means values 0..n-1.  The sorted pairs end up in
// (*keys_out, *vals_out), which point at one of the two ping-pong buffers.
struct RadixScratch {
    uint32_t* kbuf[2];
    uint32_t* vbuf[2];
    uint32_t* counts;     // radix_counts_elems
    uint32_t* scan_tmp;   // scan_tmp_elems(radix_counts_elems)
};
size_t radix_counts_elems(long n);
size_t scan_tmp_elems(long n);
void carve_radix(Carver& c, long n, RadixScratch* rs);
int radix_sort(vpmc_context* ctx, const uint32_t* keys_in, const uint32_t* vals_in, long n,
               int key_bits, const RadixScratch& rs, uint32_t** keys_out, uint32_t** vals_out);
// out[0..n) = exclusive prefix of in; out[n] = total when write_total.
int exclusive_scan(vpmc_context* ctx, const uint32_t* in, uint32_t* out, long n, uint32_t* tmp,
                   bool write_total);
int bits_for(uint64_t max_value_exclusive);

// ---------------------------------------------------------- deterministic FP64
// out[0] = sum_i a[i]*b[i] (b == nullptr: sum a[i]^2), fixed reduction tree.
int dot_f64(vpmc_context* ctx, const double* a, const double* b, long n, double* out_dev,
            double* tmp /* >= dot_tmp_elems(n) */);
size_t dot_tmp_elems(long n);

}  // namespace vpmc

// ================================================================ device side
#ifdef __CUDACC__
namespace vpmc {

constexpr float kPiF = 3.14159265358979323846f;
constexpr double kPiD = 3.14159265358979323846;

// floor(v) -> int with saturation, NaN -> 0 (cvt.rmi.s32.f32 semantics).
__device__ __forceinline__ int floor_int(float v) { return __float2int_rd(v); }

// Cubic B-spline W(r; h) exactly as include/utilities.hpp:7-17 (FP32 order).
__host__ __device__ __forceinline__ float spline_w(float r, float hw) {
    const float pi = 3.141592653589793f;
    const float sigma = 40.f / (7.f * pi * hw * hw);
    const float q = r / hw;
    if (q >= 0.f && q <= 0.5f) { const float qq = q * q; return sigma * (6.f * (qq * q - qq) + 1.f); }
    if (q > 0.5f && q < 1.f) { const float t = 1.f - q; return sigma * 2.f * t * t * t; }
    return 0.f;
}

__host__ __device__ __forceinline__ double spline_w_d(double r, double hw) {
    const double sigma = 40.0 / (7.0 * kPiD * hw * hw);
    const double q = r / hw;
    if (q <= 0.5) return sigma * (6.0 * (q * q * q - q * q) + 1.0);
    if (q < 1.0) { const double t = 1.0 - q; return sigma * 2.0 * t * t * t; }
    return 0.0;
}

// Spline mass inside q*h (radial CDF of 2 pi r W).
__host__ __device__ __forceinline__ double spline_mass_d(double q) {
    if (q <= 0.0) return 0.0;
    if (q >= 1.0) return 1.0;
    const double c = 80.0 / 7.0;
    const double q2 = q * q;
    if (q <= 0.5) return c * (1.2 * q2 * q2 * q - 1.5 * q2 * q2 + 0.5 * q2);
    const double g = q2 - 2.0 * q2 * q + 1.5 * q2 * q2 - 0.4 * q2 * q2 * q;
    return c * (0.06875 + g - 0.08125);
}

// Largest singular value of F = [[F.x, F.y], [F.z, F.w]]: the square root of
// the largest eigenvalue of F^T F (how far a deformed kernel W(|F^-1 d|)
// reaches, in units of h_w).
__host__ __device__ __forceinline__ float sigma_max(float4 F) {
    const double T = double(F.x) * F.x + double(F.y) * F.y + double(F.z) * F.z + double(F.w) * F.w;
    const double d = double(F.x) * F.w - double(F.y) * F.z;
    const double disc = T * T - 4.0 * d * d;
    const double l = 0.5 * (T + sqrt(disc > 0.0 ? disc : 0.0));
    return float(sqrt(l));
}

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -------------------------
struct U4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return uint32_t((uint64_t(a) * uint64_t(b)) >> 32);
#endif
}

__host__ __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
    constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = M0 * c.x, hi0 = mulhi32(M0, c.x);
        const uint32_t lo1 = M1 * c.z, hi1 = mulhi32(M1, c.z);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// 32 random bits -> float strictly inside (0,1).
__host__ __device__ __forceinline__ float u01(uint32_t r) {
    return (float(r >> 8) + 0.5f) * (1.0f / 16777216.0f);
}
// 32 random bits -> double strictly inside (0,1).
__host__ __device__ __forceinline__ double u01d(uint32_t r) {
    return (double(r) + 0.5) * (1.0 / 4294967296.0);
}

// ---- bounded mbarrier / bulk-copy helpers (sm_90+ PTX) -------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
// Wait with an iteration cap; false on expiry (caller flags VPMC_ERR_TIMEOUT).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t max_iter) {
    for (uint32_t i = 0; i < max_iter; ++i)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}
// 1-D bulk copy global -> shared (TMA engine), completion on `bar`.
// dst/src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Kahan / TwoSum helpers for compensated FP32 sums.
struct KSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};
// Exact TwoSum: a + b = s + e.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// Warp-wide compensated reduction of (s, c) pairs (fixed tree); all lanes get it.
// The same over aligned groups of G lanes (G a power of two <= 32); every lane
// of the warp must take part.
template <int G>
__device__ __forceinline__ void group_sum_comp_pair(float& s, float& c) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
        const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
        float t, e;
        const bool lo = (threadIdx.x & o) == 0;
        two_sum(lo ? s : s2, lo ? s2 : s, t, e);
        c = (lo ? c + c2 : c2 + c) - e;
        s = t;
    }
}
template <int G>
__device__ __forceinline__ float group_sum_comp(float s, float c) {
    group_sum_comp_pair<G>(s, c);
    return s - c;
}
// (sa - ca) - (sb - cb) of two compensated sums, the difference of the
// leading parts taken exactly: no cancellation error when the two sums are
// large and nearly equal (the two sign estimates of a velocity).
__device__ __forceinline__ float comp_diff(float sa, float ca, float sb, float cb) {
    float d, e;
    two_sum(sa, -sb, d, e);
    return d + (e - (ca - cb));
}
__device__ __forceinline__ float warp_sum_comp(float s, float c) {
    // order-independent pairing: combine (min lane, max lane) consistently
    group_sum_comp_pair<32>(s, c);
    return s - c;
}

}  // namespace vpmc
#endif  // __CUDACC__
