// vpmc_context.cu -- context, scratch memory, error reporting, small host utilities.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "vpmc_internal.cuh"

namespace vpmc {

static std::atomic<uint64_t> g_launches{0};
static thread_local char g_last_error[512] = {0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int context_release(vpmc_context* c) {
    if (c->refs.fetch_sub(1) > 1) return VPMC_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& b : c->scratch) b.release();
    if (c->d_flags) cudaFree(c->d_flags);
    if (c->h_flags) cudaFreeHost(c->h_flags);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return VPMC_OK;
}

void record_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s:%d)", cudaGetErrorString(e), what, file,
                  line);
}

int DevBuf::reserve(size_t b) {
    if (b <= bytes && p) return VPMC_OK;
    release();
    size_t want = b < 256 ? 256 : b;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, want);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        record_cuda_error(e, "cudaMalloc", __FILE__, __LINE__);
        return VPMC_ERR_NOMEM;
    }
    p = q;
    bytes = want;
    return VPMC_OK;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

int scratch(vpmc_context* ctx, int slot, size_t bytes, char** base) {
    if (slot < 0 || slot >= kScratchSlots) return VPMC_ERR_INVALID;
    DevBuf& b = ctx->scratch[slot];
    if (bytes > b.bytes) {
        // growing frees the old block: wait for work that may still use it
        VPMC_CUDA(cudaStreamSynchronize(ctx->stream));
        VPMC_TRY(b.reserve(bytes + bytes / 4));
    }
    *base = static_cast<char*>(b.p);
    return VPMC_OK;
}

int collect_flags(vpmc_context* ctx) {
    VPMC_CUDA(cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    VPMC_CUDA(cudaStreamSynchronize(ctx->stream));
    const unsigned f = *ctx->h_flags;
    if (f) {
        VPMC_CUDA(cudaMemsetAsync(ctx->d_flags, 0, sizeof(unsigned), ctx->stream));
        VPMC_CUDA(cudaStreamSynchronize(ctx->stream));
        if (f & FLAG_TIMEOUT) return VPMC_ERR_TIMEOUT;
        if (f & FLAG_CAPACITY) return VPMC_ERR_CAPACITY;
        if (f & FLAG_NONFINITE) return VPMC_ERR_NONFINITE;
        return VPMC_ERR_DEVICE;
    }
    return VPMC_OK;
}

int bits_for(uint64_t max_exclusive) {
    int b = 0;
    while (b < 64 && (uint64_t(1) << b) < max_exclusive) ++b;
    return b < 1 ? 1 : b;
}

}  // namespace vpmc

using namespace vpmc;

extern "C" {

int vpmc_abi_version(void) { return VPMC_ABI_VERSION; }

uint64_t vpmc_kernel_launch_count(void) { return g_launches.load(); }

const char* vpmc_status_string(int s) {
    switch (s) {
        case VPMC_OK: return "ok";
        case VPMC_ERR_INVALID: return "invalid argument";
        case VPMC_ERR_UNSUPPORTED: return "unsupported (this library runs on the GPU only)";
        case VPMC_ERR_CUDA: return g_last_error[0] ? g_last_error : "CUDA error";
        case VPMC_ERR_NOMEM: return "device allocation failed";
        case VPMC_ERR_TIMEOUT: return "bounded device wait expired";
        case VPMC_ERR_DEVICE: return "device-side check failed";
        case VPMC_ERR_GEOMETRY: return "domain too small for the neighbour walk";
        case VPMC_ERR_CAPACITY: return "size exceeds a fixed capacity";
        case VPMC_ERR_NOT_CONVERGED: return "iterative solve did not reach its tolerance";
        case VPMC_ERR_NONFINITE: return "non-finite value";
        default: return "unknown status";
    }
}

int vpmc_context_create(int device, void* stream, vpmc_context** out) {
    if (!out) return VPMC_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    VPMC_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(device));
    auto* c = new (std::nothrow) vpmc_context();
    if (!c) return VPMC_ERR_NOMEM;
    c->device = device;
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) { delete c; record_cuda_error(e, "props", __FILE__, __LINE__); return VPMC_ERR_CUDA; }
    c->sm_count = prop.multiProcessorCount;
    c->smem_optin = prop.sharedMemPerBlockOptin;
    if (stream) {
        c->stream = static_cast<cudaStream_t>(stream);
    } else {
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete c; record_cuda_error(e, "stream", __FILE__, __LINE__); return VPMC_ERR_CUDA; }
        c->own_stream = true;
    }
    if (cudaMalloc(&c->d_flags, sizeof(unsigned)) != cudaSuccess ||
        cudaMallocHost(&c->h_flags, sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(c->d_flags, 0, sizeof(unsigned)) != cudaSuccess) {
        vpmc_context_destroy(c);
        return VPMC_ERR_NOMEM;
    }
    *c->h_flags = 0;
    *out = c;
    return VPMC_OK;
}

int vpmc_context_destroy(vpmc_context* c) {
    if (!c) return VPMC_ERR_INVALID;
    return vpmc::context_release(c);
}


void* vpmc_context_stream(vpmc_context* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

int vpmc_context_set_wait_limit(vpmc_context* c, uint32_t polls) {
    if (!c) return VPMC_ERR_INVALID;
    c->wait_limit = polls;
    return VPMC_OK;
}

int vpmc_context_sync(vpmc_context* c) {
    if (!c) return VPMC_ERR_INVALID;
    VPMC_CUDA(cudaSetDevice(c->device));
    VPMC_CUDA(cudaStreamSynchronize(c->stream));
    return collect_flags(c);
}

size_t vpmc_context_scratch_bytes(vpmc_context* c) {
    if (!c) return 0;
    size_t s = 0;
    for (auto& b : c->scratch) s += b.bytes;
    return s;
}

void vpmc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    U4 c{ctr[0], ctr[1], ctr[2], ctr[3]};
    U4 r = philox4x32_10(c, key[0], key[1]);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
}

float vpmc_cubic_spline(float r, float h_w) { return spline_w(r, h_w); }

// build_cubic_rcdf + cdf_to_icdf (src/utilities.cu:12-96), same FP32 steps as
// the reference's CPU branch: midpoint samples of r*W(r), running sum,
// normalisation, then piecewise-linear inversion at bin centres scaled by h_w.
int vpmc_kernel_icdf_table(float h_w, int L, float* cdf, float* icdf) {
    if (L < 1 || !cdf || !(h_w > 0.f)) return VPMC_ERR_INVALID;
    const float h_a = h_w / L;
    float acc = 0.f;
    for (int i = 0; i < L; ++i) {
        const float x = (0.5f + i) * h_a;
        acc += spline_w(x, h_w) * x;
        cdf[i] = acc;
    }
    const float total = cdf[L - 1];
    for (int i = 0; i < L; ++i) cdf[i] /= total;
    if (!icdf) return VPMC_OK;
    const float dh = 1.f / L;
    for (int i = 0; i < L; ++i) {
        const float u = (i + 0.5f) * dh;
        int ptr = 0;
        while (ptr < L && u > cdf[ptr]) ++ptr;
        float idx;
        if (ptr == 0) {
            const float lam = (cdf[0] - u) / cdf[0];
            idx = (1 - lam) * 0.5f;
        } else if (ptr == L) {
            const float lam = (1 - u) / (1 - cdf[L - 1]);
            idx = (1 - lam) * (L - 0.5f);
        } else {
            const float lam = (cdf[ptr] - u) / (cdf[ptr] - cdf[ptr - 1]);
            idx = (1 - lam) * (ptr + 0.5f) + lam * (ptr - 0.5f);
        }
        icdf[i] = idx * dh * h_w;
    }
    return VPMC_OK;
}

}  // extern "C"
