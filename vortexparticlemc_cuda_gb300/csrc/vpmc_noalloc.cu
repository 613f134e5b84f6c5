// vpmc_noalloc.cu -- spatial hash build that allocates no memory.
//
// Some callers cannot allocate device memory: a host application that owns
// every byte of device memory through its own pool and forbids plugins from
// calling cudaMalloc, or a real-time loop that cannot afford cudaMalloc's
// implicit device synchronisation.  vpmc_hash_build_noalloc serves them: the
// caller passes inputs and outputs, and the radix-sort and scan scratch lives
// in one file-scope __device__ array of fixed size (kScratchBytes, about
// 4.3 MB), which every GPU that loads this library holds until the process
// exits.  Sizes beyond the array's capacity are rejected with
// VPMC_ERR_CAPACITY.
//
// The array is shared by every call: a call overwrites what the previous one
// left (nothing in it needs to start at zero), and two calls that overlap on
// the GPU (different host threads or streams) race on it.  Every call waits
// for its stream to finish before it returns -- also when it fails after
// issuing work -- so consecutive calls from one thread are safe.  The first
// call on a device looks up the array's device address (cudaGetSymbolAddress)
// and keeps it for the life of the process; make that first call before any
// stream capture.  The kept address belongs to the device's primary context:
// after cudaDeviceReset, or under another context of the same device, it is
// stale, so such callers must not use this entry point.  The stream must
// belong to the current device (VPMC_ERR_INVALID otherwise).
#include <mutex>

#include "vpmc_internal.cuh"

namespace vpmc {
int launch_fill_cells(cudaStream_t st, int rshx, int rshy, float inv_hx, float inv_hy, const int* sub,
                      const float2* pos, long N, int* cell_num, int* vp_cell);
}

namespace {

constexpr long kMaxN = 1L << 18;        // particles per call (262,144)
constexpr long kMaxCells = 1L << 20;    // rshx * rshy
// radix ping-pong keys/values (4 x kMaxN x 4 B) + digit counts + scan scratch + slack
constexpr size_t kScratchBytes = size_t(4) * kMaxN * 4 + size_t(256) * (kMaxN / 4096) * 4 + (size_t(1) << 16) +
                                 (size_t(1) << 13);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_addr[64] = {};

// Device address of the scratch array on the current device (looked up once
// per device; the symbol name is only a host-side stand-in).
int scratch_address(int dev, void** out) {
    if (dev < 0 || dev >= 64) return VPMC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            vpmc::record_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
            return VPMC_ERR_CUDA;
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return VPMC_OK;
}

}  // namespace

using namespace vpmc;

extern "C" int vpmc_hash_build_noalloc(void* stream, int rshx, int rshy, float Lx, float Ly, int N, const int* sub,
                                       const float* pos, int* cell_num, int* cell_acc, int* vp_cell, int* vp_sort) {
    if (rshx < 1 || rshy < 1 || N < 0 || !(Lx > 0.f) || !(Ly > 0.f) || !cell_num || !cell_acc) return VPMC_ERR_INVALID;
    if (N > 0 && (!pos || !vp_cell || !vp_sort)) return VPMC_ERR_INVALID;
    if (long(N) > kMaxN || long(rshx) * long(rshy) > kMaxCells) return VPMC_ERR_CAPACITY;
    int dev = 0;
    VPMC_CUDA(cudaGetDevice(&dev));
    int sdev = dev;
    VPMC_CUDA(cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &sdev));
    if (sdev != dev) return VPMC_ERR_INVALID;   // the scratch array used is the current device's
    void* base = nullptr;
    VPMC_TRY(scratch_address(dev, &base));

    // carve the fixed array exactly like the context path carves its scratch
    const long ncell = long(rshx) * rshy;
    RadixScratch rs;
    Carver c{static_cast<char*>(base), 0};
    carve_radix(c, kMaxN, &rs);
    uint32_t* cell_tmp = c.take<uint32_t>(scan_tmp_elems(ncell) + 1);
    (void)cell_tmp;
    if (c.off > kScratchBytes) return VPMC_ERR_CAPACITY;

    vpmc_context local;   // stream holder only: no allocation, no flags
    local.device = dev;
    local.stream = static_cast<cudaStream_t>(stream);
    cudaStream_t st = local.stream;
    // from here on work is queued: whatever the outcome, the call returns only
    // once the stream has drained, so no queued kernel still uses the shared
    // scratch when the next call starts
    struct DrainOnExit {
        cudaStream_t st;
        ~DrainOnExit() { (void)cudaStreamSynchronize(st); }
    } drain{st};

    VPMC_CUDA(cudaMemsetAsync(cell_num, 0, sizeof(int) * size_t(ncell), st));
    const float inv_hx = rshx / Lx;   // FillCells_cpu's FP32 expressions
    const float inv_hy = rshy / Ly;
    VPMC_TRY(launch_fill_cells(st, rshx, rshy, inv_hx, inv_hy, sub, reinterpret_cast<const float2*>(pos), long(N),
                               cell_num, vp_cell));
    VPMC_TRY(exclusive_scan(&local, reinterpret_cast<const uint32_t*>(cell_num), reinterpret_cast<uint32_t*>(cell_acc),
                            ncell, cell_tmp, false));
    if (N > 0) {
        uint32_t *ks = nullptr, *vs = nullptr;
        VPMC_TRY(radix_sort(&local, reinterpret_cast<const uint32_t*>(vp_cell), nullptr, N,
                            bits_for(uint64_t(ncell)), rs, &ks, &vs));
        VPMC_CUDA(cudaMemcpyAsync(vp_sort, vs, sizeof(int) * size_t(N), cudaMemcpyDeviceToDevice, st));
    }
    // CountingSort leaves cell_num at zero (src/cpu/hash.cpp:36-48)
    VPMC_CUDA(cudaMemsetAsync(cell_num, 0, sizeof(int) * size_t(ncell), st));
    VPMC_CUDA(cudaStreamSynchronize(st));
    return VPMC_OK;
}
