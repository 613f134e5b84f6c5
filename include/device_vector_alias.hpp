// device_vector_alias.hpp -- containers of the C++ API (replaces the
// reference's include/device_vector_alias.hpp:24-75, where dvec<T> is a
// thrust::device_vector).  Here dvec<T> is a small RAII device buffer: the
// library's C ABI takes raw device pointers, so no Thrust is needed.
#pragma once

#include <cuda_runtime_api.h>
#include <vector_types.h>

#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "vpmc.h"

namespace vpmc {

// Error type of the C++ layer: every failing vpmc_* status becomes one.
struct error : std::runtime_error {
    int status;
    error(int s, const std::string& where)
        : std::runtime_error(where + ": " + vpmc_status_string(s)), status(s) {}
};

inline void check(int status, const char* where) {
    if (status != VPMC_OK) throw error(status, where);
}

inline void check_cuda(cudaError_t e, const char* where) {
    if (e != cudaSuccess) throw error(VPMC_ERR_CUDA, std::string(where) + " (" + cudaGetErrorString(e) + ")");
}

// Thrown by the reference's CPU/OMP entry points: this build runs on the GPU only.
struct unsupported : error {
    explicit unsupported(const char* what) : error(VPMC_ERR_UNSUPPORTED, what) {}
};

// Process-wide default context per device, used by the reference-shaped free
// functions that take no context (the reference issues everything on the
// default stream).  Each vpmc_* call completes before it returns, so work on
// the context's own stream is ordered with the synchronous copies dvec does.
inline vpmc_context* default_context() {
    static vpmc_context* ctx[64] = {};
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (!ctx[dev]) check(vpmc_context_create(dev, nullptr, &ctx[dev]), "vpmc_context_create");
    return ctx[dev];
}

}  // namespace vpmc

// Device vector: contiguous device memory of n elements of T.
template <typename T>
class dvec {
public:
    dvec() = default;
    explicit dvec(size_t n) { resize(n); }
    dvec(const dvec& o) { *this = o; }
    dvec(dvec&& o) noexcept { swap(o); }
    ~dvec() { release(); }
    dvec& operator=(const dvec& o) {
        if (this != &o) {
            resize(o.n_);
            if (n_) vpmc::check_cuda(cudaMemcpy(p_, o.p_, n_ * sizeof(T), cudaMemcpyDeviceToDevice), "dvec copy");
        }
        return *this;
    }
    dvec& operator=(dvec&& o) noexcept {
        swap(o);
        return *this;
    }
    void resize(size_t n) {
        if (n == n_) return;
        T* q = nullptr;
        if (n) vpmc::check_cuda(cudaMalloc(reinterpret_cast<void**>(&q), n * sizeof(T)), "dvec resize");
        if (n_ && n) vpmc::check_cuda(cudaMemcpy(q, p_, (n < n_ ? n : n_) * sizeof(T), cudaMemcpyDeviceToDevice),
                                      "dvec resize copy");
        release();
        p_ = q;
        n_ = n;
    }
    void clear() { release(); }
    size_t size() const { return n_; }
    bool empty() const { return n_ == 0; }
    T* data() { return p_; }
    const T* data() const { return p_; }
    // host <-> device helpers
    void assign(const std::vector<T>& h) {
        resize(h.size());
        if (n_) vpmc::check_cuda(cudaMemcpy(p_, h.data(), n_ * sizeof(T), cudaMemcpyHostToDevice), "dvec assign");
    }
    std::vector<T> to_host() const {
        std::vector<T> h(n_);
        if (n_) vpmc::check_cuda(cudaMemcpy(h.data(), p_, n_ * sizeof(T), cudaMemcpyDeviceToHost), "dvec to_host");
        return h;
    }
    void fill_zero() {
        if (n_) vpmc::check_cuda(cudaMemset(p_, 0, n_ * sizeof(T)), "dvec fill_zero");
    }
    void swap(dvec& o) noexcept {
        std::swap(p_, o.p_);
        std::swap(n_, o.n_);
    }

private:
    void release() {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }
    T* p_ = nullptr;
    size_t n_ = 0;
};

template <typename T>
T* raw_ptr(dvec<T>& v) { return v.data(); }
template <typename T>
const T* raw_ptr(const dvec<T>& v) { return v.data(); }

// float2 helpers the reference defines next to its containers
inline float2 operator+(float2 a, float2 b) { return {a.x + b.x, a.y + b.y}; }
inline float2 operator-(float2 a, float2 b) { return {a.x - b.x, a.y - b.y}; }
inline float2 operator*(float2 a, float s) { return {a.x * s, a.y * s}; }
inline float2 operator*(float s, float2 a) { return {s * a.x, s * a.y}; }
