// spatial_hash.hpp -- uniform-grid spatial hash (the reference's
// include/spatial_hash.hpp:7-73): same struct and free-function names.  The
// *_cuda functions run the GPU build (bit-exact with the reference's CPU
// build); the *_cpu / *_omp functions exist for source compatibility and
// throw vpmc::unsupported (this build has no CPU path).
#pragma once

#include <span>

#include "device_vector_alias.hpp"

struct SpatialHash {
    int rshx{}, rshy{};
    dvec<int> cell_num, cell_acc;   // rshx*rshy
    dvec<int> vp_cell, vp_sort;     // particles of the subset

    void resize_cells(int rx, int ry) {
        rshx = rx;
        rshy = ry;
        const size_t cells = size_t(rx) * ry;
        cell_num.resize(cells);
        cell_acc.resize(cells);
    }
    void resize_particles(int N_max) {
        vp_cell.resize(N_max);
        vp_sort.resize(N_max);
    }
};

inline void FillCells_cpu(int, int, float, float, int, std::span<const int>, std::span<const float>,
                          std::span<const float>, std::span<int>, std::span<int>, std::span<int>) {
    throw vpmc::unsupported("FillCells_cpu");
}
inline void CountingSort_cpu(int, std::span<int>, std::span<const int>, std::span<const int>, std::span<int>) {
    throw vpmc::unsupported("CountingSort_cpu");
}
inline void FillCells_omp(int, int, float, float, int, std::span<const int>, std::span<const float>,
                          std::span<const float>, std::span<int>, std::span<int>, std::span<int>) {
    throw vpmc::unsupported("FillCells_omp");
}
inline void CountingSort_omp(int, std::span<int>, std::span<const int>, std::span<const int>, std::span<int>) {
    throw vpmc::unsupported("CountingSort_omp");
}

// FillCells_cuda (src/cuda/hash.cu:42-69): device pointers; pos is float2[*].
inline void FillCells_cuda(int rshx, int rshy, float Lx, float Ly, int N, const int* sub, const float2* pos,
                           int* cell_num, int* cell_acc, int* vp_cell) {
    vpmc::check(vpmc_fill_cells(vpmc::default_context(), rshx, rshy, Lx, Ly, N, sub,
                                reinterpret_cast<const float*>(pos), cell_num, cell_acc, vp_cell),
                "FillCells_cuda");
}

// CountingSort_cuda (src/cuda/hash.cu:71-91).  The reference's five-argument
// call has no cell count: it is then inferred from vp_cell (one device-to-host
// read; the reference synchronises the device at this point too).  A caller
// that knows it (rshx * rshy) passes it as `ncell` and the call stays on the
// device until its final wait.
inline void CountingSort_cuda(int N, int* cell_num, const int* cell_acc, const int* vp_cell, int* vp_map,
                              int ncell = 0) {
    vpmc::check(vpmc_counting_sort(vpmc::default_context(), N, ncell, cell_num, cell_acc, vp_cell, vp_map),
                "CountingSort_cuda");
}
