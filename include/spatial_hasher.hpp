// spatial_hasher.hpp -- SpatialHasher (the reference's include/spatial_hasher.hpp:
// 6-21 plus the data() accessor its callers expect, apps/vortex_method_mc.cu:64).
// Backend::CUDA builds on the GPU; CPU and OMP throw vpmc::unsupported.
#pragma once

#include <vector>

#include "spatial_hash.hpp"

enum class Backend { CPU, OMP, CUDA };

class SpatialHasher {
public:
    SpatialHasher(int rshx, int rshy, Backend b) : backend_(b) {
        if (b != Backend::CUDA) throw vpmc::unsupported("SpatialHasher CPU/OMP backend");
        hash_.resize_cells(rshx, rshy);
    }

    void resize(int N_max) { hash_.resize_particles(N_max); }

    // pos: device float2 array (dvec<float2>) of all particles; sub: device
    // int array (dvec<int>) of the subset's global indices.
    template <typename VecPos, typename VecSub>
    void build(const VecPos& pos, const VecSub& sub, float Lx, float Ly) {
        const int N = int(sub.size());
        if (size_t(N) > hash_.vp_cell.size()) hash_.resize_particles(N);
        vpmc::check(vpmc_hash_build(vpmc::default_context(), hash_.rshx, hash_.rshy, Lx, Ly, N, raw_ptr(sub),
                                    reinterpret_cast<const float*>(raw_ptr(pos)), raw_ptr(hash_.cell_num),
                                    raw_ptr(hash_.cell_acc), raw_ptr(hash_.vp_cell), raw_ptr(hash_.vp_sort)),
                    "SpatialHasher::build");
    }

    const SpatialHash& data() const { return hash_; }

private:
    SpatialHash hash_;
    Backend backend_;
};
