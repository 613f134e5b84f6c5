// monte_carlo_bs.hpp -- MIS Biot-Savart estimator types and host helpers (the
// reference's include/monte_carlo_bs.hpp:7-102).  monte_carlo_bs_cpu and the
// std::mt19937 samplers are CPU-only in the reference and throw here; the GPU
// estimator runs inside Simulation::step_cuda / vpmc_sim_velocity.
#pragma once

#include <algorithm>
#include <cmath>
#include <random>

#include "vortex_particle_mc.hpp"

struct MCBSEstimate {
    float2 main{}, left{}, right{}, top{}, bottom{};
};

struct MCBSCtx {
    const dvec<int>* sub_pos = nullptr;
    const dvec<int>* sub_neg = nullptr;
    const dvec<float>* cdf_pos = nullptr;
    const dvec<float>* cdf_neg = nullptr;
    const dvec<float>* icdf_kernel = nullptr;
    int kernel_L = 0;
    float h_w = 1.0f;
    bool periodic = false;
    float Lx = 1.0f, Ly = 1.0f;
    float InvLx = 1.0f, InvLy = 1.0f;
    float cum_pos = 1.0f, cum_neg = 1.0f;
    VorticityView pos_view{};
    VorticityView neg_view{};
};

inline MCBSEstimate monte_carlo_bs_cpu(const float2&, int, int, const float2&, const float2&, const float2&,
                                       const float2&, const ParticleSet&, const MCBSCtx&, int, int, std::mt19937&) {
    throw vpmc::unsupported("monte_carlo_bs_cpu");
}
inline float sample_kernel_radius(std::mt19937&, const float*, int, float) {
    throw vpmc::unsupported("sample_kernel_radius");
}
inline int sample_vorticity_idx_cdf(std::mt19937&, const float*, int) {
    throw vpmc::unsupported("sample_vorticity_idx_cdf");
}
inline float2 sample_disk_biot_savart(std::mt19937&, const float2&, float) {
    throw vpmc::unsupported("sample_disk_biot_savart");
}

// perp(x - y) / (2 pi (|x - y|^2 + 1e-8)), the regularised kernel of the MIS terms.
inline float2 biot_savart_kernel(const float2& x, const float2& y) {
    const float rx = x.x - y.x, ry = x.y - y.y;
    const float inv_r2 = 1.f / (rx * rx + ry * ry + 1e-8f);
    return {-ry * inv_r2 / (2 * 3.14159265358979323846f), rx * inv_r2 / (2 * 3.14159265358979323846f)};
}

// Radius of the branch-2 disk: the farthest periodic image of dst (sqrt(Lx^2+Ly^2)).
inline float SamplingDiskRadius(const float2& dst, bool periodic, const float& Lx, const float& Ly) {
    if (!periodic) return std::sqrt(Lx * Lx + Ly * Ly);
    float m = 0.f;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy) {
            const float ix = dst.x + dx * Lx, iy = dst.y + dy * Ly;
            const float ex = ix - dst.x, ey = iy - dst.y;
            m = std::max(m, ex * ex + ey * ey);
        }
    return std::sqrt(m);
}
