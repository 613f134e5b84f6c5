// monte_carlo_bs.cuh -- device-side context of the reference's MIS kernel
// (include/monte_carlo_bs.cuh:17-41) kept for layout compatibility, and the
// host equivalents of its scalar helpers.  The kernels themselves
// (monte_carlo_bs_kernel_safe, update_jacobian_from5, biot_savart_naive_kernel)
// are internal to libvpmc: the MIS step runs through Simulation::step_cuda /
// vpmc_sim_step, the direct sum through vpmc_direct_velocity_f64.
#pragma once

#include <cmath>

#include "monte_carlo_bs.hpp"

struct MCBSCtx_d {
    const int* sub_pos;
    const int* sub_neg;
    const float* cdf_pos;
    const float* cdf_neg;
    int cnt_pos;
    int cnt_neg;
    const float* icdf_kernel;
    int kernel_L;
    float h_w;
    float cum_pos;
    float cum_neg;
    float Lx, Ly;
    float InvLx;
    float InvLy;
    bool periodic;
    float dx;
    VorticityView pos_view;
    VorticityView neg_view;
};

// d - round(d/L) L (minimum image), include/monte_carlo_bs.cuh:134-138.
inline float wrap_delta(float d, float L, float /*InvL*/, bool periodic) {
    if (!periodic) return d;
    return d - std::round(d / L) * L;
}

// Plummer kernel perp(d) / (2 pi (|d|^2 + eps^2)), include/monte_carlo_bs.cuh:158-163.
inline float2 bs_kernel_2d(float2 d, float eps2) {
    const float denom = d.x * d.x + d.y * d.y + eps2;
    const float coef = 0.5f * (1.0f / 3.14159265358979323846f) / denom;
    return {-d.y * coef, d.x * coef};
}
