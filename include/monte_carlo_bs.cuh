// monte_carlo_bs.cuh -- device-side context of the reference's MIS kernel
// (include/monte_carlo_bs.cuh:17-41) kept for layout compatibility, the host
// equivalents of its scalar helpers, and host-callable replacements of its
// kernels: update_jacobian_from5 and biot_savart_naive (device arrays in,
// device arrays out, run on the library's default context).  The MIS kernel
// itself (monte_carlo_bs_kernel_safe) runs inside Simulation::step_cuda /
// vpmc_sim_step, which builds its own binned sample sets.
#pragma once

#include <cmath>
#include <numeric>
#include <vector>

#include "device_vector_alias.hpp"
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

// update_jacobian_from5 (src/cuda/monte_carlo_bs.cu:274-288): F = renorm_det1(I + dt grad u).
inline void update_jacobian_from5(int N, float dt, float dx, const float2* velC, const float2* velL,
                                  const float2* velR, const float2* velT, const float2* velB, float4* Fout) {
    vpmc::check(vpmc_update_jacobian_from5(vpmc::default_context(), N, dt, dx, reinterpret_cast<const float*>(velC),
                                           reinterpret_cast<const float*>(velL), reinterpret_cast<const float*>(velR),
                                           reinterpret_cast<const float*>(velT), reinterpret_cast<const float*>(velB),
                                           reinterpret_cast<float*>(Fout)),
                "update_jacobian_from5");
}

// biot_savart_naive_kernel (src/cuda/naive_biot_savart.cu:15-40): Plummer
// minimum-image direct sum of every particle, FP32 tiles.
inline void biot_savart_naive(const float2* pos, const float* gamma, int N, float2* out, float Lx, float Ly,
                              bool periodic, float eps) {
    std::vector<int> iota(N > 0 ? N : 1);
    std::iota(iota.begin(), iota.end(), 0);
    dvec<int> tidx;
    tidx.assign(iota);
    vpmc::check(vpmc_direct_velocity_f32(vpmc::default_context(), VPMC_DIRECT_PLUMMER, N,
                                         reinterpret_cast<const float*>(pos), gamma, N, nullptr, raw_ptr(tidx), eps,
                                         Lx, Ly, periodic ? 1 : 0, reinterpret_cast<float*>(out)),
                "biot_savart_naive");
}
