// ref_shim.cpp -- C entry points onto the REFERENCE's own CPU functions.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh together with the
// reference's unmodified CPU sources (read in place from the reference tree)
// into oracle/_ref/libvpmc_ref.so, which is git-ignored.  It exists to pin the
// oracle restatement (vpmc_oracle.cpp) and to generate tests/golden fixtures;
// nothing in the product links it.
//
// Harness-only liberties:
//   * `#define private public` to reach Simulation's subset buffers, which
//     build_subsets_cpu (src/cpu/build_particle_sets.cpp:6-42) writes;
//   * the trivial Simulation constructor (src/vortex_particle_mc.cu:75) is
//     defined here because that translation unit (a demo main + PNG output)
//     is not compiled.

#define private public
#include "vortex_particle_mc.hpp"
#undef private
#include "spatial_hash.hpp"
#include "monte_carlo_bs.hpp"
#include "utilities.hpp"

#include <cstdint>
#include <random>
#include <span>
#include <vector>

Simulation::Simulation(SimParam p) : P_(std::move(p)) {}

namespace {
VorticityView make_view(const float* pos, const float* w, int N, const int* vp_sort,
                        const int* cell_acc, int rshx, int rshy, float Lx, float Ly,
                        int cnt_view, const int* sub) {
    VorticityView v{};
    v.pos = reinterpret_cast<const float2*>(pos);
    v.F = nullptr;
    v.w = w;
    v.N = N;
    v.vp_sort = vp_sort;
    v.cell_acc = cell_acc;
    v.rshx = rshx;
    v.rshy = rshy;
    v.Lx = Lx;
    v.Ly = Ly;
    v.InvLx = 1.0f / Lx;
    v.InvLy = 1.0f / Ly;
    v.cnt_view = cnt_view;
    v.sub = sub;
    return v;
}
}  // namespace

extern "C" {

void ref_fill_cells(int rshx, int rshy, float Lx, float Ly, int N, const int* sub,
                    const float* px, const float* py, int npos, int* cell_num,
                    int* cell_acc, int* vp_cell) {
    const size_t nc = size_t(rshx) * rshy;
    FillCells_cpu(rshx, rshy, Lx, Ly, N, std::span<const int>(sub, N),
                  std::span<const float>(px, npos), std::span<const float>(py, npos),
                  std::span<int>(cell_num, nc), std::span<int>(cell_acc, nc),
                  std::span<int>(vp_cell, N));
}

void ref_counting_sort(int N, int ncell, int* cell_num, const int* cell_acc,
                       const int* vp_cell, int* vp_sort) {
    CountingSort_cpu(N, std::span<int>(cell_num, ncell), std::span<const int>(cell_acc, ncell),
                     std::span<const int>(vp_cell, N), std::span<int>(vp_sort, N));
}

void ref_fill_cells_omp(int rshx, int rshy, float Lx, float Ly, int N, const int* sub,
                        const float* px, const float* py, int npos, int* cell_num,
                        int* cell_acc, int* vp_cell) {
    const size_t nc = size_t(rshx) * rshy;
    FillCells_omp(rshx, rshy, Lx, Ly, N, std::span<const int>(sub, N),
                  std::span<const float>(px, npos), std::span<const float>(py, npos),
                  std::span<int>(cell_num, nc), std::span<int>(cell_acc, nc),
                  std::span<int>(vp_cell, N));
}

void ref_counting_sort_omp(int N, int ncell, int* cell_num, const int* cell_acc,
                           const int* vp_cell, int* vp_sort) {
    CountingSort_omp(N, std::span<int>(cell_num, ncell), std::span<const int>(cell_acc, ncell),
                     std::span<const int>(vp_cell, N), std::span<int>(vp_sort, N));
}

// Simulation::build_subsets_cpu on a fresh Simulation holding `omega`.
void ref_build_subsets(int N, const float* omega, int* sub_pos, int* sub_neg,
                       float* cdf_pos, float* cdf_neg, int* cnt, float* cum) {
    SimParam P;
    Simulation sim(P);
    sim.particles_.resize(N);
    for (int i = 0; i < N; ++i) sim.particles_.omega[i] = omega[i];
    sim.build_subsets_cpu();
    cnt[0] = sim.cnt_pos_;
    cnt[1] = sim.cnt_neg_;
    cum[0] = sim.cum_pos_;
    cum[1] = sim.cum_neg_;
    for (int k = 0; k < sim.cnt_pos_; ++k) { sub_pos[k] = sim.sub_pos_[k]; cdf_pos[k] = sim.cdf_pos_[k]; }
    for (int k = 0; k < sim.cnt_neg_; ++k) { sub_neg[k] = sim.sub_neg_[k]; cdf_neg[k] = sim.cdf_neg_[k]; }
}

void ref_build_cubic_rcdf(float h_w, int length, float* cdf) {
    std::vector<float> c;
    build_cubic_rcdf(h_w, length, c);
    for (int i = 0; i < length; ++i) cdf[i] = c[i];
}

void ref_cdf_to_icdf(const float* cdf, int length, float h_w, float* icdf) {
    std::vector<float> c(cdf, cdf + length), ic;
    cdf_to_icdf(c, h_w, ic);
    for (int i = 0; i < length; ++i) icdf[i] = ic[i];
}

float ref_spline_pdf(float r, float h_w) { return cubicSplinePDF(r, h_w); }

void ref_eval_vorticity(const float* pos, const float* w, int N, const int* vp_sort,
                        const int* cell_acc, int rshx, int rshy, float Lx, float Ly,
                        int cnt_view, const int* sub, const float* pts, int M, int sign,
                        int use_signed, int exclude_center, float h_w, int periodic,
                        float* out) {
    const VorticityView v = make_view(pos, w, N, vp_sort, cell_acc, rshx, rshy, Lx, Ly, cnt_view, sub);
    for (int m = 0; m < M; ++m) {
        const float2 p{pts[2 * m], pts[2 * m + 1]};
        out[m] = evalVorticityAbs_cpu(v, p, sign, use_signed != 0, exclude_center != 0, h_w,
                                      periodic != 0);
    }
}

// One monte_carlo_bs_cpu evaluation per target (both signs), aux as given,
// one std::mt19937(seed) for the whole target loop, as step_cpu does
// (src/cpu/simulation_step.cpp:13,31-44).  out: M x 5 float2 for sign +1,
// then M x 5 float2 for sign -1.
void ref_mc_estimates(int N, const float* pos, const float* omega,
                      const int* sub_pos, int cnt_pos, const float* cdf_pos, float cum_pos,
                      const int* vp_sort_pos, const int* cell_acc_pos,
                      const int* sub_neg, int cnt_neg, const float* cdf_neg, float cum_neg,
                      const int* vp_sort_neg, const int* cell_acc_neg,
                      int rshx, int rshy, float Lx, float Ly, float h_w, int periodic,
                      const float* dst5, int M, int aux, int N1, int N2, uint32_t seed,
                      float* out_pos, float* out_neg) {
    ParticleSet P;
    P.resize(N);
    for (int i = 0; i < N; ++i) { P.pos[i].x = pos[2 * i]; P.pos[i].y = pos[2 * i + 1]; }
    std::vector<int> sp(sub_pos, sub_pos + cnt_pos), sn(sub_neg, sub_neg + cnt_neg);
    std::vector<float> cp(cdf_pos, cdf_pos + cnt_pos), cn(cdf_neg, cdf_neg + cnt_neg);
    std::vector<float> icdf;
    MCBSCtx C;
    C.sub_pos = &sp;
    C.sub_neg = &sn;
    C.cdf_pos = &cp;
    C.cdf_neg = &cn;
    C.icdf_kernel = &icdf;
    C.kernel_L = 0;
    C.h_w = h_w;
    C.periodic = periodic != 0;
    C.Lx = Lx;
    C.Ly = Ly;
    C.InvLx = 1.0f / Lx;
    C.InvLy = 1.0f / Ly;
    C.cum_pos = cum_pos;
    C.cum_neg = cum_neg;
    C.pos_view = make_view(pos, omega, N, vp_sort_pos, cell_acc_pos, rshx, rshy, Lx, Ly, cnt_pos, sub_pos);
    C.neg_view = make_view(pos, omega, N, vp_sort_neg, cell_acc_neg, rshx, rshy, Lx, Ly, cnt_neg, sub_neg);
    std::mt19937 rng(seed);
    for (int t = 0; t < M; ++t) {
        const float* d = dst5 + 10 * t;
        const float2 a{d[0], d[1]}, l{d[2], d[3]}, r{d[4], d[5]}, tp{d[6], d[7]}, b{d[8], d[9]};
        const MCBSEstimate ep = monte_carlo_bs_cpu(a, +1, aux, l, r, tp, b, P, C, N1, N2, rng);
        const MCBSEstimate en = monte_carlo_bs_cpu(a, -1, aux, l, r, tp, b, P, C, N1, N2, rng);
        const float2* vp[5] = {&ep.main, &ep.left, &ep.right, &ep.top, &ep.bottom};
        const float2* vn[5] = {&en.main, &en.left, &en.right, &en.top, &en.bottom};
        for (int k = 0; k < 5; ++k) {
            out_pos[10 * t + 2 * k] = vp[k]->x;
            out_pos[10 * t + 2 * k + 1] = vp[k]->y;
            out_neg[10 * t + 2 * k] = vn[k]->x;
            out_neg[10 * t + 2 * k + 1] = vn[k]->y;
        }
    }
}

}  // extern "C"
