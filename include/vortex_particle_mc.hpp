// vortex_particle_mc.hpp -- C++ API of the hot path with the reference's names
// (include/vortex_particle_mc.hpp:16-209): SimParam, ParticleSet,
// VorticityView, Simulation.  Header-only; every method forwards to the C ABI
// in vpmc.h (GPU only).  Differences from the reference, by design:
//   * step_cuda runs the reference's deformation step (aux = 1, F update)
//     by default; set_deformation(false) selects the plain method;
//   * the estimator law defaults to the reference kernel's sampling law and
//     can be switched to the unbiased law (set_law);
//   * the *_cpu members throw vpmc::unsupported.
#pragma once

#include <cassert>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <random>
#include <vector>

#include "analytical_flow.hpp"
#include "device_vector_alias.hpp"
#include "spatial_hash.hpp"
#include "spatial_hasher.hpp"
#include "utilities.hpp"

struct ParticleSet {
    int N_max{0};
    int N_cur{0};

    dvec<float2> pos;
    dvec<float2> pos_left, pos_right, pos_top, pos_bottom;
    dvec<float2> pos_temp;
    dvec<float2> vel;
    dvec<float> omega;
    dvec<float> omega_field;
    dvec<float> jac;
    dvec<float4> F;

    void resize(int cap) {
        N_max = cap;
        N_cur = cap;
        pos.resize(cap);
        vel.resize(cap);
        pos_left.resize(cap);
        pos_right.resize(cap);
        pos_top.resize(cap);
        pos_bottom.resize(cap);
        pos_temp.resize(cap);
        omega.resize(cap);
        omega_field.resize(cap);
        jac.resize(cap);
        F.resize(cap);
    }
    void set_n_current(const int n) { N_cur = n; }

    float2* d_p() { return raw_ptr(pos); }
    float2* d_pt() { return raw_ptr(pos_temp); }
    float2* d_v() { return raw_ptr(vel); }
    float4* d_F() { return raw_ptr(F); }
    float* d_omega() { return raw_ptr(omega); }
    float* d_omega_field() { return raw_ptr(omega_field); }
    float* d_jac() { return raw_ptr(jac); }
    const float2* d_p() const { return raw_ptr(pos); }
    const float2* d_pt() const { return raw_ptr(pos_temp); }
    const float2* d_v() const { return raw_ptr(vel); }
    const float4* d_F() const { return raw_ptr(F); }
    const float* d_omega() const { return raw_ptr(omega); }
    const float* d_omega_field() const { return raw_ptr(omega_field); }
    const float* d_jac() const { return raw_ptr(jac); }
};

// Device-side view of one particle subset and its hash (same members as the
// reference's VorticityView).
struct VorticityView {
    const float2* pos;
    const float4* F;
    const float* w;
    int N;
    const int* vp_sort;
    const int* cell_acc;
    int rshx{}, rshy{};
    float Lx, Ly;
    float InvLx, InvLy;
    int cnt_view;
    const int* sub;
};

struct SimParam {
    float dt = 0.001f;
    float Lx = 1.f;
    float Ly = 1.f;
    int ResolutionX = 200;
    float hwr = 8.f;
    int N_max = 6000;
    int N1 = 1000;
    int N2 = 1000;

    int ResolutionY = 0;
    float h = 0.f;
    float h_w = 0.f;
    int length_iCDF = 10;
    float dx = 0.f;
    bool periodic = true;

    explicit SimParam(float dt_ = 0.01f, float Lx_ = 1.f, float Ly_ = 1.f, int resX = 200, float hwr_ = 16.f)
        : dt(dt_), Lx(Lx_), Ly(Ly_), ResolutionX(resX), hwr(hwr_) {
        assert(ResolutionX > 0 && "ResolutionX must be positive");
        h = Lx / float(ResolutionX);
        ResolutionY = int(std::round(Ly / h));
        if (ResolutionY == 0) ResolutionY = 1;
        h_w = h * hwr;
        dx = 0.5f * h_w;
    }
};

class Simulation {
public:
    ParticleSet particles_;
    SimParam P_;

    explicit Simulation(SimParam p) : P_(p) {}
    ~Simulation() {
        if (sim_) vpmc_sim_destroy(sim_);
    }
    Simulation(const Simulation&) = delete;
    Simulation& operator=(const Simulation&) = delete;

    // Simulation::init (src/vortex_particle_mc.cu:77-120): N uniform random
    // positions (std::mt19937(42)), Taylor-Green strengths fitted by CG-RBF,
    // sign subsets, hashes.
    void init(int num_of_p) {
        assert(num_of_p > 0 && num_of_p <= P_.N_max);
        particles_.resize(P_.N_max);
        particles_.set_n_current(num_of_p);
        std::vector<float2> hp(P_.N_max, float2{0.f, 0.f});
        std::vector<float> ho(P_.N_max, 0.f);
        std::mt19937 rng(42);
        std::uniform_real_distribution<float> uni(0.f, 1.f);
        ensure_icdf_kernel(20);
        for (int i = 0; i < num_of_p; ++i) {
            float2 p{uni(rng), uni(rng)};
            hp[i] = p;
            ho[i] = taylor_green_vorticity(p);
        }
        particles_.pos.assign(hp);
        particles_.omega.assign(ho);
        particles_.jac.assign(std::vector<float>(P_.N_max, 1.f));
        particles_.F.assign(std::vector<float4>(P_.N_max, float4{1.f, 0.f, 0.f, 1.f}));
        prepare_rhs_b();
        conjugate_gradient(5e-3, 1000);
        build_subsets_cuda();
        do_spatial_hashing();
    }

    // Per-sign hashes at the reference resolution rsh = Nx/int(hwr)/2
    // (src/vortex_particle_mc.cu:123-210).
    void do_spatial_hashing() {
        const int rshx = P_.ResolutionX / int(P_.hwr) / 2;
        const int rshy = P_.ResolutionY / int(P_.hwr) / 2;
        hash_one(hash_pos_, sub_pos_, cnt_pos_, rshx, rshy);
        hash_one(hash_neg_, sub_neg_, cnt_neg_, rshx, rshy);
        pos_view = makePosView();
        neg_view = makeNegView();
    }

    void build_global_hash() {
        const int N = particles_.N_cur;
        std::vector<int> iota(N);
        std::iota(iota.begin(), iota.end(), 0);
        sub_all_.assign(iota);
        const int rshx = P_.ResolutionX / int(P_.hwr) / 2;
        const int rshy = P_.ResolutionY / int(P_.hwr) / 2;
        hash_one(hash_all_, sub_all_, N, rshx, rshy);
    }

    void build_subsets_cpu() { throw vpmc::unsupported("Simulation::build_subsets_cpu"); }

    // build_subsets_cuda (src/cuda/build_particle_sets.cu:11-89), FP64 CDFs
    // (cdf64_*) plus the reference's FP32 layout (cdf_pos_/cdf_neg_).
    void build_subsets_cuda() {
        const int N = particles_.N_cur;
        sub_pos_.resize(std::max(N, 1));
        sub_neg_.resize(std::max(N, 1));
        cdf64_pos_.resize(std::max(N, 1));
        cdf64_neg_.resize(std::max(N, 1));
        cdf_pos_.resize(std::max(N, 1));
        cdf_neg_.resize(std::max(N, 1));
        int cnt[2];
        double cum[2];
        vpmc::check(vpmc_build_subsets(ctx(), N, particles_.d_omega(), raw_ptr(sub_pos_), raw_ptr(sub_neg_),
                                       raw_ptr(cdf64_pos_), raw_ptr(cdf64_neg_), raw_ptr(cdf_pos_), raw_ptr(cdf_neg_),
                                       cnt, cum),
                    "build_subsets_cuda");
        cnt_pos_ = cnt[0];
        cnt_neg_ = cnt[1];
        cum_pos_ = float(cum[0]);
        cum_neg_ = float(cum[1]);
        omega_dirty_ = true;
    }

    // prepare_rhs_b (src/vortex_particle_mc.cu:237-260): omega_field = Taylor-Green(pos).
    void prepare_rhs_b() {
        const int N = particles_.N_cur;
        std::vector<float2> hp = particles_.pos.to_host();
        std::vector<float> b(particles_.omega_field.size(), 0.f);
        for (int i = 0; i < N; ++i) b[i] = taylor_green_vorticity(hp[i]);
        particles_.omega_field.assign(b);
    }

    std::mt19937 rng;
    void step_cpu(bool) { throw vpmc::unsupported("Simulation::step_cpu"); }

    // step_cuda (src/cuda/simulation_step.cu:9-90): MIS velocity of every
    // particle with deformed kernels and the four auxiliary points, F =
    // renorm_det1(I + dt grad u), x += dt u with the periodic wrap in FP64.
    // With set_deformation(false): the plain method (F unused).
    void step_cuda(bool periodic) {
        ensure_sim(periodic);
        vpmc::check(vpmc_sim_set_particles(sim_, reinterpret_cast<const float*>(particles_.d_p()),
                                           omega_dirty_ ? particles_.d_omega() : nullptr, 0),
                    "step_cuda: set particles");
        if (omega_dirty_) vpmc::check(vpmc_sim_prepare(sim_), "step_cuda: prepare");
        omega_dirty_ = false;
        if (deformation_ != sim_deform_) {
            vpmc::check(vpmc_sim_set_deformation(sim_, deformation_ ? 1 : 0, 0.f), "step_cuda: deformation");
            sim_deform_ = deformation_;
        }
        if (deformation_)
            vpmc::check(vpmc_sim_set_F(sim_, reinterpret_cast<const float*>(particles_.d_F()), 0), "step_cuda: F");
        vpmc::check(vpmc_sim_step(sim_, 1, 1), "step_cuda");
        vpmc::check(vpmc_sim_get_particles(sim_, reinterpret_cast<float*>(particles_.d_p()), nullptr,
                                           reinterpret_cast<float*>(particles_.d_v()), 0),
                    "step_cuda: get particles");
        if (deformation_)
            vpmc::check(vpmc_sim_get_F(sim_, reinterpret_cast<float*>(particles_.d_F()), 0), "step_cuda: F out");
    }

    // compute_velocity_naive (src/cuda/simulation_step.cu:92-108): Plummer
    // minimum-image direct sum in FP32 (the reference's kernel is FP32), written
    // to particles.vel.  compute_velocity_naive_f64 gives the FP64 sum.
    void compute_velocity_naive(bool periodic, float eps_core) {
        const int N = particles_.N_cur;
        if (particles_.vel.size() < size_t(N)) particles_.vel.resize(N);
        direct_plummer_f32(periodic, eps_core, reinterpret_cast<float*>(particles_.d_v()));
    }

    void compute_velocity_naive_f64(bool periodic, float eps_core, dvec<double>& uv) {
        uv.resize(size_t(2) * std::max(particles_.N_cur, 1));
        direct_plummer(periodic, eps_core, uv);
    }

    // step_cuda_naive (src/cuda/simulation_step.cu:110-129): eps = h_w/2, FP32
    // velocities, forward Euler, periodic wrap.
    void step_cuda_naive(bool periodic) {
        const int N = particles_.N_cur;
        compute_velocity_naive(periodic, 0.5f * P_.h_w);
        vpmc::check(vpmc_advect(ctx(), N, reinterpret_cast<float*>(particles_.d_p()),
                                reinterpret_cast<const float*>(particles_.d_v()), nullptr, P_.dt, P_.Lx, P_.Ly,
                                periodic ? 1 : 0),
                    "step_cuda_naive");
    }

    inline float eval_vorticity_cpu(float2, bool) const { throw vpmc::unsupported("eval_vorticity_cpu"); }

    // test_vorticity_grid (src/vortex_particle_mc.cu:332-456): positive-part
    // field on a res x res grid from the GPU query against a direct FP64 sum
    // on the host; returns the max absolute difference.
    double test_vorticity_grid(int res) {
        std::vector<float2> g(size_t(res) * res);
        const float step = 1.f / res;
        for (int ix = 0; ix < res; ++ix)
            for (int iy = 0; iy < res; ++iy) g[size_t(ix) * res + iy] = float2{(ix + 0.5f) * step, (iy + 0.5f) * step};
        dvec<float2> pts;
        pts.assign(g);
        dvec<float> out(g.size());
        vpmc::check(vpmc_query_vorticity(ctx(), particles_.N_cur, reinterpret_cast<const float*>(particles_.d_p()),
                                         particles_.d_omega(), nullptr, int(g.size()),
                                         reinterpret_cast<const float*>(raw_ptr(pts)), +1, 0, 0, P_.h_w, P_.Lx,
                                         P_.Ly, 0, raw_ptr(out)),
                    "test_vorticity_grid");
        const std::vector<float> got = out.to_host();
        const std::vector<float2> hp = particles_.pos.to_host();
        const std::vector<float> hw = particles_.omega.to_host();
        double max_err = 0.0;
        for (size_t q = 0; q < g.size(); ++q) {
            double s = 0.0;
            for (int i = 0; i < particles_.N_cur; ++i) {
                if (!(hw[i] > 0.f)) continue;
                const double dx = double(hp[i].x) - g[q].x, dy = double(hp[i].y) - g[q].y;
                s += double(hw[i]) * double(cubicSplinePDF(float(std::sqrt(dx * dx + dy * dy)), P_.h_w));
            }
            max_err = std::max(max_err, std::fabs(s - got[q]));
        }
        return max_err;
    }

    // ensure_icdf_kernel (src/vortex_particle_mc.cu:264-279).
    void ensure_icdf_kernel(int L) {
        if (icdf_L_ == L && icdf_kernel_.size() == size_t(L)) return;
        dvec<float> cdf;
        build_cubic_rcdf(P_.h_w, L, cdf);
        cdf_to_icdf(cdf, P_.h_w, icdf_kernel_);
        icdf_L_ = L;
    }

    VorticityView makePosView(const float* w_ptr = nullptr) const {
        return view_of(hash_pos_, w_ptr, cnt_pos_, raw_ptr(sub_pos_));
    }
    VorticityView makeNegView(const float* w_ptr = nullptr) const {
        return view_of(hash_neg_, w_ptr, cnt_neg_, raw_ptr(sub_neg_));
    }
    VorticityView makePosViewNaive(const float* w_ptr = nullptr) const {
        VorticityView v = makePosView(w_ptr);
        v.vp_sort = nullptr;
        v.cell_acc = nullptr;
        v.rshx = v.rshy = 0;
        return v;
    }
    VorticityView makeNegViewNaive(const float* w_ptr = nullptr) const {
        VorticityView v = makeNegView(w_ptr);
        v.vp_sort = nullptr;
        v.cell_acc = nullptr;
        v.rshx = v.rshy = 0;
        return v;
    }
    VorticityView makeAllView(const float* w_ptr = nullptr) const {
        return view_of(hash_all_, w_ptr, particles_.N_cur, raw_ptr(sub_all_));
    }

    // -- extensions of this build (no reference counterpart) --
    void set_law(int law) {
        law_ = law;
        if (sim_) vpmc::check(vpmc_sim_set_law(sim_, law), "set_law");
    }
    // step_cuda with (default, as the reference) or without the 5-point deformation.
    void set_deformation(bool on) { deformation_ = on; }
    // Reinitialisation (the reference's README describes it; its code has
    // none): positions to the lattice, F = I, strengths re-fitted by CG-RBF to
    // the current field.  Returns {iters, relres, true relres}.
    std::vector<double> reinitialize(double tol, int max_iter, bool periodic = true) {
        ensure_sim(periodic);
        vpmc::check(vpmc_sim_set_particles(sim_, reinterpret_cast<const float*>(particles_.d_p()),
                                           particles_.d_omega(), 0),
                    "reinitialize: set particles");
        if (deformation_ != sim_deform_) {
            vpmc::check(vpmc_sim_set_deformation(sim_, deformation_ ? 1 : 0, 0.f), "reinitialize: deformation");
            sim_deform_ = deformation_;
        }
        if (deformation_)
            vpmc::check(vpmc_sim_set_F(sim_, reinterpret_cast<const float*>(particles_.d_F()), 0), "reinitialize: F");
        std::vector<double> info(3, 0.0);
        const int rc = vpmc_sim_reinit(sim_, tol, max_iter, info.data());
        if (rc != VPMC_OK && rc != VPMC_ERR_NOT_CONVERGED) vpmc::check(rc, "reinitialize");
        vpmc::check(vpmc_sim_get_particles(sim_, reinterpret_cast<float*>(particles_.d_p()), particles_.d_omega(),
                                           nullptr, 0),
                    "reinitialize: get particles");
        vpmc::check(vpmc_sim_get_F(sim_, reinterpret_cast<float*>(particles_.d_F()), 0), "reinitialize: F out");
        // the reference-shaped subsets and hashes follow the new state
        build_subsets_cuda();
        do_spatial_hashing();
        build_global_hash();
        return info;
    }
    // CG with explicit tolerance (conjugate_gradient_rbf uses the reference defaults).
    std::vector<double> conjugate_gradient(double tol, int max_iter) {
        std::vector<double> info(3, 0.0);
        const int N = particles_.N_cur;
        const int rc = vpmc_cg_rbf(ctx(), N, reinterpret_cast<const float*>(particles_.d_p()),
                                   particles_.d_omega_field(), particles_.d_omega(), P_.h_w, P_.Lx, P_.Ly,
                                   P_.periodic ? 1 : 0, tol, max_iter, info.data());
        if (rc != VPMC_OK && rc != VPMC_ERR_NOT_CONVERGED) vpmc::check(rc, "conjugate_gradient");
        omega_dirty_ = true;
        return info;
    }
    vpmc_context* ctx() const { return vpmc::default_context(); }

private:
    void hash_one(SpatialHash& H, const dvec<int>& sub, int cnt, int rshx, int rshy) {
        H.resize_cells(rshx, rshy);
        H.resize_particles(std::max(cnt, 1));
        vpmc::check(vpmc_hash_build(ctx(), rshx, rshy, P_.Lx, P_.Ly, cnt, raw_ptr(sub),
                                    reinterpret_cast<const float*>(particles_.d_p()), raw_ptr(H.cell_num),
                                    raw_ptr(H.cell_acc), raw_ptr(H.vp_cell), raw_ptr(H.vp_sort)),
                    "do_spatial_hashing");
    }

    VorticityView view_of(const SpatialHash& H, const float* w_ptr, int cnt, const int* sub) const {
        return VorticityView{particles_.d_p(), particles_.d_F(), w_ptr ? w_ptr : particles_.d_omega(),
                             particles_.N_cur, raw_ptr(H.vp_sort), raw_ptr(H.cell_acc), H.rshx, H.rshy,
                             P_.Lx, P_.Ly, 1.0f / P_.Lx, 1.0f / P_.Ly, cnt, sub};
    }

    void ensure_sim(bool periodic) {
        if (sim_ && periodic == sim_periodic_) return;
        if (sim_) vpmc_sim_destroy(sim_);
        vpmc_sim_params p{};
        p.dt = P_.dt;
        p.Lx = P_.Lx;
        p.Ly = P_.Ly;
        p.Nx = P_.ResolutionX;
        p.hwr = P_.hwr;
        p.N1 = P_.N1;
        p.N2 = P_.N2;
        p.periodic = periodic ? 1 : 0;
        p.law = law_;
        p.seed = 0x1234;
        const int n = particles_.N_cur;
        vpmc::check(vpmc_sim_create(ctx(), 1, &p, &n, &sim_), "vpmc_sim_create");
        sim_periodic_ = periodic;
        sim_deform_ = false;
        omega_dirty_ = true;
    }

    void direct_plummer(bool periodic, float eps, dvec<double>& uv) {
        const int N = particles_.N_cur;
        std::vector<int> iota(N);
        std::iota(iota.begin(), iota.end(), 0);
        dvec<int> tidx;
        tidx.assign(iota);
        vpmc::check(vpmc_direct_velocity_f64(ctx(), VPMC_DIRECT_PLUMMER, N,
                                             reinterpret_cast<const float*>(particles_.d_p()), particles_.d_omega(),
                                             N, nullptr, raw_ptr(tidx), eps, P_.Lx, P_.Ly, periodic ? 1 : 0,
                                             raw_ptr(uv)),
                    "direct Biot-Savart");
    }

    void direct_plummer_f32(bool periodic, float eps, float* out) {
        const int N = particles_.N_cur;
        std::vector<int> iota(N);
        std::iota(iota.begin(), iota.end(), 0);
        dvec<int> tidx;
        tidx.assign(iota);
        vpmc::check(vpmc_direct_velocity_f32(ctx(), VPMC_DIRECT_PLUMMER, N,
                                             reinterpret_cast<const float*>(particles_.d_p()), particles_.d_omega(),
                                             N, nullptr, raw_ptr(tidx), eps, P_.Lx, P_.Ly, periodic ? 1 : 0, out),
                    "direct Biot-Savart (FP32)");
    }

    SpatialHash hash_pos_, hash_neg_, hash_all_;
    dvec<int> sub_all_;
    dvec<int> sub_pos_, sub_neg_;
    dvec<float> cdf_pos_, cdf_neg_;
    dvec<double> cdf64_pos_, cdf64_neg_;
    int cnt_pos_{}, cnt_neg_{};
    float cum_pos_{}, cum_neg_{};
    dvec<float> cdf_kernel, icdf_kernel;
    dvec<float> icdf_kernel_;
    int icdf_L_ = 0;
    VorticityView pos_view{};
    VorticityView neg_view{};

    vpmc_sim* sim_ = nullptr;
    bool sim_periodic_ = true;
    bool deformation_ = true;
    bool sim_deform_ = false;
    bool omega_dirty_ = true;
    int law_ = VPMC_LAW_REFERENCE;
};

// evalVorticityAbs_cpu (include/vortex_particle_mc.hpp:195-201): CPU only in
// the reference; this build has no CPU path.
inline float evalVorticityAbs_cpu(const VorticityView&, const float2&, int, bool, bool, float, bool) {
    throw vpmc::unsupported("evalVorticityAbs_cpu");
}
