// api_check.cpp -- drives the C++ API (include/*.hpp, the reference's class and
// function names) on the GPU and dumps the results as raw arrays into the
// directory argv[1]; tests/test_gpu_cpp_api.py compares them with the oracle.
#include <cstdio>
#include <fstream>
#include <numeric>
#include <string>
#include <vector>

#include "cg_rbf.hpp"
#include "cg_rbf_init.cuh"
#include "monte_carlo_bs.cuh"
#include "spatial_hasher.hpp"
#include "vortex_particle_mc.hpp"

static std::string g_dir;

template <typename T>
static void dump(const std::string& name, const std::vector<T>& v) {
    std::ofstream f(g_dir + "/" + name + ".bin", std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), std::streamsize(v.size() * sizeof(T)));
}

template <typename T>
static std::vector<T> from_dev(const T* p, size_t n) {
    std::vector<T> h(n);
    if (n) vpmc::check_cuda(cudaMemcpy(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost), "from_dev");
    return h;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: api_check OUTDIR\n");
        return 2;
    }
    g_dir = argv[1];
    try {
        SimParam P(1e-3f, 1.f, 1.f, 64, 4.f);
        P.N_max = 4096;
        P.N1 = 16;
        P.N2 = 16;
        Simulation sim(P);
        sim.init(4096);
        const int N = sim.particles_.N_cur;
        dump("pos0", sim.particles_.pos.to_host());
        dump("omega", sim.particles_.omega.to_host());
        dump("omega_field", sim.particles_.omega_field.to_host());

        const VorticityView pv = sim.makePosView();
        dump("pos_sub", from_dev(pv.sub, size_t(pv.cnt_view)));
        dump("pos_vp_sort", from_dev(pv.vp_sort, size_t(pv.cnt_view)));
        dump("pos_cell_acc", from_dev(pv.cell_acc, size_t(pv.rshx) * pv.rshy));
        const VorticityView nv = sim.makeNegView();
        dump("neg_sub", from_dev(nv.sub, size_t(nv.cnt_view)));
        dump("neg_vp_sort", from_dev(nv.vp_sort, size_t(nv.cnt_view)));

        dvec<float> y{size_t(N)};
        Ax_cuda(sim, sim.particles_.d_omega(), raw_ptr(y));
        dump("Ax", y.to_host());
        {
            // x produced on a caller stream right before the call: Ax_cuda orders
            // itself after that stream's work
            cudaStream_t us = nullptr;
            vpmc::check_cuda(cudaStreamCreateWithFlags(&us, cudaStreamNonBlocking), "stream");
            dvec<float> x2{size_t(N)}, y2{size_t(N)};
            vpmc::check_cuda(cudaMemcpyAsync(raw_ptr(x2), sim.particles_.d_omega(), sizeof(float) * size_t(N),
                                             cudaMemcpyDeviceToDevice, us), "copy x");
            Ax_cuda(sim, raw_ptr(x2), raw_ptr(y2), us);
            dump("Ax_stream", y2.to_host());
            vpmc::check_cuda(cudaStreamDestroy(us), "stream");
        }

        // reference-named free functions on the all-particle subset
        std::vector<int> iota(N);
        std::iota(iota.begin(), iota.end(), 0);
        dvec<int> sub;
        sub.assign(iota);
        SpatialHash H;
        H.resize_cells(8, 8);
        H.resize_particles(N);
        FillCells_cuda(8, 8, 1.f, 1.f, N, raw_ptr(sub), sim.particles_.d_p(), raw_ptr(H.cell_num),
                       raw_ptr(H.cell_acc), raw_ptr(H.vp_cell));
        dump("fill_cell_num", H.cell_num.to_host());
        CountingSort_cuda(N, raw_ptr(H.cell_num), raw_ptr(H.cell_acc), raw_ptr(H.vp_cell), raw_ptr(H.vp_sort));
        dump("all_cell_acc", H.cell_acc.to_host());
        dump("all_vp_sort", H.vp_sort.to_host());
        dump("all_cell_num_after", H.cell_num.to_host());
        // the same with the cell count given (no device-to-host read)
        FillCells_cuda(8, 8, 1.f, 1.f, N, raw_ptr(sub), sim.particles_.d_p(), raw_ptr(H.cell_num),
                       raw_ptr(H.cell_acc), raw_ptr(H.vp_cell));
        CountingSort_cuda(N, raw_ptr(H.cell_num), raw_ptr(H.cell_acc), raw_ptr(H.vp_cell), raw_ptr(H.vp_sort), 64);
        dump("all_vp_sort_ncell", H.vp_sort.to_host());

        SpatialHasher hasher(16, 16, Backend::CUDA);
        hasher.resize(N);
        hasher.build(sim.particles_.pos, sub, 1.f, 1.f);
        dump("hasher_vp_sort", hasher.data().vp_sort.to_host());
        dump("hasher_cell_acc", hasher.data().cell_acc.to_host());

        std::vector<int> flags(6, 0);
        try { SpatialHasher bad(4, 4, Backend::CPU); } catch (const vpmc::unsupported&) { flags[0] = 1; }
        try { sim.step_cpu(true); } catch (const vpmc::unsupported&) { flags[1] = 1; }
        try { solve_cg_rbf_cpu(sim, P.h_w); } catch (const vpmc::unsupported&) { flags[2] = 1; }
        try { sim.build_subsets_cpu(); } catch (const vpmc::unsupported&) { flags[3] = 1; }

        const double grid_err = sim.test_vorticity_grid(24);
        std::vector<double> gerr{grid_err};
        dump("grid_err", gerr);

        sim.step_cuda(true);   // the reference's step: deformed kernels, aux points, F update
        dump("pos1", sim.particles_.pos.to_host());
        dump("vel1", sim.particles_.vel.to_host());
        dump("F1", sim.particles_.F.to_host());

        {   // the reference's kernels as host calls: biot_savart_naive_kernel
            dvec<float2> u{size_t(N)};
            biot_savart_naive(sim.particles_.d_p(), sim.particles_.d_omega(), N, raw_ptr(u), P.Lx, P.Ly, true,
                              0.5f * P.h_w);
            dump("naive_pos", sim.particles_.pos.to_host());
            dump("naive_u", u.to_host());
        }

        std::vector<float2> before = sim.particles_.pos.to_host();
        sim.step_cuda_naive(true);
        dump("pos_naive_before", before);
        dump("pos_naive_after", sim.particles_.pos.to_host());

        const std::vector<double> rinfo = sim.reinitialize(1e-8, 1000);
        dump("pos_reinit", sim.particles_.pos.to_host());
        dump("reinit_info", rinfo);

        const float2 d{0.3f, 0.7f};
        flags[4] = SamplingDiskRadius(d, true, 1.f, 1.f) > 1.41f && SamplingDiskRadius(d, true, 1.f, 1.f) < 1.42f;
        flags[5] = std::fabs(wrap_delta(0.8f, 1.f, 1.f, true) + 0.2f) < 1e-6f;
        dump("flags", flags);
        std::printf("api_check ok N=%d grid_err=%g\n", N, grid_err);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "api_check failed: %s\n", e.what());
        return 1;
    }
}
