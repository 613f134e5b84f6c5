// cg_rbf_init.cuh -- RBF SpMV and CG strength initialisation (the reference's
// include/cg_rbf_init.cuh:6-13): same names and defaults.
#pragma once

#include <cuda_runtime_api.h>

#include "vortex_particle_mc.hpp"

// Ax_cuda (src/cuda/cg_rbf_init.cu:33-50): y = A x over all particles of the
// simulation (device pointers).  The SpMV runs on the library context's
// stream, ordered after the work already queued on `stream` (x may be produced
// there), and completes before return, so later work on `stream` sees y.
inline void Ax_cuda(const Simulation& sim, const float* x, float* y, cudaStream_t stream = 0) {
    cudaStream_t own = static_cast<cudaStream_t>(vpmc_context_stream(sim.ctx()));
    if (stream != own) {
        cudaEvent_t ev = nullptr;
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
            throw vpmc::error(VPMC_ERR_CUDA, "Ax_cuda: event");
        const bool ok = cudaEventRecord(ev, stream) == cudaSuccess && cudaStreamWaitEvent(own, ev, 0) == cudaSuccess;
        cudaEventDestroy(ev);
        if (!ok) throw vpmc::error(VPMC_ERR_CUDA, "Ax_cuda: stream order");
    }
    vpmc::check(vpmc_rbf_matvec(sim.ctx(), sim.particles_.N_cur, reinterpret_cast<const float*>(sim.particles_.d_p()),
                                x, y, sim.P_.h_w, sim.P_.Lx, sim.P_.Ly, sim.P_.periodic ? 1 : 0, 1),
                "Ax_cuda");
}

// conjugate_gradient_rbf (src/cuda/cg_rbf_init.cu:53-116): solve A w = omega_field,
// write omega, rebuild the sign subsets and hashes.
inline void conjugate_gradient_rbf(Simulation& sim, float tol = 5e-3f, int max_iter = 1000) {
    sim.conjugate_gradient(tol, max_iter);
    sim.build_subsets_cuda();
    sim.do_spatial_hashing();
}
