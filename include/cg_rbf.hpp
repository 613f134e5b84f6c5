// cg_rbf.hpp -- the reference's CPU CG interface (include/cg_rbf.hpp:4-10).
// build_global_hash_all builds the all-particle hash on the GPU;
// solve_cg_rbf_cpu is CPU-only and throws (use conjugate_gradient_rbf).
#pragma once

#include "vortex_particle_mc.hpp"

inline void build_global_hash_all(Simulation& sim) { sim.build_global_hash(); }

inline void solve_cg_rbf_cpu(Simulation&, float, float = 3e-3f, float = 1e-8f, int = 1000) {
    throw vpmc::unsupported("solve_cg_rbf_cpu");
}
