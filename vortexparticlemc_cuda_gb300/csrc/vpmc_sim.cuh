// vpmc_sim.cuh -- the simulation handle's state and the pieces its two
// translation units share: vpmc_sim.cu (creation, the MIS step, deformation,
// reinitialisation) and vpmc_adjoint.cu (the adjoint of the step).
#pragma once

#include <vector>

#include "vpmc_grid.cuh"

namespace vpmc {
namespace sim {

constexpr int kIcdfRef = 20;      // reference iCDF table length (src/vortex_particle_mc.cu:89)
constexpr int kJitTab = 1024;     // inverse spline-radius CDF table (unbiased law)

struct InstMC {
    float Lx, Ly, hw, dt;
    float dx;              // auxiliary-point offset, SimParam::dx = h_w / 2 (include/vortex_particle_mc.hpp:132)
    int periodic, law;
    float cum9[2];         // Omega_s (x9 when periodic), FP32 copy of the FP64 totals
    int cnt[2];
    long off[2];           // offsets of the subset in sub/cdf/guide arrays
    long goff[2];          // guide table offsets (cnt+2 entries each)
    uint32_t key0, key1;   // Philox key
    int p_begin, p_end;
    float icdf[kIcdfRef];  // reference law: r = interp(icdf) * h_w
};

__device__ __forceinline__ int inst_of(const InstMC* I, int n, long t) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (I[mid].p_begin <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// SamplingDiskRadius (include/monte_carlo_bs.hpp:73-89), same FP32 steps.
__host__ __device__ __forceinline__ float disk_radius(float2 d, bool periodic, float Lx, float Ly) {
    if (!periodic) return sqrtf(Lx * Lx + Ly * Ly);
    float m = 0.f;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy) {
            const float ix = d.x + dx * Lx, iy = d.y + dy * Ly;
            const float ex = ix - d.x, ey = iy - d.y;
            m = fmaxf(m, ex * ex + ey * ey);
        }
    return sqrtf(m);
}

struct GenArgs {
    const InstMC* mc;
    int n_inst;
    const GridInst* gi;
    const float2* pos;
    const float4* F;              // deformation mode: per-particle F (branch-1 jitter F r); else nullptr
    const float2* pos_sub;        // positions in subset order, or nullptr (then sub + pos)
    const int* sub;
    const double* cdf;
    const uint2* guide;           // CDF search brackets per guide slot
    const float2* jit;            // kJitTab pairs (t[i], t[i+1]) of the inverse spline-radius CDF (units of h_w)
    const unsigned long long* step;
    long t0, nt;                  // target chunk
    int N1, N2;
    int naux;                     // disk sample sets per target: 1, or 5 (C, L, R, T, B) in deformation mode
    int* src;                     // adjoint: branch-1 source particle of each sample (-1 otherwise), or nullptr
    float2* ys;
    uint32_t* qbin;
    uint32_t* qcount;
    uint32_t* qrank;
};

// One thread per (target, sign, sample): Philox draw, branch-1 CDF / image /
// jitter or disk draw, bin + rank (vpmc_sim.cu).
__global__ void k_gen(GenArgs a);

inline int blocks_for(long n, int threads = 256) {
    long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 65535L * 16) b = 65535L * 16;
    return int(b);
}

}  // namespace sim
}  // namespace vpmc

// (internal header of the library's two simulation units)
using namespace vpmc;
using namespace vpmc::sim;

struct vpmc_sim {
    vpmc_context* ctx = nullptr;
    int n_inst = 0;
    std::vector<vpmc_sim_params> prm;
    std::vector<int> counts;
    std::vector<long> begin;
    long N = 0;
    long t_begin = 0, t_end = 0;       // targets a pass estimates and advects (a shard); all N by default
    int N1 = 0, N2 = 0;
    uint64_t step = 0;
    int k_walk = 0, qpt = 4;
    int rows = 32;                     // candidate sub-rows per cell of the evaluation grid
    bool prepared = false;
    // device state
    DevBuf mem;                        // particles, subsets, tables
    float2* pos = nullptr;
    float2* pos_next = nullptr;
    float2* vel = nullptr;
    float* omega = nullptr;
    int* sub = nullptr;                // instance i: positives at 2*b_i, negatives at 2*b_i + n_i
    double* cdf = nullptr;
    uint2* guide = nullptr;            // CDF search brackets (see k_guide)
    float2* jit = nullptr;             // paired jitter table
    float2* pos_sub = nullptr;         // positions in subset order (plain method)
    InstMC* d_mc = nullptr;
    unsigned long long* d_step = nullptr;
    std::vector<InstMC> mc;
    // grid + sample working set
    DevBuf work;
    std::vector<GridInst> plan;
    GridBufs g;
    ItemBufs it;
    QueryBufs q;
    float2* ys = nullptr;
    long ys_t0 = -1, ys_nt = 0;        // targets whose samples ys holds (last chunk of the last pass)
    float* fv = nullptr;
    double* fv64 = nullptr;            // FP64 path only
    double* cum64 = nullptr;           // per instance Omega_+-, x9 when periodic (FP64 path)
    std::vector<double> cum64_h;       // host copy (the working set is re-carved on re-planning)
    int precision = 32;
    int rbf_solver = VPMC_RBF_CG;      // strength fits of init_strengths / reinit
    // deformation mode
    int deform = 0;
    float cover = 1.f;                 // plan cover: sigma_max(F) the walk reaches
    float min_cover = 1.f;
    float sigma = 1.f;                 // sigma_max of the current F
    long long over_cap = 0;            // particle-steps with sigma_max(F) > kCoverCap
    float4* F = nullptr;
    float4* F_next = nullptr;
    unsigned* d_sig = nullptr;         // 2 words
    double* d_check = nullptr;         // autotuner: sum of |u|^2 of a pass
    // adjoint: checkpointed forward record and working set
    bool frozen = false;               // prepare keeps the sampling CDF, refreshes only Omega
    bool prepared_once = false;
    int rec_steps = 0, rec_k = 0;
    uint64_t rec_step0 = 0;
    DevBuf ckpt, seg, adj;
    DevBuf aux;                        // deformation mode: vel5 (kept across re-planning)
    float2* vel5 = nullptr;            // 5 per particle
    long chunk_targets = 0;
    long max_samples = 0;
    // graphs
    cudaGraphExec_t graph_step = nullptr;
    cudaGraphExec_t graph_vel = nullptr;
    int launches_per_step = 0;
    float eval_ms = 0.f;
    int eval_launches = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> chunk_ev;   // start/end pair per chunk around the eval launch
};

namespace vpmc {
namespace sim {

// Samples per (target, sign): N1 branch-1 samples + N2 disk samples per point.
inline long samples_per(const vpmc_sim* s) { return long(s->N1) + long(s->deform ? 5 : 1) * s->N2; }
// One MIS pass over all targets (advect: step the positions), eagerly or by graph.
int run_pass(vpmc_sim* s, bool advect, int use_graph);
// Host and device step counter (the Philox counter's step word).
int set_step_counter(vpmc_sim* s, uint64_t step);

}  // namespace sim
}  // namespace vpmc
