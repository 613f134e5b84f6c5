/*
 * vpmc_oracle.h -- CPU oracle for the vortex-particle Monte-Carlo hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, its
 * C-ABI, the C++ API or the Python binding) links, loads or calls this code.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * (and its `--impl reference` arm) use it, as the checker / CPU baseline.
 *
 * Two families of functions live here:
 *   orc_*      -- restatements of the reference's CPU functions in the same
 *                 FP32 arithmetic and the same std::mt19937 random stream,
 *                 pinned bit-for-bit (or to float rounding of libm) against
 *                 golden vectors produced by the reference's own sources
 *                 (tests/golden/make_golden.py).
 *   orc_*_f64  -- FP64 restatements of the maths the GPU path computes
 *                 (query, RBF SpMV / CG, mollified and Plummer direct sums),
 *                 used as the accuracy oracle.
 *
 * Citations are file:line inside the reference project.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirror of VorticityView (include/vortex_particle_mc.hpp:77-94).  pos is the
 * global xy-interleaved position array, w the global strengths, F optional
 * (4 floats per particle, row-major {a,b,c,d}; NULL = identity).
 * vp_sort/cell_acc NULL selects the naive O(N) walk. */
typedef struct orc_view {
    const float* pos;
    const float* F;
    const float* w;
    int          N;
    const int*   vp_sort;
    const int*   cell_acc;
    int          rshx, rshy;
    float        Lx, Ly;
    int          cnt_view;
    const int*   sub;
} orc_view;

/* Mirror of MCBSCtx (include/monte_carlo_bs.hpp:15-35). */
typedef struct orc_mcctx {
    const int*   sub_pos;
    const int*   sub_neg;
    const float* cdf_pos;
    const float* cdf_neg;
    int          cnt_pos, cnt_neg;
    float        h_w;
    int          periodic;
    float        Lx, Ly;
    float        cum_pos, cum_neg;
    orc_view     pos_view, neg_view;
} orc_mcctx;

/* ---- spatial hash: src/cpu/hash.cpp:6-34 and :36-48 ---- */
void orc_fill_cells(int rshx, int rshy, float Lx, float Ly, int N,
                    const int* sub, const float* px, const float* py,
                    int* cell_num, int* cell_acc, int* vp_cell);
void orc_counting_sort(int N, int* cell_num, const int* cell_acc,
                       const int* vp_cell, int* vp_sort);

/* ---- the OpenMP pair: src/omp/hash_omp.cpp:12-54 and :56-70 ----
 * FillCells_omp: per-thread cell histograms merged under a critical section,
 * then the exclusive scan (results equal FillCells_cpu's).  CountingSort_omp:
 * reverse loop over particles split statically over threads, each slot taken
 * by an atomic fetch-sub on cell_num, based at the PREVIOUS cell's offset
 * cell_acc[c-1] (hash_omp.cpp:65) -- so its vp_sort is wrong (runs of
 * neighbouring cells overwrite each other), as the reference's is; every
 * store stays inside [0, N).  Kept for the timed CPU baseline only.
 * nthreads <= 0 uses OpenMP's default; returns the threads used. */
int orc_fill_cells_omp(int rshx, int rshy, float Lx, float Ly, int N,
                       const int* sub, const float* px, const float* py,
                       int* cell_num, int* cell_acc, int* vp_cell, int nthreads);
int orc_counting_sort_omp(int N, int* cell_num, const int* cell_acc,
                          const int* vp_cell, int* vp_sort, int nthreads);

/* ---- sign subsets + |omega| CDF: src/cpu/build_particle_sets.cpp:6-42 ---- */
void orc_build_subsets(int N, const float* omega,
                       int* sub_pos, int* sub_neg,
                       float* cdf_pos, float* cdf_neg,
                       int* cnt /*[2]*/, float* cum /*[2]*/);
/* FP64 CDF / Omega variant (same subsets). */
void orc_build_subsets_f64(int N, const float* omega,
                           int* sub_pos, int* sub_neg,
                           double* cdf_pos, double* cdf_neg,
                           int* cnt /*[2]*/, double* cum /*[2]*/);

/* ---- kernel radial CDF / iCDF tables: src/utilities.cu:12-96 (CPU branch) ---- */
void  orc_build_cubic_rcdf(float h_w, int length, float* cdf);
void  orc_cdf_to_icdf(const float* cdf, int length, float h_w, float* icdf);
float orc_cubic_spline_pdf(float r, float h_w);   /* include/utilities.hpp:7-17 */

/* ---- vorticity queries ---- */
/* evalVorticityAbs_cpu, src/cpu/evaluate_vorticity.cpp:8-75, batched. */
void orc_eval_vorticity_cpu(const orc_view* v, const float* pts, int M,
                            int sign, int use_signed, int exclude_center,
                            float h_w, int periodic, float* out);
/* queryVorticityAbs (include/vorticity_query.cuh:15-79) restated in FP64:
 * same 3x3 hash walk (incl. its double visit of cells when rsh<3), F-deformed
 * distance, minimum image, 2*h_w cutoff. */
void orc_query_vorticity_f64(const orc_view* v, const float* pts, int M,
                             int sign, int use_signed, int exclude_center,
                             double h_w, int periodic, double* out);
/* Exact FP64 smoothed field: every particle once, nearest periodic image,
 * isotropic W (F ignored).  The value the GPU query must reproduce. */
void orc_field_exact_f64(const float* pos, const float* w, int N,
                         const float* pts, int M, int sign, int use_signed,
                         double h_w, double Lx, double Ly, int periodic,
                         double* out);

/* ---- MIS Monte-Carlo Biot-Savart: src/cpu/monte_carlo_bs.cpp:28-128,
 *      src/cpu/monte_carlo_sampling.cpp:9-45 ---- */
typedef struct orc_rng orc_rng;               /* wraps std::mt19937 */
orc_rng* orc_rng_create(uint32_t seed);
void     orc_rng_destroy(orc_rng* r);
/* One monte_carlo_bs_cpu call.  dst5 = {main, left, right, top, bottom} xy
 * (10 floats); out10 = the five float2 estimates. */
void orc_mc_bs_estimate(const orc_mcctx* ctx, const float* pos,
                        const float* dst5, int sign, int auxiliary,
                        int N1, int N2, orc_rng* rng, float* out10);
/* The per-particle body of Simulation::step_cpu (src/cpu/simulation_step.cpp:
 * 31-55) with aux = 0: u = est(+1) - est(-1) for each target, one rng for the
 * whole loop (targets in order). */
void orc_mc_velocity(const orc_mcctx* ctx, const float* pos,
                     const float* targets, int M, int N1, int N2,
                     uint32_t seed, float* vel);
/* Same estimator, OpenMP over targets, target t seeded with seed + t (so the
 * result does not depend on the thread count).  Returns threads used.  This
 * parallel loop is harness-level: the reference's step_cpu is serial.
 * law 0 = monte_carlo_bs_cpu; law 1 = the sampling law of the reference's GPU
 * kernel monte_carlo_bs_kernel_safe (jitter from `icdf` [icdf_L entries, as
 * build_cubic_rcdf/cdf_to_icdf make it], GPU query convention in FP64,
 * minimum-image alpha/r) restated with std::mt19937. */
int  orc_mc_velocity_omp(const orc_mcctx* ctx, const float* pos,
                         const float* targets, int M, int N1, int N2,
                         uint32_t seed, float* vel, int nthreads,
                         int law, const float* icdf, int icdf_L);

/* The GPU kernel's law (law 1 above) with deformation, as the reference's
 * step_cuda runs it (aux = 1): views carry F (kernels W(|F^-1 d|)), branch-1
 * jitter is F r, five targets per particle (C, L, R, T, B at offsets dx).
 * vel10 = the five u(+) - u(-) per target.  Target t seeded with seed + t. */
int  orc_mc_velocity5_omp(const orc_mcctx* ctx, const float* pos, const float* F,
                          const float* targets, int M, int N1, int N2, float dx,
                          uint32_t seed, float* vel10, int nthreads, const float* icdf,
                          int icdf_L);

/* This build's plain MIS step (both laws) restated in FP64 with FP64
 * positions, for finite-difference checks of the adjoint: the library's
 * Philox keys/counters and sampling maps, the branch-1 index drawn from the
 * |omega| CDF of omega_sample (frozen sampling law) while field weights and
 * Omega use omega, brute-force fields (3x3 images of the sample's tile for
 * the unbiased law, the periodic field for the reference law), FP64 MIS
 * terms, forward Euler with FP64 wrap.  law: 0 reference, 1 unbiased.
 * Returns -1 if omega and omega_sample differ in sign pattern. */
int orc_mis_forward_f64(const float* pos0, const float* omega, const float* omega_sample, int N, int Nx,
                        float hwr, float Lx, float Ly, int periodic, int law, int N1, int N2, float dt,
                        uint64_t seed, uint64_t step0, int nsteps, double* pos_out, int nthreads);

/* ---- RBF system: src/cuda/cg_rbf_init.cu:11-116 restated in FP64 ---- */
/* y = A x,  A_ij = W(|F_j^-1 (x_j - x_i)|) via the all-particle 3x3 walk. */
void orc_rbf_matvec_f64(const orc_view* all_view, const double* x, double* y,
                        double h_w, int periodic, int nthreads);
/* CG as conjugate_gradient_rbf: x0 = b / W(0), stop at |r|/|b| < tol.
 * Returns iterations; *relres = final recursive relative residual,
 * *true_relres = |b - A x|/|b| recomputed at exit. */
int  orc_cg_rbf_f64(const orc_view* all_view, const float* b, double* x,
                    double h_w, int periodic, double tol, int max_iter,
                    double* relres, double* true_relres, int nthreads);

/* ---- direct Biot-Savart sums ---- */
/* Velocity of the smoothed field: sum over the 3x3 periodic images (or just
 * the domain when !periodic) of omega_i * perp(d)/(2 pi |d|^2) * M(|d|/h_w),
 * M = cubic-spline mass inside radius |d|.  This is the integral the MIS
 * estimator estimates (unbiased law). */
void orc_direct_mollified_f64(const float* pos, const float* omega, int N,
                              const float* pts, int M, double h_w,
                              double Lx, double Ly, int periodic,
                              double* out_uv, int nthreads);
/* The same velocity for deformed kernels W(|F_i^-1 (y - x_i)|) (F row-major
 * per particle, NULL = identity): the Biot-Savart integral of each blob by
 * quadrature in FP64 -- Gauss-Legendre in blob coordinates when the target
 * is more than 3 sigma_max h_w away, else rays from the target's preimage
 * (exact ray/circle splits, GL along each ray, trapezoid or windowed GL in
 * angle).  The mean of the unbiased deformed MIS estimator. */
void orc_direct_deformed_f64(const float* pos, const float* omega, const float* F, int N,
                             const float* pts, int M, double h_w, double Lx, double Ly,
                             int periodic, double* out_uv, int nthreads);
/* biot_savart_naive_kernel (src/cuda/naive_biot_savart.cu:15-40) in FP64:
 * Plummer core eps, minimum image, j == i skipped.  Targets are particle
 * indices. */
void orc_direct_plummer_f64(const float* pos, const float* omega, int N,
                            const int* tidx, int M, double eps,
                            double Lx, double Ly, int periodic,
                            double* out_uv, int nthreads);
/* Spline mass inside radius q*h_w (q in [0,1], 1 beyond). */
double orc_spline_mass(double q);

/* Version / self-description string. */
const char* orc_version(void);

#ifdef __cplusplus
}
#endif
