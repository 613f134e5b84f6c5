/*
 * vpmc.h -- C ABI of the GB300 (sm_103a) vortex-particle Monte-Carlo hot path.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns a
 * vpmc_status (0 = success) and never aborts.  Device pointers are CUDA
 * global-memory addresses on the context's device; entry points whose name
 * ends in `_host` take host pointers and do the copies themselves.  Work is
 * issued on the context's stream; a call returns when its results are
 * complete unless documented otherwise.  A context (and every handle made
 * from it) must not be used by two host threads at once.
 *
 * The comment on each entry point cites the reference interface it replaces
 * (file:line inside the reference project GargantuaOmni/VortexParticleMC_cuda).
 * Layouts follow the reference: positions are float2 (x,y interleaved), the
 * deformation F is float4 {a,b,c,d} (row-major 2x2), strengths are float.
 */
#ifndef VPMC_H
#define VPMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VPMC_ABI_VERSION 1

typedef enum vpmc_status {
    VPMC_OK = 0,
    VPMC_ERR_INVALID = 1,        /* bad argument (NULL, negative size, ...)        */
    VPMC_ERR_UNSUPPORTED = 2,    /* backend/feature not provided (CPU/OMP paths)   */
    VPMC_ERR_CUDA = 3,           /* a CUDA runtime call failed                     */
    VPMC_ERR_NOMEM = 4,          /* device allocation failed                       */
    VPMC_ERR_TIMEOUT = 5,        /* a bounded device wait expired                  */
    VPMC_ERR_DEVICE = 6,         /* a kernel reported an internal error            */
    VPMC_ERR_GEOMETRY = 7,       /* domain/grid too small for the neighbour walk   */
    VPMC_ERR_CAPACITY = 8,       /* a size exceeds a documented maximum            */
    VPMC_ERR_NOT_CONVERGED = 9,  /* iterative solve stopped before its tolerance   */
    VPMC_ERR_NONFINITE = 10      /* NaN/Inf found in an input or a result          */
} vpmc_status;

typedef struct vpmc_context vpmc_context;
typedef struct vpmc_sim vpmc_sim;

/* Estimator law for the MIS Biot-Savart velocity.
 *   VPMC_LAW_REFERENCE reproduces the sampling law of
 *     monte_carlo_bs_kernel_safe (src/cuda/monte_carlo_bs.cu:144-271):
 *     branch-1 jitter radius = iCDF table * h_w (the table already holds h_w),
 *     disk radius R*sqrt(u) weighted as alpha/r, minimum-image r in alpha/r,
 *     periodic field query.  Biased (its mean is not the Biot-Savart integral),
 *     kept for variance parity and like-for-like speed.
 *   VPMC_LAW_UNBIASED draws the branch-1 jitter from the cubic spline itself,
 *     the disk radius uniformly in r (density alpha/r), uses raw distances
 *     and restricts the field to the 3x3 periodic images the branch-1 density
 *     covers, so its mean is the velocity of the smoothed field. */
typedef enum vpmc_law { VPMC_LAW_REFERENCE = 0, VPMC_LAW_UNBIASED = 1 } vpmc_law;

/* Direct-sum kernels. */
typedef enum vpmc_direct_kernel {
    VPMC_DIRECT_MOLLIFIED = 0,  /* smoothed-field velocity, 3x3 periodic images (oracle of the MC mean) */
    VPMC_DIRECT_PLUMMER = 1     /* biot_savart_naive_kernel: Plummer core, minimum image, j != i        */
} vpmc_direct_kernel;

/* ------------------------------------------------------------------ context */
/* Create a context on `device`.  `stream` may be NULL (the context creates a
 * non-blocking stream) or a cudaStream_t the caller owns.  No reference
 * counterpart: the reference runs everything on the default stream. */
int vpmc_context_create(int device, void* stream, vpmc_context** out);
int vpmc_context_destroy(vpmc_context* ctx);
/* Stream the context issues work on (a cudaStream_t). */
void* vpmc_context_stream(vpmc_context* ctx);
/* Wait for all work issued on the context; returns the first pending error. */
int vpmc_context_sync(vpmc_context* ctx);
/* Bytes of device scratch the context currently holds. */
size_t vpmc_context_scratch_bytes(vpmc_context* ctx);
const char* vpmc_status_string(int status);
int vpmc_abi_version(void);
/* Number of kernels this library has launched in this process (all contexts):
 * a counter for benchmarks that report GPU launch counts. */
uint64_t vpmc_kernel_launch_count(void);
/* Bounded device waits.  The field-evaluation kernel stages candidates with
 * bulk copies and waits for them on an mbarrier; each wait polls at most
 * `polls` times (default VPMC_WAIT_LIMIT_DEFAULT, far beyond any copy's
 * latency), then the kernel lets the copy in flight land, stops, and the call
 * returns VPMC_ERR_TIMEOUT with the context still usable.  0 makes every such
 * wait give up at once: a way to exercise that error path without a fault.
 * No reference counterpart (its only device check is an unused trap,
 * src/utilities.cu:99-103). */
#define VPMC_WAIT_LIMIT_DEFAULT (1u << 26)
int vpmc_context_set_wait_limit(vpmc_context* ctx, uint32_t polls);

/* --------------------------------------------------------------- hash (a1-a3)
 * Uniform-grid spatial hash of a particle subset, bit-exact with the
 * reference's deterministic CPU build (cells ascending, members ascending by
 * local index within a cell). */

/* FillCells_cuda, src/cuda/hash.cu:42-69 (and FillCells_cpu, src/cpu/hash.cpp:
 * 6-34).  For i < N: j = sub[i]; cell = clamp(floor(x*rshx/Lx)) * rshy +
 * clamp(floor(y*rshy/Ly)); vp_cell[i] = cell; cell_num = per-cell counts;
 * cell_acc = exclusive prefix of cell_num.  All pointers are device pointers;
 * cell_num/cell_acc hold rshx*rshy ints. */
int vpmc_fill_cells(vpmc_context* ctx, int rshx, int rshy, float Lx, float Ly, int N,
                    const int* sub, const float* pos, int* cell_num, int* cell_acc,
                    int* vp_cell);

/* CountingSort_cuda, src/cuda/hash.cu:71-91 (CountingSort_cpu, src/cpu/hash.cpp:
 * 36-48).  vp_sort[cell_acc[c] + k] = k-th local index (ascending) of cell c;
 * cell_num is left all-zero as the reference leaves it.  `ncell` = number of
 * cells (the reference infers it); pass <= 0 to have it computed (one extra
 * device-to-host read).  Deterministic, unlike the reference's atomicSub
 * scatter. */
int vpmc_counting_sort(vpmc_context* ctx, int N, int ncell, int* cell_num,
                       const int* cell_acc, const int* vp_cell, int* vp_sort);

/* FillCells + CountingSort in one call (the pair Simulation::do_spatial_hashing
 * issues per subset, src/vortex_particle_mc.cu:140-164).  cell_num may be NULL. */
int vpmc_hash_build(vpmc_context* ctx, int rshx, int rshy, float Lx, float Ly, int N,
                    const int* sub, const float* pos, int* cell_num, int* cell_acc,
                    int* vp_cell, int* vp_sort);

/* Same as vpmc_hash_build with host buffers (copies in and out). */
int vpmc_hash_build_host(vpmc_context* ctx, int rshx, int rshy, float Lx, float Ly, int N,
                         int n_pos, const int* sub, const float* pos, int* cell_num,
                         int* cell_acc, int* vp_cell, int* vp_sort);

/* Allocation-free variant of vpmc_hash_build, with no counterpart in the
 * reference.  For callers that cannot allocate device memory -- a host
 * application that owns all device memory and forbids plugins to call
 * cudaMalloc, or a real-time loop that cannot take cudaMalloc's implicit
 * device synchronisation.  No context: work runs on `stream` (a cudaStream_t;
 * NULL = the legacy default stream) and the call returns when it is done.
 * It calls no cudaMalloc/cudaFree and no allocating library routine; its
 * radix-sort and scan scratch is a fixed ~4.3 MB __device__ array inside the
 * library that every GPU using the library holds until process exit.
 * Limits: N <= 262144 particles and rshx*rshy <= 1048576 cells, otherwise
 * VPMC_ERR_CAPACITY.  All calls share that scratch, so calls that overlap on
 * the GPU (two host threads, or two streams) race; every call waits for its
 * stream to finish before it returns (also on an error after work was
 * queued), so consecutive calls are safe.  `stream` must belong to the
 * current device (VPMC_ERR_INVALID otherwise).  The first call on a device
 * looks up the scratch array's address and keeps it for the process: make
 * it before any stream capture, and do not use this entry point after
 * cudaDeviceReset or under a non-primary context (the kept address would be
 * stale).  Results are identical to vpmc_hash_build (device pointers, same
 * layouts). */
int vpmc_hash_build_noalloc(void* stream, int rshx, int rshy, float Lx, float Ly, int N,
                            const int* sub, const float* pos, int* cell_num, int* cell_acc,
                            int* vp_cell, int* vp_sort);

/* --------------------------------------------------------------- subsets (a4)
 * build_subsets_cuda, src/cuda/build_particle_sets.cu:11-89: split particle
 * indices by the sign of omega (zeros belong to neither), |omega| prefix sums
 * normalised to a CDF, and the totals.  The CDF and totals are FP64 (the
 * reference is FP32).  cdf32_* (optional, may be NULL) receive the FP32 copy
 * the reference's layout uses.  cnt[2] and cum[2] are HOST pointers. */
int vpmc_build_subsets(vpmc_context* ctx, int N, const float* omega, int* sub_pos,
                       int* sub_neg, double* cdf_pos, double* cdf_neg, float* cdf32_pos,
                       float* cdf32_neg, int* cnt, double* cum);

/* --------------------------------------------------------- kernel table (a5)
 * build_cubic_rcdf + cdf_to_icdf, src/utilities.cu:12-96 (host arithmetic, same
 * FP32 steps).  Writes `length` floats each to HOST arrays (icdf may be NULL). */
int vpmc_kernel_icdf_table(float h_w, int length, float* cdf, float* icdf);

/* Cubic B-spline W(r; h_w), include/utilities.hpp:7-17, host evaluation. */
float vpmc_cubic_spline(float r, float h_w);

/* ------------------------------------------------------ vorticity query (a7)
 * queryVorticityAbs, include/vorticity_query.cuh:15-79, for M points at once:
 *   out[m] = sum_i  wv_i * W(|F_i^-1 d_i|; h_w),  d_i = x_i - p_m (nearest
 *   periodic image when periodic), over particles with omega_i > 0 (sign > 0),
 *   omega_i < 0 (sign < 0) or all (sign == 0); wv_i = omega_i if use_signed
 *   else |omega_i|; exclude_center drops pairs closer than 1e-6.
 * F may be NULL (identity).  Points are wrapped into the domain when periodic
 * and give 0 outside it otherwise.  Each particle contributes once, also when
 * the reference's hash would have fewer than 3 cells per axis (where its
 * 3x3 walk visits cells twice).  pos/omega/F/pts/out are device pointers. */
int vpmc_query_vorticity(vpmc_context* ctx, int N, const float* pos, const float* omega,
                         const float* F, int M, const float* pts, int sign,
                         int use_signed, int exclude_center, float h_w, float Lx,
                         float Ly, int periodic, float* out);

/* The same query with every pair and the sum in FP64 (the plain FP64 GPU path
 * of the query: the FP32 strengths, split exactly into two floats, times the
 * spline evaluated in FP64); isotropic kernels only, no exclude_center.
 * out: M doubles (device).  No reference counterpart (an FP64 comparison
 * path for queryVorticityAbs, include/vorticity_query.cuh:15-79). */
int vpmc_query_vorticity_f64(vpmc_context* ctx, int N, const float* pos, const float* omega,
                             int M, const float* pts, int sign, int use_signed, float h_w,
                             float Lx, float Ly, int periodic, double* out);

/* ---------------------------------------------------------- RBF / CG (a10)
 * Ax_cuda, src/cuda/cg_rbf_init.cu:33-50 (matvec_kernel :11-31):
 *   y_i = sum_j x_j W(|x_j - x_i|; h_w) over all particles (nearest image).
 * `precise` != 0 evaluates and accumulates in-support pairs in FP64; 0 uses
 * FP32 pair arithmetic with compensated FP32 sums.  Device pointers. */
int vpmc_rbf_matvec(vpmc_context* ctx, int N, const float* pos, const float* x, float* y,
                    float h_w, float Lx, float Ly, int periodic, int precise);

/* conjugate_gradient_rbf, src/cuda/cg_rbf_init.cu:53-116: solve A w = b with
 * A as above, w0 = b / W(0), stop when |r|/|b| < tol or after max_iter
 * iterations.  Dot products and norms are FP64.  omega_out (device) receives
 * w.  info (HOST, may be NULL) receives {iterations, recursive |r|/|b|,
 * true |b - A w|/|b| recomputed with the FP64 SpMV}.  Returns
 * VPMC_ERR_NOT_CONVERGED (with omega_out written) when max_iter is reached. */
int vpmc_cg_rbf(vpmc_context* ctx, int N, const float* pos, const float* b,
                float* omega_out, float h_w, float Lx, float Ly, int periodic,
                double tol, int max_iter, double* info);

/* vpmc_cg_rbf with an FP64 right-hand side (device, N doubles): a field
 * sampled in FP64 keeps its structure (e.g. a lattice Fourier mode stays an
 * exact eigenvector of A), which its FP32 rounding does not. */
int vpmc_cg_rbf_f64rhs(vpmc_context* ctx, int N, const float* pos, const double* b,
                       float* omega_out, float h_w, float Lx, float Ly, int periodic,
                       double tol, int max_iter, double* info);

/* The same system solved by MINRES (Paige & Saunders 1975) instead of CG,
 * from the same starting point w0 = b / W(0), with the FP64 SpMV and FP64
 * vectors, dots and norms.  The RBF matrix is symmetric but indefinite (the
 * cubic spline's 2-D symbol is negative at high wavenumbers) with eigenvalues
 * near zero on both sides, where CG can stall or break down; MINRES
 * minimises |b - A w| over the same Krylov space, so the residual falls
 * monotonically.  Stops when the recursive |r|/|b| < tol.  info (HOST, may be
 * NULL) = {iterations, recursive |r|/|b|, true |b - A w|/|b|}; returns
 * VPMC_ERR_NOT_CONVERGED (with omega_out written) after max_iter.  No
 * reference counterpart: an alternative to conjugate_gradient_rbf
 * (src/cuda/cg_rbf_init.cu:53-116) for fields that are not lattice modes. */
int vpmc_minres_rbf(vpmc_context* ctx, int N, const float* pos, const float* b,
                    float* omega_out, float h_w, float Lx, float Ly, int periodic,
                    double tol, int max_iter, double* info);
int vpmc_minres_rbf_f64rhs(vpmc_context* ctx, int N, const float* pos, const double* b,
                           float* omega_out, float h_w, float Lx, float Ly, int periodic,
                           double tol, int max_iter, double* info);

/* ------------------------------------------------------ direct sums (a11)
 * biot_savart_naive_kernel, src/cuda/naive_biot_savart.cu:15-40, in FP64.
 * VPMC_DIRECT_PLUMMER: targets are particle indices `tidx` (M of them),
 *   u_i = sum_{j != i} omega_j perp(d)/(2 pi (|d|^2 + eps^2)), d minimum image.
 * VPMC_DIRECT_MOLLIFIED: targets are points `pts` (M of them), velocity of the
 *   smoothed field over the 3x3 periodic images (or the domain alone when
 *   !periodic): sum omega_j perp(d)/(2 pi |d|^2) M(|d|/h_w), M the spline mass.
 * out_uv: 2*M doubles (device).  param = eps (Plummer) or h_w (mollified). */
int vpmc_direct_velocity_f64(vpmc_context* ctx, int kernel, int N, const float* pos,
                             const float* omega, int M, const float* pts, const int* tidx,
                             double param, double Lx, double Ly, int periodic,
                             double* out_uv);

/* The same direct sums in FP32 tiles: the deterministic "P" particle method
 * of the reference (biot_savart_naive_kernel is FP32), for P-vs-MC
 * comparisons.  param = eps (Plummer) or h_w (mollified); out_uv: 2*M floats
 * (device).  Fixed-order sums (deterministic). */
int vpmc_direct_velocity_f32(vpmc_context* ctx, int kernel, int N, const float* pos,
                             const float* omega, int M, const float* pts, const int* tidx,
                             float param, float Lx, float Ly, int periodic, float* out_uv);

/* ------------------------------------------------- simulation (a8, a9, a12)
 * SimParam, include/vortex_particle_mc.hpp:96-134; one entry per instance.
 * h = Lx/Nx, h_w = h*hwr, dx = h_w/2 are derived as the reference does.  */
typedef struct vpmc_sim_params {
    float    dt;
    float    Lx, Ly;
    int      Nx;          /* ResolutionX */
    float    hwr;         /* h_w / h     */
    int      N1, N2;      /* MIS samples per target and sign (same for all instances) */
    int      periodic;
    int      law;         /* vpmc_law */
    uint64_t seed;        /* Philox key; instance index is mixed in */
} vpmc_sim_params;

/* Create a simulation of `n_inst` independent instances (an ensemble; 1 for a
 * single run).  counts[k] = particles of instance k; instances are stored
 * back to back in the order given.  Mirrors Simulation(SimParam) +
 * ParticleSet::resize (include/vortex_particle_mc.hpp:34-50,136-192). */
int vpmc_sim_create(vpmc_context* ctx, int n_inst, const vpmc_sim_params* prms,
                    const int* counts, vpmc_sim** out);
int vpmc_sim_destroy(vpmc_sim* sim);
int vpmc_sim_num_particles(vpmc_sim* sim);

/* Upload positions (2N floats) and strengths (N floats).  is_host selects
 * host or device source pointers.  omega may be NULL (left unchanged).
 * Invalidates subsets/CDFs (rebuilt by vpmc_sim_prepare). */
int vpmc_sim_set_particles(vpmc_sim* sim, const float* pos, const float* omega, int is_host);
int vpmc_sim_get_particles(vpmc_sim* sim, float* pos, float* omega, float* vel, int is_host);

/* Simulation::init's strength initialisation (src/vortex_particle_mc.cu:99-105,
 * prepare_rhs_b :237-260, conjugate_gradient_rbf): b = omega_field (device,
 * N floats; NULL = Taylor-Green 4 pi sin(2 pi x) sin(2 pi y), include/
 * analytical_flow.hpp:24-28, evaluated in FP64), solved per instance by
 * vpmc_cg_rbf (vpmc_cg_rbf_f64rhs for the Taylor-Green field).
 * info (HOST, may be NULL): 3 doubles per instance as vpmc_cg_rbf. */
int vpmc_sim_init_strengths(vpmc_sim* sim, const float* omega_field, double tol,
                            int max_iter, double* info);

/* Solver of the strength fits vpmc_sim_init_strengths and vpmc_sim_reinit
 * make: VPMC_RBF_CG (default, the reference's conjugate_gradient_rbf) or
 * VPMC_RBF_MINRES (vpmc_minres_rbf). */
typedef enum vpmc_rbf_solver { VPMC_RBF_CG = 0, VPMC_RBF_MINRES = 1 } vpmc_rbf_solver;
int vpmc_sim_set_rbf_solver(vpmc_sim* sim, int solver);

/* Sign subsets + FP64 |omega| CDFs + sampling tables for every instance
 * (build_subsets_cuda).  Strengths are conserved, so this runs once after
 * the strengths are set, not per step. */
int vpmc_sim_prepare(vpmc_sim* sim);

/* Simulation::step_cuda (src/cuda/simulation_step.cu:9-90) without the
 * kernel deformation (aux=0, F=I): rebuild the hash, estimate
 * u = u(+) - u(-) with the MIS estimator, x += dt*u, wrap x into the domain
 * in FP64.  nsteps steps; the first call captures a CUDA graph per step
 * shape and later calls replay it (use_graph != 0). */
int vpmc_sim_step(vpmc_sim* sim, int nsteps, int use_graph);

/* The MIS velocity at the current positions without moving them (for
 * estimator checks).  vel: 2N floats, device.  `step` selects the Philox
 * stream (the step counter is not advanced). */
int vpmc_sim_velocity(vpmc_sim* sim, uint64_t step, float* vel);

/* One step with host buffers: copies pos_in (2N) to the device, steps,
 * copies positions and velocities back (2N each). */
int vpmc_sim_step_host(vpmc_sim* sim, const float* pos_in, float* pos_out, float* vel_out);

/* Forward-Euler update with the FP64 periodic wrap, x += dt*u (the position
 * update of Simulation::step_cuda / step_cuda_naive, src/cuda/simulation_step.cu:
 * 77-89, 115-128).  Velocities come from vel (float2) or, if vel is NULL, from
 * vel64 (double2).  Device pointers. */
int vpmc_advect(vpmc_context* ctx, int N, float* pos, const float* vel, const double* vel64, float dt,
                float Lx, float Ly, int periodic);

/* Deformation mode (the reference's Simulation::step_cuda, src/cuda/
 * simulation_step.cu:9-90, which runs monte_carlo_bs_kernel_safe with aux = 1
 * and update_jacobian_from5): each particle carries F (row-major
 * {F11, F12, F21, F22}, identity at creation); vorticity kernels become
 * W(|F^-1 d|), branch-1 jitter becomes F r, every target gets the four
 * auxiliary points x -/+ dx e_x, x +/- dx e_y (dx = h_w / 2) with their own
 * N2 disk samples each and a share of the N1 branch-1 samples, and each step
 * ends with F = renorm_det1(I + dt grad u) from central differences of the
 * auxiliary velocities.  on = 0 returns to the plain method (F kept, unused).
 * The grid walk reaches cover * h_w with cover >= sigma_max(F) (rounded up to
 * 1/16, re-planned between steps when F stretches further, at most 2 = the
 * reach of the reference's 3x3 walk of 2 h_w cells); min_cover (<= 2) forces
 * a wider reach.  FP32 only (VPMC_ERR_UNSUPPORTED with precision 64). */
int vpmc_sim_set_deformation(vpmc_sim* sim, int on, float min_cover);
/* update_jacobian_from5 + renorm_det1 (src/cuda/monte_carlo_bs.cu:274-288,
 * include/monte_carlo_bs.cuh:140-150) for callers that hold the five velocity
 * arrays (float2, device; velC is not read, as in the reference): F_out
 * (float4, device) = renorm_det1(I + dt grad u) with grad u from central
 * differences of L/R/T/B at offset dx, in FP32 as the reference. */
int vpmc_update_jacobian_from5(vpmc_context* ctx, int N, float dt, float dx, const float* velC,
                               const float* velL, const float* velR, const float* velT,
                               const float* velB, float* F_out);

/* F of every particle (4N floats); set_F rejects det F <= 0 or non-finite F. */
int vpmc_sim_set_F(vpmc_sim* sim, const float* F, int is_host);
int vpmc_sim_get_F(vpmc_sim* sim, float* F, int is_host);
/* Deformation mode: the five velocities (C, L, R, T, B; u(+) - u(-)) of the
 * last pass, 10N floats (the reference's velC..velB). */
int vpmc_sim_get_aux_velocities(vpmc_sim* sim, float* vel5, int is_host);
/* info[0] = sigma_max of the current F, info[1] = cover in use, info[2] =
 * particle-steps whose new F stretched beyond 2 (not covered), info[3] = 1 in
 * deformation mode. */
int vpmc_sim_deform_info(vpmc_sim* sim, double* info);

/* Reinitialisation (README.md:319-321 and :416-420 of the reference; not in
 * its code): for every instance, the current field (signed, deformed kernels
 * in deformation mode) is evaluated at a fresh cell-centred Nx x Ny lattice,
 * positions move to that lattice, F is reset to the identity, and the
 * strengths are re-fitted by CG-RBF to the evaluated field (tol, max_iter as
 * in vpmc_cg_rbf; info: 3 per instance).  Needs N_i = Nx * Ny per instance.
 * Returns VPMC_ERR_NOT_CONVERGED (after finishing) if some CG did not reach tol. */
int vpmc_sim_reinit(vpmc_sim* sim, double tol, int max_iter, double* info);

/* Field rasterisation for validation images (the grid diagnostic of
 * Simulation::test_vorticity_grid, src/vortex_particle_mc.cu:332-456): the
 * field of instance inst at the cell centres of a res_x x res_y grid over its
 * domain (ix-major), sign 0 = signed field, +1 / -1 = |omega| of the
 * positive / negative particles (deformed kernels in deformation mode).
 * out: res_x * res_y floats (device). */
int vpmc_sim_vorticity_grid(vpmc_sim* sim, int inst, int res_x, int res_y, int sign, float* out);

/* ---------------------------------------------------------------- adjoint
 * Gradients of a loss of the final positions with respect to the initial
 * positions and the strengths, through nsteps plain-method MIS steps with
 * the forward's own samples (common random numbers: the same Philox streams;
 * the discrete CDF-index and image choices are held fixed, i.e. the pathwise
 * derivative).  No counterpart in the reference.
 *   vpmc_sim_record: run nsteps from the current state, keeping positions
 *     every k_ckpt steps (and the final state) on the device.
 *   vpmc_sim_adjoint: given dL/dX_T (2N doubles, device), recompute each
 *     segment from its checkpoint and run the adjoint steps backwards; writes
 *     dL/dX_0 (2N doubles) and dL/domega (N doubles); the simulation is left
 *     in the recorded final state.  The trajectory is the forward's (its
 *     precision); the adjoint's field values and gradients at the samples,
 *     its transposed sums and its MIS-term derivatives take their terms in
 *     the forward's precision (for the FP32 path: FP32 pairs summed into
 *     FP64 per candidate run, the transposed sums compensated in FP32 per
 *     work item, FP32 MIS-term derivatives); every accumulation across
 *     runs, items and samples is FP64.
 *     flags: VPMC_ADJ_SCORE adds the score-function term of the discrete
 *     branch-1 draw (P(I = J) = |omega_J| / Omega), which makes dL/domega an
 *     unbiased estimate of the gradient of the expected trajectory; without
 *     it dL/domega is the exact derivative of the frozen-sampling estimator.
 *   vpmc_sim_freeze_sampling: on = keep the |omega| CDF (sampling law) of
 *     the last prepare when strengths change, refreshing only Omega; for
 *     finite-difference checks of the pathwise derivative.  The sign of
 *     every strength must stay (VPMC_ERR_INVALID otherwise).
 * Deformation mode: VPMC_ERR_UNSUPPORTED. */
int vpmc_sim_record(vpmc_sim* sim, int nsteps, int k_ckpt);
enum { VPMC_ADJ_SCORE = 1 };
int vpmc_sim_adjoint(vpmc_sim* sim, const double* dL_dXT, double* dL_dX0, double* dL_domega, int flags);
int vpmc_sim_freeze_sampling(vpmc_sim* sim, int on);

/* Shard of the targets: MIS passes (steps, velocity passes) estimate and
 * advect only the particles [begin, end) of the instance-concatenated order;
 * every particle stays a source (the hash and the field cover all N).  A
 * target's samples depend only on its instance, its instance-local index and
 * the step (the Philox counter), so a shard's velocities and positions are
 * bit-identical to the whole run's as long as all positions agree: a sharded
 * run on several GPUs all-gathers the updated positions after each step.
 * Particles outside the range keep their positions and velocities.  Not with
 * deformation mode or the adjoint (VPMC_ERR_UNSUPPORTED).  Default: [0, N).
 * No reference counterpart (the reference runs on one GPU). */
int vpmc_sim_set_target_range(vpmc_sim* sim, long long begin, long long end);
int vpmc_sim_get_target_range(vpmc_sim* sim, long long* begin, long long* end);

/* Change the estimator law / seed / step counter of an existing simulation. */
int vpmc_sim_set_law(vpmc_sim* sim, int law);
int vpmc_sim_set_seed(vpmc_sim* sim, uint64_t seed);
int vpmc_sim_set_step(vpmc_sim* sim, uint64_t step);
uint64_t vpmc_sim_get_step(vpmc_sim* sim);

/* Arithmetic of the MIS step: 32 (default: FP32 pair arithmetic with
 * compensated sums) or 64 (the plain FP64 path of the same estimator: field
 * values, MIS terms, sums and the Euler update in FP64; sample points are
 * drawn as in FP32 mode).  The FP64 path is the baseline the FP32 path is
 * measured against; on GB300 FP64 runs at a small fraction of the FP32 rate. */
int vpmc_sim_set_precision(vpmc_sim* sim, int bits);

/* Neighbour-walk tuning: cells per h_w (1 <= k <= 8; the walk covers the
 * (2k+1)^2 cells around a bin minus the corner cells beyond reach) and
 * queries per thread in the field-evaluation kernel (4, 6 or 8), or 1 for the
 * tensor-core evaluation (squared distances of 128 queries x 128 candidates
 * per tcgen05 multiply; plain kernels only, deformed kernels keep 4).
 * 0 = default (k = 2, 4 queries per thread). */
int vpmc_sim_set_tuning(vpmc_sim* sim, int k_walk, int queries_per_thread);
int vpmc_sim_get_tuning(vpmc_sim* sim, int* k_walk, int* queries_per_thread);

/* Autotuner (no reference counterpart): times one full MIS velocity pass per
 * candidate (k_walk, queries_per_thread) in {2..8}x{4} + {3,4,6,8}x{6} + {2,3,4,6,8}x{8}
 * + {3..8}x{1} (the tensor-core evaluation; not with deformed kernels), keeps
 * the fastest, and caches the choice in-process by (hwr, samples per target,
 * particles per h_w^2).  Results do not depend on the choice beyond FP32
 * rounding of the field sums, and the autotuner checks that: each
 * candidate's sum of |u|^2 over the targets must agree with the candidates'
 * median to 1e-4 (relative), else VPMC_ERR_DEVICE (a kernel variant gave
 * different results).  Outputs (HOST, may be NULL): chosen k, queries per
 * thread, and the best pass time in ms (-1 when cached). */
int vpmc_sim_autotune(vpmc_sim* sim, int* k_walk, int* queries_per_thread, float* best_ms);

/* Kernels launched per step by the last captured or eager pass, and the
 * device time (ms, CUDA events on the context stream) of the field-evaluation
 * launches of the last step completed by vpmc_sim_step.  No reference
 * counterpart (instrumentation). */
int vpmc_sim_last_stats(vpmc_sim* sim, int* launches_per_step, float* eval_ms);

/* Sizes of the step: info[8] = {particles, targets per chunk, chunks per step,
 * bins, cells per axis (instance 0), walk half-width k, samples per target,
 * eval launches in the last timed step}.  No reference counterpart. */
int vpmc_sim_geometry(vpmc_sim* sim, long long* info);

/* Sample points of the last chunk drawn by the last MIS pass (a step, a
 * velocity pass or an autotuner pass): count (x, y) pairs from sample index
 * `first` into the HOST array xy, where sample (t - t0) * samples_per_target
 * + sign * samples_per_target / 2 + j is sample j of target t and the given
 * sign (0: positive strengths, 1: negative); *t0 (may be NULL) receives the
 * chunk's first target.  Points are as drawn (before the periodic wrap).
 * VPMC_ERR_INVALID when no pass has drawn samples since the working set was
 * last (re)allocated or reused, or when the range leaves the chunk.  No
 * reference counterpart (instrumentation: the in-support pair count of the
 * evaluation's roofline). */
int vpmc_sim_read_samples(vpmc_sim* sim, long long first, long long count, long long* t0, float* xy);

/* Field values of the same samples (HOST array of count doubles; the FP32
 * path's values are widened): the smoothed |omega| field of the sample's sign
 * subset at the sample point, as the MIS terms use it -- with the unbiased
 * law the sum over the 3x3 periodic images {-1,0,1}^2 of the particles seen
 * from the unwrapped point, with the reference law the periodic field at the
 * wrapped point; 0 for a sample the law drops.  Same indexing and validity
 * rules as vpmc_sim_read_samples.  No reference counterpart (parity
 * instrumentation of queryVorticityAbs inside monte_carlo_bs_kernel_safe,
 * src/cuda/monte_carlo_bs.cu:214-218). */
int vpmc_sim_read_field(vpmc_sim* sim, long long first, long long count, long long* t0, double* f);

/* ---------------------------------------------------------------- misc */
/* Philox4x32-10 (Salmon et al., SC'11) block function, host evaluation:
 * out[4] = philox(ctr[4], key[2]).  Exposed for known-answer tests. */
void vpmc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out);

#ifdef __cplusplus
}
#endif
#endif /* VPMC_H */
