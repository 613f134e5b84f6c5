// vpmc_grid.cuh -- cell-binned particle sets and the field-evaluation kernel.
//
// Every field query in the library (vorticity queries, MIS sample values, the
// RBF SpMV) runs through the same structure:
//   * particles ("candidates") are sorted stably by bin = (instance, sign set,
//     cell) on a grid whose cell side s >= h_w / k, and gathered into an AoS
//     32-byte record array (coordinates and weight duplicated for packed math)
//     so each cell is one contiguous run;
//   * query points are binned by the cell of their wrapped position;
//   * one CTA takes a bin (or a chunk of it), stages the (2k+1)^2 neighbour
//     cells -- at most 2(2k+1) contiguous runs, one per column and periodic
//     wrap -- into shared memory with bulk (TMA) copies, and evaluates every
//     query of the bin against them.  Periodic images are folded into a
//     per-run offset of the query point, so the inner loop has no branches.
#pragma once

#include "vpmc_internal.cuh"

namespace vpmc {

// Geometry of one instance on the evaluation grid (device visible).
struct GridInst {
    float Lx, Ly;
    float inv_sx, inv_sy;   // gx/Lx, gy/Ly
    int gx, gy;             // cells per axis
    int k;                  // walk half width in cells
    int bin_base;           // first bin of the instance
    int nsets;              // candidate sets (2 = sign split, 1 = one set)
    int periodic;
    float hw;               // support radius h_w
    float reach;            // radius the walk must cover: h_w x cover (sigma_max of deformed kernels)
    float inv_hw;           // 1/h_w
    float A, B;             // 3/h_w^3, -3/h_w^2: W/(2 sigma) = min(0.5 + r^2 (A r + B), (1 - r/h_w)^3)
    float two_sigma;        // 2 * 40 / (7 pi h_w^2)
    int p_begin, p_end;     // particle range of the instance
};

// Candidate record (32 bytes): coordinates and weight duplicated so that one
// shared-memory broadcast load feeds packed f32x2 operands for two queries.
// w = weight (FP32 hi part), wl = the FP32 remainder (for FP64 SpMV weights).
struct __align__(16) Cand {
    float x, x2, y, y2;
    float w, w2, wl, pad;
};

// Candidate record of a deformed kernel W(|F^-1 d|) (64 bytes).  In global
// memory: f = {x, y, g11, g12, g22, w, wl, 0, ...}, G = F^-T F^-1 the metric
// (|F^-1 d|^2 = d^T G d).  Staged in shared memory it is rewritten, per run,
// into the bin-local expanded form of r^2 as a polynomial in the query point
// q (coefficients duplicated for packed math):
//   r^2 = e + g11 qx^2 + 2 g12 qx qy + g22 qy^2 + a qx + b qy,
//   a = -2 (G c)_x, b = -2 (G c)_y, e = c^T G c   (c = local candidate position).
struct __align__(16) CandF {
    float f[16];
};

// Query record: wrapped position, output slot, image flags (16 bytes).
struct QRec {
    float x, y;
    uint32_t id;
    uint32_t flags;   // bits 0-2: kx+2, bits 3-5: ky+2 (unwrapped image of the point)
};

struct Item {
    uint32_t bin;
    uint32_t qbeg;
    uint32_t qcnt;
    uint32_t inst;
};

// Packed FP32x2 arithmetic (sm_100+ f32x2 instructions): one instruction
// serves two queries.  Operands are 64-bit register pairs {lo, hi}.
typedef unsigned long long f2x;
__device__ __forceinline__ f2x pk2(float a, float b) {
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void up2(f2x v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2x add2(f2x a, f2x b) {
    f2x r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
    f2x r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
    f2x r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// 1/sqrt(3): the packed spline works with sqrt(3) r/h (see packed_run).
constexpr float kInvSqrt3 = 0.57735026918962576f;

__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// One column of a bin's walk (lane = 0 .. 2k of a warp; column ox = lane - k
// cells from the bin's cell (cx, cy) in x): the grid column gxx it reads, the
// periodic image sxi it lies in, and its sub-rows [r0[h], r1[h]] in up to two
// runs (a periodic column wrapping in y splits; image syi[h]).  The column is
// at least dx from every point of the bin's cell, so its candidates within
// reach lie within dy = sqrt(reach^2 - dx^2) of the cell in y: sub-rows
// [cy R - m, cy R + R - 1 + m] (1e-3 of a sub-row of tolerance: the pairs it
// can skip lie within 0.2% of the kernel's support edge, where W / W(0) <
// 1e-7).  Runs left empty have r0 > r1.
__device__ __forceinline__ void walk_column(const GridInst& G, int cx, int cy, int R, int lane, int& gxx, int& sxi,
                                            int (&r0)[2], int (&r1)[2], int (&syi)[2]) {
    const int gyR = G.gy * R;
    const float sx = 1.f / G.inv_sx, reach2 = G.reach * G.reach;
    const int ox = lane - G.k;
    gxx = cx + ox;
    sxi = 0;
    r0[0] = r0[1] = 1;
    r1[0] = r1[1] = 0;
    syi[0] = syi[1] = 0;
    const float dx = ox == 0 ? 0.f : float(abs(ox) - 1) * sx;
    bool col = ox <= G.k && dx * dx <= reach2;
    if (col) {
        if (G.periodic) {
            if (gxx < 0) { gxx += G.gx; sxi = -1; }
            else if (gxx >= G.gx) { gxx -= G.gx; sxi = 1; }
        } else if (gxx < 0 || gxx >= G.gx) {
            col = false;
        }
    }
    if (!col) return;
    const int m = min(int(ceilf(sqrtf(reach2 - dx * dx) * G.inv_sy * float(R) - 1e-3f)), G.k * R);
    const int ylo = cy * R - m, yhi = cy * R + R - 1 + m;
    if (G.periodic) {
        if (ylo < 0) {
            r0[0] = 0; r1[0] = yhi;
            r0[1] = ylo + gyR; r1[1] = gyR - 1; syi[1] = -1;
        } else if (yhi >= gyR) {
            r0[0] = ylo; r1[0] = gyR - 1;
            r0[1] = 0; r1[1] = yhi - gyR; syi[1] = 1;
        } else {
            r0[0] = ylo; r1[0] = yhi;
        }
    } else {
        r0[0] = max(ylo, 0); r1[0] = min(yhi, gyR - 1);
    }
}

enum EvalMode : int {
    EVAL_FIELD = 0,      // out_f32[id] = sum w W          (periodic / plain field)
    EVAL_FIELD9 = 1,     // as FIELD, only images m in {-1,0,1}^2 of the unwrapped point
    EVAL_FIELD_EXC = 2,  // as FIELD, pairs closer than 1e-6 skipped (exclude_center)
    EVAL_SPMV64 = 3,     // out_f64[id] = sum (w + w_lo) W, in-support pairs in FP64
    EVAL_SPMV32 = 4,     // out_f64[id] = compensated FP32 sum
    EVAL_FIELD64 = 5,    // as FIELD, every pair in FP64 (weight w + wl), out_f64[id]
    EVAL_FIELD9_64 = 6,  // as FIELD9 in FP64
    EVAL_FIELD_F = 7,    // as FIELD with deformed kernels W(|F^-1 d|) (CandF records)
    EVAL_FIELD9_F = 8,   // as FIELD9 with deformed kernels
    EVAL_FIELD_F_EXC = 9,// as FIELD_EXC with deformed kernels (pairs with |F^-1 d| < 1e-6 skipped)
    // FP64 value and gradient (adjoint): out_f64[3 id + {0, 1, 2}] = {f, df/dqx, df/dqy}
    EVAL_GRAD64 = 10,    // f(q) = sum w W(|q - c|)
    EVAL_GRAD9_64 = 11,  // same with the FIELD9 image mask of the query
    // the two GRAD modes with the pairs in FP32 (weights w only) and the run sums
    // in FP64: the adjoint of the FP32-compensated step
    EVAL_GRAD32 = 12,
    EVAL_GRAD9_32 = 13,
    // the transposed sums G(x_p) = sum_s a_s W(|x_p - y_s|) and its gradient,
    // computed from the sample side: the queries are the samples (weight
    // qweight[id] * 2 sigma), the candidates the particles;
    // out_f64[3 slot + {0, 1, 2}] += {sum_s a_s W, sum_s a_s dW/dx_p} with slot
    // the particle's candidate index (grid order), one FP64 atomic per
    // (item, particle).  SCAT*_64: pairs in FP64; SCAT*_32: pairs in FP32, each
    // particle's sum over an item's samples compensated (TwoSum), so the result
    // does not depend on the samples' placement order beyond FP64 rounding.
    EVAL_SCAT64 = 14,
    EVAL_SCAT9_64 = 15,  // with each sample's FIELD9 image mask
    EVAL_SCAT32 = 16,
    EVAL_SCAT9_32 = 17,
};

__host__ __device__ constexpr bool eval_grad(int mode) {
    return mode == EVAL_GRAD64 || mode == EVAL_GRAD9_64 || mode == EVAL_GRAD32 || mode == EVAL_GRAD9_32;
}

__host__ __device__ constexpr bool eval_scat(int mode) {
    return mode == EVAL_SCAT64 || mode == EVAL_SCAT9_64 || mode == EVAL_SCAT32 || mode == EVAL_SCAT9_32;
}

__host__ __device__ constexpr bool eval_deformed(int mode) {
    return mode == EVAL_FIELD_F || mode == EVAL_FIELD9_F || mode == EVAL_FIELD_F_EXC;
}

enum SetMode : int {
    SET_SIGN_SPLIT = 0,  // set 0: omega > 0, set 1: omega < 0; weight |omega| * 2 sigma
    SET_ONE_SIGNED = 1,  // one set, all particles; weight omega (value or external vector)
    SET_POS_ONLY = 2,    // one set, omega > 0
    SET_NEG_ONLY = 3,    // one set, omega < 0
    SET_ONE_ABS = 4,     // one set, all particles; weight |omega|
};

constexpr uint32_t kNoBin = 0xffffffffu;

// Host description of an instance before planning.
struct InstDesc {
    float Lx, Ly, hw;
    int periodic;
    int p_begin, p_end;
    float cover = 1.f;   // the walk covers cover * h_w: the largest stretch sigma_max(F) of a deformed kernel
};

// Plan the grid: fills `out` (n entries) and returns the bin count, or a
// negative vpmc_status on geometry errors.  k <= 0 selects the default.
long grid_plan(const InstDesc* in, int n, int k, int nsets, GridInst* out);
int default_k();

// Device-side working set of one grid (caller owns the memory).
struct GridBufs {
    GridInst* inst = nullptr;   // device copy of the plan
    int n_inst = 0;
    long nbins = 0;
    int rows = 1;               // candidate sub-rows per cell (candidates sorted by cell, then sub-row in y)
    long n = 0;                 // particles covered
    uint32_t* keys = nullptr;   // n
    uint32_t* count = nullptr;  // nbins * rows + 1
    uint32_t* start = nullptr;  // nbins * rows + 1: candidate range of sub-row (bin * rows + r)
    uint32_t* cstart = nullptr; // nbins + 1: candidate range of a whole bin (= start when rows == 1)
    Cand* cand = nullptr;       // n
    CandF* candf = nullptr;     // n (deformed kernels only)
    uint32_t* perm = nullptr;   // n: sorted slot -> particle (points into rs buffers)
    RadixScratch rs{};
};
void carve_grid(Carver& c, long n, long nbins, int n_inst, GridBufs* g, bool deformed = false, int rows = 1);

// Bin keys + counts + stable sort + ranges + gather.  weights == nullptr uses
// omega (SET_SIGN_SPLIT scales |omega| by 2 sigma, SET_ONE_SIGNED by
// 2 sigma too).  Writes g.cand / g.start / g.perm; with F (per particle,
// row-major {F11, F12, F21, F22}) it writes the deformed records g.candf.
int grid_build(vpmc_context* ctx, GridBufs& g, const float2* pos, const float* omega, int set_mode,
               const float4* F = nullptr);
// Overwrite candidate weights from a vector in sorted order: cand[p].z/.w =
// hi/lo FP32 split of scale * x[p] (FP64 in, for the SpMV).
int grid_set_weights_sorted(vpmc_context* ctx, GridBufs& g, const double* x_sorted, double scale);

// Work items for queries that are already grouped by bin: qstart[b]..qstart[b+1].
struct ItemBufs {
    Item* items = nullptr;
    uint32_t* n_items = nullptr;    // device scalar
    uint32_t* per_bin = nullptr;    // nbins + 1
    uint32_t* item_start = nullptr; // nbins + 1
    uint32_t* counter = nullptr;    // work counter (device scalar)
    uint32_t* scan_tmp = nullptr;
    long max_items = 0;
};
void carve_items(Carver& c, long nbins, long max_queries, ItemBufs* it);
// chunk = queries per item = 256 * queries-per-thread of the eval launch.
int make_items(vpmc_context* ctx, const GridBufs& g, const uint32_t* qstart, ItemBufs& it, int chunk);
int query_chunk(int qpt);

// Query binning for points/samples: bin ids (kNoBin = skip) -> counts -> scan
// -> scatter into QRec by bin (order inside a bin is irrelevant).
struct QueryBufs {
    uint32_t* qbin = nullptr;    // per point
    uint32_t* qcount = nullptr;  // nbins + 1
    uint32_t* qstart = nullptr;  // nbins + 1
    uint32_t* qfill = nullptr;   // nbins
    uint32_t* qrank = nullptr;   // per point: rank inside its bin (only without the staged placement)
    QRec* qrec = nullptr;        // max points
    uint4* tmp = nullptr;        // max points (staged placement of ranked points: super-bins)
    uint4* tmp2 = nullptr;       // max points (staged placement: slot windows)
    uint32_t* super_fill = nullptr;
    uint32_t* win_fill = nullptr;
    uint32_t* scan_tmp = nullptr;
};
void carve_queries(Carver& c, long nbins, long max_points, QueryBufs* q, bool two_pass = false);
// Bin arbitrary points (one instance `inst_of` lookup per point by index range
// `point_inst` == nullptr -> instance 0).  set = candidate set to query.
int bin_points(vpmc_context* ctx, const GridBufs& g, QueryBufs& q, const float2* pts, long M, int set,
               int field9);
// Scatter points whose bins are already in q.qbin (counts in q.qcount).
int scatter_points(vpmc_context* ctx, const GridBufs& g, QueryBufs& q, const float2* pts, long M,
                   int field9);
// Same for points whose bins are counted in q.qcount: with q.tmp carved
// through super-bins and bin windows in three streaming passes (slots inside
// a bin assigned in shared memory); otherwise each point's rank inside its
// bin must be in q.qrank.
int scatter_ranked(vpmc_context* ctx, const GridBufs& g, QueryBufs& q, const float2* pts, long M);

// sigma_max over F[0..n) (+inf if some F is non-finite or has det <= 0);
// d_words: 2 device words of scratch.  Synchronises the stream.
int grid_max_sigma(vpmc_context* ctx, const float4* F, long n, unsigned* d_words, float* sigma);

struct EvalLaunch {
    int mode = EVAL_FIELD;
    int rows = -1;             // candidate sub-rows per cell of the candidate ranges (-1: the grid's)
    int qpt = 4;               // queries per thread (FIELD modes: 4, 6 or 8, or 1 = the tensor-core evaluation; others: 4)
    float* out_f32 = nullptr;
    double* out_f64 = nullptr;
    const double* qweight = nullptr;   // SCAT modes: weight of each query, by query id
};
int launch_eval(vpmc_context* ctx, const GridBufs& g, const QRec* qrec, ItemBufs& it, const EvalLaunch& L);

// The FIELD / FIELD9 evaluation with the squared distances on the tensor cores
// (vpmc_eval_tc.cu; selected by EvalLaunch::qpt == 1, items of 128 queries).
struct EvalTcArgs {
    const GridInst* inst;
    const uint32_t* cstart;   // candidate range per sub-row
    int rows;                 // sub-rows per cell
    const Cand* cand;
    const QRec* qrec;
    const Item* items;
    const uint32_t* n_items;
    uint32_t* counter;
    float* out;               // out[id] = sum w W
    unsigned* flags;
    uint32_t wait_limit;
};
int launch_eval_tc(vpmc_context* ctx, const EvalTcArgs& a, bool field9);

}  // namespace vpmc
