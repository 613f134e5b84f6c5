// vpmc_eval_tc.cu -- field evaluation (FIELD / FIELD9 modes) with the squared
// distances on the 5th-generation tensor cores.
//
// The evaluation sums, for every query q of a bin, w W(|q - c|) over the
// candidates c of the bin's walk (include/vorticity_query.cuh:15-79 and
// src/cuda/monte_carlo_bs.cu:144-271 evaluate the same field pair by pair).
// In the bin's local frame the scaled squared distance is a rank-4 product,
//   s2 = kappa (|q|^2 + |c|^2 - 2 q.c) = [qx qy Q2 1] . [X Y 1 C2],
//   kappa = -3/h^2, X = -2 kappa cx, Y = -2 kappa cy, Q2 = kappa |q|^2, C2 = kappa |c|^2,
// so a 128-query x N-candidate tile of s2 is one tcgen05 MMA of kind tf32.  Each
// operand is split into a TF32 head and a TF32 remainder (x = h + l) and the
// three products h.h + h.l + l.h are summed in FP32 by the MMA (K = 10 of 16
// used), which keeps s2 at FP32 accuracy.  The accumulator tile lives in
// tensor memory; each warp reads its 32 query rows back (tcgen05.ld) and the
// CUDA cores only evaluate the spline (one square root on the XU, the rest on
// the FMA pipe) and the weighted sum -- the part of the pair work the tensor
// cores cannot do.
//
// Four CTAs per SM, each four warps = one item (a bin and up to 128 of its
// queries, one query per TMEM lane) with 128 TMEM columns = the accumulator of
// one batch of 128 candidate columns.  Per item: the A operand from the queries;
// the walk over the (2k+1) columns of cells around the bin (one column per
// lane of warp 0), each run trimmed to the sub-rows within reach of the item's
// query box; the runs laid out as columns grouped by periodic image (FIELD9:
// each group padded to 32 columns, so a 32-column chunk has one image).  The
// batches of 128 columns run one after another (operands built, multiplied,
// summed); the bulk copies (TMA engine) of batch b + 1's runs land in shared
// memory while batch b is multiplied and summed.  Four CTAs keep the SM's
// pipes busy while one waits for its multiply or copies.
//
// The autotuner (tuning value 1) times this kernel against the one-warp
// CUDA-core evaluation.  On the 2048^2 Taylor-Green step (k_walk 7) it took
// 318 ms against 261 ms: it is bound by latency (the per-batch barrier, the
// multiply's round trip, the per-item walk and staging), which four CTAs of
// four warps -- all the TMEM columns allow -- cannot hide as the one-warp
// kernel's 24 independent warps per SM do.  Warp-specialised (a producer warp,
// two CTAs per SM) and software-pipelined (two TMEM buffers) forms measured
// slower still (544, 405-518 ms).
//
#include "vpmc_grid.cuh"

namespace vpmc {

namespace {

constexpr int kTcThreads = 128;              // 4 warps = TMEM lanes 0-127
constexpr int kTcCols = 128;                 // candidate columns per batch
constexpr int kTcTmemCols = kTcCols;         // one accumulator tile
constexpr int kTcCtasPerSm = 512 / kTcTmemCols;
constexpr int kTcMaxK = 8;
constexpr int kTcMaxPieces = 2 * (2 * kTcMaxK + 1);
constexpr uint32_t kTcDrainLimit = VPMC_WAIT_LIMIT_DEFAULT;
// dynamic shared memory: the A tile (8 KB), the B tile (8 KB), two raw
// staging buffers, two weight rows (a warp may still sum batch b while another
// builds batch b + 1); 48 KB so that no more than four CTAs (the TMEM budget)
// are resident on an SM (4 x 52 KB of the 228 KB with the static part)
constexpr size_t kTcSmA = 0, kTcSmB = 8192, kTcSmRaw = kTcSmB + kTcCols * 64,
                 kTcSmW = kTcSmRaw + 2 * kTcCols * sizeof(Cand);
constexpr size_t kTcSmem = 48 * 1024;
static_assert(kTcSmW + 2 * kTcCols * sizeof(float) <= kTcSmem, "shared memory layout");

struct TcPiece {
    uint32_t gstart, cnt;   // trimmed candidate run in global memory
    uint32_t col;           // its first column (item column space)
    float ox, oy;           // origin of its local frame: bin centre + image offset
    int img;                // (mx + 2) | (my + 2) << 3
};

// tcgen05 shared-memory matrix descriptor, no swizzle, K-major: core matrices
// of 8 rows x 16 bytes, `lbo` bytes apart along K, `sbo` bytes apart along M/N.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor: D FP32, A and B TF32, both K-major, M = 128, N columns.
__device__ __forceinline__ uint32_t tc_idesc(uint32_t n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive TMEM columns of this warp's 32 lanes -> 32 registers (async
// until tc_wait32 on the same registers, which ties their uses after the wait).
__device__ __forceinline__ void tc_ld32(uint32_t (&R)[32], uint32_t taddr) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(R[0]), "=r"(R[1]), "=r"(R[2]), "=r"(R[3]), "=r"(R[4]), "=r"(R[5]), "=r"(R[6]), "=r"(R[7]),
          "=r"(R[8]), "=r"(R[9]), "=r"(R[10]), "=r"(R[11]), "=r"(R[12]), "=r"(R[13]), "=r"(R[14]), "=r"(R[15]),
          "=r"(R[16]), "=r"(R[17]), "=r"(R[18]), "=r"(R[19]), "=r"(R[20]), "=r"(R[21]), "=r"(R[22]), "=r"(R[23]),
          "=r"(R[24]), "=r"(R[25]), "=r"(R[26]), "=r"(R[27]), "=r"(R[28]), "=r"(R[29]), "=r"(R[30]), "=r"(R[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tc_wait32(uint32_t (&R)[32]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "+r"(R[7]),
                   "+r"(R[8]), "+r"(R[9]), "+r"(R[10]), "+r"(R[11]), "+r"(R[12]), "+r"(R[13]), "+r"(R[14]),
                   "+r"(R[15]), "+r"(R[16]), "+r"(R[17]), "+r"(R[18]), "+r"(R[19]), "+r"(R[20]), "+r"(R[21]),
                   "+r"(R[22]), "+r"(R[23]), "+r"(R[24]), "+r"(R[25]), "+r"(R[26]), "+r"(R[27]), "+r"(R[28]),
                   "+r"(R[29]), "+r"(R[30]), "+r"(R[31])
                 :
                 : "memory");
}
// FP32 -> TF32 (round to nearest; the low 13 bits cleared)
__device__ __forceinline__ float tf32_round(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// One operand row (16 TF32 values, 64 bytes) into the no-swizzle K-major tile:
// row m, k-core j (4 values) at (m / 8) * 512 + j * 128 + (m % 8) * 16.
__device__ __forceinline__ void put_row(float* tile, int m, float4 k0, float4 k1, float4 k2, float4 k3) {
    char* base = reinterpret_cast<char*>(tile) + (m >> 3) * 512 + (m & 7) * 16;
    *reinterpret_cast<float4*>(base) = k0;
    *reinterpret_cast<float4*>(base + 128) = k1;
    *reinterpret_cast<float4*>(base + 256) = k2;
    *reinterpret_cast<float4*>(base + 384) = k3;
}

// Bulk copies of the candidate runs that fall into columns [b*128, (b+1)*128)
// of the item into `dst` (column order), by the lanes of one warp; completion
// (with the byte count) on `bar`.
__device__ __forceinline__ void issue_batch(const TcPiece* pcs, int np, uint32_t b, Cand* dst,
                                            const Cand* __restrict__ cand, uint64_t* bar, int lane) {
    const uint32_t lo = b * uint32_t(kTcCols), hi = lo + uint32_t(kTcCols);
    uint32_t bytes = 0;
    for (int p = lane; p < np; p += 32) {
        const uint32_t c0 = max(pcs[p].col, lo), c1 = min(pcs[p].col + pcs[p].cnt, hi);
        if (c0 < c1) bytes += (c1 - c0) * uint32_t(sizeof(Cand));
    }
    bytes = __reduce_add_sync(0xffffffffu, bytes);
    if (lane == 0) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, bytes);
    }
    __syncwarp();
    fence_proxy_async_smem();
    for (int p = lane; p < np; p += 32) {
        const TcPiece pc = pcs[p];
        const uint32_t c0 = max(pc.col, lo), c1 = min(pc.col + pc.cnt, hi);
        if (c0 < c1)
            bulk_g2s(dst + (c0 - lo), cand + (pc.gstart + (c0 - pc.col)), (c1 - c0) * uint32_t(sizeof(Cand)), bar);
    }
}

// Sum of one 32-column chunk into acc: s2 from TMEM, spline on the CUDA cores
// (the packed form of the one-warp kernel: t = (1 - r/h)+ from one square
// root, W / 2 sigma = min(1/2 + s2 t, t^3)), weights from shared memory.
__device__ __forceinline__ float chunk_sum(const uint32_t (&R)[32], const float* __restrict__ w, float acc) {
    const f2x HALF = pk2(0.5f, 0.5f);
#pragma unroll
    for (int i = 0; i < 32; i += 4) {
        const float4 w4 = *reinterpret_cast<const float4*>(w + i);
        const float wv[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int j = 0; j < 4; j += 2) {
            const float sa = __uint_as_float(R[i + j]), sb = __uint_as_float(R[i + j + 1]);
            const float ra = sqrt_approx(fabsf(sa)), rb = sqrt_approx(fabsf(sb));
            const f2x t = pk2(__saturatef(fmaf(-kInvSqrt3, ra, 1.f)), __saturatef(fmaf(-kInvSqrt3, rb, 1.f)));
            const f2x in = fma2(pk2(sa, sb), t, HALF);
            const f2x t3 = mul2(mul2(t, t), t);
            float ia, ib, ta, tb;
            up2(in, ia, ib);
            up2(t3, ta, tb);
            acc = fmaf(wv[j], fminf(ia, ta), acc);
            acc = fmaf(wv[j + 1], fminf(ib, tb), acc);
        }
    }
    return acc;
}

// B operand rows and weights of the batch's columns [b * 128, b * 128 + 128):
// column c (thread c) from the staged run that holds it,
//   [X_h, X_l, X_h, Y_h, Y_l, Y_h, 1, 1, C2_h, C2_l, 0 x 6],
// padding columns zero with weight zero; the chunk images (FIELD9) from the
// chunks' first columns.
// `cur` is the thread's piece cursor: its columns only grow from batch to
// batch, so the run holding the column is found by stepping forward.
__device__ __forceinline__ void build_b(const TcPiece* s_pc, int np, uint32_t b, uint32_t bcols, const Cand* raw,
                                        float* sB, float* sW, int* chimg, float kap, int tid, int& cur) {
    if (uint32_t(tid) >= bcols) return;
    const uint32_t gc = b * uint32_t(kTcCols) + uint32_t(tid);
    while (cur + 1 < np && s_pc[cur + 1].col <= gc) ++cur;
    const TcPiece pc = s_pc[cur];
    float lx = 0.f, ly = 0.f, w = 0.f;
    if (gc >= pc.col && gc < pc.col + pc.cnt) {
        const Cand cd = raw[tid];
        lx = cd.x - pc.ox;
        ly = cd.y - pc.oy;
        w = cd.w;
    }
    const float X = -2.f * kap * lx, Y = -2.f * kap * ly, C2 = kap * fmaf(lx, lx, ly * ly);
    const float Xh = tf32_round(X), Xl = tf32_round(X - Xh);
    const float Yh = tf32_round(Y), Yl = tf32_round(Y - Yh);
    const float Ch = tf32_round(C2), Cl = tf32_round(C2 - Ch);
    put_row(sB, tid, make_float4(Xh, Xl, Xh, Yh), make_float4(Yl, Yh, 1.f, 1.f), make_float4(Ch, Cl, 0.f, 0.f),
            make_float4(0.f, 0.f, 0.f, 0.f));
    sW[tid] = w;
    if ((tid & 31) == 0) chimg[tid >> 5] = pc.img;
}

template <bool kField9>
__global__ void __launch_bounds__(kTcThreads, kTcCtasPerSm) k_eval_tc(EvalTcArgs a) {
    extern __shared__ __align__(1024) unsigned char s_dyn[];
    float* const sA = reinterpret_cast<float*>(s_dyn + kTcSmA);
    float* const sB = reinterpret_cast<float*>(s_dyn + kTcSmB);
    Cand* const sRaw = reinterpret_cast<Cand*>(s_dyn + kTcSmRaw);    // [2][kTcCols]
    float* const sW2 = reinterpret_cast<float*>(s_dyn + kTcSmW);     // [2][kTcCols]
    __shared__ TcPiece s_pc[kTcMaxPieces];
    __shared__ float4 s_box[kTcThreads / 32];
    __shared__ __align__(16) float s_zero[32];
    __shared__ int s_chimg[2][kTcCols / 32];
    __shared__ int s_np;
    __shared__ uint32_t s_ncols, s_item, s_tmem;
    __shared__ __align__(8) uint64_t s_bar_raw[2], s_bar_mma, s_bar_drain;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        mbar_init(&s_bar_raw[0], 1);
        mbar_init(&s_bar_raw[1], 1);
        mbar_init(&s_bar_mma, 1);
        mbar_init(&s_bar_drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_item = atomicAdd(a.counter, 1u);
    }
    if (tid < 32) s_zero[tid] = 0.f;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(uint32_t(kTcTmemCols))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t lim = a.wait_limit;
    // Phases of the two raw-staging barriers and the multiply barrier (every
    // thread waits on every one of them, so all agree while no wait expires);
    // batches are numbered across items (g), staging slots alternate by g.  Thread 0 also
    // tracks the copies it has not yet seen land and whether it multiplied.
    // `bad` marks an expired wait: the CTA leaves at its next barrier
    // (__syncthreads_or), so the decision is uniform.
    uint32_t rph = 0u, mph = 0u, pend_raw = 0u;   // mph: bit 0, the multiply barrier's phase
    bool issued_mma = false;
    int bad = 0, aborted = 0;
    uint32_t g = 0;

    for (;;) {
        const uint32_t item = s_item;
        if (item >= *a.n_items) break;
        uint32_t next_item = 0;
        if (tid == 0) next_item = atomicAdd(a.counter, 1u);
        const Item it = a.items[item];
        const GridInst G = a.inst[it.inst];
        const uint32_t local = it.bin - uint32_t(G.bin_base);
        const uint32_t ncell = uint32_t(G.gx * G.gy);
        const uint32_t set = local / ncell, cell = local % ncell;
        const int cx = int(cell) / G.gy, cy = int(cell) % G.gy;
        // bin centre (wrapped coordinates): origin of the local frame
        const float ocx = (float(cx) + 0.5f) / G.inv_sx, ocy = (float(cy) + 0.5f) / G.inv_sy;
        const float kap = G.B;

        // this thread's query = row tid of the A tile:
        //   [qx_h, qx_h, qx_l, qy_h, qy_h, qy_l, Q2_h, Q2_l, 1, 1, 0 x 6]
        const bool qv = uint32_t(tid) < it.qcnt;
        QRec qr{0.f, 0.f, 0u, 2u | (2u << 3)};
        if (qv) qr = a.qrec[it.qbeg + uint32_t(tid)];
        const float ax = qr.x - ocx, ay = qr.y - ocy;
        {
            float4 k0 = make_float4(0.f, 0.f, 0.f, 0.f), k1 = k0, k2 = k0;
            if (qv) {
                const float xh = tf32_round(ax), xl = tf32_round(ax - xh);
                const float yh = tf32_round(ay), yl = tf32_round(ay - yh);
                const float q2 = kap * fmaf(ax, ax, ay * ay);
                const float q2h = tf32_round(q2), q2l = tf32_round(q2 - q2h);
                k0 = make_float4(xh, xh, xl, yh);
                k1 = make_float4(yh, yl, q2h, q2l);
                k2 = make_float4(1.f, 1.f, 0.f, 0.f);
            }
            put_row(sA, tid, k0, k1, k2, make_float4(0.f, 0.f, 0.f, 0.f));
        }
        // bounding box of the item's queries in the local frame
        {
            float bx0 = qv ? ax : INFINITY, bx1 = qv ? ax : -INFINITY;
            float by0 = qv ? ay : INFINITY, by1 = qv ? ay : -INFINITY;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
                bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
                by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
                by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
            }
            if (lane == 0) s_box[warp] = make_float4(bx0, bx1, by0, by1);
        }
        __syncthreads();

        if (warp == 0) {
            // the walk, one column of cells per lane (2 k + 1 <= 17 columns, up to
            // two runs each where a periodic column wraps in y), each run trimmed to
            // the sub-rows within reach of the item's query box
            float4 bb = s_box[0];
#pragma unroll
            for (int w = 1; w < kTcThreads / 32; ++w) {
                const float4 o = s_box[w];
                bb = make_float4(fminf(bb.x, o.x), fmaxf(bb.y, o.y), fminf(bb.z, o.z), fmaxf(bb.w, o.w));
            }
            const int R = a.rows, gyR = G.gy * R;
            const uint32_t colbase = (uint32_t(G.bin_base) + set * ncell) * uint32_t(R);
            const float sx = 1.f / G.inv_sx;
            const float srow = 1.f / (G.inv_sy * float(R)), inv_srow = G.inv_sy * float(R);
            const float rm = G.reach * 1.001f;
            int gxx, sxi, r0[2], r1[2], syi[2];
            walk_column(G, cx, cy, R, lane, gxx, sxi, r0, r1, syi);
            uint32_t gs[2] = {0u, 0u}, cn[2] = {0u, 0u};
            int img[2] = {0, 0};
            float fox[2] = {0.f, 0.f}, foy[2] = {0.f, 0.f};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (r0[h] > r1[h]) continue;
                const float qdx = -float(sxi) * G.Lx, qdy = -float(syi[h]) * G.Ly;
                const float x0 = float(gxx) / G.inv_sx - ocx - qdx;
                const float y0 = float(r0[h]) * srow - ocy - qdy;
                const float dxw = fmaxf(0.f, fmaxf(x0 - bb.y, bb.x - (x0 + sx)));
                if (!(dxw < rm)) continue;
                const float dy = sqrtf(fmaf(rm, rm, -dxw * dxw));
                const int ilo = max(int(floorf(fmaf(bb.z - dy - y0, inv_srow, -0.01f))), 0);
                const int ihi = min(int(floorf(fmaf(bb.w + dy - y0, inv_srow, 0.01f))), r1[h] - r0[h]);
                if (ilo > ihi) continue;
                const uint32_t b0 = colbase + uint32_t(gxx * gyR + r0[h]);
                const uint32_t t0 = a.cstart[b0 + uint32_t(ilo)], t1 = a.cstart[b0 + uint32_t(ihi) + 1u];
                if (t1 <= t0) continue;
                gs[h] = t0;
                cn[h] = t1 - t0;
                img[h] = kField9 ? ((sxi + 2) | ((syi[h] + 2) << 3)) : 0;
                fox[h] = ocx + qdx;
                foy[h] = ocy + qdy;
            }
            // columns: the runs grouped by image in a fixed order (the image code),
            // walk order inside a group; FIELD9 pads each group to 32 columns
            const int cl0 = cn[0] ? (kField9 ? ((img[0] & 7) - 1) * 3 + ((img[0] >> 3) & 7) - 1 : 0) : -1;   // 0..8
            const int cl1 = cn[1] ? (kField9 ? ((img[1] & 7) - 1) * 3 + ((img[1] >> 3) & 7) - 1 : 0) : -1;
            unsigned present = __reduce_or_sync(0xffffffffu, (cl0 >= 0 ? 1u << cl0 : 0u) | (cl1 >= 0 ? 1u << cl1 : 0u));
            const unsigned lt = (1u << lane) - 1u;
            uint32_t ccol = 0;
            int cslot = 0;
            while (present) {
                const int cl = __ffs(present) - 1;
                present &= present - 1u;
                const uint32_t c0 = cl0 == cl ? cn[0] : 0u, c1 = cl1 == cl ? cn[1] : 0u;
                uint32_t incl = c0 + c1;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
                const uint32_t ex = incl - c0 - c1;
                const unsigned m0 = __ballot_sync(0xffffffffu, c0 > 0u), m1 = __ballot_sync(0xffffffffu, c1 > 0u);
                const int sl = cslot + __popc(m0 & lt) + __popc(m1 & lt);
                if (c0) s_pc[sl] = TcPiece{gs[0], c0, ccol + ex, fox[0], foy[0], img[0]};
                if (c1) s_pc[sl + (c0 ? 1 : 0)] = TcPiece{gs[1], c1, ccol + ex + c0, fox[1], foy[1], img[1]};
                cslot += __popc(m0) + __popc(m1);
                ccol += kField9 ? ((tot + 31u) & ~31u) : tot;
            }
            if (!kField9) ccol = (ccol + 31u) & ~31u;
            __syncwarp();
            // the first batch's runs (staging slot by the batch number across items)
            if (ccol > 0) {
                issue_batch(s_pc, cslot, 0u, sRaw + (g & 1u) * kTcCols, a.cand, &s_bar_raw[g & 1u], lane);
                pend_raw |= 1u << (g & 1u);
            }
            if (lane == 0) {
                s_np = cslot;
                s_ncols = ccol;
            }
        }
        __syncthreads();

        const int np = s_np;
        const uint32_t ncols = s_ncols;
        const uint32_t nbat = (ncols + uint32_t(kTcCols) - 1u) / uint32_t(kTcCols);
        const bool wrows = uint32_t(warp * 32) < it.qcnt;   // this warp holds queries
        // FIELD9: the query's unwrapped image code (the chunk's image is combined with it)
        const int qmx = int(qr.flags & 7u) - 2, qmy = int((qr.flags >> 3) & 7u) - 2;
        float acc = 0.f;
        int cur = 0;   // piece cursor of this thread's B-operand column
        // batch b of the item is batch g + b overall: staging slot and weight row (g + b) & 1
        for (uint32_t b = 0; b < nbat; ++b) {
            const uint32_t gb = g + b, sl = gb & 1u;
            const uint32_t bcols = min(uint32_t(kTcCols), ncols - b * uint32_t(kTcCols));
            if (mbar_wait_bounded(&s_bar_raw[sl], (rph >> sl) & 1u, lim)) {
                rph ^= 1u << sl;
                pend_raw &= ~(1u << sl);
            } else {
                bad = 1;
            }
            build_b(s_pc, np, b, bcols, sRaw + sl * kTcCols, sB, sW2 + sl * kTcCols, s_chimg[sl], kap, tid, cur);
            fence_proxy_async_smem();   // operand tiles visible to the tensor core
            // the barrier also shows every warp done reading the TMEM tile of batch b - 1
            tc_fence_before();
            if (__syncthreads_or(bad)) break;
            if (tid == 0) {
                tc_fence_after();
                const uint32_t idesc = tc_idesc(bcols);
                const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
                tc_mma(tmem, tc_desc(a0, 128u, 512u), tc_desc(b0, 128u, 512u), idesc, 0u);
                tc_mma(tmem, tc_desc(a0 + 256u, 128u, 512u), tc_desc(b0 + 256u, 128u, 512u), idesc, 1u);
                tc_commit(&s_bar_mma);
                issued_mma = true;
            }
            // the next batch's runs into the other staging slot (batch b - 1's, read before the barrier)
            if (warp == 0 && b + 1u < nbat) {
                issue_batch(s_pc, np, b + 1u, sRaw + (sl ^ 1u) * kTcCols, a.cand, &s_bar_raw[sl ^ 1u], lane);
                pend_raw |= 1u << (sl ^ 1u);
            }
            const bool done = mbar_wait_bounded(&s_bar_mma, mph & 1u, lim);
            if (done) mph ^= 1u;
            else bad = 1;
            // tcgen05.ld is warp-collective: a warp reads only if all its lanes saw the multiply end
            if (!__all_sync(0xffffffffu, done)) continue;   // the next barrier ends the item
            tc_fence_after();
            if (wrows) {
                const uint32_t nch = bcols >> 5;
                const uint32_t tb = tmem + (uint32_t(warp * 32) << 16);
                const float* sW = sW2 + sl * kTcCols;
                // chunk weights: this query's image mask decides whether a chunk counts
                const float* wp[kTcCols / 32];
#pragma unroll
                for (int j = 0; j < kTcCols / 32; ++j) {
                    bool use = true;
                    if (kField9 && uint32_t(j) < nch) {
                        const int ci = s_chimg[sl][j];
                        const int mx = qmx + (ci & 7) - 2, my = qmy + ((ci >> 3) & 7) - 2;
                        use = mx >= -1 && mx <= 1 && my >= -1 && my <= 1;
                    }
                    wp[j] = use ? sW + 32 * j : s_zero;
                }
                // two register sets: the next chunk's load overlaps this chunk's sum
                uint32_t RA[32], RB[32];
                tc_ld32(RA, tb);
                tc_wait32(RA);
                if (nch > 1) tc_ld32(RB, tb + 32u);
                acc = chunk_sum(RA, wp[0], acc);
                if (nch > 1) {
                    tc_wait32(RB);
                    if (nch > 2) tc_ld32(RA, tb + 64u);
                    acc = chunk_sum(RB, wp[1], acc);
                }
                if (nch > 2) {
                    tc_wait32(RA);
                    if (nch > 3) tc_ld32(RB, tb + 96u);
                    acc = chunk_sum(RA, wp[2], acc);
                }
                if (nch > 3) {
                    tc_wait32(RB);
                    acc = chunk_sum(RB, wp[3], acc);
                }
            }
            tc_fence_before();
        }
        g += nbat;
        if (qv && !bad) a.out[qr.id] = acc;
        if (tid == 0) s_item = next_item;
        tc_fence_before();
        if (__syncthreads_or(bad)) {
            aborted = 1;
            break;
        }
    }
    __syncthreads();
    if (aborted && tid == 0) {
        atomicOr(a.flags, FLAG_TIMEOUT);
        // let every copy and multiply still in flight land before TMEM is freed
        for (uint32_t i = 0; i < 2; ++i)
            if ((pend_raw >> i) & 1u) (void)mbar_wait_bounded(&s_bar_raw[i], (rph >> i) & 1u, kTcDrainLimit);
        if (issued_mma) {
            tc_commit(&s_bar_drain);
            (void)mbar_wait_bounded(&s_bar_drain, 0u, kTcDrainLimit);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(uint32_t(kTcTmemCols))
                     : "memory");
    }
}

}  // namespace

int launch_eval_tc(vpmc_context* ctx, const EvalTcArgs& a, bool field9) {
    static bool configured[2][64] = {};
    const int dev = ctx->device;
    auto kern = field9 ? k_eval_tc<true> : k_eval_tc<false>;
    if (dev < 64 && !configured[field9][dev]) {
        VPMC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTcSmem)));
        VPMC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       int(cudaSharedmemCarveoutMaxShared)));
        configured[field9][dev] = true;
    }
    // a persistent grid of the TMEM budget per SM (the shared-memory size keeps
    // more from being resident; a CTA that found the columns taken would wait
    // in tcgen05.alloc until another exits)
    VPMC_LAUNCH(kern, ctx->sm_count * kTcCtasPerSm, kTcThreads, kTcSmem, ctx->stream, a);
    return VPMC_OK;
}

}  // namespace vpmc
