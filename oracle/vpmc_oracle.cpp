// vpmc_oracle.cpp -- CPU oracle (test infrastructure only; see vpmc_oracle.h).
//
// The orc_* functions restate the reference's CPU path in the same FP32
// expression order and with the same std::mt19937 stream, so that they can be
// pinned against golden vectors produced by the reference's own sources.
// Build with -ffp-contract=off: the reference was compiled for x86-64 without
// FMA contraction, and aarch64 gcc contracts a*b+c by default.
//
// Deliberate differences from the reference, each noted where it occurs:
//   * float -> int conversions saturate (NaN -> 0) instead of being UB;
//   * an empty sign subset contributes nothing instead of indexing sub[-1].

#include "vpmc_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr float  kPiF = 3.14159265358979323846f;
constexpr double kPiD = 3.14159265358979323846;

struct f2 { float x, y; };

// int(std::floor(v)) with saturation instead of UB (NaN -> 0).
inline int floor_to_int(float v) {
    if (!(v == v)) return 0;
    float f = std::floor(v);
    if (f >= 2147483648.0f) return 2147483647;
    if (f < -2147483648.0f) return -2147483647 - 1;
    return static_cast<int>(f);
}
// int(v) (truncation) with the same saturation.
inline int trunc_to_int(float v) {
    if (!(v == v)) return 0;
    if (v >= 2147483648.0f) return 2147483647;
    if (v < -2147483648.0f) return -2147483647 - 1;
    return static_cast<int>(v);
}

// Cubic B-spline, include/utilities.hpp:7-17 (same FP32 operation order).
inline float spline_pdf_f(float r, float hw) {
    const float pi = 3.141592653589793f;
    const float sigma = 40.f / (7.f * pi * hw * hw);
    const float q = r / hw;
    if (q >= 0.f && q <= 0.5f) {
        const float qq = q * q;
        return sigma * (6.f * (qq * q - qq) + 1.f);
    }
    if (q > 0.5f && q < 1.f) {
        const float t = 1.f - q;
        return sigma * 2.f * t * t * t;
    }
    return 0.f;
}

inline double spline_pdf_d(double r, double hw) {
    const double sigma = 40.0 / (7.0 * kPiD * hw * hw);
    const double q = r / hw;
    if (q >= 0.0 && q <= 0.5) return sigma * (6.0 * (q * q * q - q * q) + 1.0);
    if (q > 0.5 && q < 1.0) { const double t = 1.0 - q; return sigma * 2.0 * t * t * t; }
    return 0.0;
}

inline f2 ld2(const float* p, long i) { return f2{p[2 * i], p[2 * i + 1]}; }

// ---------------------------------------------------------------------------
// evalVorticityAbs_cpu, src/cpu/evaluate_vorticity.cpp:8-75.
// Note the reference keeps pos = (0,0) on the non-periodic path (only the
// periodic branch assigns it), so a non-periodic in-domain query evaluates
// the field at the origin; restated as-is.
float eval_vort_cpu(const orc_view& v, f2 p, int sign, bool use_signed,
                    bool exclude_center, float hw, bool periodic) {
    f2 q{0.f, 0.f};
    if (periodic) {
        q.x = p.x - std::floor(p.x / v.Lx) * v.Lx;
        q.y = p.y - std::floor(p.y / v.Ly) * v.Ly;
    } else {
        if (p.x < 0.f || p.x > v.Lx || p.y < 0.f || p.y > v.Ly) return 0.f;
    }
    float acc = 0.f;
    const float cellx = v.Lx / v.rshx;
    const float celly = v.Ly / v.rshy;
    auto visit = [&](int I) {
        f2 d{v.pos[2 * I] - q.x, v.pos[2 * I + 1] - q.y};
        if (periodic) {
            if (d.x > v.Lx - 2 * cellx) d.x -= v.Lx;
            if (d.x < -v.Lx + 2 * cellx) d.x += v.Lx;
            if (d.y > v.Ly - 2 * celly) d.y -= v.Ly;
            if (d.y < -v.Ly + 2 * celly) d.y += v.Ly;
        }
        const float r2 = d.x * d.x + d.y * d.y;
        if (r2 > hw * hw || (exclude_center && r2 < 1e-12f)) return;
        const float wi = v.w[I];
        const float wval = use_signed ? wi : std::fabs(wi);
        if (sign > 0 && wi <= 0) return;
        if (sign < 0 && wi >= 0) return;
        acc += wval * spline_pdf_f(std::sqrt(r2), hw);
    };
    if (v.vp_sort && v.cell_acc) {
        const int cx = std::min(trunc_to_int(q.x * v.rshx / v.Lx), v.rshx - 1);
        const int cy = std::min(trunc_to_int(q.y * v.rshy / v.Ly), v.rshy - 1);
        const int ncell = v.rshx * v.rshy;
        for (int ox = -1; ox <= 1; ++ox)
            for (int oy = -1; oy <= 1; ++oy) {
                int gx = cx + ox, gy = cy + oy;
                if (periodic) {
                    gx = (gx % v.rshx + v.rshx) % v.rshx;
                    gy = (gy % v.rshy + v.rshy) % v.rshy;
                } else if (gx < 0 || gy < 0 || gx >= v.rshx || gy >= v.rshy) {
                    continue;
                }
                const int c = gx * v.rshy + gy;
                const int beg = v.cell_acc[c];
                const int end = (c + 1 < ncell) ? v.cell_acc[c + 1] : v.cnt_view;
                for (int k = beg; k < end; ++k) visit(v.sub[v.vp_sort[k]]);
            }
    } else {
        for (int I = 0; I < v.N; ++I) visit(I);
    }
    return acc;
}

// queryVorticityAbs, include/vorticity_query.cuh:15-79, in FP64.
double query_vort_f64(const orc_view& v, double px, double py, int sign,
                      bool use_signed, bool exclude_center, double hw,
                      bool periodic) {
    if (periodic) {
        px = px - std::floor(px / v.Lx) * v.Lx;
        py = py - std::floor(py / v.Ly) * v.Ly;
    } else if (px < 0.0 || px > v.Lx || py < 0.0 || py > v.Ly) {
        return 0.0;
    }
    const int cx = std::min(static_cast<int>(px / v.Lx * v.rshx), v.rshx - 1);
    const int cy = std::min(static_cast<int>(py / v.Ly * v.rshy), v.rshy - 1);
    const int ncell = v.rshx * v.rshy;
    double acc = 0.0;
    for (int ox = -1; ox <= 1; ++ox)
        for (int oy = -1; oy <= 1; ++oy) {
            int gx = cx + ox, gy = cy + oy;
            if (periodic) {
                gx = (gx % v.rshx + v.rshx) % v.rshx;
                gy = (gy % v.rshy + v.rshy) % v.rshy;
            } else if (gx < 0 || gy < 0 || gx >= v.rshx || gy >= v.rshy) {
                continue;
            }
            const int c = gx * v.rshy + gy;
            const int beg = v.cell_acc[c];
            const int end = (c + 1 < ncell) ? v.cell_acc[c + 1] : v.cnt_view;
            for (int k = beg; k < end; ++k) {
                const int I = v.sub[v.vp_sort[k]];
                double a = 1, b = 0, cc = 0, d = 1;
                if (v.F) { a = v.F[4 * I]; b = v.F[4 * I + 1]; cc = v.F[4 * I + 2]; d = v.F[4 * I + 3]; }
                const double det = a * d - b * cc;
                double dx = double(v.pos[2 * I]) - px, dy = double(v.pos[2 * I + 1]) - py;
                if (periodic) {
                    if (dx > 0.5 * v.Lx) dx -= v.Lx;
                    if (dx < -0.5 * v.Lx) dx += v.Lx;
                    if (dy > 0.5 * v.Ly) dy -= v.Ly;
                    if (dy < -0.5 * v.Ly) dy += v.Ly;
                }
                const double lx = (d * dx - b * dy) / det;
                const double ly = (-cc * dx + a * dy) / det;
                const double rad = std::hypot(lx, ly);
                if (rad > 2.0 * hw) continue;
                if (exclude_center && rad < 1e-6) continue;
                const double wi = v.w[I];
                if (sign > 0 && wi <= 0) continue;
                if (sign < 0 && wi >= 0) continue;
                acc += (use_signed ? wi : std::fabs(wi)) * spline_pdf_d(rad, hw);
            }
        }
    return acc;
}

// ---- MC sampling helpers: src/cpu/monte_carlo_sampling.cpp:9-45,
//      include/monte_carlo_bs.hpp:60-102 ----
using Rng = std::mt19937;

inline float unif(Rng& g) {
    std::uniform_real_distribution<float> U(0.f, 1.f);
    return U(g);
}

int sample_cdf_index(Rng& g, const float* cdf, int n) {
    const float u = unif(g);
    const int j = static_cast<int>(std::upper_bound(cdf, cdf + n, u) - cdf);
    return j == n ? n - 1 : j;
}

f2 sample_disk(Rng& g, f2 c, float R) {
    const float phi = 2.f * kPiF * unif(g);
    const float u = unif(g);
    const float r = R * std::sqrt(u);
    return f2{c.x + r * std::cos(phi), c.y + r * std::sin(phi)};
}

f2 sample_image_shift(Rng& g) {
    f2 d{0.f, 0.f};
    const float ux = unif(g);
    const float uy = unif(g);
    if (ux < 1.f / 3.f) d.x = -1.f; else if (ux > 2.f / 3.f) d.x = 1.f;
    if (uy < 1.f / 3.f) d.y = -1.f; else if (uy > 2.f / 3.f) d.y = 1.f;
    return d;
}

float disk_radius(f2 dst, bool periodic, float Lx, float Ly) {
    if (!periodic) return std::sqrt(Lx * Lx + Ly * Ly);
    float m = 0.f;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy) {
            const f2 img{dst.x + dx * Lx, dst.y + dy * Ly};
            const f2 d{img.x - dst.x, img.y - dst.y};
            m = std::max(m, d.x * d.x + d.y * d.y);
        }
    return std::sqrt(m);
}

// biot_savart_kernel, include/monte_carlo_bs.hpp:60-66 (1e-8 regulariser).
inline f2 bs_kernel(f2 x, f2 y) {
    const f2 r{x.x - y.x, x.y - y.y};
    const float inv_r2 = 1.f / (r.x * r.x + r.y * r.y + 1e-8f);
    return f2{-r.y * inv_r2 / (2 * kPiF), r.x * inv_r2 / (2 * kPiF)};
}

// mis_contrib, src/cpu/monte_carlo_bs.cpp:11-26 (raw distance on the CPU path).
inline f2 mis_term(f2 dst, f2 sp, float om, float w1, float w2, float cum, float alpha) {
    if (om <= 0.f) return f2{0.f, 0.f};
    const f2 r{dst.x - sp.x, dst.y - sp.y};
    const float rn = std::max(std::sqrt(r.x * r.x + r.y * r.y), 1e-6f);
    const f2 k = bs_kernel(dst, sp);
    const float denom = w1 * om / cum + w2 * alpha / rn;
    const float s = om / denom;
    return f2{k.x * s, k.y * s};
}

inline void add(f2& a, f2 b) { a.x += b.x; a.y += b.y; }

// mis_contrib_dev (src/cuda/monte_carlo_bs.cu:35-51): as mis_term but the
// distance in alpha/r is the minimum image (wrap_delta, include/monte_carlo_bs.cuh:134-138).
inline f2 mis_term_gpu(f2 dst, f2 sp, float om, float w1, float w2, float cum, float alpha,
                       bool per, float Lx, float Ly) {
    if (om <= 0.f) return f2{0.f, 0.f};
    f2 r{dst.x - sp.x, dst.y - sp.y};
    if (per) { r.x = r.x - std::round(r.x / Lx) * Lx; r.y = r.y - std::round(r.y / Ly) * Ly; }
    const float rn = std::max(std::sqrt(r.x * r.x + r.y * r.y), 1e-6f);
    const f2 k = bs_kernel(dst, sp);
    const float denom = w1 * om / cum + w2 * alpha / rn;
    const float s = om / denom;
    return f2{k.x * s, k.y * s};
}

// monte_carlo_bs_cpu, src/cpu/monte_carlo_bs.cpp:28-128 (law 0), or the
// sampling law of monte_carlo_bs_kernel_safe (src/cuda/monte_carlo_bs.cu:
// 144-271) restated on the CPU with std::mt19937 (law 1): branch-1 jitter
// radius interp(icdf)*h_w with icdf already scaled by h_w (include/
// monte_carlo_bs.cuh:78-97, src/utilities.cu:87), the GPU query convention
// (queryVorticityAbs, here in FP64) and minimum-image alpha/r.
void mc_estimate(const orc_mcctx& C, const float* pos, const f2* dst, int sign,
                 int aux, int N1, int N2, Rng& g, f2* out, int law = 0,
                 const float* icdf = nullptr, int icdf_L = 0, const float* Fj = nullptr) {
    const float w1 = float(N1) / float(N1 + N2);
    const float w2 = float(N2) / float(N1 + N2);
    f2 s[5] = {};
    float cum = (sign > 0) ? C.cum_pos : C.cum_neg;
    const bool per = C.periodic != 0;
    if (per) cum *= 9.f;
    const orc_view& V = sign > 0 ? C.pos_view : C.neg_view;
    const float* cdf = sign > 0 ? C.cdf_pos : C.cdf_neg;
    const int* sub = sign > 0 ? C.sub_pos : C.sub_neg;
    const int n = sign > 0 ? C.cnt_pos : C.cnt_neg;
    auto alpha_of = [&](f2 d) { return 1.f / (2.f * kPiF * disk_radius(d, per, C.Lx, C.Ly)); };

    for (int i = 0; i < N1; ++i) {
        if (n == 0) break;                       // reference would read sub[-1]
        const int loc = sample_cdf_index(g, cdf, n);
        const int p = sub[loc];
        f2 sp = ld2(pos, p);
        if (per) {
            const f2 d = sample_image_shift(g);
            sp.x += d.x * C.Lx;
            sp.y += d.y * C.Ly;
        }
        if (law == 1) {
            const float u = unif(g);
            const float f = u * (icdf_L - 1);
            const int i0 = int(f), i1 = std::min(i0 + 1, icdf_L - 1);
            const float t = f - i0;
            const float rr = (icdf[i0] * (1.f - t) + icdf[i1] * t) * C.h_w;
            const float th = 2.f * kPiF * unif(g);
            const float jx = rr * std::cos(th), jy = rr * std::sin(th);
            if (Fj) {   // mul_mat2(F, r), include/monte_carlo_bs.cuh:99-103
                const float* f = Fj + 4 * p;
                sp.x += f[0] * jx + f[1] * jy;
                sp.y += f[2] * jx + f[3] * jy;
            } else {
                sp.x += jx;
                sp.y += jy;
            }
            const float om = float(query_vort_f64(V, sp.x, sp.y, sign, false, false, C.h_w, per));
            add(s[0], mis_term_gpu(dst[0], sp, om, w1, w2, cum, alpha_of(dst[0]), per, C.Lx, C.Ly));
            if (aux)
                for (int a = 1; a < 5; ++a)
                    add(s[a], mis_term_gpu(dst[a], sp, om, w1, w2, cum, alpha_of(dst[a]), per, C.Lx, C.Ly));
            continue;
        }
        const float om = eval_vort_cpu(V, sp, sign, false, false, C.h_w, per);
        add(s[0], mis_term(dst[0], sp, om, w1, w2, cum, alpha_of(dst[0])));
        if (aux)
            for (int a = 1; a < 5; ++a) add(s[a], mis_term(dst[a], sp, om, w1, w2, cum, alpha_of(dst[a])));
    }
    for (int i = 0; i < N2; ++i) {
        for (int a = 0; a < (aux ? 5 : 1); ++a) {
            const float R = disk_radius(dst[a], per, C.Lx, C.Ly);
            const float al = 1.f / (2.f * kPiF * R);
            const f2 sp = sample_disk(g, dst[a], R);
            if (law == 1) {
                const float om = float(query_vort_f64(V, sp.x, sp.y, sign, false, false, C.h_w, per));
                add(s[a], mis_term_gpu(dst[a], sp, om, w1, w2, cum, al, per, C.Lx, C.Ly));
                continue;
            }
            const float om = eval_vort_cpu(V, sp, sign, false, false, C.h_w, per);
            add(s[a], mis_term(dst[a], sp, om, w1, w2, cum, al));
        }
    }
    const float inv = 1.f / float(N1 + N2);
    for (int a = 0; a < 5; ++a) out[a] = f2{s[a].x * inv, s[a].y * inv};
}

// Nearest-image FP64 difference.
inline double min_img(double d, double L) { return d - L * std::nearbyint(d / L); }

// Enclosed cubic-spline mass inside q (closed form of the radial CDF).
inline double spline_mass_d(double q) {
    if (q <= 0.0) return 0.0;
    if (q >= 1.0) return 1.0;
    const double c = 80.0 / 7.0;
    if (q <= 0.5) {
        const double q2 = q * q;
        return c * (1.2 * q2 * q2 * q - 1.5 * q2 * q2 + 0.5 * q2);
    }
    auto G = [](double s) { const double s2 = s * s; return s2 - 2.0 * s2 * s + 1.5 * s2 * s2 - 0.4 * s2 * s2 * s; };
    return c * (0.06875 + G(q) - G(0.5));
}

int threads_or_default(int nthreads) {
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

}  // namespace

// ===========================================================================
extern "C" {

const char* orc_version(void) { return "vpmc-oracle 1 (restatement of the reference CPU path + FP64 maths)"; }

float orc_cubic_spline_pdf(float r, float h_w) { return spline_pdf_f(r, h_w); }
double orc_spline_mass(double q) { return spline_mass_d(q); }

void orc_fill_cells(int rshx, int rshy, float Lx, float Ly, int N,
                    const int* sub, const float* px, const float* py,
                    int* cell_num, int* cell_acc, int* vp_cell) {
    const int ncell = rshx * rshy;
    std::fill(cell_num, cell_num + ncell, 0);
    const float inv_hx = rshx / Lx;
    const float inv_hy = rshy / Ly;
    for (int i = 0; i < N; ++i) {
        const int j = sub[i];
        const int ix = std::clamp(floor_to_int(px[j] * inv_hx), 0, rshx - 1);
        const int iy = std::clamp(floor_to_int(py[j] * inv_hy), 0, rshy - 1);
        const int c = ix * rshy + iy;
        vp_cell[i] = c;
        ++cell_num[c];
    }
    if (ncell > 0) cell_acc[0] = 0;
    for (int c = 1; c < ncell; ++c) cell_acc[c] = cell_acc[c - 1] + cell_num[c - 1];
}

void orc_counting_sort(int N, int* cell_num, const int* cell_acc,
                       const int* vp_cell, int* vp_sort) {
    for (int i = N - 1; i >= 0; --i) {
        const int c = vp_cell[i];
        vp_sort[--cell_num[c] + cell_acc[c]] = i;
    }
}

int orc_fill_cells_omp(int rshx, int rshy, float Lx, float Ly, int N, const int* sub, const float* px,
                       const float* py, int* cell_num, int* cell_acc, int* vp_cell, int nthreads) {
    const int ncell = rshx * rshy;
    std::fill(cell_num, cell_num + ncell, 0);
    const float inv_hx = rshx / Lx;
    const float inv_hy = rshy / Ly;
    int used = 1;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
    {
#pragma omp single
        used = omp_get_num_threads();
        std::vector<int> local(size_t(ncell), 0);
#pragma omp for schedule(static)
        for (int i = 0; i < N; ++i) {
            const int j = sub[i];
            const int ix = std::clamp(floor_to_int(px[j] * inv_hx), 0, rshx - 1);
            const int iy = std::clamp(floor_to_int(py[j] * inv_hy), 0, rshy - 1);
            const int c = ix * rshy + iy;
            vp_cell[i] = c;
            ++local[size_t(c)];
        }
#pragma omp critical
        for (int c = 0; c < ncell; ++c) cell_num[c] += local[size_t(c)];
    }
    int acc = 0;
    for (int c = 0; c < ncell; ++c) {
        cell_acc[c] = acc;
        acc += cell_num[c];
    }
    return used;
}

int orc_counting_sort_omp(int N, int* cell_num, const int* cell_acc, const int* vp_cell, int* vp_sort,
                          int nthreads) {
    int used = 1;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
    {
#pragma omp single
        used = omp_get_num_threads();
#pragma omp for schedule(static)
        for (int i = N - 1; i >= 0; --i) {
            const int c = vp_cell[i];
            const int base = c == 0 ? 0 : cell_acc[c - 1];
            int old;
#pragma omp atomic capture
            old = cell_num[c]--;
            vp_sort[old - 1 + base] = i;
        }
    }
    return used;
}

void orc_build_subsets(int N, const float* omega, int* sub_pos, int* sub_neg,
                       float* cdf_pos, float* cdf_neg, int* cnt, float* cum) {
    int np = 0, nn = 0;
    float cp = 0.f, cn = 0.f;
    for (int i = 0; i < N; ++i) {
        const float w = omega[i];
        if (w > 0) { sub_pos[np] = i; cp += w; cdf_pos[np++] = cp; }
        else if (w < 0) { sub_neg[nn] = i; cn -= w; cdf_neg[nn++] = cn; }
    }
    if (cp > 0.f) { const float inv = 1.0f / cp; for (int k = 0; k < np; ++k) cdf_pos[k] *= inv; }
    if (cn > 0.f) { const float inv = 1.0f / cn; for (int k = 0; k < nn; ++k) cdf_neg[k] *= inv; }
    cnt[0] = np; cnt[1] = nn; cum[0] = cp; cum[1] = cn;
}

void orc_build_subsets_f64(int N, const float* omega, int* sub_pos, int* sub_neg,
                           double* cdf_pos, double* cdf_neg, int* cnt, double* cum) {
    int np = 0, nn = 0;
    double cp = 0.0, cn = 0.0;
    for (int i = 0; i < N; ++i) {
        const double w = omega[i];
        if (w > 0) { sub_pos[np] = i; cp += w; cdf_pos[np++] = cp; }
        else if (w < 0) { sub_neg[nn] = i; cn -= w; cdf_neg[nn++] = cn; }
    }
    for (int k = 0; k < np; ++k) cdf_pos[k] /= cp;
    for (int k = 0; k < nn; ++k) cdf_neg[k] /= cn;
    cnt[0] = np; cnt[1] = nn; cum[0] = cp; cum[1] = cn;
}

void orc_build_cubic_rcdf(float h_w, int length, float* cdf) {
    const float h_a = h_w / length;
    float acc = 0.f;
    for (int i = 0; i < length; ++i) {
        const float x = (0.5f + i) * h_a;
        acc += spline_pdf_f(x, h_w) * x;
        cdf[i] = acc;
    }
    const float total = cdf[length - 1];
    for (int i = 0; i < length; ++i) cdf[i] /= total;
}

void orc_cdf_to_icdf(const float* cdf, int L, float h_w, float* icdf) {
    const float dh = 1.f / L;
    auto lookup = [&](float u) -> float {
        int ptr = 0;
        while (ptr < L && u > cdf[ptr]) ++ptr;
        if (ptr == 0) { const float lam = (cdf[0] - u) / cdf[0]; return (1 - lam) * 0.5f; }
        if (ptr == L) { const float lam = (1 - u) / (1 - cdf[L - 1]); return (1 - lam) * (L - 0.5f); }
        const float lam = (cdf[ptr] - u) / (cdf[ptr] - cdf[ptr - 1]);
        return (1 - lam) * (ptr + 0.5f) + lam * (ptr - 0.5f);
    };
    for (int i = 0; i < L; ++i) {
        const float u = (i + 0.5f) * dh;
        icdf[i] = lookup(u) * dh * h_w;
    }
}

void orc_eval_vorticity_cpu(const orc_view* v, const float* pts, int M, int sign,
                            int use_signed, int exclude_center, float h_w,
                            int periodic, float* out) {
    for (int m = 0; m < M; ++m)
        out[m] = eval_vort_cpu(*v, ld2(pts, m), sign, use_signed != 0,
                               exclude_center != 0, h_w, periodic != 0);
}

void orc_query_vorticity_f64(const orc_view* v, const float* pts, int M, int sign,
                             int use_signed, int exclude_center, double h_w,
                             int periodic, double* out) {
    for (int m = 0; m < M; ++m)
        out[m] = query_vort_f64(*v, pts[2 * m], pts[2 * m + 1], sign, use_signed != 0,
                                exclude_center != 0, h_w, periodic != 0);
}

void orc_field_exact_f64(const float* pos, const float* w, int N, const float* pts,
                         int M, int sign, int use_signed, double h_w, double Lx,
                         double Ly, int periodic, double* out) {
#pragma omp parallel for schedule(static)
    for (int m = 0; m < M; ++m) {
        double px = pts[2 * m], py = pts[2 * m + 1];
        if (periodic) {
            px -= std::floor(px / Lx) * Lx;
            py -= std::floor(py / Ly) * Ly;
        }
        double acc = 0.0;
        for (int i = 0; i < N; ++i) {
            const double wi = w[i];
            if (sign > 0 && wi <= 0) continue;
            if (sign < 0 && wi >= 0) continue;
            double dx = double(pos[2 * i]) - px, dy = double(pos[2 * i + 1]) - py;
            if (periodic) { dx = min_img(dx, Lx); dy = min_img(dy, Ly); }
            const double r = std::sqrt(dx * dx + dy * dy);
            if (r >= h_w) continue;
            acc += (use_signed ? wi : std::fabs(wi)) * spline_pdf_d(r, h_w);
        }
        out[m] = acc;
    }
}

struct orc_rng { Rng g; };
orc_rng* orc_rng_create(uint32_t seed) { return new orc_rng{Rng(seed)}; }
void orc_rng_destroy(orc_rng* r) { delete r; }

void orc_mc_bs_estimate(const orc_mcctx* ctx, const float* pos, const float* dst5,
                        int sign, int auxiliary, int N1, int N2, orc_rng* rng,
                        float* out10) {
    f2 dst[5], out[5];
    for (int a = 0; a < 5; ++a) dst[a] = ld2(dst5, a);
    mc_estimate(*ctx, pos, dst, sign, auxiliary, N1, N2, rng->g, out);
    for (int a = 0; a < 5; ++a) { out10[2 * a] = out[a].x; out10[2 * a + 1] = out[a].y; }
}

void orc_mc_velocity(const orc_mcctx* ctx, const float* pos, const float* targets,
                     int M, int N1, int N2, uint32_t seed, float* vel) {
    Rng g(seed);
    for (int t = 0; t < M; ++t) {
        f2 dst[5];
        for (int a = 0; a < 5; ++a) dst[a] = ld2(targets, t);
        f2 vp[5], vn[5];
        mc_estimate(*ctx, pos, dst, +1, 0, N1, N2, g, vp);
        mc_estimate(*ctx, pos, dst, -1, 0, N1, N2, g, vn);
        vel[2 * t] = vp[0].x - vn[0].x;
        vel[2 * t + 1] = vp[0].y - vn[0].y;
    }
}

int orc_mc_velocity_omp(const orc_mcctx* ctx, const float* pos, const float* targets,
                        int M, int N1, int N2, uint32_t seed, float* vel, int nthreads,
                        int law, const float* icdf, int icdf_L) {
    const int nt = threads_or_default(nthreads);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
    for (int t = 0; t < M; ++t) {
        Rng g(seed + static_cast<uint32_t>(t));
        f2 dst[5];
        for (int a = 0; a < 5; ++a) dst[a] = ld2(targets, t);
        f2 vp[5], vn[5];
        mc_estimate(*ctx, pos, dst, +1, 0, N1, N2, g, vp, law, icdf, icdf_L);
        mc_estimate(*ctx, pos, dst, -1, 0, N1, N2, g, vn, law, icdf, icdf_L);
        vel[2 * t] = vp[0].x - vn[0].x;
        vel[2 * t + 1] = vp[0].y - vn[0].y;
    }
    return nt;
}

int orc_mc_velocity5_omp(const orc_mcctx* ctx, const float* pos, const float* F,
                         const float* targets, int M, int N1, int N2, float dx,
                         uint32_t seed, float* vel10, int nthreads, const float* icdf,
                         int icdf_L) {
    const int nt = threads_or_default(nthreads);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
    for (int t = 0; t < M; ++t) {
        Rng g(seed + static_cast<uint32_t>(t));
        const f2 x = ld2(targets, t);
        // monte_carlo_bs_kernel_safe's auxiliary points (src/cuda/monte_carlo_bs.cu:163-167)
        const f2 dst[5] = {x, f2{x.x - dx, x.y}, f2{x.x + dx, x.y}, f2{x.x, x.y + dx}, f2{x.x, x.y - dx}};
        f2 vp[5], vn[5];
        mc_estimate(*ctx, pos, dst, +1, 1, N1, N2, g, vp, 1, icdf, icdf_L, F);
        mc_estimate(*ctx, pos, dst, -1, 1, N1, N2, g, vn, 1, icdf, icdf_L, F);
        for (int a = 0; a < 5; ++a) {
            vel10[10 * t + 2 * a] = vp[a].x - vn[a].x;
            vel10[10 * t + 2 * a + 1] = vp[a].y - vn[a].y;
        }
    }
    return nt;
}

namespace {

// ---- this build's MIS estimator restated in FP64 (for finite differences) ----
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the uniform maps the
// product uses; key = mix32 of the seed, counter = (sample | sign << 31,
// target, step lo, step hi).
struct P4 { uint32_t x, y, z, w; };
P4 philox(P4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = uint64_t(0xD2511F53u) * c.x, p1 = uint64_t(0xCD9E8D57u) * c.z;
        c = P4{uint32_t(p1 >> 32) ^ c.y ^ k0, uint32_t(p1), uint32_t(p0 >> 32) ^ c.w ^ k1, uint32_t(p0)};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}
inline double u01f(uint32_t r) { return double((float(r >> 8) + 0.5f) * (1.0f / 16777216.0f)); }
inline double u01dd(uint32_t r) { return (double(r) + 0.5) * (1.0 / 4294967296.0); }
uint32_t mix32(uint64_t v) {
    v ^= v >> 33;
    v *= 0xff51afd7ed558ccdULL;
    v ^= v >> 33;
    v *= 0xc4ceb9fe1a85ec53ULL;
    v ^= v >> 33;
    return uint32_t(v);
}

}  // namespace

int orc_mis_forward_f64(const float* pos0, const float* omega, const float* omega_sample, int N, int Nx,
                        float hwr, float Lx, float Ly, int periodic, int law, int N1, int N2, float dt,
                        uint64_t seed, uint64_t step0, int nsteps, double* pos_out, int nthreads) {
    const int nt = threads_or_default(nthreads);
    // SimParam: h = Lx / Nx, h_w = h * hwr in FP32
    const float hf = Lx / float(Nx);
    const double hw = double(hf * hwr);
    const uint32_t k0 = mix32(seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL);
    const uint32_t k1 = mix32(seed ^ 0xA4093822299F31D0ULL);
    // sampling law (frozen): subsets and FP64 |omega| CDF of omega_sample
    std::vector<int> sub[2];
    std::vector<double> cdf[2];
    for (int i = 0; i < N; ++i) {
        const float w = omega_sample[i];
        if (w == 0.f) continue;
        const int s = w > 0.f ? 0 : 1;
        sub[s].push_back(i);
        cdf[s].push_back((cdf[s].empty() ? 0.0 : cdf[s].back()) + std::fabs(double(w)));
    }
    for (int s = 0; s < 2; ++s)
        for (auto& c : cdf[s]) c /= cdf[s].back();
    // Omega of the current strengths (x9 when periodic); the sign pattern must match
    double cum[2] = {0.0, 0.0};
    for (int i = 0; i < N; ++i) {
        if ((omega[i] > 0.f) != (omega_sample[i] > 0.f) || (omega[i] < 0.f) != (omega_sample[i] < 0.f)) return -1;
        if (omega[i] != 0.f) cum[omega[i] > 0.f ? 0 : 1] += std::fabs(double(omega[i]));
    }
    const double f9 = periodic ? 9.0 : 1.0;
    // jitter tables: reference law = the reference's 20-entry iCDF, unbiased = inverse radial mass
    float rc[20], icdf[20];
    orc_build_cubic_rcdf(float(hw), 20, rc);
    orc_cdf_to_icdf(rc, 20, float(hw), icdf);
    std::vector<float> jit(1025);
    for (int i = 0; i <= 1024; ++i) {
        const double u = double(i) / 1024;
        double lo = 0.0, hi = 1.0;
        for (int it = 0; it < 80; ++it) {
            const double mid = 0.5 * (lo + hi);
            if (spline_mass_d(mid) < u) lo = mid; else hi = mid;
        }
        jit[i] = float(0.5 * (lo + hi));
    }
    jit[0] = 0.f;
    jit[1024] = 1.f;
    const int Q = N1 + N2;
    const double w1 = double(N1) / Q, w2 = double(N2) / Q;
    const double R = std::sqrt(double(Lx) * Lx + double(Ly) * Ly), alpha = 1.0 / (2.0 * kPiD * R);
    const double sigma = 40.0 / (7.0 * kPiD * hw * hw);
    std::vector<double> X(2 * size_t(N)), Xn(2 * size_t(N));
    for (int i = 0; i < 2 * N; ++i) X[i] = pos0[i];
    auto field = [&](int s, double yx, double yy) {
        double f = 0.0;
        const int lo = periodic ? -1 : 0, hi = periodic ? 1 : 0;
        for (int J : sub[s]) {
            const double aw = std::fabs(double(omega[J]));
            for (int mx = lo; mx <= hi; ++mx)
                for (int my = lo; my <= hi; ++my) {
                    const double dx = yx - (X[2 * J] + mx * Lx), dy = yy - (X[2 * J + 1] + my * Ly);
                    const double r = std::sqrt(dx * dx + dy * dy);
                    if (r >= hw) continue;
                    const double q = r / hw;
                    f += aw * sigma * (q <= 0.5 ? 6.0 * (q * q * q - q * q) + 1.0 : 2.0 * (1 - q) * (1 - q) * (1 - q));
                }
        }
        return f;
    };
    for (int n = 0; n < nsteps; ++n) {
        const uint64_t step = step0 + uint64_t(n);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
        for (int t = 0; t < N; ++t) {
            const double x = X[2 * t], y0 = X[2 * t + 1];
            double u[2] = {0.0, 0.0};
            for (int s = 0; s < 2; ++s) {
                const int ns = int(sub[s].size());
                double ax = 0.0, ay = 0.0;
                for (int j = 0; j < Q; ++j) {
                    const P4 r = philox(P4{uint32_t(j) | (uint32_t(s) << 31), uint32_t(t), uint32_t(step),
                                           uint32_t(step >> 32)}, k0, k1);
                    double yx, yy;
                    if (j < N1) {
                        if (ns == 0) continue;
                        const double uu = u01dd(r.x);
                        int idx = int(std::upper_bound(cdf[s].begin(), cdf[s].end(), uu) - cdf[s].begin());
                        idx = std::min(idx, ns - 1);
                        const int p = sub[s][idx];
                        yx = X[2 * p];
                        yy = X[2 * p + 1];
                        if (periodic) {
                            const int m9 = std::min(int(float(u01f(r.y)) * 9.f), 8);
                            yx += double(m9 / 3 - 1) * Lx;
                            yy += double(m9 % 3 - 1) * Ly;
                        }
                        double rr;
                        const float ur = float(u01f(r.z));
                        if (law == 0) {
                            const float f = ur * 19.f;
                            const int i0 = int(f), i1 = std::min(i0 + 1, 19);
                            const float tt = f - float(i0);
                            rr = double(icdf[i0] * (1.f - tt) + icdf[i1] * tt) * hw;
                        } else {
                            const float f = ur * 1024.f;
                            const int i0 = std::min(int(f), 1023);
                            const float tt = f - float(i0);
                            rr = double(jit[i0] * (1.f - tt) + jit[i0 + 1] * tt) * hw;
                        }
                        const double th = 2.0 * kPiD * u01f(r.w);
                        yx += rr * std::cos(th);
                        yy += rr * std::sin(th);
                    } else {
                        const double phi = 2.0 * kPiD * u01f(r.x), ur = u01f(r.y);
                        const double rr = law == 0 ? R * std::sqrt(ur) : R * ur;
                        yx = x + rr * std::cos(phi);
                        yy = y0 + rr * std::sin(phi);
                    }
                    // field at the sample: unbiased law = the 3x3 images around the
                    // sample's own tile; reference law = the periodic field
                    double f = 0.0;
                    if (periodic) {
                        const double kx = std::floor(yx / Lx), ky = std::floor(yy / Ly);
                        if (law == 1) {
                            if (std::fabs(kx) > 2.0 || std::fabs(ky) > 2.0) continue;
                            f = field(s, yx, yy);
                        } else {
                            f = field(s, yx - kx * Lx, yy - ky * Ly);
                        }
                    } else {
                        if (yx < 0.0 || yx > Lx || yy < 0.0 || yy > Ly) continue;
                        f = field(s, yx, yy);
                    }
                    if (!(f > 0.0)) continue;
                    const double rx = x - yx, ry = y0 - yy;
                    const double c = cum[s] * f9;
                    double sc;
                    if (law == 0) {
                        double wx = rx, wy = ry;
                        if (periodic) { wx = rx - std::round(rx / Lx) * Lx; wy = ry - std::round(ry / Ly) * Ly; }
                        const double rn = std::max(std::sqrt(wx * wx + wy * wy), 1e-6);
                        const double inv = 1.0 / (rx * rx + ry * ry + 1e-8);
                        sc = f / (w1 * f / c + w2 * alpha / rn) * inv / (2.0 * kPiD);
                    } else {
                        const double r2 = rx * rx + ry * ry;
                        if (!(r2 > 0.0)) continue;
                        const double rn = std::sqrt(r2);
                        const double p2 = rn < R ? alpha / rn : 0.0;
                        sc = f / ((w1 * f / c + w2 * p2) * (2.0 * kPiD * r2));
                    }
                    ax += -ry * sc;
                    ay += rx * sc;
                }
                const double sg = s == 0 ? 1.0 : -1.0;
                u[0] += sg * ax / Q;
                u[1] += sg * ay / Q;
            }
            double nx = x + double(dt) * u[0], ny = y0 + double(dt) * u[1];
            if (periodic) {
                nx -= std::floor(nx / Lx) * Lx;
                ny -= std::floor(ny / Ly) * Ly;
            }
            Xn[2 * t] = nx;
            Xn[2 * t + 1] = ny;
        }
        X.swap(Xn);
    }
    for (int i = 0; i < 2 * N; ++i) pos_out[i] = X[i];
    return 0;
}

void orc_rbf_matvec_f64(const orc_view* all_view, const double* x, double* y,
                        double h_w, int periodic, int nthreads) {
    const orc_view& V = *all_view;
    const int N = V.N;
    const int nt = threads_or_default(nthreads);
    const int ncell = V.rshx * V.rshy;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int i = 0; i < N; ++i) {
        double px = V.pos[2 * i], py = V.pos[2 * i + 1];
        if (periodic) {
            px -= std::floor(px / V.Lx) * V.Lx;
            py -= std::floor(py / V.Ly) * V.Ly;
        } else if (px < 0.0 || px > V.Lx || py < 0.0 || py > V.Ly) {
            y[i] = 0.0;
            continue;
        }
        const int cx = std::min(static_cast<int>(px / V.Lx * V.rshx), V.rshx - 1);
        const int cy = std::min(static_cast<int>(py / V.Ly * V.rshy), V.rshy - 1);
        double acc = 0.0;
        for (int ox = -1; ox <= 1; ++ox)
            for (int oy = -1; oy <= 1; ++oy) {
                int gx = cx + ox, gy = cy + oy;
                if (periodic) {
                    gx = (gx % V.rshx + V.rshx) % V.rshx;
                    gy = (gy % V.rshy + V.rshy) % V.rshy;
                } else if (gx < 0 || gy < 0 || gx >= V.rshx || gy >= V.rshy) {
                    continue;
                }
                const int c = gx * V.rshy + gy;
                const int beg = V.cell_acc[c];
                const int end = (c + 1 < ncell) ? V.cell_acc[c + 1] : V.cnt_view;
                for (int k = beg; k < end; ++k) {
                    const int J = V.sub[V.vp_sort[k]];
                    double a = 1, b = 0, cc = 0, d = 1;
                    if (V.F) { a = V.F[4 * J]; b = V.F[4 * J + 1]; cc = V.F[4 * J + 2]; d = V.F[4 * J + 3]; }
                    const double det = a * d - b * cc;
                    double dx = double(V.pos[2 * J]) - px, dy = double(V.pos[2 * J + 1]) - py;
                    if (periodic) {
                        if (dx > 0.5 * V.Lx) dx -= V.Lx;
                        if (dx < -0.5 * V.Lx) dx += V.Lx;
                        if (dy > 0.5 * V.Ly) dy -= V.Ly;
                        if (dy < -0.5 * V.Ly) dy += V.Ly;
                    }
                    const double rad = std::hypot((d * dx - b * dy) / det, (-cc * dx + a * dy) / det);
                    if (rad > 2.0 * h_w) continue;
                    acc += x[J] * spline_pdf_d(rad, h_w);
                }
            }
        y[i] = acc;
    }
}

int orc_cg_rbf_f64(const orc_view* all_view, const float* b, double* x, double h_w,
                   int periodic, double tol, int max_iter, double* relres,
                   double* true_relres, int nthreads) {
    const int N = all_view->N;
    std::vector<double> r(N), p(N), Ap(N), bb(N);
    for (int i = 0; i < N; ++i) bb[i] = b[i];
    const double diag = spline_pdf_d(0.0, h_w);
    for (int i = 0; i < N; ++i) x[i] = bb[i] / diag;
    orc_rbf_matvec_f64(all_view, x, Ap.data(), h_w, periodic, nthreads);
    double bnorm2 = 0.0, rr = 0.0;
    for (int i = 0; i < N; ++i) { r[i] = bb[i] - Ap[i]; p[i] = r[i]; rr += r[i] * r[i]; bnorm2 += bb[i] * bb[i]; }
    const double bnorm = std::sqrt(bnorm2);
    int it = 0;
    double res = bnorm > 0 ? std::sqrt(rr) / bnorm : 0.0;
    while (it < max_iter && res >= tol && bnorm > 0) {
        orc_rbf_matvec_f64(all_view, p.data(), Ap.data(), h_w, periodic, nthreads);
        double pAp = 0.0;
        for (int i = 0; i < N; ++i) pAp += p[i] * Ap[i];
        if (pAp == 0.0) break;
        const double alpha = rr / pAp;
        double rr_new = 0.0;
        for (int i = 0; i < N; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; rr_new += r[i] * r[i]; }
        ++it;
        res = std::sqrt(rr_new) / bnorm;
        if (res < tol) break;
        const double beta = rr_new / rr;
        for (int i = 0; i < N; ++i) p[i] = r[i] + beta * p[i];
        rr = rr_new;
    }
    if (relres) *relres = res;
    if (true_relres) {
        orc_rbf_matvec_f64(all_view, x, Ap.data(), h_w, periodic, nthreads);
        double s = 0.0;
        for (int i = 0; i < N; ++i) { const double e = bb[i] - Ap[i]; s += e * e; }
        *true_relres = bnorm > 0 ? std::sqrt(s) / bnorm : 0.0;
    }
    return it;
}

void orc_direct_mollified_f64(const float* pos, const float* omega, int N,
                              const float* pts, int M, double h_w, double Lx,
                              double Ly, int periodic, double* out_uv, int nthreads) {
    const int nt = threads_or_default(nthreads);
    const int lo = periodic ? -1 : 0, hi = periodic ? 1 : 0;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
    for (int m = 0; m < M; ++m) {
        const double px = pts[2 * m], py = pts[2 * m + 1];
        double u = 0.0, v = 0.0;
        for (int i = 0; i < N; ++i) {
            const double wi = omega[i];
            if (wi == 0.0) continue;
            for (int ix = lo; ix <= hi; ++ix)
                for (int iy = lo; iy <= hi; ++iy) {
                    const double dx = px - (double(pos[2 * i]) + ix * Lx);
                    const double dy = py - (double(pos[2 * i + 1]) + iy * Ly);
                    const double r2 = dx * dx + dy * dy;
                    if (r2 == 0.0) continue;
                    const double k = spline_mass_d(std::sqrt(r2) / h_w) / (2.0 * kPiD * r2);
                    u += wi * (-dy * k);
                    v += wi * (dx * k);
                }
        }
        out_uv[2 * m] = u;
        out_uv[2 * m + 1] = v;
    }
}

namespace {

// Gauss-Legendre nodes/weights on [-1, 1]: Newton iteration on P_n from the
// Chebyshev-like initial guesses (the textbook method).
struct GL {
    std::vector<double> x, w;
    explicit GL(int n) : x(n), w(n) {
        for (int i = 0; i < n; ++i) {
            double z = std::cos(kPiD * (i + 0.75) / (n + 0.5)), pp = 1.0;
            for (int it = 0; it < 100; ++it) {
                double p1 = 1.0, p2 = 0.0;
                for (int j = 1; j <= n; ++j) {
                    const double p3 = p2;
                    p2 = p1;
                    p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
                }
                pp = n * (z * p1 - p2) / (z * z - 1.0);
                const double dz = p1 / pp;
                z -= dz;
                if (std::fabs(dz) < 1e-16) break;
            }
            x[i] = z;
            w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
        }
    }
};

// Unnormalised radial profile of the cubic B-spline (utilities.hpp:7-17
// without the 40/(7 pi h^2) factor) at q = |v|/h.
inline double spline_shape(double q) {
    if (q < 0.5) return 6.0 * (q * q * q - q * q) + 1.0;
    if (q < 1.0) { const double t = 1.0 - q; return 2.0 * t * t * t; }
    return 0.0;
}

// g(theta) = integral over rho >= 0 of W-shape(|v + rho e| / h): pieces split
// where the ray crosses |.| = h/2, h and at its closest approach, GL on each.
double ray_integral(double vx, double vy, double ex, double ey, double h, const GL& gl) {
    const double b = vx * ex + vy * ey, c0 = vx * vx + vy * vy;
    const double dh = b * b - c0 + h * h;
    if (dh <= 0.0) return 0.0;
    const double sh = std::sqrt(dh);
    const double lo = std::max(0.0, -b - sh), hi = -b + sh;
    if (hi <= lo) return 0.0;
    double cut[6];
    int nc = 0;
    cut[nc++] = lo;
    const double di = b * b - c0 + 0.25 * h * h;
    double pts[3];
    int np = 0;
    if (di > 0.0) { const double si = std::sqrt(di); pts[np++] = -b - si; pts[np++] = -b + si; }
    pts[np++] = -b;
    std::sort(pts, pts + np);
    for (int k = 0; k < np; ++k) if (pts[k] > lo && pts[k] < hi) cut[nc++] = pts[k];
    cut[nc++] = hi;
    double acc = 0.0;
    for (int k = 0; k + 1 < nc; ++k) {
        const double a0 = cut[k], a1 = cut[k + 1], hm = 0.5 * (a1 - a0), cm = 0.5 * (a1 + a0);
        double part = 0.0;
        for (size_t g = 0; g < gl.x.size(); ++g) {
            const double r = cm + hm * gl.x[g];
            const double qx = vx + r * ex, qy = vy + r * ey;
            part += gl.w[g] * spline_shape(std::sqrt(qx * qx + qy * qy) / h);
        }
        acc += hm * part;
    }
    return acc;
}

}  // namespace

void orc_direct_deformed_f64(const float* pos, const float* omega, const float* F, int N,
                             const float* pts, int M, double h_w, double Lx, double Ly,
                             int periodic, double* out_uv, int nthreads) {
    const int nt = threads_or_default(nthreads);
    const int lo = periodic ? -1 : 0, hi = periodic ? 1 : 0;
    const double norm = 40.0 / (7.0 * kPiD * h_w * h_w);
    const GL gr(12), gt(48), gf(10);
    const int n_trap = 1024;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int m = 0; m < M; ++m) {
        const double px = pts[2 * m], py = pts[2 * m + 1];
        double u = 0.0, v = 0.0;
        for (int i = 0; i < N; ++i) {
            const double wi = omega[i];
            if (wi == 0.0) continue;
            double a = 1, b = 0, c = 0, d = 1;
            if (F) { a = F[4 * i]; b = F[4 * i + 1]; c = F[4 * i + 2]; d = F[4 * i + 3]; }
            const double det = a * d - b * c, adet = std::fabs(det);
            // sigma_max(F): reach of the deformed support
            const double T = a * a + b * b + c * c + d * d;
            const double smax = std::sqrt(0.5 * (T + std::sqrt(std::max(T * T - 4.0 * det * det, 0.0))));
            for (int ix = lo; ix <= hi; ++ix)
                for (int iy = lo; iy <= hi; ++iy) {
                    const double rx = px - (double(pos[2 * i]) + ix * Lx);
                    const double ry = py - (double(pos[2 * i + 1]) + iy * Ly);
                    const double dist = std::sqrt(rx * rx + ry * ry);
                    double su = 0.0, sv = 0.0;
                    if (dist > 3.0 * smax * h_w) {
                        // smooth kernel over the blob: polar GL in v-space, y = c + F v
                        for (int pc = 0; pc < 2; ++pc) {
                            const double r0 = pc == 0 ? 0.0 : 0.5 * h_w, r1 = pc == 0 ? 0.5 * h_w : h_w;
                            for (size_t g = 0; g < gf.x.size(); ++g) {
                                const double rr = 0.5 * (r0 + r1) + 0.5 * (r1 - r0) * gf.x[g];
                                const double wr = 0.5 * (r1 - r0) * gf.w[g] * rr * spline_shape(rr / h_w);
                                for (int k = 0; k < 64; ++k) {
                                    const double th = 2.0 * kPiD * (k + 0.5) / 64.0;
                                    const double vx = rr * std::cos(th), vy = rr * std::sin(th);
                                    const double dx = rx - (a * vx + b * vy), dy = ry - (c * vx + d * vy);
                                    const double kk = wr * (2.0 * kPiD / 64.0) / (2.0 * kPiD * (dx * dx + dy * dy));
                                    su += -dy * kk;
                                    sv += dx * kk;
                                }
                            }
                        }
                    } else {
                        // rays from the singular point v* = F^-1 (x - c): K dv = -perp(F e)/(2 pi |F e|^2) drho dtheta
                        const double vx = (d * rx - b * ry) / det, vy = (-c * rx + a * ry) / det;
                        const double vr = std::sqrt(vx * vx + vy * vy);
                        auto add_dir = [&](double th, double wt) {
                            const double ex = std::cos(th), ey = std::sin(th);
                            const double g = ray_integral(vx, vy, ex, ey, h_w, gr);
                            if (g == 0.0) return;
                            const double fx = a * ex + b * ey, fy = c * ex + d * ey;
                            const double s = -wt * g / (2.0 * kPiD * (fx * fx + fy * fy));
                            su += s * (-fy);
                            sv += s * fx;
                        };
                        if (vr < h_w) {
                            for (int k = 0; k < n_trap; ++k) add_dir(2.0 * kPiD * k / n_trap, 2.0 * kPiD / n_trap);
                        } else {
                            const double phi0 = std::atan2(-vy, -vx), be = std::asin(std::min(1.0, h_w / vr));
                            const double bi = std::asin(std::min(1.0, 0.5 * h_w / vr));
                            const double edges[4] = {-be, -bi, bi, be};
                            for (int pc = 0; pc < 3; ++pc) {
                                const double t0 = edges[pc], t1 = edges[pc + 1];
                                for (size_t g = 0; g < gt.x.size(); ++g)
                                    add_dir(phi0 + 0.5 * (t0 + t1) + 0.5 * (t1 - t0) * gt.x[g], 0.5 * (t1 - t0) * gt.w[g]);
                            }
                        }
                    }
                    u += wi * adet * norm * su;
                    v += wi * adet * norm * sv;
                }
        }
        out_uv[2 * m] = u;
        out_uv[2 * m + 1] = v;
    }
}

void orc_direct_plummer_f64(const float* pos, const float* omega, int N, const int* tidx,
                            int M, double eps, double Lx, double Ly, int periodic,
                            double* out_uv, int nthreads) {
    const int nt = threads_or_default(nthreads);
    const double e2 = eps * eps;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int m = 0; m < M; ++m) {
        const int i = tidx[m];
        double u = 0.0, v = 0.0;
        for (int j = 0; j < N; ++j) {
            if (j == i) continue;
            double dx = double(pos[2 * i]) - double(pos[2 * j]);
            double dy = double(pos[2 * i + 1]) - double(pos[2 * j + 1]);
            if (periodic) { dx = min_img(dx, Lx); dy = min_img(dy, Ly); }
            const double c = 1.0 / (2.0 * kPiD * (dx * dx + dy * dy + e2));
            u += omega[j] * (-dy * c);
            v += omega[j] * (dx * c);
        }
        out_uv[2 * m] = u;
        out_uv[2 * m + 1] = v;
    }
}

}  // extern "C"
