// utilities.hpp -- cubic B-spline and kernel radial tables (the reference's
// include/utilities.hpp:7-17, src/utilities.cu:12-96), host side.
#pragma once

#include <vector>

#include "device_vector_alias.hpp"

// W(r; h_w) = 40/(7 pi h_w^2) * {6(q^3 - q^2) + 1, q <= 1/2; 2(1-q)^3, q < 1; 0}
inline float cubicSplinePDF(float r, float h_w) { return vpmc_cubic_spline(r, h_w); }

// Radial CDF of r W(r) at `length` midpoints, normalised (device output).
inline void build_cubic_rcdf(float h_w, int length, dvec<float>& cdf) {
    std::vector<float> c(length), ic(length);
    vpmc::check(vpmc_kernel_icdf_table(h_w, length, c.data(), ic.data()), "build_cubic_rcdf");
    cdf.assign(c);
}

// Piecewise-linear inverse of that CDF at bin centres, scaled by h_w.
inline void cdf_to_icdf(const dvec<float>& cdf, float h_w, dvec<float>& icdf) {
    std::vector<float> c(cdf.size()), ic(cdf.size());
    vpmc::check(vpmc_kernel_icdf_table(h_w, int(cdf.size()), c.data(), ic.data()), "cdf_to_icdf");
    icdf.assign(ic);
}
