// analytical_flow.hpp -- Taylor-Green vortex (the reference's
// include/analytical_flow.hpp:12-31): u = (sin 2pi x cos 2pi y, -cos 2pi x sin 2pi y),
// omega = 4 pi sin 2pi x sin 2pi y.
#pragma once

#include <cmath>

#include <vector_types.h>

constexpr float TWO_PI = 6.28318530717958647692f;

inline float2 taylor_green_velocity(float x, float y) {
    return {std::sin(TWO_PI * x) * std::cos(TWO_PI * y), -std::cos(TWO_PI * x) * std::sin(TWO_PI * y)};
}
inline float2 taylor_green_velocity(const float2& p) { return taylor_green_velocity(p.x, p.y); }
inline float taylor_green_vorticity(float x, float y) {
    return 4.0f * 3.14159265358979323846f * std::sin(TWO_PI * x) * std::sin(TWO_PI * y);
}
inline float taylor_green_vorticity(const float2& p) { return taylor_green_vorticity(p.x, p.y); }
