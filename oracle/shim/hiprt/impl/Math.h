/*
 * Clean-room stand-in for the HIPRT scalar/vector helpers the reference calls as hiprt::
 * (src/HostDeviceCommon/Math.h:358-436 of the reference). The definitions are the textbook
 * ones, evaluated left to right: dot = x*x' + y*y' + z*z', cross by the determinant rule,
 * normalize = v / sqrt(dot(v, v)). Test infrastructure only.
 */
#ifndef GBPT_SHIM_HIPRT_MATH_H
#define GBPT_SHIM_HIPRT_MATH_H

#include <hiprt/hiprt_vec.h>
#include <cmath>

namespace hiprt
{
constexpr float Pi = 3.14159265358979323846f;

template <typename T> inline T min(T a, T b) { return a < b ? a : b; }
template <typename T> inline T max(T a, T b) { return a > b ? a : b; }
template <typename T> inline T clamp(T x, T lo, T hi) { return min(max(x, lo), hi); }

inline float dot(const hiprtFloat3& a, const hiprtFloat3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline hiprtFloat3 cross(const hiprtFloat3& a, const hiprtFloat3& b)
{
    return make_hiprtFloat3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline hiprtFloat3 normalize(const hiprtFloat3& a) { return a / std::sqrt(dot(a, a)); }
} // namespace hiprt

#endif
