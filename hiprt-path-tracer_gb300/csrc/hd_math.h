// Small float3 vector type and helpers usable from device code (nvcc) and from the host build
// that the CPU tests compile (tests/native), so that one source of the BSDF and sampling code
// runs in both.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#include <cuda_runtime.h>
#ifndef GBPT_HD
#define GBPT_HD __device__ __forceinline__
#endif
// a device function kept out of line: rarely taken code whose inlined copy would raise the
// register count of the kernels that call it
#define GBPT_HD_OUTLINE static __device__ __noinline__
#else
#include <cmath>
#include <cstring>
#ifndef GBPT_HD
#define GBPT_HD inline
#endif
#define GBPT_HD_OUTLINE inline
#endif

namespace gbpt {
namespace hd {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kTwoPi = 6.28318530717958647693f;

struct V3
{
    float x, y, z;
};
GBPT_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
GBPT_HD V3 v3(float s) { return V3{s, s, s}; }
GBPT_HD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
GBPT_HD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
GBPT_HD V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
GBPT_HD V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
GBPT_HD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
GBPT_HD V3 operator*(float s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }
GBPT_HD V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
GBPT_HD V3 operator/(float s, V3 a) { return v3(s / a.x, s / a.y, s / a.z); }
GBPT_HD V3 operator+(V3 a, float s) { return v3(a.x + s, a.y + s, a.z + s); }
GBPT_HD V3 operator-(float s, V3 a) { return v3(s - a.x, s - a.y, s - a.z); }
GBPT_HD V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
GBPT_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GBPT_HD V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
GBPT_HD float length(V3 a) { return sqrtf(dot(a, a)); }
GBPT_HD V3 normalize(V3 a) { return a / sqrtf(dot(a, a)); }
GBPT_HD float max_comp(V3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
GBPT_HD bool is_black(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
GBPT_HD bool is_white(V3 a) { return a.x == 1.0f && a.y == 1.0f && a.z == 1.0f; }
// Rec. 709-like weights the reference uses for luminance (src/HostDeviceCommon/Color.h:90)
GBPT_HD float luminance(V3 c) { return 0.3086f * c.x + 0.6094f * c.y + 0.0820f * c.z; }
GBPT_HD float clampf(float lo, float hi, float x) { return fminf(hi, fmaxf(lo, x)); }
GBPT_HD V3 clamp3(float lo, float hi, V3 a) { return v3(clampf(lo, hi, a.x), clampf(lo, hi, a.y), clampf(lo, hi, a.z)); }
// (1 - t) * a + t * b, the blend form the reference uses everywhere
GBPT_HD float lerp(float a, float b, float t) { return (1.0f - t) * a + t * b; }
GBPT_HD V3 lerp(V3 a, V3 b, float t) { return (1.0f - t) * a + t * b; }
GBPT_HD float sq(float x) { return x * x; }
GBPT_HD float pow6(float x)
{
    const float x2 = x * x;
    const float x4 = x2 * x2;
    return x4 * x2;
}
GBPT_HD V3 exp3(V3 a) { return v3(expf(a.x), expf(a.y), expf(a.z)); }
GBPT_HD V3 log3(V3 a) { return v3(logf(a.x), logf(a.y), logf(a.z)); }
GBPT_HD V3 sqrt3(V3 a) { return v3(sqrtf(a.x), sqrtf(a.y), sqrtf(a.z)); }
GBPT_HD V3 pow3(V3 a, float e) { return v3(powf(a.x, e), powf(a.y, e), powf(a.z, e)); }
GBPT_HD V3 reflect(V3 d, V3 n) { return 2.0f * dot(d, n) * n - d; }

}  // namespace hd
}  // namespace gbpt
