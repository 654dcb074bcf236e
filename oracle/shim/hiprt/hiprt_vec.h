/*
 * Clean-room stand-in for the HIPRT vector types used by the reference's host-compiled device
 * code (HIPRT itself is an absent submodule). Written from the usage in
 * src/HostDeviceCommon/Math.h:9-40 of the reference: plain structs with x/y/z/w members,
 * make_* constructors and component-wise arithmetic. Test infrastructure only.
 */
#ifndef GBPT_SHIM_HIPRT_VEC_H
#define GBPT_SHIM_HIPRT_VEC_H

#include <cmath>
// The reference relies on these arriving transitively through the HIPRT headers.
#include <fstream>
#include <string>
#include <vector>
#include <algorithm>
#include <atomic>

// Device compilers (HIP, CUDA) declare float overloads of the math functions in the global
// namespace, so the reference's device code computes cos(float), sqrt(float), pow(float, float)
// in float on the GPU. A plain host build would pick the C double versions instead; these
// using-declarations make the host build compute in float like the reference's GPU path.
using std::acos;
using std::asin;
using std::atan2;
using std::cos;
using std::exp;
using std::fabs;
using std::log;
using std::pow;
using std::sin;
using std::sqrt;
using std::tan;

#ifndef HIPRT_HOST_DEVICE
#define HIPRT_HOST_DEVICE
#define HIPRT_DEVICE
#define HIPRT_HOST
#define HIPRT_INLINE inline
#endif

struct hiprtFloat2 { float x, y; };
struct hiprtFloat3 { float x, y, z; };
struct hiprtFloat4 { float x, y, z, w; };
struct hiprtInt2 { int x, y; };
struct hiprtInt3 { int x, y, z; };
struct hiprtInt4 { int x, y, z, w; };
struct hiprtUint2 { unsigned int x, y; };

inline hiprtFloat4 make_hiprtFloat4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline hiprtFloat4 make_hiprtFloat4(const hiprtFloat3& a, float w) { return {a.x, a.y, a.z, w}; }
// The reference's device compilers evaluate a call's arguments left to right, and some of its
// kernels draw random numbers inside one call (make_float2(rng() - 0.5f, rng() - 0.5f),
// src/Device/includes/ReSTIR/UtilsTemporal.h:65, UtilsSpatial.h:155,199). A host compiler may
// evaluate them in another order (g++ on x86-64 goes right to left), so the float vector
// constructors are macros over braced lists, whose elements C++ evaluates left to right.
struct hiprtFloat2Args
{
    hiprtFloat2 v;
    hiprtFloat2Args(float x, float y) : v{x, y} {}
    explicit hiprtFloat2Args(float s) : v{s, s} {}
};
struct hiprtFloat3Args
{
    hiprtFloat3 v;
    hiprtFloat3Args(float x, float y, float z) : v{x, y, z} {}
    explicit hiprtFloat3Args(float s) : v{s, s, s} {}
    explicit hiprtFloat3Args(const hiprtFloat4& a) : v{a.x, a.y, a.z} {}
};
#define make_hiprtFloat2(...) (hiprtFloat2Args{__VA_ARGS__}.v)
#define make_hiprtFloat3(...) (hiprtFloat3Args{__VA_ARGS__}.v)
inline hiprtInt2 make_hiprtInt2(int x, int y) { return {x, y}; }
inline hiprtInt3 make_hiprtInt3(int x, int y, int z) { return {x, y, z}; }
inline hiprtInt4 make_hiprtInt4(int x, int y, int z, int w) { return {x, y, z, w}; }
inline hiprtUint2 make_hiprtUint2(unsigned int x, unsigned int y) { return {x, y}; }

#define GBPT_SHIM_BINOPS(T, S, N)                                                               \
    inline T operator+(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = (&a.x)[i] + (&b.x)[i]; return r; } \
    inline T operator-(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = (&a.x)[i] - (&b.x)[i]; return r; } \
    inline T operator*(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = (&a.x)[i] * (&b.x)[i]; return r; } \
    inline T operator/(const T& a, const T& b) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = (&a.x)[i] / (&b.x)[i]; return r; } \
    inline T operator+(const T& a, S s) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = (&a.x)[i] + s; return r; }               \
    inline T operator-(const T& a, S s) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = (&a.x)[i] - s; return r; }               \
    inline T operator*(const T& a, S s) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = (&a.x)[i] * s; return r; }               \
    inline T operator/(const T& a, S s) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = (&a.x)[i] / s; return r; }               \
    inline T operator+(S s, const T& a) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = s + (&a.x)[i]; return r; }               \
    inline T operator-(S s, const T& a) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = s - (&a.x)[i]; return r; }               \
    inline T operator*(S s, const T& a) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = s * (&a.x)[i]; return r; }               \
    inline T operator/(S s, const T& a) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = s / (&a.x)[i]; return r; }               \
    inline T operator-(const T& a) { T r; for (int i = 0; i < N; i++) (&r.x)[i] = -(&a.x)[i]; return r; }                     \
    inline T& operator+=(T& a, const T& b) { a = a + b; return a; }                                                           \
    inline T& operator-=(T& a, const T& b) { a = a - b; return a; }                                                           \
    inline T& operator*=(T& a, const T& b) { a = a * b; return a; }                                                           \
    inline T& operator/=(T& a, const T& b) { a = a / b; return a; }                                                           \
    inline T& operator+=(T& a, S s) { a = a + s; return a; }                                                                  \
    inline T& operator-=(T& a, S s) { a = a - s; return a; }                                                                  \
    inline T& operator*=(T& a, S s) { a = a * s; return a; }                                                                  \
    inline T& operator/=(T& a, S s) { a = a / s; return a; }

GBPT_SHIM_BINOPS(hiprtFloat2, float, 2)
GBPT_SHIM_BINOPS(hiprtFloat3, float, 3)
GBPT_SHIM_BINOPS(hiprtFloat4, float, 4)
GBPT_SHIM_BINOPS(hiprtInt2, int, 2)
GBPT_SHIM_BINOPS(hiprtInt3, int, 3)
GBPT_SHIM_BINOPS(hiprtInt4, int, 4)
#undef GBPT_SHIM_BINOPS

#endif
