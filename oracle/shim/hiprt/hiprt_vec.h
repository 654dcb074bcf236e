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

inline hiprtFloat2 make_hiprtFloat2(float x, float y) { return {x, y}; }
inline hiprtFloat2 make_hiprtFloat2(float s) { return {s, s}; }
inline hiprtFloat3 make_hiprtFloat3(float x, float y, float z) { return {x, y, z}; }
inline hiprtFloat3 make_hiprtFloat3(float s) { return {s, s, s}; }
inline hiprtFloat3 make_hiprtFloat3(const hiprtFloat4& a) { return {a.x, a.y, a.z}; }
inline hiprtFloat4 make_hiprtFloat4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline hiprtFloat4 make_hiprtFloat4(const hiprtFloat3& a, float w) { return {a.x, a.y, a.z, w}; }
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
