/*
 * Clean-room stand-in for the HIPRT ray/hit types as the reference uses them on its CPU path:
 * hiprtRay{origin,minT,direction,maxT} and hiprtHit{primID,uv,normal,t,hasHit()}.
 * hiprtHit::t defaults to -1 because the reference's CPU BVH treats t == -1 as "no hit yet"
 * (src/Renderer/BVH.h:174 of the reference). Opaque handles are plain pointers. Test
 * infrastructure only.
 */
#ifndef GBPT_SHIM_HIPRT_TYPES_H
#define GBPT_SHIM_HIPRT_TYPES_H

#include <hiprt/hiprt_vec.h>
#include <cstdint>

constexpr uint32_t hiprtInvalidValue = ~0u;

struct hiprtRay
{
    hiprtFloat3 origin = {0.f, 0.f, 0.f};
    float minT = 0.0f;
    hiprtFloat3 direction = {0.f, 0.f, 0.f};
    float maxT = 1e38f;
};

struct hiprtHit
{
    uint32_t primID = hiprtInvalidValue;
    hiprtFloat2 uv = {0.f, 0.f};
    hiprtFloat3 normal = {0.f, 0.f, 0.f};
    float t = -1.0f;
    bool hasHit() const { return primID != hiprtInvalidValue; }
};

typedef void* hiprtGeometry;
typedef void* hiprtFuncTable;
struct hiprtGlobalStackBuffer { uint32_t stackSize; uint32_t stackCount; void* stackData; };
typedef void* hiprtContext;
typedef int hiprtTraversalHint;
constexpr int hiprtTraversalHintDefault = 0;

#endif
