// The volume a path travels in: the reference's nested-dielectric interior stack (RayVolumeState,
// src/Device/includes/RayVolumeState.h:20-80, with NestedDielectricsInteriorStack,
// src/Device/includes/NestedDielectrics.h:119-258; Schmidt and Budge 2002, "Simple Nested
// Dielectrics in Ray Traced Images").
//
// Four entries of 32 bits: priority (4 bits) | topmost << 4 | odd parity << 5 | material << 6,
// entry 0 the air (material 0x3FFFFFF, priority 0). Every hit pushes its material: the parity of
// the material's entries says whether the hit enters or leaves it, the last entered material is
// the medium on the other side, and a hit on a lower-priority material inside a higher-priority
// one would be skipped (the priorities used here never allow it: a material without transmission
// has priority 15 and its entry is popped again by every continuation leaving it, a transmissive
// one 0). The continuation's BSDF sample pops what it leaves behind (vol_after_sample). The
// distance travelled inside a volume feeds Beer-Lambert absorption when the path refracts out
// (principled_beer_absorption, src/Device/includes/BSDFs/Principled.h:332-357).
//
// Per path slot the stack is 16 bytes (uint4) and the state 16 bytes (int4: incident material,
// outgoing material, position | inside << 8, distance bits). Every index below is a compile-time
// constant after unrolling, so the entries stay in registers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "principled.h"
#include "render_common.h"

namespace gbpt {

struct VolumeStack
{
    static constexpr uint32_t kAir = 0x3FFFFFFu;  // NestedDielectricsInteriorStack::MAX_MATERIAL_INDEX
    uint32_t e[4];
    int pos;
    int incident, outgoing;
    bool inside;
    float distance;

    static __device__ __forceinline__ uint32_t mat(uint32_t x) { return (x >> 6) & kAir; }
    static __device__ __forceinline__ bool topmost(uint32_t x) { return (x >> 4) & 1u; }
    static __device__ __forceinline__ bool odd(uint32_t x) { return (x >> 5) & 1u; }
    static __device__ __forceinline__ int prio(uint32_t x) { return (int)(x & 15u); }

    // RayVolumeState's constructor: every entry the air, odd parity, topmost, priority 0
    __device__ __forceinline__ void reset()
    {
#pragma unroll
        for (int i = 0; i < 4; i++) e[i] = (kAir << 6) | (1u << 5) | (1u << 4);
        pos = 0;
        incident = outgoing = -1;
        inside = false;
        distance = 0.0f;
    }

    __device__ __forceinline__ void load(const uint4* stack, const int4* state, int64_t slot)
    {
        const uint4 s = stack[slot];
        const int4 t = state[slot];
        e[0] = s.x;
        e[1] = s.y;
        e[2] = s.z;
        e[3] = s.w;
        incident = t.x;
        outgoing = t.y;
        pos = t.z & 0xFF;
        inside = (t.z >> 8) & 1;
        distance = __int_as_float(t.w);
    }

    __device__ __forceinline__ void store(uint4* stack, int4* state, int64_t slot) const
    {
        stack[slot] = make_uint4(e[0], e[1], e[2], e[3]);
        state[slot] = make_int4(incident, outgoing, pos | (inside ? 256 : 0), __float_as_int(distance));
    }

    // NestedDielectricsInteriorStack::push: returns true when the boundary would be skipped
    __device__ __forceinline__ bool push(int m, int priority)
    {
        if (pos == 3) return false;
        const uint32_t um = (uint32_t)m & kAir;
        int last = 0;  // the last entered material: topmost odd entry of another material
        int prev = -1; // the topmost entry of this material
#pragma unroll
        for (int i = 0; i < 4; i++)
        {
            if (i <= pos && mat(e[i]) != um && topmost(e[i]) && odd(e[i])) last = i;
            if (i <= pos && mat(e[i]) == um) prev = i;
        }
        bool par = true;
        uint32_t last_entry = e[0];
#pragma unroll
        for (int i = 0; i < 4; i++)
        {
            if (i == prev)
            {
                par = !odd(e[i]);
                e[i] &= ~(1u << 4);
            }
            if (i == last) last_entry = e[i];
        }
        inside = !par;
        pos++;
        const uint32_t entry = (um << 6) | ((par ? 1u : 0u) << 5) | (1u << 4) | ((uint32_t)priority & 15u);
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (i == pos) e[i] = entry;
        if (priority < prio(last_entry)) return true;
        incident = par ? (int)mat(last_entry) : m;
        outgoing = par ? m : (int)mat(last_entry);
        return false;
    }

    // NestedDielectricsInteriorStack::pop
    __device__ __forceinline__ void pop(bool in)
    {
        uint32_t top = 0;
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (i == pos) top = mat(e[i]);
        if (pos > 0) pos--;
        if (in)
        {
            int prev = -1;
#pragma unroll
            for (int i = 0; i < 4; i++)
                if (i <= pos && mat(e[i]) == top) prev = i;
            if (prev >= 0)
            {
#pragma unroll
                for (int i = 1; i < 4; i++)
                    if (i > prev && i <= pos) e[i - 1] = e[i];
            }
            if (pos > 0) pos--;
        }
        int k = -1;
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (i <= pos && mat(e[i]) == top) k = i;
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (i == k) e[i] |= 1u << 4;
    }
};

// The dielectric priority the reference's material packing gives a material (CPUMaterial::make_safe,
// src/HostDeviceCommon/Material/MaterialCPU.h:200-212, stored in an unsigned char): 255 without
// transmission, else the default 0
__device__ __forceinline__ int dielectric_priority(const gbpt_principled_material& m)
{
    return (m.specular_transmission == 0.0f && m.diffuse_transmission == 0.0f) ? 255 : 0;
}

__device__ __forceinline__ float volume_ior(const SceneView& s, int mat)
{
    return (mat < 0 || (uint32_t)mat == VolumeStack::kAir) ? 1.0f : s.pmats[mat].ior;
}

// The BSDF's view of the volume state at a hit: the media on both sides, whether the hit leaves
// the material, and the Beer-Lambert attenuation of the volume being left (1 when it is the air or
// its absorption colour is white)
__device__ __forceinline__ bsdf::Medium volume_medium(const SceneView& s, const VolumeStack& v)
{
    bsdf::Medium md;
    md.inside = v.inside;
    md.eta_incident = volume_ior(s, v.incident);
    md.eta_outgoing = volume_ior(s, v.outgoing);
    md.absorbing = false;
    md.beer = v3(1.0f);
    if (v.incident >= 0 && (uint32_t)v.incident != VolumeStack::kAir)
    {
        const gbpt_principled_material& a = s.pmats[v.incident];
        const V3 c = v3(a.absorption_color[0], a.absorption_color[1], a.absorption_color[2]);
        if (!(c.x == 1.0f && c.y == 1.0f && c.z == 1.0f))
        {
            const float d = fmaxf(v.distance, 1.0e-6f);
            md.absorbing = true;
            md.beer = v3(expf(logf(c.x) / a.absorption_at_distance * d), expf(logf(c.y) / a.absorption_at_distance * d),
                         expf(logf(c.z) / a.absorption_at_distance * d));
        }
    }
    return md;
}

// A hit: push its material; inside a volume the segment's length is travelled distance
// (trace_main_path_ray, src/Device/includes/Intersect.h:232-245)
__device__ __forceinline__ void volume_hit(VolumeStack& v, const gbpt_principled_material& pm, int mat, float t)
{
    v.push(mat, dielectric_priority(pm));
    if (v.inside) v.distance += t;
}

// The stack updates of a continuation sample (the BSDF sample that updates the ray's volume
// state): a reflective lobe pops (principled_bsdf_sample, Principled.h:1851-1857), so does a
// glass reflection or a thin-walled refraction (principled_glass_sample, :793, :821); the
// evaluation of the sampled direction then pops when it refracts out of a volume through the
// glass lobe (principled_glass_eval, :536-556, past its early exits) or the diffuse-transmission
// lobe (:844-860), and restarts the travelled distance.
__device__ __forceinline__ void volume_after_sample(const SceneView& s, VolumeStack& v, const bsdf::Material& m, V3 view,
                                                    V3 ns, V3 ng, V3 wi, int lobe)
{
    const bool through = lobe == GBPT_LOBE_GLASS_REFLECT || lobe == GBPT_LOBE_GLASS_REFRACT ||
                         lobe == GBPT_LOBE_DIFFUSE_TRANSMISSION;
    if (!through) v.pop(false);
    if (lobe == GBPT_LOBE_GLASS_REFLECT || (lobe == GBPT_LOBE_GLASS_REFRACT && m.thin_walled)) v.pop(false);
    if (dot(wi, ng) < 0.0f && !through) return;
    const bsdf::Lobes w = bsdf::lobe_weights(m, !v.inside);
    const float nov = dot(view, ns), nol = dot(wi, ns);
    const bool from_volume = v.incident >= 0 && (uint32_t)v.incident != VolumeStack::kAir;
    if (w.glass > 0.0f && fabsf(nol) >= 1.0e-8f && !(nol * nov > 0.0f))
    {
        float eta = volume_ior(s, v.outgoing) / volume_ior(s, v.incident);
        if (fabsf(eta - 1.0f) < 1.0e-5f) eta = 1.0f + 1.0e-5f;
        const float rough = bsdf::thin_walled_roughness(m.thin_walled, m.roughness, eta);
        V3 h;
        if (rough <= bsdf::kRoughnessClamp)
            h = ns;
        else if (m.thin_walled)
            h = normalize((wi - ns * (2.0f * nol)) + view);
        else
            h = normalize(wi * eta + view);
        if (dot(h, ns) < 0.0f) h = -h;
        if (!(dot(wi, h) * nol < 0.0f || dot(view, h) * nov < 0.0f))
        {
            if (m.thin_walled)
                v.pop(v.inside);
            else if (from_volume)
            {
                v.distance = 0.0f;
                if (v.inside) v.pop(v.inside);
            }
        }
    }
    if (w.diffuse_transmission > 0.0f && nol < 0.0f && !(nov * nol > 0.0f) && from_volume)
    {
        v.distance = 0.0f;
        if (v.inside) v.pop(v.inside);
    }
}

}  // namespace gbpt
