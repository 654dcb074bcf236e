/*
 * TEST INFRASTRUCTURE ONLY — the library's principled BSDF (hiprt-path-tracer_gb300/csrc/
 * principled.h, pinned to the reference's own principled_bsdf_eval / _sample by the BSDF golden
 * vectors) compiled for the host behind the oracles' BSDF callback interface, so that the path
 * tracing and ReSTIR oracles can run where the reference tree (and oracle/_ref/libref.so) is not
 * present. Used only by bench.py's CPU baselines of the principled workloads; every parity test
 * uses the reference's own BSDF (oracle/ref_bsdf.cpp).
 *
 * Callbacks (the signatures of ref_principled_eval_one / ref_principled_sample_one):
 *   material: 64 floats, the gbpt_principled_material record (include/gbpt_bsdf.h);
 *   query: 16 floats (view, shading normal, geometric normal, light, eta incident, eta outgoing,
 *     inside, incident lobe);
 *   eval -> out[4] = f rgb, pdf; sample(seed) -> out[8] = direction, f rgb, pdf, the Xorshift32
 *     state after sampling (bits), *lobe = the sampled lobe.
 */
#include <cstdint>
#include <cstring>

#include "principled.h"

namespace {
using namespace gbpt::bsdf;
using gbpt::hd::v3;
using gbpt::hd::V3;

Medium medium(const float* q)
{
    Medium md;
    md.eta_incident = q[12];
    md.eta_outgoing = q[13];
    md.inside = q[14] != 0.0f;
    return md;
}

// The material keeps a pointer to its record (for its extension lobes): the record lives in the
// caller's frame for as long as the material is used
gbpt_principled_material record(const float* w)
{
    gbpt_principled_material rec;
    static_assert(sizeof(gbpt_principled_material) == 64 * sizeof(float), "64-word material records");
    std::memcpy(&rec, w, sizeof(rec));
    return rec;
}
}  // namespace

extern "C" {

void host_principled_eval_one(const float* mat, const float* q, float* out)
{
    Query qq;
    qq.view = v3(q[0], q[1], q[2]);
    qq.ns = v3(q[3], q[4], q[5]);
    qq.ng = v3(q[6], q[7], q[8]);
    qq.light = v3(q[9], q[10], q[11]);
    float pdf = 0.0f;
    const gbpt_principled_material rec = record(mat);
    const V3 f = eval(load_material(rec), medium(q), false, qq, (int)q[15], pdf);
    out[0] = f.x;
    out[1] = f.y;
    out[2] = f.z;
    out[3] = pdf;
}

void host_principled_sample_one(const float* mat, const float* q, uint32_t seed, float* out, int32_t* lobe)
{
    Xorshift32 rng{seed};
    V3 dir = v3(0.0f, 0.0f, 0.0f);
    int lb = 0;
    float pdf = 0.0f;
    const gbpt_principled_material rec = record(mat);
    const V3 f = sample(load_material(rec), medium(q), false, v3(q[0], q[1], q[2]), v3(q[3], q[4], q[5]),
                        v3(q[6], q[7], q[8]), rng, dir, lb, pdf);
    out[0] = dir.x;
    out[1] = dir.y;
    out[2] = dir.z;
    out[3] = f.x;
    out[4] = f.y;
    out[5] = f.z;
    out[6] = pdf;
    std::memcpy(out + 7, &rng.state, 4);
    *lobe = lb;
}

}  // extern "C"
