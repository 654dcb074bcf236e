// TEST INFRASTRUCTURE ONLY — host build of the shared principled BSDF
// (hiprt-path-tracer_gb300/csrc/principled.h) so that CPU-only test runs check it against the
// golden vectors of the reference's own BSDF before any GPU run; the GPU tests then check the
// CUDA build against the same vectors. Same material and query layouts as include/gbpt_bsdf.h.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "principled.h"

namespace {
using namespace gbpt::bsdf;
using gbpt::hd::v3;
using gbpt::hd::V3;

void load(const gbpt_bsdf_query& s, Query& q, Medium& md)
{
    q.view = v3(s.view[0], s.view[1], s.view[2]);
    q.ns = v3(s.shading_normal[0], s.shading_normal[1], s.shading_normal[2]);
    q.ng = v3(s.geometric_normal[0], s.geometric_normal[1], s.geometric_normal[2]);
    q.light = v3(s.to_light[0], s.to_light[1], s.to_light[2]);
    md.eta_incident = s.eta_incident;
    md.eta_outgoing = s.eta_outgoing;
    md.inside = s.inside != 0;
    md.wavelength = std::fabs(s.wavelength);
}
}  // namespace

extern "C" {

void emu_bsdf_eval(const gbpt_principled_material* mats, const int32_t* mi, const gbpt_bsdf_query* qs, int64_t n,
                   int height_correlated, float* out)
{
    for (int64_t i = 0; i < n; i++)
    {
        Query q;
        Medium md;
        load(qs[i], q, md);
        float pdf;
        const V3 f = eval(load_material(mats[mi[i]]), md, height_correlated != 0, q, qs[i].incident_lobe, pdf);
        out[4 * i] = f.x;
        out[4 * i + 1] = f.y;
        out[4 * i + 2] = f.z;
        out[4 * i + 3] = pdf;
    }
}

void emu_bsdf_sample(const gbpt_principled_material* mats, const int32_t* mi, const gbpt_bsdf_query* qs,
                     const uint32_t* seeds, int64_t n, int height_correlated, float* out, int32_t* lobes,
                     uint32_t* rng_out)
{
    for (int64_t i = 0; i < n; i++)
    {
        Query q;
        Medium md;
        load(qs[i], q, md);
        Xorshift32 rng{seeds[i]};
        V3 dir = v3(0.0f);
        int lobe = 0;
        float pdf;
        const V3 f = sample(load_material(mats[mi[i]]), md, height_correlated != 0, q.view, q.ns, q.ng, rng, dir, lobe, pdf);
        float* o = out + 8 * i;
        o[0] = dir.x;
        o[1] = dir.y;
        o[2] = dir.z;
        o[3] = f.x;
        o[4] = f.y;
        o[5] = f.z;
        o[6] = pdf;
        o[7] = 0.0f;
        lobes[i] = lobe;
        rng_out[i] = rng.state;
    }
}

}  // extern "C"
