/*
 * TEST INFRASTRUCTURE ONLY — the CPU oracle for ray/scene intersection.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library, and only
 * as a checker or as the timed CPU baseline. Nothing in the GPU product path calls it.
 *
 * It restates the reference's CPU intersection path in plain C++ over flat arrays:
 *   - Moller-Trumbore triangle test, same operation order and epsilon
 *       (src/Renderer/Triangle.h:20-63 of the reference);
 *   - the 7-plane k-DOP bounding volume and its slab test
 *       (src/Renderer/BoundingVolume.h:16-131, plane normals src/Renderer/BVH.cpp:12-20);
 *   - the octree build: triangles inserted one by one in index order, midpoint octants of the
 *       centroid of each triangle's bounding box, split when a leaf holds more than 8 triangles,
 *       depth limit 32, child boxes as the reference computes them (including the
 *       'min + (0, middle, 0)' offsets of children 2, 4 and 6)
 *       (src/Renderer/BVH.h:43-134, src/Renderer/BVH.cpp:23-65, src/Renderer/Triangle.cpp:8-11);
 *   - the near-first priority-queue traversal with its early exit and first-found tie rule
 *       (src/Renderer/BVH.h:136-223);
 *   - the self-hit filter on the last hit primitive (src/Device/functions/FilterFunction.h:37-45,
 *       alpha testing off);
 *   - the shadow-ray decision 'closest hit t < t_max - 1e-4' (src/Device/includes/Intersect.h:276-324):
 *       callers pass tmax = t_max - 1e-4f and this file tests t < tmax.
 * Built with -ffp-contract=off so that every float operation rounds like the reference's.
 *
 * Parity pin: tests/test_oracle_ref.py checks this restatement against the reference's own
 * BVH.cpp/Triangle.h compiled behind clean-room shims (oracle/_ref, built by oracle/Makefile).
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <queue>
#include <thread>
#include <vector>

namespace {

struct V3 { float x, y, z; };

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
// The reference's hippt::min/max are 'a < b ? a : b' / 'a > b ? a : b' (src/HostDeviceCommon/Math.h).
inline float fmin_ref(float a, float b) { return a < b ? a : b; }
inline float fmax_ref(float a, float b) { return a > b ? a : b; }
inline V3 vmin(V3 a, V3 b) { return v3(fmin_ref(a.x, b.x), fmin_ref(a.y, b.y), fmin_ref(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return v3(fmax_ref(a.x, b.x), fmax_ref(a.y, b.y), fmax_ref(a.z, b.z)); }

constexpr int kPlanes = 7;

struct PlaneSet
{
    V3 n[kPlanes];
    PlaneSet()
    {
        const float s = std::sqrt(3.0f) / 3;
        n[0] = v3(1, 0, 0);
        n[1] = v3(0, 1, 0);
        n[2] = v3(0, 0, 1);
        n[3] = v3(s, s, s);
        n[4] = v3(-s, s, s);
        n[5] = v3(-s, -s, s);
        n[6] = v3(s, -s, s);
    }
};
const PlaneSet& planes()
{
    static PlaneSet p;
    return p;
}

struct Tri { V3 a, b, c; };

// Moller-Trumbore as src/Renderer/Triangle.h:20-63: returns true and fills t,u,v on a hit.
inline bool mt_intersect(const Tri& tri, V3 org, V3 dir, float& t_out, float& u_out, float& v_out)
{
    const float EPS = 0.0000001f;
    V3 e1 = sub(tri.b, tri.a);
    V3 e2 = sub(tri.c, tri.a);
    V3 h = cross(dir, e2);
    float a = dot(e1, h);
    if (a > -EPS && a < EPS)
        return false;
    float f = 1.0f / a;
    V3 s = sub(org, tri.a);
    float u = f * dot(s, h);
    if (u < 0.0f || u > 1.0f)
        return false;
    V3 q = cross(s, e1);
    float v = f * dot(dir, q);
    if (v < 0.0f || u + v > 1.0f)
        return false;
    float t = f * dot(e2, q);
    if (t > EPS)
    {
        t_out = t;
        u_out = u;
        v_out = v;
        return true;
    }
    return false;
}

struct KDop
{
    float dn[kPlanes], df[kPlanes];
    KDop()
    {
        for (int i = 0; i < kPlanes; i++) { dn[i] = INFINITY; df[i] = -INFINITY; }
    }
    void extend(const KDop& o)
    {
        for (int i = 0; i < kPlanes; i++) { dn[i] = fmin_ref(dn[i], o.dn[i]); df[i] = fmax_ref(df[i], o.df[i]); }
    }
    void extend(const Tri& t)
    {
        KDop k;
        const V3* vs[3] = {&t.a, &t.b, &t.c};
        for (int i = 0; i < kPlanes; i++)
            for (int j = 0; j < 3; j++)
            {
                float d = dot(planes().n[i], *vs[j]);
                k.dn[i] = fmin_ref(k.dn[i], d);
                k.df[i] = fmax_ref(k.df[i], d);
            }
        extend(k);
    }
    // Slab test of src/Renderer/BoundingVolume.h:106-131 (divisions, swap on negative denominators).
    bool hit(float& t_near, const float* den, const float* num) const
    {
        t_near = -INFINITY;
        float t_far = INFINITY;
        for (int i = 0; i < kPlanes; i++)
        {
            float d = den[i];
            if (d == 0.0f)
                continue;
            float tn = (dn[i] - num[i]) / d;
            float tf = (df[i] - num[i]) / d;
            if (d < 0.0f)
                std::swap(tn, tf);
            t_near = fmax_ref(t_near, tn);
            t_far = fmin_ref(t_far, tf);
            if (t_far < t_near)
                return false;
        }
        return true;
    }
};

struct Node
{
    V3 mn, mx;
    bool leaf = true;
    int32_t child[8];
    std::vector<int32_t> tris;
    KDop vol;
};

struct Hit
{
    float t = -1.0f, u = 0.0f, v = 0.0f;
    int32_t prim = -1;
};

struct Octree
{
    std::vector<Tri> tris;
    std::vector<Node> nodes;  // nodes[0] is the root
    int max_depth = 32;
    int leaf_max = 8;

    int new_node(V3 mn, V3 mx)
    {
        nodes.emplace_back();
        nodes.back().mn = mn;
        nodes.back().mx = mx;
        return (int)nodes.size() - 1;
    }

    static V3 centroid(const Tri& t)
    {
        V3 lo = vmin(t.a, vmin(t.b, t.c));
        V3 hi = vmax(t.a, vmax(t.b, t.c));
        V3 s = add(lo, hi);
        return v3(s.x / 2, s.y / 2, s.z / 2);
    }

    // Child boxes exactly as the reference computes them (src/Renderer/BVH.h:71-84).
    void make_children(int ni)
    {
        V3 mn = nodes[ni].mn, mx = nodes[ni].mx;
        float mx_ = (mn.x + mx.x) / 2, my = (mn.y + mx.y) / 2, mz = (mn.z + mx.z) / 2;
        int c[8];
        c[0] = new_node(mn, v3(mx_, my, mz));
        c[1] = new_node(v3(mx_, mn.y, mn.z), v3(mx.x, my, mz));
        c[2] = new_node(add(mn, v3(0, my, 0)), v3(mx_, mx.y, mz));
        c[3] = new_node(v3(mx_, my, mn.z), v3(mx.x, mx.y, mz));
        c[4] = new_node(add(mn, v3(0, 0, mz)), v3(mx_, my, mx.z));
        c[5] = new_node(v3(mx_, mn.y, mz), v3(mx.x, my, mx.z));
        c[6] = new_node(add(mn, v3(0, my, mz)), v3(mx_, mx.y, mx.z));
        c[7] = new_node(v3(mx_, my, mz), mx);
        for (int i = 0; i < 8; i++) nodes[ni].child[i] = c[i];
    }

    void insert_into_children(int ni, int tri, int depth)
    {
        V3 c = centroid(tris[tri]);
        const Node& n = nodes[ni];
        float mx_ = (n.mn.x + n.mx.x) / 2, my = (n.mn.y + n.mx.y) / 2, mz = (n.mn.z + n.mx.z) / 2;
        int oct = 0;
        if (c.x > mx_) oct += 1;
        if (c.y > my) oct += 2;
        if (c.z > mz) oct += 4;
        insert(nodes[ni].child[oct], tri, depth + 1);
    }

    void insert(int ni, int tri, int depth)
    {
        bool depth_hit = max_depth != -1 && depth == max_depth;
        if (nodes[ni].leaf || depth_hit)
        {
            nodes[ni].tris.push_back(tri);
            if ((int)nodes[ni].tris.size() > leaf_max && !depth_hit)
            {
                nodes[ni].leaf = false;
                make_children(ni);
                std::vector<int32_t> moved;
                moved.swap(nodes[ni].tris);
                for (int t : moved) insert_into_children(ni, t, depth);
            }
        }
        else
            insert_into_children(ni, tri, depth);
    }

    const KDop& compute_volume(int ni)
    {
        if (nodes[ni].leaf)
        {
            for (int t : nodes[ni].tris) nodes[ni].vol.extend(tris[t]);
        }
        else
        {
            for (int i = 0; i < 8; i++)
            {
                KDop k = compute_volume(nodes[ni].child[i]);
                nodes[ni].vol.extend(k);
            }
        }
        return nodes[ni].vol;
    }

    void build()
    {
        V3 mn = v3(INFINITY, INFINITY, INFINITY), mx = v3(-INFINITY, -INFINITY, -INFINITY);
        for (const Tri& t : tris)
        {
            mn = vmin(mn, t.a); mn = vmin(mn, t.b); mn = vmin(mn, t.c);
            mx = vmax(mx, t.a); mx = vmax(mx, t.b); mx = vmax(mx, t.c);
        }
        nodes.clear();
        nodes.reserve(tris.size() / 2 + 16);
        new_node(mn, mx);
        for (int i = 0; i < (int)tris.size(); i++) insert(0, i, 0);
        compute_volume(0);
    }

    struct QE
    {
        int node;
        float t_near;
        bool operator>(const QE& o) const { return t_near > o.t_near; }
    };

    // src/Renderer/BVH.h:148-223, with the self-hit filter and minT check of the leaf loop.
    bool intersect_node(int ni, V3 org, V3 dir, float min_t, int last_prim, Hit& hit, float& t_near_out,
                        const float* den, const float* num) const
    {
        float ignored;
        if (!nodes[ni].vol.hit(ignored, den, num))
            return false;
        const Node& n = nodes[ni];
        if (n.leaf)
        {
            for (int ti : n.tris)
            {
                float t, u, v;
                if (mt_intersect(tris[ti], org, dir, t, u, v))
                {
                    if (t < min_t) continue;
                    if (ti == last_prim) continue;
                    if (t < hit.t || hit.t == -1)
                    {
                        hit.t = t; hit.u = u; hit.v = v; hit.prim = ti;
                    }
                }
            }
            t_near_out = hit.t;
            return t_near_out > 0;
        }
        std::priority_queue<QE, std::vector<QE>, std::greater<QE>> q;
        for (int i = 0; i < 8; i++)
        {
            float tn;
            if (nodes[n.child[i]].vol.hit(tn, den, num))
                q.push(QE{n.child[i], tn});
        }
        bool found = false;
        float closest = 100000000, dist = 100000000;
        while (!q.empty())
        {
            QE top = q.top();
            q.pop();
            if (intersect_node(top.node, org, dir, min_t, last_prim, hit, dist, den, num))
            {
                closest = std::min(closest, dist);
                found = true;
                if (q.empty() || closest < q.top().t_near)
                {
                    t_near_out = closest;
                    return true;
                }
            }
        }
        if (!found)
            return false;
        t_near_out = closest;
        return true;
    }

    Hit closest(V3 org, V3 dir, float min_t, int last_prim) const
    {
        float den[kPlanes], num[kPlanes];
        for (int i = 0; i < kPlanes; i++)
        {
            den[i] = dot(planes().n[i], dir);
            num[i] = dot(planes().n[i], org);
        }
        Hit h;
        float ignored;
        intersect_node(0, org, dir, min_t, last_prim, h, ignored, den, num);
        return h;
    }
};

Tri load_tri(const float* v, int64_t i)
{
    const float* p = v + 9 * i;
    return Tri{v3(p[0], p[1], p[2]), v3(p[3], p[4], p[5]), v3(p[6], p[7], p[8])};
}

template <typename F>
void parallel_for(int64_t n, int nthreads, F&& body)
{
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (nthreads == 1 || n < 1024)
    {
        for (int64_t i = 0; i < n; i++) body(i);
        return;
    }
    std::atomic<int64_t> next{0};
    const int64_t chunk = 1024;
    std::vector<std::thread> pool;
    for (int w = 0; w < nthreads; w++)
        pool.emplace_back([&]() {
            for (;;)
            {
                int64_t s = next.fetch_add(chunk);
                if (s >= n) break;
                int64_t e = std::min(n, s + chunk);
                for (int64_t i = s; i < e; i++) body(i);
            }
        });
    for (auto& t : pool) t.join();
}

} // namespace

extern "C" {

/* Triangle soup: tri_verts holds 9 floats per triangle (a, b, c). */
void* orc_octree_build(const float* tri_verts, int64_t n_tris, int max_depth, int leaf_max)
{
    Octree* o = new Octree();
    o->max_depth = max_depth;
    o->leaf_max = leaf_max;
    o->tris.resize(n_tris);
    for (int64_t i = 0; i < n_tris; i++) o->tris[i] = load_tri(tri_verts, i);
    o->build();
    return o;
}

void orc_octree_free(void* h) { delete static_cast<Octree*>(h); }

int64_t orc_octree_node_count(void* h) { return (int64_t) static_cast<Octree*>(h)->nodes.size(); }

/* Rays: origin_tmin and dir_tmax hold 4 floats per ray; last_prim one int per ray (-1 = none).
 * Hits: 4 words per ray (t, u, v as float; prim as int32, -1 on a miss with t = -1). The
 * closest-hit query ignores tmax, as the reference's CPU traversal does. */
void orc_octree_closest(void* h, const float* origin_tmin, const float* dir_tmax, const int32_t* last_prim,
                        int64_t n, float* hits, int nthreads)
{
    const Octree* o = static_cast<const Octree*>(h);
    parallel_for(n, nthreads, [&](int64_t i) {
        const float* a = origin_tmin + 4 * i;
        const float* d = dir_tmax + 4 * i;
        Hit r = o->closest(v3(a[0], a[1], a[2]), v3(d[0], d[1], d[2]), a[3], last_prim ? last_prim[i] : -1);
        float* out = hits + 4 * i;
        out[0] = r.t; out[1] = r.u; out[2] = r.v;
        std::memcpy(out + 3, &r.prim, 4);
    });
}

/* Scene accelerator for the path-tracing and ReSTIR oracles (an orc_octree_build handle over the
 * triangles their next calls pass; NULL: their exhaustive test). */
static void* g_scene_accel = nullptr;
void orc_set_scene_accel(void* octree) { g_scene_accel = octree; }
void* orc_scene_accel() { return g_scene_accel; }

/* One ray (origin o[3], direction d[3], minimum t 0): the closest hit's triangle (-1: none) and
 * its t. The path-tracing and ReSTIR oracles trace through this when a scene accelerator is set
 * (orc_set_scene_accel), e.g. for CPU baselines on scenes too large for their exhaustive test. */
int32_t orc_octree_closest_one(void* h, const float* o, const float* d, int32_t skip, float* t_out)
{
    const Octree* oc = static_cast<const Octree*>(h);
    Hit r = oc->closest(v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2]), 0.0f, skip);
    *t_out = r.t;
    return r.prim;
}

/* Shadow rays: occluded[i] = 1 iff the closest accepted hit has t < dir_tmax[4*i+3]. */
void orc_octree_occluded(void* h, const float* origin_tmin, const float* dir_tmax, const int32_t* last_prim,
                         int64_t n, uint8_t* occluded, int nthreads)
{
    const Octree* o = static_cast<const Octree*>(h);
    parallel_for(n, nthreads, [&](int64_t i) {
        const float* a = origin_tmin + 4 * i;
        const float* d = dir_tmax + 4 * i;
        Hit r = o->closest(v3(a[0], a[1], a[2]), v3(d[0], d[1], d[2]), a[3], last_prim ? last_prim[i] : -1);
        occluded[i] = (r.prim >= 0 && r.t < d[3]) ? 1 : 0;
    });
}

/* Exhaustive Moller-Trumbore closest hit over every triangle (small scenes). Ties on t keep the
 * lowest triangle index, which is the GPU kernels' tie rule. Honours tmin and tmax (t < tmax). */
void orc_brute_closest(const float* tri_verts, int64_t n_tris, const float* origin_tmin, const float* dir_tmax,
                       const int32_t* last_prim, int64_t n, float* hits, int nthreads)
{
    parallel_for(n, nthreads, [&](int64_t i) {
        const float* a = origin_tmin + 4 * i;
        const float* d = dir_tmax + 4 * i;
        V3 org = v3(a[0], a[1], a[2]), dir = v3(d[0], d[1], d[2]);
        int lp = last_prim ? last_prim[i] : -1;
        Hit best;
        for (int64_t k = 0; k < n_tris; k++)
        {
            float t, u, v;
            if (!mt_intersect(load_tri(tri_verts, k), org, dir, t, u, v)) continue;
            if (t < a[3] || !(t < d[3]) || k == lp) continue;
            if (best.prim < 0 || t < best.t)
            {
                best.t = t; best.u = u; best.v = v; best.prim = (int32_t)k;
            }
        }
        float* out = hits + 4 * i;
        out[0] = best.t; out[1] = best.u; out[2] = best.v;
        std::memcpy(out + 3, &best.prim, 4);
    });
}

/* One Moller-Trumbore test (tie/edge classification of mismatches). Returns 1 on a hit. */
int orc_mt_intersect(const float* tri9, const float* origin3, const float* dir3, float* tuv)
{
    Tri t = load_tri(tri9, 0);
    return mt_intersect(t, v3(origin3[0], origin3[1], origin3[2]), v3(dir3[0], dir3[1], dir3[2]), tuv[0], tuv[1], tuv[2]) ? 1 : 0;
}

} // extern "C"
