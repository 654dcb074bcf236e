// Host BVH builder: binned SAH binary tree, collapsed to 8-wide quantised nodes by the
// cost-optimal (dynamic-programming) collapse of the same paper, which also merges subtrees of up
// to 3 triangles into one leaf where that costs less.
//
// Replaces the reference's GPU BVH build through HIPRT (hiprtBuildGeometry in
// src/HIPRT-Orochi/HIPRTScene.h:87-150 of the reference, whose algorithm lives in the absent HIPRT
// submodule). The layout follows the compressed wide BVH of Ylitie, Karras and Laine,
// "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs" (HPG 2017):
// 8 children per node, 8-bit child boxes relative to a per-node origin and power-of-two scale,
// children placed in slots by ray octant so that traversal order is near-first.
#include "bvh.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <thread>

namespace gbpt {
namespace {

struct Box
{
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const float* l, const float* h)
    {
        for (int a = 0; a < 3; a++)
        {
            lo[a] = std::min(lo[a], l[a]);
            hi[a] = std::max(hi[a], h[a]);
        }
    }
    void grow(const Box& b) { grow(b.lo, b.hi); }
    float half_area() const
    {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0.0f)) return 0.0f;
        return dx * dy + dy * dz + dz * dx;
    }
};

struct BNode
{
    Box box;
    int32_t left = -1;  // right child = left + 1; -1 marks a leaf
    int32_t begin = 0;  // the subtree's triangles are idx[begin, begin + n_tris)
    int32_t count = 0;  // triangles of a binary leaf (0 for an internal node)
    int32_t n_tris = 0;
};

struct Builder
{
    const BuildParams& params;
    std::vector<float> plo, phi, pc;  // per primitive: box lo/hi and centroid, 3 floats each
    std::vector<int32_t> idx;         // primitive order (leaves index into it)
    std::vector<BNode> nodes;
    std::atomic<int32_t> next_node{1};
    std::atomic<int> live_threads{0};
    int max_threads = 1;

    explicit Builder(const BuildParams& p) : params(p) {}

    int32_t alloc_pair() { return next_node.fetch_add(2); }

    void build(int32_t ni, int32_t begin, int32_t end)
    {
        BNode& node = nodes[ni];
        Box box, cbox;
        for (int32_t i = begin; i < end; i++)
        {
            int32_t p = idx[i];
            box.grow(&plo[3 * p], &phi[3 * p]);
            cbox.grow(&pc[3 * p], &pc[3 * p]);
        }
        node.box = box;
        const int32_t count = end - begin;
        node.begin = begin;
        node.n_tris = count;
        if (count <= params.max_leaf)
        {
            node.begin = begin;
            node.count = count;
            node.left = -1;
            return;
        }

        // at most 4 bins per triangle of the node (at least 16): the bottom levels' binning cost
        // follows their size; measured: the same tree quality, build 1.41 -> 1.17 s (2.3M tris)
        const int B = std::min(params.sah_bins, std::max(16, 4 * count));
        int best_axis = -1, best_split = -1;
        float best_cost = INFINITY;
        std::vector<Box> bin_box(B);
        std::vector<int32_t> bin_cnt(B);
        std::vector<float> left_area(B), left_cnt(B);
        for (int a = 0; a < 3; a++)
        {
            float ext = cbox.hi[a] - cbox.lo[a];
            if (!(ext > 0.0f)) continue;
            float k = B / ext;
            std::fill(bin_box.begin(), bin_box.end(), Box());
            std::fill(bin_cnt.begin(), bin_cnt.end(), 0);
            for (int32_t i = begin; i < end; i++)
            {
                int32_t p = idx[i];
                int b = std::min(B - 1, std::max(0, (int)((pc[3 * p + a] - cbox.lo[a]) * k)));
                bin_box[b].grow(&plo[3 * p], &phi[3 * p]);
                bin_cnt[b]++;
            }
            Box acc;
            int32_t n = 0;
            for (int b = 0; b < B - 1; b++)
            {
                acc.grow(bin_box[b]);
                n += bin_cnt[b];
                left_area[b] = acc.half_area();
                left_cnt[b] = (float)n;
            }
            acc = Box();
            n = 0;
            for (int b = B - 1; b >= 1; b--)
            {
                acc.grow(bin_box[b]);
                n += bin_cnt[b];
                float lc = left_cnt[b - 1];
                if (lc <= 0.0f || n == 0) continue;
                float cost = left_area[b - 1] * lc + acc.half_area() * (float)n;
                if (cost < best_cost)
                {
                    best_cost = cost;
                    best_axis = a;
                    best_split = b;
                }
            }
        }

        int32_t mid;
        if (best_axis < 0)
        {
            mid = begin + count / 2;  // all centroids coincide: split the range in half
        }
        else
        {
            const int a = best_axis;
            const float k = B / (cbox.hi[a] - cbox.lo[a]);
            const float lo = cbox.lo[a];
            auto it = std::partition(idx.begin() + begin, idx.begin() + end, [&](int32_t p) {
                int b = std::min(B - 1, std::max(0, (int)((pc[3 * p + a] - lo) * k)));
                return b < best_split;
            });
            mid = (int32_t)(it - idx.begin());
            if (mid == begin || mid == end)
            {
                mid = begin + count / 2;
                std::nth_element(idx.begin() + begin, idx.begin() + mid, idx.begin() + end,
                                 [&](int32_t x, int32_t y) { return pc[3 * x + a] < pc[3 * y + a]; });
            }
        }

        int32_t l = alloc_pair();
        node.left = l;
        node.count = 0;
        if (count > 65536 && live_threads.load() < max_threads)
        {
            live_threads++;
            std::thread t([this, l, begin, mid]() {
                build(l, begin, mid);
                live_threads--;
            });
            build(l + 1, mid, end);
            t.join();
        }
        else
        {
            build(l, begin, mid);
            build(l + 1, mid, end);
        }
    }
};

// SAH weights of the wide collapse: a node visit against one triangle test. Measured on the
// traversal benchmark (binary leaves of 1 triangle, 64 bins; Mrays/s): 0.3 -> 1784, 0.6 -> 1805,
// 1.0 -> 1783 (Ylitie et al. use 0.3 with their triangle test).
constexpr float kNodeCost = 1.0f;
constexpr float kTriCost = 0.6f;

struct Child
{
    int32_t bnode;
    bool leaf;
};

// 2^e as a float, e in [-126, 127].
float pow2f(int e)
{
    uint32_t bits = (uint32_t)(e + 127) << 23;
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

}  // namespace

std::string build_wide_bvh(const int32_t* indices, const float* positions, int64_t n_vertices, int64_t n_tris,
                           const BuildParams& params, HostBVH& out, bool& too_deep)
{
    too_deep = false;
    auto t0 = std::chrono::steady_clock::now();
    if (n_tris < 0 || n_vertices < 0) return "negative sizes";
    if (n_tris > (int64_t)std::numeric_limits<int32_t>::max() / 4) return "too many triangles";
    if (params.max_leaf < 1 || params.max_leaf > kMaxLeafTriangles) return "max_leaf_size must be in 1..3";
    if (params.sah_bins < 2 || params.sah_bins > 256) return "sah_bins must be in 2..256";

    Builder b(params);
    b.max_threads = params.threads > 0 ? params.threads : (int)std::max(1u, std::thread::hardware_concurrency());
    b.plo.resize(3 * n_tris);
    b.phi.resize(3 * n_tris);
    b.pc.resize(3 * n_tris);
    b.idx.reserve(n_tris);
    for (int64_t t = 0; t < n_tris; t++)
    {
        const float* v[3];
        bool ok = true;
        for (int k = 0; k < 3; k++)
        {
            int32_t vi = indices[3 * t + k];
            if (vi < 0 || vi >= n_vertices) return "triangle " + std::to_string(t) + " has an out-of-range vertex index";
            v[k] = positions + 3 * (int64_t)vi;
            for (int a = 0; a < 3; a++) ok = ok && std::isfinite(v[k][a]);
        }
        if (!ok) continue;  // Moller-Trumbore never reports a hit on a non-finite triangle
        for (int a = 0; a < 3; a++)
        {
            float lo = std::min(v[0][a], std::min(v[1][a], v[2][a]));
            float hi = std::max(v[0][a], std::max(v[1][a], v[2][a]));
            b.plo[3 * t + a] = lo;
            b.phi[3 * t + a] = hi;
            b.pc[3 * t + a] = 0.5f * (lo + hi);
        }
        b.idx.push_back((int32_t)t);
    }
    const int32_t n_valid = (int32_t)b.idx.size();

    out = HostBVH();
    out.n_input_triangles = n_tris;

    if (n_valid == 0)
    {
        // Empty structure: one node with no children; every ray misses.
        WideNode root;
        std::memset(&root, 0, sizeof(root));
        root.ex = root.ey = root.ez = 127;
        out.nodes.push_back(root);
        out.wide_depth = 1;
        out.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return "";
    }

    b.nodes.resize(std::max<int64_t>(1, 2 * (int64_t)n_valid));
    b.build(0, 0, n_valid);
    out.n_binary_nodes = b.next_node.load();

    // ---- cost-optimal collapse to 8-wide nodes (Ylitie, Karras and Laine, HPG 2017, section 3):
    // cost[n][i-1] is the least SAH cost of the subtree under binary node n spread over at most i
    // slots of a wide node, where a slot holds a leaf of at most 3 triangles (area x kTriCost per
    // triangle) or a wide node (area x kNodeCost plus its own 8 slots), solved children first.
    const int32_t nb = (int32_t)out.n_binary_nodes;
    std::vector<std::array<float, 8>> cost(nb);
    std::vector<std::array<int8_t, 8>> split(nb);  // i = 1: 1 leaf / 0 wide node; i > 1: k (0: fewer slots)
    auto eval_node = [&](int32_t n) {
        const BNode& bn = b.nodes[n];
        const float area = bn.box.half_area();
        const float leaf = bn.n_tris <= kMaxLeafTriangles ? area * kTriCost * (float)bn.n_tris : INFINITY;
        if (bn.left < 0)
        {
            cost[n].fill(leaf);
            split[n].fill(0);
            split[n][0] = 1;
            return;
        }
        const auto& cl = cost[bn.left];
        const auto& cr = cost[bn.left + 1];
        float dist[8];
        int8_t arg[8];
        for (int i = 2; i <= 8; i++)
        {
            dist[i - 1] = INFINITY;
            arg[i - 1] = 0;
            for (int k = 1; k < i; k++)
            {
                const float c = cl[k - 1] + cr[i - k - 1];
                if (c < dist[i - 1])
                {
                    dist[i - 1] = c;
                    arg[i - 1] = (int8_t)k;
                }
            }
        }
        const float wide = area * kNodeCost + dist[7];
        cost[n][0] = std::min(leaf, wide);
        split[n][0] = leaf <= wide ? 1 : 0;
        for (int i = 2; i <= 8; i++)
        {
            if (dist[i - 1] < cost[n][i - 2])
            {
                cost[n][i - 1] = dist[i - 1];
                split[n][i - 1] = arg[i - 1];
            }
            else
            {
                cost[n][i - 1] = cost[n][i - 2];
                split[n][i - 1] = 0;
            }
        }
    };
    // children before parents; subtrees of more than 65536 triangles solve their two children on
    // separate threads (as the binary build does)
    std::atomic<int> dp_threads{1};
    std::function<void(int32_t)> solve = [&](int32_t n) {
        const BNode& bn = b.nodes[n];
        if (bn.left >= 0)
        {
            if (bn.n_tris > 65536 && dp_threads.load() < b.max_threads)
            {
                dp_threads++;
                std::thread t([&solve, &dp_threads, l = bn.left]() {
                    solve(l);
                    dp_threads--;
                });
                solve(bn.left + 1);
                t.join();
            }
            else
            {
                solve(bn.left);
                solve(bn.left + 1);
            }
        }
        eval_node(n);
    };
    solve(0);
    // the slots of the wide node of binary node n: its subtree spread over at most 8 slots
    auto gather = [&](int32_t n, Child* kids) {
        int nk = 0;
        struct Item
        {
            int32_t node;
            int slots;
        };
        Item stack[64];
        int sp = 0;
        const BNode& bn = b.nodes[n];
        // the wide node itself distributes its 8 slots over its two children
        int best_k = 1;
        float best = INFINITY;
        for (int k = 1; k < 8; k++)
        {
            const float c = cost[bn.left][k - 1] + cost[bn.left + 1][8 - k - 1];
            if (c < best)
            {
                best = c;
                best_k = k;
            }
        }
        stack[sp++] = {bn.left + 1, 8 - best_k};
        stack[sp++] = {bn.left, best_k};
        while (sp > 0)
        {
            Item it = stack[--sp];
            while (it.slots > 1 && split[it.node][it.slots - 1] == 0) it.slots--;
            if (it.slots == 1)
            {
                kids[nk++] = {it.node, split[it.node][0] == 1};
                continue;
            }
            const int k = split[it.node][it.slots - 1];
            const int32_t l = b.nodes[it.node].left;
            stack[sp++] = {l + 1, it.slots - k};
            stack[sp++] = {l, k};
        }
        return nk;
    };

    // ---- collapse to 8-wide, breadth first ----
    struct Pending
    {
        int32_t wide;
        int32_t bnode;
        int depth;
    };
    std::vector<Pending> queue;
    out.nodes.reserve(out.n_binary_nodes / 4 + 16);
    out.nodes.emplace_back();
    queue.push_back({0, 0, 1});
    int max_depth = 1;
    std::vector<int32_t> order_tris;
    order_tris.reserve(n_valid);

    for (size_t qi = 0; qi < queue.size(); qi++)
    {
        const Pending pend = queue[qi];
        max_depth = std::max(max_depth, pend.depth);
        const BNode& bn = b.nodes[pend.bnode];

        Child kids[8];
        int nk = 0;
        if (bn.left < 0 || (pend.bnode == 0 && split[0][0] == 1))
            kids[nk++] = {pend.bnode, true};  // the whole scene is one leaf
        else
            nk = gather(pend.bnode, kids);

        // Union box and octant slot assignment (greedy on the offset of each child's centre).
        Box ub;
        for (int i = 0; i < nk; i++) ub.grow(b.nodes[kids[i].bnode].box);
        double cen[3];
        for (int a = 0; a < 3; a++) cen[a] = 0.5 * ((double)ub.lo[a] + (double)ub.hi[a]);
        struct Score
        {
            double s;
            int child, slot;
        };
        Score scores[64];
        int ns = 0;
        for (int i = 0; i < nk; i++)
        {
            const Box& cb = b.nodes[kids[i].bnode].box;
            double off[3];
            for (int a = 0; a < 3; a++) off[a] = 0.5 * ((double)cb.lo[a] + (double)cb.hi[a]) - cen[a];
            for (int s = 0; s < 8; s++)
            {
                double d = ((s & 4) ? off[0] : -off[0]) + ((s & 2) ? off[1] : -off[1]) + ((s & 1) ? off[2] : -off[2]);
                scores[ns++] = {d, i, s};
            }
        }
        std::sort(scores, scores + ns, [](const Score& x, const Score& y) {
            if (x.s != y.s) return x.s > y.s;
            if (x.child != y.child) return x.child < y.child;
            return x.slot < y.slot;
        });
        int slot_of[8], child_in_slot[8];
        for (int i = 0; i < 8; i++) { slot_of[i] = -1; child_in_slot[i] = -1; }
        for (int k = 0; k < ns; k++)
        {
            const Score& sc = scores[k];
            if (slot_of[sc.child] >= 0 || child_in_slot[sc.slot] >= 0) continue;
            slot_of[sc.child] = sc.slot;
            child_in_slot[sc.slot] = sc.child;
        }

        WideNode wn;
        std::memset(&wn, 0, sizeof(wn));

        // Quantisation frame: origin rounded down below the (slightly padded) union box, per-axis
        // power-of-two scale with room for a one-step outward margin on every child bound.
        float p[3];
        float scale[3];
        for (int a = 0; a < 3; a++)
        {
            double L = ub.lo[a], H = ub.hi[a];
            double mag = std::max(std::max(std::fabs(L), std::fabs(H)), H - L);
            double pad = std::max(mag * std::ldexp(1.0, -22), 1e-30);
            float pf = (float)(L - pad);
            if ((double)pf > L - pad) pf = std::nextafter(pf, -INFINITY);
            double ext = (H + pad) - (double)pf;
            int e = (ext > 0.0) ? (int)std::ceil(std::log2(ext / 253.0)) : -100;
            while (std::ldexp(253.0, e) < ext) e++;
            e = std::max(-100, std::min(100, e));
            p[a] = pf;
            scale[a] = pow2f(e);
            (&wn.ex)[a] = (uint8_t)(e + 127);
        }
        wn.px = p[0];
        wn.py = p[1];
        wn.pz = p[2];

        uint8_t* qlo[3] = {wn.qlo_x, wn.qlo_y, wn.qlo_z};
        uint8_t* qhi[3] = {wn.qhi_x, wn.qhi_y, wn.qhi_z};
        wn.child_base = (uint32_t)out.nodes.size();
        wn.tri_base = (uint32_t)order_tris.size();
        uint32_t tri_off = 0;
        uint8_t imask = 0;
        for (int s = 0; s < 8; s++)
        {
            int ci = child_in_slot[s];
            if (ci < 0) continue;
            const BNode& cn = b.nodes[kids[ci].bnode];
            for (int a = 0; a < 3; a++)
            {
                double lo = std::floor(((double)cn.box.lo[a] - (double)p[a]) / (double)scale[a]) - 1.0;
                double hi = std::ceil(((double)cn.box.hi[a] - (double)p[a]) / (double)scale[a]) + 1.0;
                qlo[a][s] = (uint8_t)std::max(0.0, std::min(255.0, lo));
                qhi[a][s] = (uint8_t)std::max(0.0, std::min(255.0, hi));
            }
            if (kids[ci].leaf)
            {
                uint32_t cnt = (uint32_t)cn.n_tris;
                static const uint8_t unary[4] = {0, 1, 3, 7};
                wn.meta[s] = (uint8_t)((unary[cnt] << 5) | tri_off);
                for (int32_t k = 0; k < cn.n_tris; k++) order_tris.push_back(b.idx[cn.begin + k]);
                tri_off += cnt;
            }
            else
            {
                wn.meta[s] = (uint8_t)((1u << 5) | (24u + (uint32_t)s));
                imask |= (uint8_t)(1u << s);
                int32_t wi = (int32_t)out.nodes.size();
                out.nodes.emplace_back();
                queue.push_back({wi, kids[ci].bnode, pend.depth + 1});
            }
        }
        wn.imask = imask;
        out.nodes[pend.wide] = wn;
    }

    out.wide_depth = max_depth;
    if (max_depth >= kTraversalStack)
    {
        too_deep = true;
        return "8-wide BVH depth " + std::to_string(max_depth) + " exceeds the traversal stack (" +
               std::to_string(kTraversalStack) + ")";
    }

    // ---- triangle records in leaf order ----
    out.tris.resize(order_tris.size() * 12);
    for (size_t k = 0; k < order_tris.size(); k++)
    {
        int32_t t = order_tris[k];
        const float* va = positions + 3 * (int64_t)indices[3 * t + 0];
        const float* vb = positions + 3 * (int64_t)indices[3 * t + 1];
        const float* vc = positions + 3 * (int64_t)indices[3 * t + 2];
        float* r = &out.tris[12 * k];
        r[0] = va[0];
        r[1] = va[1];
        r[2] = va[2];
        std::memcpy(&r[3], &t, 4);
        for (int a = 0; a < 3; a++)
        {
            r[4 + a] = vb[a];
            r[8 + a] = vc[a];
        }
        r[7] = 0.0f;
        r[11] = 0.0f;
    }
    out.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return "";
}

}  // namespace gbpt
