// Internal layout of the 8-wide BVH shared by the host builder and the CUDA traversal kernels.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace gbpt {

// One 8-wide node: 80 bytes, read by the kernels as five 16-byte words.
//   word 0: origin p (x, y, z), then the per-axis scale exponents and the internal-child mask
//   word 1: child base index, triangle base index, 8 child meta bytes
//   words 2-4: per-child quantised box bounds, qlo/qhi per axis, 8 bytes each
// Child box on axis a = [p_a + qlo_a * 2^(e_a - 127), p_a + qhi_a * 2^(e_a - 127)].
// Meta byte of a child: 0 = empty slot; internal child = 0b001'11sss (24 + slot);
// leaf child = unary triangle count in bits 5-7 (0b001/0b011/0b111), triangle offset from the
// node's triangle base in bits 0-4.
struct alignas(16) WideNode
{
    float px, py, pz;
    uint8_t ex, ey, ez, imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo_x[8], qlo_y[8];
    uint8_t qlo_z[8], qhi_x[8];
    uint8_t qhi_y[8], qhi_z[8];
};
static_assert(sizeof(WideNode) == 80, "WideNode must be 80 bytes");

// Stored triangle: three float4 (vertex a + primitive index bits, vertex b, vertex c) = 48 bytes.
// The vertices themselves, not edges: the watertight test needs a shared vertex to be the same
// value in every triangle that uses it, and Moller-Trumbore forms its edges b - a, c - a at run
// time exactly as the reference does.
constexpr int kTriangleWords = 3;
constexpr int kMaxLeafTriangles = 3;
constexpr int kTraversalStack = 48;  // >= maximum wide depth accepted at build

struct HostBVH
{
    std::vector<WideNode> nodes;
    std::vector<float> tris;  // 12 floats per stored triangle
    int64_t n_input_triangles = 0;
    int64_t n_binary_nodes = 0;
    int wide_depth = 0;
    double build_seconds = 0.0;
};

// Defaults measured on the traversal benchmark (2.3M triangles, 16M rays; Mrays/s): 32 bins with
// binary leaves of 3 and the greedy collapse 1496, 64 bins with leaves of 2 (greedy) 1730, 64 bins
// with leaves of 1 and the cost-optimal collapse (which merges up to 3 triangles per wide-node
// leaf) 1805, 128 bins 1884; the last is also the fastest on the path-tracing workloads (Cornell
// box 7% faster than greedy leaves of 2) and needs the fewest nodes. max_leaf bounds the binary
// tree's leaves.
struct BuildParams
{
    int sah_bins = 128;
    int max_leaf = 1;
    int threads = 0;
};

// Returns an empty string on success, else an error message. 'too_deep' is set when the wide
// tree would exceed the traversal stack.
std::string build_wide_bvh(const int32_t* indices, const float* positions, int64_t n_vertices, int64_t n_tris,
                           const BuildParams& params, HostBVH& out, bool& too_deep);

}  // namespace gbpt
