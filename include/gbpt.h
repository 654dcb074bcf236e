/*
 * gbpt — GB300-native (sm_103a) render path: C ABI.
 *
 * Plain C types only (pointers, sizes, PODs): no CUDA, C++ or torch types cross this boundary.
 * Device pointers are CUdeviceptr-compatible addresses passed as void* / typed pointers; every
 * stream argument is a cudaStream_t passed as void* (NULL = the legacy default stream).
 * Every entry point returns a gbpt_status and never exits or traps; gbpt_last_error() returns a
 * thread-local message for the last failure on the calling thread.
 *
 * Each declaration cites the reference interface it replaces (file:line in
 * TomClabault/HIPRT-Path-Tracer).
 */
#ifndef GBPT_H
#define GBPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBPT_API __attribute__((visibility("default")))

/* Replaces the reference's abort-on-error macros OROCHI_CHECK_ERROR / HIPRT_CHECK_ERROR
 * (src/HIPRT-Orochi/HIPRTOrochiUtils.cpp:15-48), which log and exit(EXIT_FAILURE). */
typedef enum gbpt_status {
    GBPT_OK = 0,
    GBPT_ERROR_INVALID_ARG = 1,
    GBPT_ERROR_OOM = 2,
    GBPT_ERROR_CUDA = 3,
    GBPT_ERROR_TIMEOUT = 4,
    GBPT_ERROR_NAN = 5,
    GBPT_ERROR_UNSUPPORTED = 6,
    GBPT_ERROR_BVH_TOO_DEEP = 7
} gbpt_status;

GBPT_API const char* gbpt_status_string(gbpt_status s);
GBPT_API const char* gbpt_last_error(void);
GBPT_API int32_t gbpt_version(void);

/* ------------------------------------------------------------------------------------------
 * Acceleration structure.
 * Replaces HIPRTGeometry::build_bvh (src/HIPRT-Orochi/HIPRTScene.h:87-150), i.e.
 * hiprtCreateGeometry + hiprtBuildGeometry over a hiprtTriangleMeshPrimitive
 * {indices, vertices} (src/HIPRT-Orochi/HIPRTScene.h:152-155), and its OOM retry path
 * (:118-139) which here becomes GBPT_ERROR_OOM.
 * Build: binned SAH (sah_bins bins, leaves of at most max_leaf_size triangles), collapsed to
 * 8-wide nodes by a cost-optimal dynamic program (leaves of up to 3 triangles), with 8-bit
 * quantised child boxes (80 B per node), uploaded to the device.
 * ---------------------------------------------------------------------------------------- */
typedef struct gbpt_bvh gbpt_bvh;

typedef struct gbpt_bvh_params {
    int32_t sah_bins;      /* 0 -> 128 */
    int32_t max_leaf_size; /* 0 -> 1; 1..3: leaves of the binary SAH tree (the collapse to 8-wide
                              nodes merges subtrees of up to 3 triangles into one leaf where
                              that lowers the SAH cost) */
    int32_t num_threads;   /* host build threads; 0 -> hardware concurrency */
} gbpt_bvh_params;

typedef struct gbpt_bvh_stats {
    int64_t n_triangles;     /* triangles given */
    int64_t n_bvh_triangles; /* triangles referenced by leaves (non-finite ones are left out) */
    int64_t n_nodes;         /* 8-wide nodes */
    int64_t n_binary_nodes;  /* nodes of the binned-SAH binary tree before collapsing */
    int32_t wide_depth;      /* levels of 8-wide nodes (traversal stack bound) */
    int32_t node_bytes;      /* bytes per 8-wide node (80) */
    int32_t triangle_bytes;  /* bytes per stored triangle record (48) */
    int32_t reserved;
    int64_t device_bytes;    /* device memory held by the structure */
    double build_seconds;    /* host build time (binning + collapse + encode) */
    double upload_seconds;   /* host-to-device upload time */
} gbpt_bvh_stats;

/* indices: 3*n_triangles int32 (host); positions: 3*n_vertices float (host). */
GBPT_API gbpt_status gbpt_bvh_build(const int32_t* indices, const float* positions, int64_t n_vertices,
                                    int64_t n_triangles, const gbpt_bvh_params* params, gbpt_bvh** out);
GBPT_API gbpt_status gbpt_bvh_get_stats(const gbpt_bvh* bvh, gbpt_bvh_stats* out);
GBPT_API gbpt_status gbpt_bvh_destroy(gbpt_bvh* bvh);

/* ------------------------------------------------------------------------------------------
 * Ray queries over SoA ray queues (device memory, 16-byte aligned):
 *   origin_tmin[4*i..]  = origin.xyz, tmin   (hiprtRay.origin / .minT)
 *   dir_tmax[4*i..]     = direction.xyz, tmax (hiprtRay.direction / .maxT; a hit counts iff t < tmax)
 *   last_prim[i]        = primitive to ignore (self-hit filter; -1 = none)
 * Closest-hit output hits[4*i..] = t, u, v (float), prim (int32 bits); prim = -1 and t = -1 on a miss.
 *
 * gbpt_trace_closest replaces hiprtGeomTraversalClosest + the filter function as called by
 *   trace_main_path_ray (src/Device/includes/Intersect.h:200-270, traversal macros :22-69,
 *   filter src/Device/functions/FilterFunction.h:22-75 with alpha testing off) and, on the CPU,
 *   BVH::intersect (src/Renderer/BVH.h:132-223).
 * gbpt_trace_any replaces hiprtGeomTraversalAnyHit as called by evaluate_shadow_ray_occluded
 *   (src/Device/includes/Intersect.h:276-324): occluded[i] = 1 iff some accepted hit has t < tmax.
 *   Callers pass tmax = t_max - 1e-4f as the reference does.
 * The triangle test is Moller-Trumbore with the reference's operation order and epsilon
 * (src/Renderer/Triangle.h:20-63), evaluated without FMA contraction, so t/u/v are bit-identical
 * to the reference's CPU results; ties on t resolve to the lowest primitive index.
 * ---------------------------------------------------------------------------------------- */
GBPT_API gbpt_status gbpt_trace_closest(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                        const int32_t* last_prim, int64_t n_rays, float* hits, void* stream);
GBPT_API gbpt_status gbpt_trace_any(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                    const int32_t* last_prim, int64_t n_rays, uint8_t* occluded, void* stream);

/* Host-buffer variants (the end-to-end entry points): copy the rays host->device, trace, copy
 * the results device->host, and synchronise the stream before returning. Host buffers should be
 * pinned for full copy bandwidth. Scratch device buffers are allocated stream-ordered. */
GBPT_API gbpt_status gbpt_trace_closest_host(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                             const int32_t* last_prim, int64_t n_rays, float* hits, void* stream);
GBPT_API gbpt_status gbpt_trace_any_host(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                         const int32_t* last_prim, int64_t n_rays, uint8_t* occluded, void* stream);

/* Instrumented traversal (same kernels, counting build): adds to counters[0] the 8-wide nodes
 * visited and to counters[1] the triangles tested over the batch (device int64[2]). Used to
 * compute algorithmic bytes per ray for the roofline. any_hit selects the shadow-ray kernel. */
GBPT_API gbpt_status gbpt_trace_count(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                      const int32_t* last_prim, int64_t n_rays, int32_t any_hit,
                                      unsigned long long* counters, void* stream);

/* ------------------------------------------------------------------------------------------
 * Launch configuration and autotuning of the traversal kernels. Every configuration returns the
 * same results (the closest hit does not depend on the visiting order; any-hit returns the
 * occlusion bit); only the speed differs, and it depends on the ray batch's coherence.
 * ---------------------------------------------------------------------------------------- */
enum {
    GBPT_TRACE_KERNEL_PER_RAY = 1,    /* one thread per ray */
    GBPT_TRACE_KERNEL_PERSISTENT = 2, /* persistent warps: lane refill + triangle postponing */
    GBPT_TRACE_KERNEL_FETCH = 3       /* persistent warps: each lane fetches its next ray when done */
};
typedef struct gbpt_trace_config {
    int32_t kernel;          /* GBPT_TRACE_KERNEL_* */
    int32_t block;           /* threads per block: 32, 64, 128 or 256 */
    int32_t refill_below;    /* PERSISTENT: refill a warp when fewer lanes than this trace (1..32) */
    int32_t postpone_below;  /* PERSISTENT: triangle steps need this many lanes, else postponed (0..32) */
    int32_t blocks_per_sm;   /* PERSISTENT and FETCH: blocks per SM of the grid (1..64) */
    int32_t shared_stack;    /* traversal-stack entries per thread kept in shared memory (0, 8 or 16;
                                deeper entries in local memory); 0 in configurations written before */
    int32_t triangle_test;   /* GBPT_TRIANGLE_* [GBPT_TRIANGLE_MOLLER_TRUMBORE]; the autotuner keeps it */
    int32_t top_levels;      /* 1: each block first copies the 73 nodes nearest the root (the top three
                                levels of the 8-wide BVH, 5.8 KB) into shared memory and fetches them
                                from there; needs shared_stack 0 [0] */
    int32_t reserved[4];
} gbpt_trace_config;


/* Ray/triangle test of a traversal (gbpt_trace_config.triangle_test):
 *   GBPT_TRIANGLE_MOLLER_TRUMBORE: the reference's Moller-Trumbore (src/Renderer/Triangle.h:20-63)
 *     in its operation order, rounded step by step: hits bit-identical to the reference's CPU
 *     traversal (the parity mode); not watertight at shared edges;
 *   GBPT_TRIANGLE_WATERTIGHT: Woop, Benthin and Wald 2013 (JCGT 2:1): no ray passes between two
 *     triangles that share an edge (the production mode). t, u, v agree with Moller-Trumbore to
 *     float rounding away from edges. */
enum { GBPT_TRIANGLE_MOLLER_TRUMBORE = 0, GBPT_TRIANGLE_WATERTIGHT = 1 };

/* The configuration gbpt_trace_closest (any_hit = 0) / gbpt_trace_any (any_hit = 1) and their
 * host variants use for this BVH (defaults: persistent closest-hit, per-ray any-hit). */
GBPT_API gbpt_status gbpt_bvh_set_trace_config(gbpt_bvh* bvh, int32_t any_hit, const gbpt_trace_config* cfg);
GBPT_API gbpt_status gbpt_bvh_get_trace_config(const gbpt_bvh* bvh, int32_t any_hit, gbpt_trace_config* cfg);
/* Traversal with an explicit configuration (NULL: the BVH's). */
GBPT_API gbpt_status gbpt_trace_closest_cfg(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                            const int32_t* last_prim, int64_t n_rays, float* hits,
                                            const gbpt_trace_config* cfg, void* stream);
GBPT_API gbpt_status gbpt_trace_any_cfg(const gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                        const int32_t* last_prim, int64_t n_rays, uint8_t* occluded,
                                        const gbpt_trace_config* cfg, void* stream);
/* Autotuner: times candidate configurations (kernel, block size, shared-memory stack depth, refill
 * and postpone thresholds, resident blocks) on the given device ray batch with CUDA events, coordinate by coordinate from
 * the current best, each candidate run twice and its faster run kept; writes the fastest to *best
 * and its time per launch to *best_ms (either may be NULL). Results go to scratch memory. Stores
 * the result as the BVH's configuration for the class when store != 0. Synchronous. */
GBPT_API gbpt_status gbpt_trace_autotune(gbpt_bvh* bvh, const float* origin_tmin, const float* dir_tmax,
                                         const int32_t* last_prim, int64_t n_rays, int32_t any_hit, int32_t store,
                                         gbpt_trace_config* best, float* best_ms, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBPT_H */
