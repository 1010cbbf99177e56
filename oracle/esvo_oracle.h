/*
 * CPU oracle for the sparse-voxel-DAG ray traversal.  TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of Cubiquity's ESVO ray cast over its flat node
 * store.  It exists so that tests, the smoke check and the CPU-baseline leg of
 * the benchmark can check the CUDA path against an independent implementation
 * on the same bytes.  The product library never links, loads or calls it.
 *
 * Parity of this restatement with the reference itself is pinned by
 *   - tests/golden/ fixtures: outputs produced by the reference's own intersectVolume
 *     (src/library/raytracing.cpp, compiled by oracle/Makefile into oracle/_ref)
 *     on seeded scenes built through the reference's Volume::setVoxel + bake;
 *   - tests/test_oracle_vs_ref.py, which runs both side by side wherever the
 *     reference sources are available.
 *
 * Node layout (src/library/storage.h:62, storage.cpp:110-122): node i occupies
 * u32 words [8i, 8i+8).  Slots 0..255 are material nodes whose eight children
 * all equal their own index.  A child value of 0 is empty, 1..255 a uniform
 * material, >= 256 an internal node.
 */
#ifndef CBQ_ESVO_ORACLE_H
#define CBQ_ESVO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same 32-byte layout as the reference's SubDAG (src/library/raytracing.h:57-65). */
typedef struct orc_subdag {
    int32_t  lower[3];
    int32_t  height;
    uint32_t pad0;
    uint32_t node;
    uint32_t pad1, pad2;
} orc_subdag;

/* Per-ray outputs (any pointer may be NULL).  position/normal/voxel hold 3
 * values per ray, interleaved x,y,z. */
typedef struct orc_hits {
    uint8_t*  hit;
    float*    distance;
    uint32_t* material;
    float*    position;
    float*    normal;
    int32_t*  voxel;
    uint8_t*  status;
} orc_hits;

/* Per-ray status codes (shared with the CUDA path). */
#define ORC_RAY_OK          0u
#define ORC_RAY_ITER_LIMIT  1u   /* iteration cap reached; result reported as a miss */
#define ORC_RAY_STUCK       2u   /* a step that moved nowhere (NaN slab); reported as a miss */

#define ORC_MAX_ITERATIONS  (1u << 17)

/* findSubDAGs (src/library/raytracing.cpp:43-97).  Returns 0 on success, a
 * negative value if a node index is out of range. */
int orc_find_subdags(const uint32_t* nodes, uint64_t node_count, uint32_t root,
                     orc_subdag out[8]);

/* intersectVolume (src/library/raytracing.cpp:397-478) over a batch of rays.
 * orig4/dir4: 4 floats per ray (x, y, z, tmax|pad).  use_tmax != 0 turns a hit
 * with distance > tmax into a miss (post-filter).  nthreads <= 0 uses all
 * online CPUs.  Returns 0 on success. */
int orc_intersect_batch(const uint32_t* nodes, uint64_t node_count,
                        const orc_subdag subdags[8],
                        const float* orig4, const float* dir4, uint64_t n,
                        int compute_surface, float max_footprint, int use_tmax,
                        const orc_hits* out, int nthreads);

/* As orc_intersect_batch; with unwritten_slot_is_start_node != 0 a descent-
 * stack slot that was never written reads as the walk's start node instead of
 * node 0.  The reference leaves those slots uninitialised, so a ray whose
 * result changes between the two settings depends on undefined values there;
 * tests use this to identify and list such rays. */
int orc_intersect_batch_ex(const uint32_t* nodes, uint64_t node_count,
                           const orc_subdag subdags[8],
                           const float* orig4, const float* dir4, uint64_t n,
                           int compute_surface, float max_footprint, int use_tmax,
                           const orc_hits* out, int nthreads, int unwritten_slot_is_start_node);

/* Counts the node fetches (dependent child loads) each ray performs. */
int orc_count_fetches(const uint32_t* nodes, uint64_t node_count,
                      const orc_subdag subdags[8],
                      const float* orig4, const float* dir4, uint64_t n,
                      int compute_surface, float max_footprint,
                      uint32_t* fetches_out, int nthreads);

/* Double-precision brute-force oracle: the nearest non-empty material leaf
 * whose exact box [v-0.5, v+0.5] the ray enters with exit > 0, in the spirit
 * of traceRayRef (src/library/raytracing.cpp:480-535) but with exact integer
 * node bounds and a double slab test throughout.  distance is double. */
int orc_trace_fp64_batch(const uint32_t* nodes, uint64_t node_count,
                         const orc_subdag subdags[8],
                         const float* orig4, const float* dir4, uint64_t n,
                         uint8_t* hit, double* distance, uint32_t* material,
                         int nthreads);

/* The integer hit voxel shared by both sides:
 * voxel = floor(position - 0.5f*normal + 0.5f), no contraction, saturating. */
void orc_hit_voxel(const float p[3], const float nrm[3], int32_t v[3]);

#ifdef __cplusplus
}
#endif

#endif
