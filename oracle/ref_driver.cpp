// Batch driver around the reference implementation.  TEST INFRASTRUCTURE ONLY.
//
// oracle/Makefile compiles this file together with the reference's own library
// sources (src/library/{storage,raytracing,utility,base,geometry}.cpp, read in
// place from the reference checkout, never copied) into oracle/_ref/libcbq_ref.so.
// It exposes a small C ABI so the Python tests can
//   - build volumes through the reference's Volume::setVoxel + bake
//     (src/library/storage.cpp:396-437, 387-394),
//   - load/save the reference's .dag format (storage.cpp:505-542),
//   - run the reference's intersectVolume (raytracing.cpp:397-478) and
//     traceRayRef (raytracing.cpp:521-535) over batches of rays on all cores.
// The outputs are the checker for the oracle restatement and for the CUDA path.
#include "raytracing.h"
#include "storage.h"
#include "utility.h"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <unistd.h>
#include <vector>

using namespace Cubiquity;

namespace {

int32_t sat_f2i(float f)
{
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f < -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}

// The integer hit voxel (a field the reference lacks), defined identically on
// every side: floor(position - 0.5f * normal + 0.5f), one rounding per step.
void hit_voxel(const float p[3], const float n[3], int32_t v[3])
{
    for (int i = 0; i < 3; i++) {
        volatile float half = 0.5f * n[i];
        volatile float a = p[i] - half;
        volatile float b = a + 0.5f;
        v[i] = sat_f2i(std::floor((float)b));
    }
}

template <typename F>
void parallel_for(uint64_t n, int nthreads, F&& body)
{
    if (nthreads <= 0) nthreads = (int)std::thread::hardware_concurrency();
    if (nthreads <= 0) nthreads = 1;
    std::atomic<uint64_t> next{0};
    const uint64_t chunk = 1024;
    auto work = [&]() {
        for (;;) {
            uint64_t b = next.fetch_add(chunk);
            if (b >= n) break;
            uint64_t e = std::min(n, b + chunk);
            for (uint64_t i = b; i < e; i++) body(i);
        }
    };
    if (nthreads == 1) { work(); return; }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) th.emplace_back(work);
    for (auto& t : th) t.join();
}

} // namespace

extern "C" {

void* ref_volume_new() { return new Volume(); }

void ref_volume_free(void* v) { delete static_cast<Volume*>(v); }

int ref_volume_set_voxels(void* v, const int32_t* xyz, const uint8_t* mat, uint64_t n)
{
    Volume* vol = static_cast<Volume*>(v);
    for (uint64_t i = 0; i < n; i++) vol->setVoxel(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], mat[i]);
    return 0;
}

void ref_volume_fill(void* v, uint8_t m) { static_cast<Volume*>(v)->fill(m); }

void ref_volume_bake(void* v) { static_cast<Volume*>(v)->bake(); }

uint32_t ref_volume_root(void* v) { return Internals::getRootNodeIndex(*static_cast<Volume*>(v)); }

uint64_t ref_volume_node_count(void* v)
{
    return Internals::getNodes(*static_cast<Volume*>(v)).unsharedNodesEnd();
}

int ref_volume_copy_nodes(void* v, uint32_t* dst, uint64_t cap_nodes)
{
    const Internals::NodeStore& ns = Internals::getNodes(*static_cast<Volume*>(v));
    const uint64_t count = ns.unsharedNodesEnd();
    if (count > cap_nodes) return -1;
    std::memcpy(dst, ns.rawBytesPtr(), count * 32u);
    return 0;
}

uint8_t ref_volume_voxel(void* v, int32_t x, int32_t y, int32_t z)
{
    return static_cast<Volume*>(v)->voxel(x, y, z);
}

int ref_volume_load(const char* path, void** out)
{
    Volume* vol = new Volume();
    if (!vol->load(path)) { delete vol; return -1; }
    *out = vol;
    return 0;
}

int ref_volume_save(void* v, const char* path)
{
    static_cast<Volume*>(v)->save(path);
    return 0;
}

// Builds a reference Volume holding exactly the given node array by writing it
// to a temporary .dag file and reading it back with Volume::load.
int ref_volume_from_nodes(const uint32_t* nodes, uint64_t node_count, uint32_t root, void** out)
{
    if (node_count < Internals::MaterialCount) return -1;
    char tmpl[] = "/tmp/cbq_ref_XXXXXX";
    int fd = mkstemp(tmpl);
    if (fd < 0) return -2;
    FILE* f = fdopen(fd, "wb");
    const uint32_t internal = (uint32_t)(node_count - Internals::MaterialCount);
    fwrite(&root, 4, 1, f);
    fwrite(&internal, 4, 1, f);
    fwrite(nodes + 8u * Internals::MaterialCount, 32, internal, f);
    fclose(f);
    int rc = ref_volume_load(tmpl, out);
    unlink(tmpl);
    return rc;
}

int ref_find_subdags(void* v, SubDAG* out)
{
    Volume* vol = static_cast<Volume*>(v);
    SubDAGArray a = findSubDAGs(Internals::getNodes(*vol), Internals::getRootNodeIndex(*vol));
    for (int i = 0; i < 8; i++) out[i] = a[i];
    return 0;
}

// intersectVolume over a batch.  orig4/dir4 hold 4 floats per ray; the fourth is
// ignored (the reference has no tmax).  Any output pointer may be null.
int ref_intersect_batch(void* v, const SubDAG* sd, const float* o4, const float* d4, uint64_t n,
                        int compute_surface, float max_footprint, uint8_t* hit, double* distance,
                        uint32_t* material, float* position, float* normal, int32_t* voxel,
                        int nthreads)
{
    const Volume& vol = *static_cast<Volume*>(v);
    SubDAGArray subdags;
    for (int i = 0; i < 8; i++) subdags[i] = sd[i];
    parallel_for(n, nthreads, [&](uint64_t i) {
        RayVolumeIntersection r = intersectVolume(vol, subdags, o4[4 * i], o4[4 * i + 1], o4[4 * i + 2],
                                                  d4[4 * i], d4[4 * i + 1], d4[4 * i + 2],
                                                  compute_surface != 0, max_footprint);
        if (hit) hit[i] = r.hit ? 1 : 0;
        if (distance) distance[i] = r.distance;
        if (material) material[i] = r.material;
        float p[3] = { r.position.x, r.position.y, r.position.z };
        float nn[3] = { r.normal.x, r.normal.y, r.normal.z };
        if (position) { position[3 * i] = p[0]; position[3 * i + 1] = p[1]; position[3 * i + 2] = p[2]; }
        if (normal) { normal[3 * i] = nn[0]; normal[3 * i + 1] = nn[1]; normal[3 * i + 2] = nn[2]; }
        if (voxel) {
            int32_t vv[3] = { 0, 0, 0 };
            if (r.hit) hit_voxel(p, nn, vv);
            voxel[3 * i] = vv[0]; voxel[3 * i + 1] = vv[1]; voxel[3 * i + 2] = vv[2];
        }
    });
    return 0;
}

// traceRayRef (the reference's brute-force tracer) over a batch.
int ref_trace_ray_ref_batch(void* v, const float* o4, const float* d4, uint64_t n, uint8_t* hit,
                            double* distance, uint32_t* material, int nthreads)
{
    Volume& vol = *static_cast<Volume*>(v);
    parallel_for(n, nthreads, [&](uint64_t i) {
        RayVolumeIntersection r = traceRayRef(vol, o4[4 * i], o4[4 * i + 1], o4[4 * i + 2],
                                              d4[4 * i], d4[4 * i + 1], d4[4 * i + 2]);
        if (hit) hit[i] = r.hit ? 1 : 0;
        if (distance) distance[i] = r.distance;
        if (material) material[i] = r.material;
    });
    return 0;
}

} // extern "C"
