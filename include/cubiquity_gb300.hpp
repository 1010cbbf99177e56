// C++ drop-in shim over the C ABI of cubiquity_gb300.h, header-only.
//
// Mirrors the reference's ray-cast interface (src/library/raytracing.h:48-81)
// so that a caller of Cubiquity::intersectVolume can switch to the GPU by
// changing the namespace and the volume argument:
//
//   Cubiquity::SubDAGArray subDAGs = Cubiquity::findSubDAGs(nodes, root);      // reference
//   Cubiquity::RayVolumeIntersection r = Cubiquity::intersectVolume(volume, subDAGs, ox, oy, oz,
//                                                                    dx, dy, dz, true);
// becomes
//   cbq::Volume gpu(nodes_ptr, node_count, root);        // uploads once (SSBO-0 equivalent)
//   cbq::RayVolumeIntersection r = cbq::intersectVolume(gpu, gpu.subDAGs(), ox, oy, oz, dx, dy, dz, true);
//
// Both of the reference's overloads are here (six floats, raytracing.h:72-75;
// Ray3f, raytracing.h:77).  The SubDAGs passed must be the volume's own (those
// of findSubDAGs on the same nodes and root); others raise cbq::Error.
//
// The single-ray overload exists for API compatibility (collision picking,
// viewer.cpp:152-163); throughput callers use intersectVolumes() on batches.
// Errors surface as cbq::Error exceptions on the C++ side only; the C ABI below
// never throws.
#pragma once

#include "cubiquity_gb300.h"

#include <array>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace cbq {

struct vec3 {
    float x, y, z;
};

// The reference's Ray3f (geometry.h:229-250, Ray3<vec3f>): origin then
// direction, 24 bytes.
struct Ray3f {
    vec3 mOrigin;
    vec3 mDir;
    Ray3f() = default;
    Ray3f(const vec3& origin, const vec3& dir) : mOrigin(origin), mDir(dir) {}
};
static_assert(sizeof(Ray3f) == 24, "layout must match the reference");

// Byte layout identical to the reference's RayVolumeIntersection (48 bytes:
// bool hit @0, double distance @8, uint material @16, vec3 position @20,
// vec3 normal @32), so results can be handed to code compiled against it.
struct RayVolumeIntersection {
    bool hit;
    double distance;
    unsigned int material;
    vec3 position;
    vec3 normal;
};
static_assert(sizeof(RayVolumeIntersection) == 48, "layout must match the reference");
static_assert(offsetof(RayVolumeIntersection, distance) == 8, "layout must match the reference");
static_assert(offsetof(RayVolumeIntersection, material) == 16, "layout must match the reference");
static_assert(offsetof(RayVolumeIntersection, position) == 20, "layout must match the reference");
static_assert(offsetof(RayVolumeIntersection, normal) == 32, "layout must match the reference");

using SubDAG = cbq_subdag;
using SubDAGArray = std::array<SubDAG, 8>;

constexpr float MAX_FOOTPRINT_DISABLED = CBQ_MAX_FOOTPRINT_DISABLED;

struct Error : std::runtime_error {
    cbq_status status;
    Error(cbq_status s, const char* what) : std::runtime_error(std::string(what) + ": " + cbq_status_string(s)), status(s) {}
};

inline void check(cbq_status s, const char* what)
{
    if (s != CBQ_OK) throw Error(s, what);
}

// findSubDAGs (raytracing.h:69) on a host node array.
inline SubDAGArray findSubDAGs(const uint32_t* nodes, uint64_t node_count, uint32_t root)
{
    SubDAGArray a;
    check(cbq_find_subdags(nodes, node_count, root, a.data()), "findSubDAGs");
    return a;
}

// A device-resident volume: owns the cbq_dag handle.
class Volume {
public:
    Volume(const uint32_t* nodes, uint64_t node_count, uint32_t root)
    {
        check(cbq_dag_create(nodes, node_count, root, &dag_), "cbq_dag_create");
        cbq_dag_info info;
        check(cbq_dag_get_info(dag_, &info), "cbq_dag_get_info");
        for (int i = 0; i < 8; i++) subdags_[i] = info.subdags[i];
    }
    ~Volume() { if (dag_) cbq_dag_destroy(dag_); }
    Volume(const Volume&) = delete;
    Volume& operator=(const Volume&) = delete;

    const cbq_dag* handle() const { return dag_; }
    const SubDAGArray& subDAGs() const { return subdags_; }

private:
    cbq_dag* dag_ = nullptr;
    SubDAGArray subdags_;
};

// Batched intersectVolume over host arrays.  The SubDAGs are the volume's own
// (a cbq_dag computes them at creation, as the reference's callers do after
// each edit, pathtracing_demo.cpp:335-338).
inline void intersectVolumes(const Volume& volume, const float* origins_xyz, const float* dirs_xyz, size_t n,
                             bool computeSurfaceProperties, float maxFootprint, RayVolumeIntersection* out)
{
    std::vector<float> o(4 * n), d(4 * n);
    for (size_t i = 0; i < n; i++) {
        for (int a = 0; a < 3; a++) {
            o[4 * i + a] = origins_xyz[3 * i + a];
            d[4 * i + a] = dirs_xyz[3 * i + a];
        }
        o[4 * i + 3] = 0.0f;
        d[4 * i + 3] = 0.0f;
    }
    std::vector<uint8_t> hit(n);
    std::vector<float> dist(n), pos(3 * n), nrm(3 * n);
    std::vector<uint32_t> mat(n);
    cbq_hits h{};
    h.hit = hit.data();
    h.distance = dist.data();
    h.material = mat.data();
    h.position = pos.data();
    h.normal = nrm.data();
    cbq_query q{computeSurfaceProperties ? 1 : 0, maxFootprint, 0u, 0u};
    check(cbq_intersect_host(volume.handle(), o.data(), d.data(), n, &q, &h), "intersectVolumes");
    for (size_t i = 0; i < n; i++) {
        RayVolumeIntersection& r = out[i];
        r = RayVolumeIntersection{};
        r.hit = hit[i] != 0;
        r.distance = (double)dist[i];  // the reference widens the same FP32 value
        r.material = mat[i];
        r.position = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        r.normal = {nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
    }
}

// True when `a` holds the same SubDAGs as `b` (lower bound, height and root
// node of all eight; padding ignored).
inline bool sameSubDAGs(const SubDAGArray& a, const SubDAGArray& b)
{
    for (int i = 0; i < 8; i++) {
        const SubDAG& x = a[i];
        const SubDAG& y = b[i];
        if (x.lower_bound[0] != y.lower_bound[0] || x.lower_bound[1] != y.lower_bound[1] ||
            x.lower_bound[2] != y.lower_bound[2] || x.node_height != y.node_height || x.node_index != y.node_index)
            return false;
    }
    return true;
}

// intersectVolume (raytracing.h:77), one ray given as a Ray3f.  The device
// traverses with the SubDAGs the volume computed when it was uploaded, which
// equal findSubDAGs of the same nodes and root; SubDAGs of anything else (a
// different root, an older version of the volume) are refused with
// cbq::Error(CBQ_ERR_INVALID_ARGUMENT) rather than silently replaced.
inline RayVolumeIntersection intersectVolume(const Volume& volume, const SubDAGArray& subDAGs, Ray3f ray,
                                             bool computeSurfaceProperties,
                                             float maxFootprint = MAX_FOOTPRINT_DISABLED)
{
    if (!sameSubDAGs(subDAGs, volume.subDAGs()))
        throw Error(CBQ_ERR_INVALID_ARGUMENT, "intersectVolume: the SubDAGs are not this volume's");
    const float o[3] = {ray.mOrigin.x, ray.mOrigin.y, ray.mOrigin.z};
    const float d[3] = {ray.mDir.x, ray.mDir.y, ray.mDir.z};
    RayVolumeIntersection r;
    intersectVolumes(volume, o, d, 1, computeSurfaceProperties, maxFootprint, &r);
    return r;
}

// intersectVolume (raytracing.h:72-76), one ray as six floats: forwards to the
// Ray3f form, as the reference does (raytracing.cpp:397-405).
inline RayVolumeIntersection intersectVolume(const Volume& volume, const SubDAGArray& subDAGs, float ray_orig_x,
                                             float ray_orig_y, float ray_orig_z, float ray_dir_x, float ray_dir_y,
                                             float ray_dir_z, bool computeSurfaceProperties,
                                             float maxFootprint = MAX_FOOTPRINT_DISABLED)
{
    return intersectVolume(volume, subDAGs,
                           Ray3f(vec3{ray_orig_x, ray_orig_y, ray_orig_z}, vec3{ray_dir_x, ray_dir_y, ray_dir_z}),
                           computeSurfaceProperties, maxFootprint);
}

}  // namespace cbq
