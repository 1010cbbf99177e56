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

// intersectVolume (raytracing.h:72-75), one ray.  `subDAGs` must be the
// volume's own SubDAGs; it is accepted for signature compatibility.
inline RayVolumeIntersection intersectVolume(const Volume& volume, const SubDAGArray& subDAGs, float ray_orig_x,
                                             float ray_orig_y, float ray_orig_z, float ray_dir_x, float ray_dir_y,
                                             float ray_dir_z, bool computeSurfaceProperties,
                                             float maxFootprint = MAX_FOOTPRINT_DISABLED)
{
    (void)subDAGs;
    const float o[3] = {ray_orig_x, ray_orig_y, ray_orig_z};
    const float d[3] = {ray_dir_x, ray_dir_y, ray_dir_z};
    RayVolumeIntersection r;
    intersectVolumes(volume, o, d, 1, computeSurfaceProperties, maxFootprint, &r);
    return r;
}

}  // namespace cbq
