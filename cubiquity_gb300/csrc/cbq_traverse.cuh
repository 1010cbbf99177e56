// Device-side ESVO traversal of the sparse voxel DAG (sm_103a).
//
// One ray per thread.  The floating-point operations are those of the
// reference's intersectVolume / intersectRayNodeESVO (src/library/
// raytracing.cpp:213-478) in the same order with one rounding each: this file
// must be compiled with -fmad=false (no contraction) and IEEE division
// (-prec-div=true, the default without fast math).  min/max follow std::min /
// std::max, i.e. `(b < a) ? b : a`, never fminf/fmaxf (different NaN rules).
//
// Integer state is packed: the child id is a 3-bit mask, positions are three
// i32 registers with wrapping arithmetic, and the descent stack is indexed by
// node height as in the reference, with a bitmask of the slots written by the
// current sub-DAG walk (a slot never written reads as node 0, the empty node).
#pragma once

#include <cfloat>
#include <cstdint>

namespace cbq {
namespace dev {

constexpr uint32_t kMaterialCount = 256u;
constexpr uint32_t kMaxFetches = 1u << 17;
// The flat kernels index the node store with 32-bit word offsets.
constexpr uint64_t kFlatMaxNodes = 1ull << 29;
constexpr uint32_t kRayOk = 0u, kRayIterLimit = 1u, kRayStuck = 2u;

struct SubDag {
    int32_t lx, ly, lz;   // lower bound (signed voxel coordinates)
    int32_t height;
    uint32_t node;
    uint32_t pad[3];
};

struct DagParams {
    const uint32_t* __restrict__ nodes;
    SubDag sd[8];
};

struct QueryParams {
    int32_t compute_surface;
    float max_footprint;
    uint32_t flags;
    uint32_t image_width;  // flat kernels: rays dealt in 4x8 tiles of an image this wide (0: in order)
};

struct HitsOut {
    uint8_t* hit;
    float* distance;
    uint32_t* material;
    float* position;
    float* normal;
    int32_t* voxel;
    uint8_t* status;
};

struct RayResult {
    bool hit;
    float distance;
    uint32_t material;
    float px, py, pz;
    float nx, ny, nz;
    uint32_t status;
};

__device__ __forceinline__ float min2_ref(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float max2_ref(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float min3_ref(float x, float y, float z) { return min2_ref(min2_ref(x, y), z); }
__device__ __forceinline__ float max3_ref(float x, float y, float z) { return max2_ref(max2_ref(x, y), z); }

__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

__device__ __forceinline__ uint32_t load_child(const uint32_t* __restrict__ nodes, uint32_t node, uint32_t slot)
{
    return __ldg(nodes + ((size_t)node * 8u + slot));
}

// The same with the word index in 32 bits, for stores of fewer than 2^29
// nodes (the flat kernels' condition, kFlatMaxNodes): one multiply-add less.
__device__ __forceinline__ uint32_t load_child32(const uint32_t* __restrict__ nodes, uint32_t node, uint32_t slot)
{
    return __ldg(nodes + (node * 8u + slot));
}

// Child `slot` of node reference `node` in the compact store (the occupancy
// mask is the reference's low byte, the packed children start at unit
// node >> 8 of 8 bytes): an empty child costs no load.  `loads` counts loads.
__device__ __forceinline__ uint32_t load_child_compact(const uint32_t* __restrict__ nodes, uint32_t node,
                                                       uint32_t slot, uint32_t& loads)
{
    const uint32_t m = node & 0xffu;
    if (!((m >> slot) & 1u)) return 0u;
    loads++;
    return __ldg(nodes + ((node >> 8) * 2u + __popc(m & ((1u << slot) - 1u))));  // offsets < 2^25 words
}

// WIDE: 64-bit word index (the nested and integer-position kernels, any store
// size); otherwise the store has fewer than 2^29 nodes.
template <bool COMPACT, bool WIDE = false>
__device__ __forceinline__ uint32_t child_of(const uint32_t* __restrict__ nodes, uint32_t node, uint32_t slot,
                                             uint32_t& loads)
{
    if constexpr (COMPACT) {
        return load_child_compact(nodes, node, slot, loads);
    } else {
        loads++;
        return WIDE ? load_child(nodes, node, slot) : load_child32(nodes, node, slot);
    }
}

// Per-ray constants in the reflected frame.
struct RayFrame {
    float ox, oy, oz;      // (origin + 0.5) * sign
    float ix, iy, iz;      // 1 / |dir|
    uint32_t sign_bits;
};

// findFirstChild (raytracing.cpp:178-196) as a 3-bit child id.
__device__ __forceinline__ uint32_t first_child(const RayFrame& f, float entry, int32_t cx, int32_t cy, int32_t cz)
{
    const float mx = ((float)cx - f.ox) * f.ix;
    const float my = ((float)cy - f.oy) * f.iy;
    const float mz = ((float)cz - f.oz) * f.iz;
    uint32_t id = (mx < entry ? 1u : 0u) | (my < entry ? 2u : 0u) | (mz < entry ? 4u : 0u);
    if (entry <= 0.0f) {
        id |= (f.ox >= (float)cx ? 1u : 0u) | (f.oy >= (float)cy ? 2u : 0u) | (f.oz >= (float)cz ? 4u : 0u);
    }
    return id;
}

// hasLargeFootprint = (childNodeSize / tChildExit) > maxFootprint
// (raytracing.cpp:276).  With the LOD disabled (maxFootprint < 0) and a positive
// exit the quotient is positive, so the division is skipped; every other case
// divides exactly as the reference does.
__device__ __forceinline__ bool large_footprint(int32_t cns, float t_exit, float mf)
{
    if (mf < 0.0f && t_exit > 0.0f) return true;
    return ((float)cns / t_exit) > mf;
}

// Stack held in a per-thread local array (L1-resident).
struct LocalStack {
    alignas(16) uint32_t slot[32];
    __device__ __forceinline__ void put(int h, uint32_t v) { slot[h & 31] = v; }
    __device__ __forceinline__ uint32_t get(int h) const { return slot[h & 31]; }
    // Zeroes every slot (eight 16-byte stores); `top` is for the shared form.
    __device__ __forceinline__ void clear(int /*top*/)
    {
#pragma unroll
        for (int i = 0; i < 8; i++) reinterpret_cast<uint4*>(slot)[i] = make_uint4(0u, 0u, 0u, 0u);
    }
};

// Stack held in shared memory, one column per thread: slot h at
// base[(h - 1) * stride].  Heights run 1..max_height.
struct SharedStack {
    uint32_t* base;
    uint32_t stride;
    __device__ __forceinline__ void put(int h, uint32_t v) { base[(uint32_t)(h - 1) * stride] = v; }
    __device__ __forceinline__ uint32_t get(int h) const { return base[(uint32_t)(h - 1) * stride]; }
    // Zeroes slots 1..top.
    __device__ __forceinline__ void clear(int top)
    {
        for (int h = 1; h <= top; h++) put(h, 0u);
    }
};

struct EsvoOut {
    bool hit;
    float distance;
    uint32_t material;
    float nx, ny, nz;
};

// findNearestMaterial (raytracing.cpp:134-162).
// `fetches` counts child probes (the reference's loads, which also bound the
// walk); `loads` the loads actually made (fewer in the compact layout).
template <bool COMPACT = false, bool WIDE = false>
__device__ __forceinline__ uint32_t nearest_material(const uint32_t* __restrict__ nodes, uint32_t node,
                                                     uint32_t sign_bits, uint32_t& fetches, uint32_t& status,
                                                     uint32_t& loads)
{
    const uint32_t order = (0x76534210u | 0x88888888u) ^ (sign_bits * 0x11111111u);
    while (node >= kMaterialCount) {
        for (uint32_t ids = order; ids != 0u; ids >>= 4) {
            const uint32_t c = child_of<COMPACT, WIDE>(nodes, node, ids & 7u, loads);
            fetches++;
            if (c > 0u) { node = c; break; }
        }
        if (fetches >= kMaxFetches) { status = kRayIterLimit; return 0u; }
    }
    return node;
}

// intersectRayNodeESVO (raytracing.cpp:213-371).
template <typename Stack>
__device__ __forceinline__ EsvoOut esvo(const uint32_t* __restrict__ nodes, const RayFrame& f, uint32_t node,
                                        int32_t px, int32_t py, int32_t pz, int height, const QueryParams& q,
                                        Stack& stack, uint32_t& fetches, uint32_t& status)
{
    EsvoOut res;
    res.hit = false;
    res.distance = 0.0f;
    res.material = 0u;
    res.nx = res.ny = res.nz = 0.0f;

    const uint32_t node_size = 1u << height;
    const float t0x = ((float)px - f.ox) * f.ix;
    const float t0y = ((float)py - f.oy) * f.iy;
    const float t0z = ((float)pz - f.oz) * f.iz;
    const float t1x = (((float)px + (float)node_size) - f.ox) * f.ix;
    const float t1y = (((float)py + (float)node_size) - f.oy) * f.iy;
    const float t1z = (((float)pz + (float)node_size) - f.oz) * f.iz;
    const float entry = max3_ref(t0x, t0y, t0z);
    const float exit_ = min3_ref(t1x, t1y, t1z);
    if (!(entry < exit_)) return res;

    const int start_h = height;
    int h = height;
    int32_t cns = (int32_t)(node_size >> 1);
    uint32_t cid = first_child(f, entry, wadd(px, cns), wadd(py, cns), wadd(pz, cns));
    int32_t cx = wadd(px, (cid & 1u) ? cns : 0);
    int32_t cy = wadd(py, (cid & 2u) ? cns : 0);
    int32_t cz = wadd(pz, (cid & 4u) ? cns : 0);
    float last_exit = exit_;
    uint32_t written = 0u;  // bit h: stack slot h written during this walk

    for (;;) {
        const float c1x = ((float)wadd(cx, cns) - f.ox) * f.ix;
        const float c1y = ((float)wadd(cy, cns) - f.oy) * f.iy;
        const float c1z = ((float)wadd(cz, cns) - f.oz) * f.iz;
        const float tcx = min3_ref(c1x, c1y, c1z);

        if (fetches >= kMaxFetches) { status = kRayIterLimit; res.hit = false; return res; }
        const uint32_t child = load_child(nodes, node, cid ^ f.sign_bits);
        fetches++;

        if (child > 0u) {
            const float c0x = ((float)cx - f.ox) * f.ix;
            const float c0y = ((float)cy - f.oy) * f.iy;
            const float c0z = ((float)cz - f.oz) * f.iz;
            const float tce = max3_ref(c0x, c0y, c0z);
            if (child >= kMaterialCount && large_footprint(cns, tcx, q.max_footprint)) {
                if (tcx < last_exit) { stack.put(h, node); written |= 1u << h; }
                last_exit = tcx;
                h--;
                node = child;
                cns /= 2;
                cid = first_child(f, tce, wadd(cx, cns), wadd(cy, cns), wadd(cz, cns));
                cx = wadd(cx, (cid & 1u) ? cns : 0);
                cy = wadd(cy, (cid & 2u) ? cns : 0);
                cz = wadd(cz, (cid & 4u) ? cns : 0);
            } else {
                res.hit = true;
                res.distance = tce;
                if (q.compute_surface) {
                    uint32_t loads = 0;
                    res.material = nearest_material<false, true>(nodes, child, f.sign_bits, fetches, status, loads);
                    if (status != kRayOk) { res.hit = false; return res; }
                    const float sx = (f.sign_bits & 1u) ? 1.0f : -1.0f;  // -rayDirSign
                    const float sy = (f.sign_bits & 2u) ? 1.0f : -1.0f;
                    const float sz = (f.sign_bits & 4u) ? 1.0f : -1.0f;
                    res.nx = __fmul_rn(tce == c0x ? 1.0f : 0.0f, sx);
                    res.ny = __fmul_rn(tce == c0y ? 1.0f : 0.0f, sy);
                    res.nz = __fmul_rn(tce == c0z ? 1.0f : 0.0f, sz);
                }
                return res;
            }
        } else {
            const uint32_t flips = (c1x <= tcx ? 1u : 0u) | (c1y <= tcx ? 2u : 0u) | (c1z <= tcx ? 4u : 0u);
            if (flips == 0u) { status = kRayStuck; res.hit = false; return res; }
            cid ^= flips;
            const int32_t ox = cx, oy = cy, oz = cz;
            if (flips & 1u) cx = wadd(cx, cns);
            if (flips & 2u) cy = wadd(cy, cns);
            if (flips & 4u) cz = wadd(cz, cns);
            if ((cid & flips) != flips) {
                const uint32_t diff = (uint32_t)(ox ^ cx) | (uint32_t)(oy ^ cy) | (uint32_t)(oz ^ cz);
                const int msb = 31 - __clz(diff);
                h = msb + 1;
                if (h > start_h) return res;  // left the sub-DAG
                node = (written & (1u << h)) ? stack.get(h) : 0u;
                cns = (int32_t)(1u << msb);
                cid = (uint32_t)((cx >> msb) & 1) | ((uint32_t)((cy >> msb) & 1) << 1) |
                      ((uint32_t)((cz >> msb) & 1) << 2);
                cx = wadd((int32_t)((uint32_t)(cx >> h) << h), (cid & 1u) ? cns : 0);
                cy = wadd((int32_t)((uint32_t)(cy >> h) << h), (cid & 2u) ? cns : 0);
                cz = wadd((int32_t)((uint32_t)(cz >> h) << h), (cid & 4u) ? cns : 0);
                last_exit = 0.0f;
            }
        }
    }
}

// intersectVolume (raytracing.cpp:407-478) for one ray.
template <typename Stack>
__device__ __forceinline__ RayResult intersect_volume(const DagParams& dag, float4 o, float4 d, const QueryParams& q,
                                                      Stack& stack, uint32_t* fetch_count)
{
    RayResult r;
    r.hit = false;
    r.distance = 0.0f;
    r.material = 0u;
    r.px = r.py = r.pz = 0.0f;
    r.nx = r.ny = r.nz = 0.0f;
    r.status = kRayOk;

    const uint32_t sbx = d.x < 0.0f, sby = d.y < 0.0f, sbz = d.z < 0.0f;
    RayFrame f;
    f.sign_bits = sbx | (sby << 1) | (sbz << 2);
    const float sx = sbx ? -1.0f : 1.0f, sy = sby ? -1.0f : 1.0f, sz = sbz ? -1.0f : 1.0f;
    f.ox = __fmul_rn(__fadd_rn(o.x, 0.5f), sx);
    f.oy = __fmul_rn(__fadd_rn(o.y, 0.5f), sy);
    f.oz = __fmul_rn(__fadd_rn(o.z, 0.5f), sz);
    const float rdx = fabsf(d.x), rdy = fabsf(d.y), rdz = fabsf(d.z);
    // 1 / |dir|: the correctly rounded reciprocal, the same value as the IEEE division.
    f.ix = __frcp_rn(rdx);
    f.iy = __frcp_rn(rdy);
    f.iz = __frcp_rn(rdz);

    uint32_t oct = 0u;
    float dx = (-f.ox) / rdx, dy = (-f.oy) / rdy, dz = (-f.oz) / rdz;
    if (dx < 0.0f) { oct += 1u; dx = __fadd_rn(dx, FLT_MAX); }
    if (dy < 0.0f) { oct += 2u; dy = __fadd_rn(dy, FLT_MAX); }
    if (dz < 0.0f) { oct += 4u; dz = __fadd_rn(dz, FLT_MAX); }

    uint32_t fetches = 0u;
    do {
        const SubDag& s = dag.sd[oct ^ f.sign_bits];
        if (s.node > 0u) {
            const int32_t ns = (int32_t)(1u << s.height);
            // lowerBound * rayDirSign - signBit * nodeSize, wrapping (raytracing.cpp:454-456)
            const int32_t lx = (int32_t)((sbx ? 0u - (uint32_t)s.lx : (uint32_t)s.lx) - (sbx ? (uint32_t)ns : 0u));
            const int32_t ly = (int32_t)((sby ? 0u - (uint32_t)s.ly : (uint32_t)s.ly) - (sby ? (uint32_t)ns : 0u));
            const int32_t lz = (int32_t)((sbz ? 0u - (uint32_t)s.lz : (uint32_t)s.lz) - (sbz ? (uint32_t)ns : 0u));
            const EsvoOut e = esvo(dag.nodes, f, s.node, lx, ly, lz, s.height, q, stack, fetches, r.status);
            if (r.status != kRayOk) break;
            if (e.hit) {
                r.hit = true;
                r.distance = e.distance;
                r.material = e.material;
                r.nx = e.nx;
                r.ny = e.ny;
                r.nz = e.nz;
                r.px = __fadd_rn(o.x, __fmul_rn(d.x, e.distance));
                r.py = __fadd_rn(o.y, __fmul_rn(d.y, e.distance));
                r.pz = __fadd_rn(o.z, __fmul_rn(d.z, e.distance));
                break;
            }
        }
        const float md = min3_ref(dx, dy, dz);
        const uint32_t before = oct;
        if (dx <= md) { oct += 1u; dx = __fadd_rn(dx, FLT_MAX); }
        if (dy <= md) { oct += 2u; dy = __fadd_rn(dy, FLT_MAX); }
        if (dz <= md) { oct += 4u; dz = __fadd_rn(dz, FLT_MAX); }
        if (oct == before) {  // NaN distances: the reference would revisit this octant forever
            r.status = kRayStuck;
            break;
        }
    } while (oct <= 7u);

    if ((q.flags & 1u) && r.hit && !(r.distance <= o.w)) {
        r.hit = false;
        r.distance = 0.0f;
        r.material = 0u;
        r.px = r.py = r.pz = 0.0f;
        r.nx = r.ny = r.nz = 0.0f;
    }
    if (fetch_count) *fetch_count = fetches;
    return r;
}

// Hit records are written once and not read back by the kernel: streaming
// (evict-first) stores keep them from displacing the node store in L2.
__device__ __forceinline__ void write_result(const HitsOut& out, size_t i, const RayResult& r)
{
    if (out.hit) __stcs(out.hit + i, (uint8_t)(r.hit ? 1 : 0));
    if (out.distance) __stcs(out.distance + i, r.distance);
    if (out.material) __stcs(out.material + i, r.material);
    if (out.position) {
        __stcs(out.position + 3 * i, r.px);
        __stcs(out.position + 3 * i + 1, r.py);
        __stcs(out.position + 3 * i + 2, r.pz);
    }
    if (out.normal) {
        __stcs(out.normal + 3 * i, r.nx);
        __stcs(out.normal + 3 * i + 1, r.ny);
        __stcs(out.normal + 3 * i + 2, r.nz);
    }
    if (out.voxel) {
        int32_t vx = 0, vy = 0, vz = 0;
        if (r.hit) {
            vx = __float2int_rd(__fadd_rn(__fsub_rn(r.px, __fmul_rn(0.5f, r.nx)), 0.5f));
            vy = __float2int_rd(__fadd_rn(__fsub_rn(r.py, __fmul_rn(0.5f, r.ny)), 0.5f));
            vz = __float2int_rd(__fadd_rn(__fsub_rn(r.pz, __fmul_rn(0.5f, r.nz)), 0.5f));
        }
        __stcs(out.voxel + 3 * i, vx);
        __stcs(out.voxel + 3 * i + 1, vy);
        __stcs(out.voxel + 3 * i + 2, vz);
    }
    if (out.status) __stcs(out.status + i, (uint8_t)r.status);
}

}  // namespace dev
}  // namespace cbq
