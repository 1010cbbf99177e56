// Flat ("while-while") form of the ESVO traversal for sm_103a.
//
// The reference's control flow (raytracing.cpp:397-478 around :213-371) is two
// nested loops with early exits: an octant walk, and inside it the ESVO
// descend/advance/pop loop.  Run per thread as written, the lanes of a warp
// leave those loops at different times and drift apart (measured: 1.8-2.8
// active lanes per instruction).  Here the same arithmetic is re-expressed as a
// per-lane state machine driven by a single loop: every iteration each lane
// performs at most one ESVO step (plus any octant transitions), so the warp
// reconverges at the top of every iteration.  In the persistent form, lanes
// whose ray is done pull new rays from a global counter (warp-aggregated).
//
// Floating-point operations are those of cbq_traverse.cuh / the reference, in
// the same order (compile with -fmad=false).  Child positions are carried as
// floats updated by exact float additions; the host only selects this form
// when every SubDAG's reflected coordinates lie within +-2^21, where
// (float)(a + b) == (float)a + (float)b and p + 1.5 * 2^23 is exact with a
// fixed exponent, so the integer bits the pop's XOR/MSB logic needs are the
// low bits of that sum's bit pattern (no float/int conversion).
#pragma once

#include "../../include/cubiquity_gb300.h"
#include "cbq_traverse.cuh"

namespace cbq {
namespace dev {

// Float positions p with |p| <= 2^21: the bit pattern of p + kPosBias is
// 0x4B400000 + p (two's complement), exactly, so its low 22 bits are p's.
constexpr float kPosBias = 12582912.0f;  // 1.5 * 2^23

enum : uint32_t { kLaneIdle = 0u, kLaneEnter = 1u, kLaneNext = 2u, kLaneWalk = 3u };

struct Lane {
    float4 o, d;                 // the ray as given (o.w = tmax)
    float rox, roy, roz;         // reflected origin
    float ix, iy, iz;            // 1 / |dir|
    float ddx, ddy, ddz;         // octant walk distances (distToOrigin)
    uint32_t sign, oct;
    // ESVO walk state
    uint32_t node, cid;
    bool fresh;                  // walk not started: its descent stack is still to be cleared
    int32_t cns;
    float fx, fy, fz, fcns;      // child position and size as exact floats (float-position form)
    int32_t px, py, pz;          // child position as wrapping i32 (integer-position form)
    int h, start_h;
    float last_exit;
    uint32_t fetches, status, mode;
    bool fast;                   // no slab distance can be NaN or -0: min/max need no NaN ordering
    uint32_t held;               // finished in this step batch: 0 no, 1 miss (status set), 2 hit at child `node`
    uint32_t loads;              // node loads made (fetches minus skipped empty children)
    uint32_t job;                // batch kernel: index of the lane's job
    uint64_t ray;                // ray index within its job
    const uint32_t* nodes;       // batch kernel: the job's node store
};

// Where a lane's volume, rays and outputs are.  The lane functions below are
// templates over this "source" so that the single-volume kernel and the
// multi-volume batch kernel share the same arithmetic.  COMPACT selects the
// node store layout; COUNT_LOADS is the fetch-count pass (cbq_count_fetches),
// which writes per ray the node loads (child probes in the reference layout,
// fewer in the compact one) to fetch_out.  It is a separate instantiation, so
// the traversal kernels carry no counting code (measured: 1-2% faster).
template <bool COMPACT, bool COUNT_LOADS = false, bool INT_POS = false>
struct FlatCtxT {
    static constexpr bool kCompact = COMPACT;
    // INT_POS: child positions as wrapping i32 converted to float where a slab
    // plane is needed (the reference's own arithmetic, any coordinates, 64-bit
    // node offsets); otherwise exact floats (coordinates within +-2^21, fewer
    // than 2^29 nodes).
    static constexpr bool kIntPos = INT_POS;
    DagParams dag;
    QueryParams q;
    HitsOut out;
    const float4* __restrict__ orig;
    const float4* __restrict__ dir;
    uint32_t* __restrict__ fetch_out;

    __device__ __forceinline__ const QueryParams& query(const Lane&) const { return q; }
    __device__ __forceinline__ const uint32_t* nodes(const Lane&) const { return dag.nodes; }
    // Ray of work item g: g itself, or with an image width (q.image_width, a
    // multiple of 4 dividing the launch into whole 8-row bands) the pixel of
    // tile g / 32 (tiles of 4 x 8 pixels, a band's tiles left to right) at
    // place g % 32 (row-major in the tile): a bijection of [0, n).
    __device__ __forceinline__ uint64_t ray_slot(uint64_t g) const
    {
        const uint32_t w = q.image_width;
        if (w == 0u) return g;
        const uint32_t t = (uint32_t)(g >> 5), k = (uint32_t)g & 31u;
        const uint32_t per_band = w >> 2;
        const uint32_t band = t / per_band, col = t - band * per_band;
        return (uint64_t)(band * 8u + (k >> 2)) * w + col * 4u + (k & 3u);
    }
    __device__ __forceinline__ const SubDag& subdag(const Lane&, uint32_t k) const { return dag.sd[k]; }
    // Rays are read once: streaming loads (evict-first) leave L2 to the node store.
    __device__ __forceinline__ float4 ray_origin(const Lane&, uint64_t i) const { return __ldcs(orig + i); }
    __device__ __forceinline__ float4 ray_direction(const Lane&, uint64_t i) const { return __ldcs(dir + i); }
    __device__ __forceinline__ void write(const Lane& L, const RayResult& r) const
    {
        write_result(out, L.ray, r);
        if constexpr (COUNT_LOADS) fetch_out[L.ray] = COMPACT ? L.loads : L.fetches;
    }
};

__device__ __forceinline__ uint32_t first_child_f(const Lane& L, float entry, float fcx, float fcy, float fcz)
{
    const float mx = (fcx - L.rox) * L.ix;
    const float my = (fcy - L.roy) * L.iy;
    const float mz = (fcz - L.roz) * L.iz;
    uint32_t id = (mx < entry ? 1u : 0u) | (my < entry ? 2u : 0u) | (mz < entry ? 4u : 0u);
    if (entry <= 0.0f) {
        id |= (L.rox >= fcx ? 1u : 0u) | (L.roy >= fcy ? 2u : 0u) | (L.roz >= fcz ? 4u : 0u);
    }
    return id;
}

// The same with each axis's bit also returned as a predicate, for callers that
// move the child position by it (cheaper than unpacking the id again).
__device__ __forceinline__ uint32_t first_child_p(const Lane& L, float entry, float fcx, float fcy, float fcz,
                                                  bool& bx, bool& by, bool& bz)
{
    bx = ((fcx - L.rox) * L.ix) < entry;
    by = ((fcy - L.roy) * L.iy) < entry;
    bz = ((fcz - L.roz) * L.iz) < entry;
    if (entry <= 0.0f) {
        bx = bx || L.rox >= fcx;
        by = by || L.roy >= fcy;
        bz = bz || L.roz >= fcz;
    }
    return (uint32_t)bx | ((uint32_t)by << 1) | ((uint32_t)bz << 2);
}

// Per-ray set-up: intersectVolume up to the octant loop (raytracing.cpp:409-434).
template <typename Src>
__device__ __forceinline__ void lane_begin(Lane& L, const Src& c, uint64_t i)
{
    L.ray = i;
    L.o = c.ray_origin(L, i);
    L.d = c.ray_direction(L, i);
    const uint32_t sbx = L.d.x < 0.0f, sby = L.d.y < 0.0f, sbz = L.d.z < 0.0f;
    L.sign = sbx | (sby << 1) | (sbz << 2);
    const float sx = sbx ? -1.0f : 1.0f, sy = sby ? -1.0f : 1.0f, sz = sbz ? -1.0f : 1.0f;
    L.rox = __fmul_rn(__fadd_rn(L.o.x, 0.5f), sx);
    L.roy = __fmul_rn(__fadd_rn(L.o.y, 0.5f), sy);
    L.roz = __fmul_rn(__fadd_rn(L.o.z, 0.5f), sz);
    const float rdx = fabsf(L.d.x), rdy = fabsf(L.d.y), rdz = fabsf(L.d.z);
    // 1 / |dir|: the correctly rounded reciprocal, the same value as the IEEE division.
    L.ix = __frcp_rn(rdx);
    L.iy = __frcp_rn(rdy);
    L.iz = __frcp_rn(rdz);
    // With every |dir| component normal (>= FLT_MIN, not NaN) and a finite
    // reflected origin, a slab distance (plane - o') * (1/|dir|) is a finite
    // difference times a finite positive number: never NaN, and never -0
    // (planes are floats of integers, so plane - o' is +0 when they are
    // equal).  For such rays fminf/fmaxf give the bits of the reference's
    // std::min/std::max compositions.
    L.fast = rdx >= FLT_MIN && rdy >= FLT_MIN && rdz >= FLT_MIN && fabsf(L.rox) <= FLT_MAX &&
             fabsf(L.roy) <= FLT_MAX && fabsf(L.roz) <= FLT_MAX;
    L.oct = 0u;
    L.ddx = (-L.rox) / rdx;
    L.ddy = (-L.roy) / rdy;
    L.ddz = (-L.roz) / rdz;
    if (L.ddx < 0.0f) { L.oct += 1u; L.ddx = __fadd_rn(L.ddx, FLT_MAX); }
    if (L.ddy < 0.0f) { L.oct += 2u; L.ddy = __fadd_rn(L.ddy, FLT_MAX); }
    if (L.ddz < 0.0f) { L.oct += 4u; L.ddz = __fadd_rn(L.ddz, FLT_MAX); }
    L.fetches = 0u;
    L.loads = 0u;
    L.status = kRayOk;
    L.mode = kLaneEnter;
}

// Writes the result of ray L.ray and frees the lane.
template <typename Src>
__device__ __forceinline__ void lane_finish(Lane& L, const Src& c, bool hit, float dist, uint32_t material,
                                            float nx, float ny, float nz)
{
    RayResult r;
    r.hit = hit;
    r.distance = hit ? dist : 0.0f;
    r.material = hit ? material : 0u;
    r.nx = hit ? nx : 0.0f;
    r.ny = hit ? ny : 0.0f;
    r.nz = hit ? nz : 0.0f;
    r.px = r.py = r.pz = 0.0f;
    if (hit) {
        r.px = __fadd_rn(L.o.x, __fmul_rn(L.d.x, dist));
        r.py = __fadd_rn(L.o.y, __fmul_rn(L.d.y, dist));
        r.pz = __fadd_rn(L.o.z, __fmul_rn(L.d.z, dist));
    }
    r.status = L.status;
    if ((c.query(L).flags & 1u) && r.hit && !(r.distance <= L.o.w)) {
        r.hit = false;
        r.distance = 0.0f;
        r.material = 0u;
        r.px = r.py = r.pz = 0.0f;
        r.nx = r.ny = r.nz = 0.0f;
    }
    c.write(L, r);
    L.mode = kLaneIdle;
}

// A finish inside the step loop.  The lane only records how it ended (a miss,
// with its status; or a hit at child `node` of the current child position) and
// flush_held completes the result after the step batch, for all the warp's
// lanes that finished in it at once: finishes are spread over the steps, so
// completing each at once ran the result code at a few active lanes.
__device__ __forceinline__ void lane_hold_miss(Lane& L)
{
    L.held = 1u;
    L.mode = kLaneIdle;
}

// Completes a held result with the reference's operations: the entry distance
// max3(childT0) (raytracing.cpp:270-271), the material (findNearestMaterial,
// :310) and the normal vec3(equal(tChildEntry, childT0)) * -rayDirSign
// (:317-318).  For rays on the fast min/max path max3 gives the same bits.
template <typename Src>
__device__ __forceinline__ void flush_held(Lane& L, const Src& c)
{
    if (!L.held) return;
    const uint32_t kind = L.held;
    L.held = 0u;
    if (kind == 1u) {
        lane_finish(L, c, false, 0.0f, 0u, 0.0f, 0.0f, 0.0f);
        return;
    }
    constexpr bool INT = Src::kIntPos;
    const float c0x = ((INT ? (float)L.px : L.fx) - L.rox) * L.ix;
    const float c0y = ((INT ? (float)L.py : L.fy) - L.roy) * L.iy;
    const float c0z = ((INT ? (float)L.pz : L.fz) - L.roz) * L.iz;
    const float tce = max3_ref(c0x, c0y, c0z);
    uint32_t material = 0u;
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    if (c.query(L).compute_surface) {
        material = nearest_material<Src::kCompact, INT>(c.nodes(L), L.node, L.sign, L.fetches, L.status, L.loads);
        if (L.status != kRayOk) {
            lane_finish(L, c, false, 0.0f, 0u, 0.0f, 0.0f, 0.0f);
            return;
        }
        nx = __fmul_rn(tce == c0x ? 1.0f : 0.0f, (L.sign & 1u) ? 1.0f : -1.0f);
        ny = __fmul_rn(tce == c0y ? 1.0f : 0.0f, (L.sign & 2u) ? 1.0f : -1.0f);
        nz = __fmul_rn(tce == c0z ? 1.0f : 0.0f, (L.sign & 4u) ? 1.0f : -1.0f);
    }
    lane_finish(L, c, true, tce, material, nx, ny, nz);
}

// One octant transition (raytracing.cpp:469-475).
template <typename Src>
__device__ __forceinline__ void lane_next(Lane& L, const Src& c)
{
    const float md = min3_ref(L.ddx, L.ddy, L.ddz);
    const uint32_t before = L.oct;
    if (L.ddx <= md) { L.oct += 1u; L.ddx = __fadd_rn(L.ddx, FLT_MAX); }
    if (L.ddy <= md) { L.oct += 2u; L.ddy = __fadd_rn(L.ddy, FLT_MAX); }
    if (L.ddz <= md) { L.oct += 4u; L.ddz = __fadd_rn(L.ddz, FLT_MAX); }
    if (L.oct == before) {  // NaN distances: the reference would revisit this octant forever
        L.status = kRayStuck;
        lane_finish(L, c, false, 0.0f, 0u, 0.0f, 0.0f, 0.0f);
    } else if (L.oct > 7u) {
        lane_finish(L, c, false, 0.0f, 0u, 0.0f, 0.0f, 0.0f);
    } else {
        L.mode = kLaneEnter;
    }
}

// Enters the SubDAG of the current octant: the slab test and set-up at the top
// of intersectRayNodeESVO (raytracing.cpp:218-250, 443-460).
template <typename Src>
__device__ __forceinline__ void lane_enter(Lane& L, const Src& c)
{
    const SubDag& s = c.subdag(L, L.oct ^ L.sign);
    if (s.node == 0u) {
        L.mode = kLaneNext;
        return;
    }
    const uint32_t sbx = L.sign & 1u, sby = (L.sign >> 1) & 1u, sbz = (L.sign >> 2) & 1u;
    const uint32_t ns = 1u << s.height;
    const int32_t px = (int32_t)((sbx ? 0u - (uint32_t)s.lx : (uint32_t)s.lx) - (sbx ? ns : 0u));
    const int32_t py = (int32_t)((sby ? 0u - (uint32_t)s.ly : (uint32_t)s.ly) - (sby ? ns : 0u));
    const int32_t pz = (int32_t)((sbz ? 0u - (uint32_t)s.lz : (uint32_t)s.lz) - (sbz ? ns : 0u));
    const float fpx = (float)px, fpy = (float)py, fpz = (float)pz, fns = (float)ns;
    const float t0x = (fpx - L.rox) * L.ix;
    const float t0y = (fpy - L.roy) * L.iy;
    const float t0z = (fpz - L.roz) * L.iz;
    const float t1x = ((fpx + fns) - L.rox) * L.ix;
    const float t1y = ((fpy + fns) - L.roy) * L.iy;
    const float t1z = ((fpz + fns) - L.roz) * L.iz;
    const float entry = max3_ref(t0x, t0y, t0z);
    const float exit_ = min3_ref(t1x, t1y, t1z);
    if (!(entry < exit_)) {
        L.mode = kLaneNext;
        return;
    }
    L.start_h = s.height;
    L.h = s.height;
    L.node = s.node;
    L.cns = (int32_t)(ns >> 1);
    if constexpr (Src::kIntPos) {
        L.cid = first_child_f(L, entry, (float)wadd(px, L.cns), (float)wadd(py, L.cns), (float)wadd(pz, L.cns));
        L.px = wadd(px, (L.cid & 1u) ? L.cns : 0);
        L.py = wadd(py, (L.cid & 2u) ? L.cns : 0);
        L.pz = wadd(pz, (L.cid & 4u) ? L.cns : 0);
    } else {
        L.fcns = (float)L.cns;
        L.cid = first_child_f(L, entry, fpx + L.fcns, fpy + L.fcns, fpz + L.fcns);
        L.fx = fpx + ((L.cid & 1u) ? L.fcns : 0.0f);
        L.fy = fpy + ((L.cid & 2u) ? L.fcns : 0.0f);
        L.fz = fpz + ((L.cid & 4u) ? L.fcns : 0.0f);
    }
    L.last_exit = exit_;
    L.fresh = true;
    L.mode = kLaneWalk;
}

// min3/max3 of slab distances: the reference's NaN-ordered forms, or (FAST,
// the lane's ray has Lane::fast) one fminf/fmaxf per pair, the same bits.
template <bool FAST>
__device__ __forceinline__ float slab_min3(float x, float y, float z)
{
    if constexpr (FAST) return fminf(fminf(x, y), z);
    else return min3_ref(x, y, z);
}
template <bool FAST>
__device__ __forceinline__ float slab_max3(float x, float y, float z)
{
    if constexpr (FAST) return fmaxf(fmaxf(x, y), z);
    else return max3_ref(x, y, z);
}

// One iteration of the ESVO loop (raytracing.cpp:253-367).
template <bool FAST, typename Src, typename Stack>
__device__ __forceinline__ void lane_walk(Lane& L, const Src& c, Stack& stack)
{
    constexpr bool INT = Src::kIntPos;
    // Exit planes: vec3(childPos + childNodeSize) (raytracing.cpp:259-260).
    const float c1x = ((INT ? (float)wadd(L.px, L.cns) : L.fx + L.fcns) - L.rox) * L.ix;
    const float c1y = ((INT ? (float)wadd(L.py, L.cns) : L.fy + L.fcns) - L.roy) * L.iy;
    const float c1z = ((INT ? (float)wadd(L.pz, L.cns) : L.fz + L.fcns) - L.roz) * L.iz;
    const float tcx = slab_min3<FAST>(c1x, c1y, c1z);
    const uint32_t child = child_of<Src::kCompact, INT>(c.nodes(L), L.node, L.cid ^ L.sign, L.loads);
    L.fetches++;
    if (child > 0u) {
        if (child >= kMaterialCount && large_footprint(L.cns, tcx, c.query(L).max_footprint)) {
            const float c0x = ((INT ? (float)L.px : L.fx) - L.rox) * L.ix;
            const float c0y = ((INT ? (float)L.py : L.fy) - L.roy) * L.iy;
            const float c0z = ((INT ? (float)L.pz : L.fz) - L.roz) * L.iz;
            const float tce = slab_max3<FAST>(c0x, c0y, c0z);
            if (tcx < L.last_exit) stack.put(L.h, L.node);
            L.last_exit = tcx;
            L.h--;
            L.node = child;
            L.cns >>= 1;
            if constexpr (INT) {
                L.cid = first_child_f(L, tce, (float)wadd(L.px, L.cns), (float)wadd(L.py, L.cns),
                                      (float)wadd(L.pz, L.cns));
                if (L.cid & 1u) L.px = wadd(L.px, L.cns);
                if (L.cid & 2u) L.py = wadd(L.py, L.cns);
                if (L.cid & 4u) L.pz = wadd(L.pz, L.cns);
            } else {
                L.fcns = (float)L.cns;
                const float mcx = L.fx + L.fcns, mcy = L.fy + L.fcns, mcz = L.fz + L.fcns;
                bool bx, by, bz;
                L.cid = first_child_p(L, tce, mcx, mcy, mcz, bx, by, bz);
                L.fx = bx ? mcx : L.fx;
                L.fy = by ? mcy : L.fy;
                L.fz = bz ? mcz : L.fz;
            }
        } else {  // a hit at this child: completed by flush_held
            L.node = child;
            L.held = 2u;
            L.mode = kLaneIdle;
        }
        return;
    }
    const bool ax = c1x <= tcx, ay = c1y <= tcx, az = c1z <= tcx;
    const uint32_t flips = (uint32_t)ax | ((uint32_t)ay << 1) | ((uint32_t)az << 2);
    // With slab distances that cannot be NaN (FAST), tcx is one of the three
    // and that axis flips: only the reference's form can get stuck here.
    if (!FAST && !(ax || ay || az)) {
        L.status = kRayStuck;
        lane_hold_miss(L);
        return;
    }
    L.cid ^= flips;
    float ofx = 0.0f, ofy = 0.0f, ofz = 0.0f;  // float positions before the advance
    if constexpr (INT) {
        if (ax) L.px = wadd(L.px, L.cns);
        if (ay) L.py = wadd(L.py, L.cns);
        if (az) L.pz = wadd(L.pz, L.cns);
    } else {
        ofx = L.fx;
        ofy = L.fy;
        ofz = L.fz;
        if (ax) L.fx += L.fcns;
        if (ay) L.fy += L.fcns;
        if (az) L.fz += L.fcns;
    }
    if ((L.cid & flips) != flips) {
        // The pop (raytracing.cpp:339-361) on integer positions: the wrapping
        // i32 ones, or the biased bit patterns of the float ones, whose low 22
        // bits are the integer's.  The highest differing bit is the same in
        // both below bit 21; at bit 21 or above (a sign change included) both
        // leave the SubDAG, whose height is at most 21.
        const uint32_t cx = INT ? (uint32_t)L.px : __float_as_uint(L.fx + kPosBias);
        const uint32_t cy = INT ? (uint32_t)L.py : __float_as_uint(L.fy + kPosBias);
        const uint32_t cz = INT ? (uint32_t)L.pz : __float_as_uint(L.fz + kPosBias);
        uint32_t diff;
        if constexpr (INT) {  // on a flipped axis the position before the advance was p - childSize
            const uint32_t cs = (uint32_t)L.cns;
            diff = (ax ? (cx ^ (cx - cs)) : 0u) | (ay ? (cy ^ (cy - cs)) : 0u) | (az ? (cz ^ (cz - cs)) : 0u);
        } else {  // before against after: an axis that did not move gives 0
            diff = (cx ^ __float_as_uint(ofx + kPosBias)) | (cy ^ __float_as_uint(ofy + kPosBias)) |
                   (cz ^ __float_as_uint(ofz + kPosBias));
        }
        const int msb = 31 - __clz(diff);
        const int h = msb + 1;
        if (h > L.start_h) {  // left the sub-DAG: on to the next octant
            L.mode = kLaneNext;
            return;
        }
        L.h = h;
        L.node = stack.get(h);
        L.cns = (int32_t)(1u << msb);
        const uint32_t keep = 0u - (uint32_t)L.cns;
        if constexpr (INT) {
            L.cid = ((cx >> msb) & 1u) | (((cy >> msb) & 1u) << 1) | (((cz >> msb) & 1u) << 2);
            L.px = (int32_t)(cx & keep);
            L.py = (int32_t)(cy & keep);
            L.pz = (int32_t)(cz & keep);
        } else {
            // Bit msb (< 21) of each axis, gathered at msb..msb+2, then shifted down.
            const uint32_t m = (uint32_t)L.cns;
            L.cid = ((cx & m) + ((cy & m) << 1) + ((cz & m) << 2)) >> msb;
            L.fcns = __uint_as_float((uint32_t)(127 + msb) << 23);  // 2^msb
            L.fx = __uint_as_float(cx & keep) - kPosBias;
            L.fy = __uint_as_float(cy & keep) - kPosBias;
            L.fz = __uint_as_float(cz & keep) - kPosBias;
        }
        L.last_exit = 0.0f;
    }
}

// Up to `steps` ESVO steps.  The reference ends a ray when a step starts with
// the fetch budget spent (raytracing.cpp:253 with the cap): the steps here are
// bounded by the budget left, and a lane still walking with the budget spent
// ends exactly as that next step would have ended it.
template <bool FAST, typename Src, typename Stack>
__device__ __forceinline__ void lane_walk_steps(Lane& L, const Src& c, Stack& stack, uint32_t steps)
{
    if (L.mode != kLaneWalk) return;
    if (L.fresh) {  // each SubDAG walk starts on a zeroed stack (never-written slots read as node 0)
        stack.clear(L.start_h);
        L.fresh = false;
    }
    const uint32_t budget = kMaxFetches - L.fetches;  // > 0: a walking lane is below the cap
    // Every step makes one fetch, so the fetch count doubles as the step counter.
    const uint32_t end = L.fetches + (steps < budget ? steps : budget);
    while (L.fetches < end && L.mode == kLaneWalk) lane_walk<FAST>(L, c, stack);
    if (L.mode == kLaneWalk && L.fetches >= kMaxFetches) {
        L.status = kRayIterLimit;
        lane_hold_miss(L);
    }
}

// The walk of a whole warp (all 32 lanes must call it): the FAST min/max when
// every walking lane's ray allows it, else the reference's forms; then the
// results of the rays that finished in it are written.
template <typename Src, typename Stack>
__device__ __forceinline__ void warp_walk_steps(Lane& L, const Src& c, Stack& stack, uint32_t steps)
{
    if (__all_sync(0xffffffffu, L.mode != kLaneWalk || L.fast))
        lane_walk_steps<true>(L, c, stack, steps);
    else
        lane_walk_steps<false>(L, c, stack, steps);
    flush_held(L, c);
}

// Octant transitions until the lane walks a SubDAG or has finished.  Bounded:
// every kLaneNext raises `oct` (or finishes the ray), every kLaneEnter walks or
// moves on, so at most 16 transitions happen.
template <typename Src>
__device__ __forceinline__ void lane_settle(Lane& L, const Src& c)
{
    while (L.mode == kLaneEnter || L.mode == kLaneNext) {
        if (L.mode == kLaneNext)
            lane_next(L, c);
        else
            lane_enter(L, c);
    }
}

}  // namespace dev

// Launch shape of the single-volume flat kernel.
struct FlatLaunch {
    bool persistent = false;
    uint64_t* counter = nullptr;     // persistent: work counter (zeroed by the launch)
    int block = 64;
    uint32_t refill_min = 8;
    bool local_stack = false;        // descent stack in local memory instead of shared
    const uint32_t* perm = nullptr;  // octant-sorted order (from launch_octant_sort), or null
    uint32_t steps = 1;              // ESVO steps per outer loop iteration
    bool registers56 = false;        // persistent local-stack form held to 56 registers
};

}  // namespace cbq

struct cbq_dag;
namespace cbq {
cbq_status launch_flat(const cbq_dag* dag, const dev::DagParams& dp, const dev::QueryParams& q,
                       const dev::HitsOut& out, const float4* orig, const float4* dir, uint64_t n,
                       uint32_t* fetch_out, const FlatLaunch& fl, cudaStream_t stream);
// Groups ray indices by octant (direction sign bits) into perm[n]; counts16 is
// 16 uint32 of scratch (zeroed here).
cbq_status launch_octant_sort(const float4* dir, uint64_t n, uint32_t* counts16, uint32_t* perm, int device,
                              cudaStream_t stream);
bool float_positions_exact(const cbq_dag* dag);
// Loads every persistent flat traversal kernel on the current device.
cbq_status preload_persistent_kernels();
}  // namespace cbq
