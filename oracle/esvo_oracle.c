/*
 * CPU oracle for the sparse-voxel-DAG ray traversal.  TEST INFRASTRUCTURE ONLY:
 * only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
 * it, always as the checker, never as the product path.
 *
 * A plain-C restatement of the reference's ESVO ray cast.  The floating-point
 * operations are the reference's, in the reference's order, one rounding per
 * operation (build with -ffp-contract=off), so results are bit-identical to
 * src/library/raytracing.cpp compiled the same way.  Integer state is kept as
 * bitmasks and scalars rather than the reference's Vec3<int>; every integer
 * operation on positions wraps modulo 2^32 as the reference's i32 arithmetic
 * does in practice.
 *
 * Deviations, all confined to cases where the reference hangs or reads
 * uninitialised memory:
 *   - the descent stack starts zeroed (the reference leaves it uninitialised;
 *     a read of a never-written slot needs a degenerate rounding tie);
 *   - an advance step that moves nowhere (a NaN slab from a zero direction
 *     component with the origin on a node plane) would repeat forever in the
 *     reference; here it ends the ray with status ORC_RAY_STUCK;
 *   - more than ORC_MAX_ITERATIONS node fetches end the ray with ORC_RAY_ITER_LIMIT.
 */
#include "esvo_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ---- helpers: reference semantics of std::min/std::max and GLSL findMSB ---- */

/* std::min(a, b) == (b < a) ? b : a; used by min3 (raytracing.cpp:168-171). */
static inline float fmin2_ref(float a, float b) { return (b < a) ? b : a; }
/* std::max(a, b) == (a < b) ? b : a; used by max3 (raytracing.cpp:173-176). */
static inline float fmax2_ref(float a, float b) { return (a < b) ? b : a; }
static inline float min3_ref(float x, float y, float z) { return fmin2_ref(fmin2_ref(x, y), z); }
static inline float max3_ref(float x, float y, float z) { return fmax2_ref(fmax2_ref(x, y), z); }

/* Unsigned findMSB: index of the highest set bit, -1 for 0 (raytracing.cpp:16-24). */
static inline int msb_u32(uint32_t v) { return v ? 31 - __builtin_clz(v) : -1; }

static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
/* (v >> h) << h with an arithmetic right shift, as i32 on the reference's targets. */
static inline int32_t floor_to_pow2(int32_t v, int h)
{
    int32_t s = v >> h;
    return (int32_t)((uint32_t)s << h);
}

static inline int32_t sat_f2i(float f)
{
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f < -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}

void orc_hit_voxel(const float p[3], const float nrm[3], int32_t v[3])
{
    for (int i = 0; i < 3; i++) {
        float half = 0.5f * nrm[i];
        float a = p[i] - half;
        float b = a + 0.5f;
        v[i] = sat_f2i(floorf(b));
    }
}

/* ---- findSubDAG / findSubDAGs (raytracing.cpp:43-97) ---- */

int orc_find_subdags(const uint32_t* nodes, uint64_t node_count, uint32_t root, orc_subdag out[8])
{
    if (root >= node_count) return -1;
    for (uint32_t oct = 0; oct < 8; oct++) {
        int height = 32;
        int32_t lb[3] = { INT32_MIN, INT32_MIN, INT32_MIN };
        uint32_t only = oct;
        uint32_t next = nodes[(uint64_t)root * 8 + only];
        uint32_t node = 0;
        uint32_t count = 1;
        while (count == 1) {
            height--;
            node = next;
            if (node >= node_count) return -2;
            lb[0] ^= (int32_t)((uint32_t)((only >> 0) & 1u) << height);
            lb[1] ^= (int32_t)((uint32_t)((only >> 1) & 1u) << height);
            lb[2] ^= (int32_t)((uint32_t)((only >> 2) & 1u) << height);
            count = 0;
            for (uint32_t i = 0; i < 8; i++) {
                uint32_t c = nodes[(uint64_t)node * 8 + i];
                if (c > 0) { next = c; count++; only = i; }
            }
            if (height == 0 && count == 1) break; /* cannot occur in a well-formed DAG */
        }
        memset(&out[oct], 0, sizeof(out[oct]));
        out[oct].lower[0] = lb[0];
        out[oct].lower[1] = lb[1];
        out[oct].lower[2] = lb[2];
        out[oct].height = height;
        out[oct].node = node;
    }
    return 0;
}

/* ---- per-ray traversal ---- */

typedef struct ray_ctx {
    const uint32_t* nodes;
    float o[3];       /* reflected origin: (origin + 0.5) * sign */
    float inv[3];     /* 1 / |dir| */
    float neg_sign[3];/* -rayDirSign, used for normals */
    uint32_t sign_bits;
    int compute_surface;
    float max_footprint;
    uint32_t fetches;
    uint32_t status;
    int fill_start;   /* never-written stack slots read as the walk's start node instead of 0 */
} ray_ctx;

typedef struct esvo_out {
    int hit;
    float distance;
    uint32_t material;
    float normal[3];
} esvo_out;

static inline uint32_t fetch(ray_ctx* r, uint32_t node, uint32_t slot)
{
    r->fetches++;
    return r->nodes[(uint64_t)node * 8 + slot];
}

/* findNearestMaterial (raytracing.cpp:134-162). */
static uint32_t nearest_material(ray_ctx* r, uint32_t node)
{
    const uint32_t order = (0x76534210u | 0x88888888u) ^ (r->sign_bits * 0x11111111u);
    while (node >= 256u) {
        uint32_t found = 0;
        for (uint32_t ids = order; ids != 0; ids >>= 4) {
            uint32_t c = fetch(r, node, ids & 7u);
            if (c > 0) { node = c; found = 1; break; }
        }
        if (r->fetches >= ORC_MAX_ITERATIONS) { r->status = ORC_RAY_ITER_LIMIT; return 0; }
        if (!found) continue; /* all-empty internal node: the reference spins; the cap ends it */
    }
    return node;
}

/* findFirstChild (raytracing.cpp:178-196), returning the child id as a 3-bit mask. */
static inline uint32_t first_child(const ray_ctx* r, float entry, int32_t cx, int32_t cy, int32_t cz)
{
    float mx = ((float)cx - r->o[0]) * r->inv[0];
    float my = ((float)cy - r->o[1]) * r->inv[1];
    float mz = ((float)cz - r->o[2]) * r->inv[2];
    uint32_t id = (mx < entry ? 1u : 0u) | (my < entry ? 2u : 0u) | (mz < entry ? 4u : 0u);
    if (entry <= 0.0f) {
        id |= (r->o[0] >= (float)cx ? 1u : 0u) | (r->o[1] >= (float)cy ? 2u : 0u) |
              (r->o[2] >= (float)cz ? 4u : 0u);
    }
    return id;
}

/* intersectRayNodeESVO (raytracing.cpp:213-371). */
static esvo_out esvo(ray_ctx* r, uint32_t node, int32_t px, int32_t py, int32_t pz, int height)
{
    esvo_out res;
    memset(&res, 0, sizeof(res));

    const uint32_t node_size = 1u << height;
    const float t0x = ((float)px - r->o[0]) * r->inv[0];
    const float t0y = ((float)py - r->o[1]) * r->inv[1];
    const float t0z = ((float)pz - r->o[2]) * r->inv[2];
    const float t1x = (((float)px + (float)node_size) - r->o[0]) * r->inv[0];
    const float t1y = (((float)py + (float)node_size) - r->o[1]) * r->inv[1];
    const float t1z = (((float)pz + (float)node_size) - r->o[2]) * r->inv[2];
    const float entry = max3_ref(t0x, t0y, t0z);
    const float exit_ = min3_ref(t1x, t1y, t1z);
    if (!(entry < exit_)) return res;

    const int start_h = height;
    int h = height;
    int32_t cns = (int32_t)(node_size / 2u);
    uint32_t cid = first_child(r, entry, wadd(px, cns), wadd(py, cns), wadd(pz, cns));
    int32_t cx = wadd(px, (cid & 1u) ? cns : 0);
    int32_t cy = wadd(py, (cid & 2u) ? cns : 0);
    int32_t cz = wadd(pz, (cid & 4u) ? cns : 0);
    float last_exit = exit_;
    uint32_t stack[33];
    for (int q = 0; q < 33; q++) stack[q] = r->fill_start ? node : 0u;

    do {
        const float c1x = ((float)wadd(cx, cns) - r->o[0]) * r->inv[0];
        const float c1y = ((float)wadd(cy, cns) - r->o[1]) * r->inv[1];
        const float c1z = ((float)wadd(cz, cns) - r->o[2]) * r->inv[2];
        const float tcx = min3_ref(c1x, c1y, c1z);

        if (r->fetches >= ORC_MAX_ITERATIONS) { r->status = ORC_RAY_ITER_LIMIT; res.hit = 0; return res; }
        const uint32_t child = fetch(r, node, cid ^ r->sign_bits);

        if (child > 0) {
            const float c0x = ((float)cx - r->o[0]) * r->inv[0];
            const float c0y = ((float)cy - r->o[1]) * r->inv[1];
            const float c0z = ((float)cz - r->o[2]) * r->inv[2];
            const float tce = max3_ref(c0x, c0y, c0z);
            const int internal = child >= 256u;
            const int large = ((float)cns / tcx) > r->max_footprint;
            if (internal && large) {
                if (tcx < last_exit) stack[h] = node;
                last_exit = tcx;
                h--;
                node = child;
                cns /= 2;
                cid = first_child(r, tce, wadd(cx, cns), wadd(cy, cns), wadd(cz, cns));
                cx = wadd(cx, (cid & 1u) ? cns : 0);
                cy = wadd(cy, (cid & 2u) ? cns : 0);
                cz = wadd(cz, (cid & 4u) ? cns : 0);
            } else {
                res.hit = 1;
                res.distance = tce;
                if (r->compute_surface) {
                    res.material = nearest_material(r, child);
                    if (r->status != ORC_RAY_OK) { res.hit = 0; return res; }
                    res.normal[0] = (tce == c0x ? 1.0f : 0.0f) * r->neg_sign[0];
                    res.normal[1] = (tce == c0y ? 1.0f : 0.0f) * r->neg_sign[1];
                    res.normal[2] = (tce == c0z ? 1.0f : 0.0f) * r->neg_sign[2];
                }
            }
        } else {
            const uint32_t flips = (c1x <= tcx ? 1u : 0u) | (c1y <= tcx ? 2u : 0u) | (c1z <= tcx ? 4u : 0u);
            if (flips == 0) { r->status = ORC_RAY_STUCK; res.hit = 0; return res; }
            cid ^= flips;
            const int32_t ox = cx, oy = cy, oz = cz;
            if (flips & 1u) cx = wadd(cx, cns);
            if (flips & 2u) cy = wadd(cy, cns);
            if (flips & 4u) cz = wadd(cz, cns);
            if ((cid & flips) != flips) {
                const uint32_t diff = (uint32_t)(ox ^ cx) | (uint32_t)(oy ^ cy) | (uint32_t)(oz ^ cz);
                const int msb = msb_u32(diff);
                h = msb + 1;
                if (h > start_h) break;          /* leaves the sub-DAG: loop ends */
                node = stack[h];
                cns = (int32_t)(1u << msb);
                cid = (uint32_t)((cx >> msb) & 1) | ((uint32_t)((cy >> msb) & 1) << 1) |
                      ((uint32_t)((cz >> msb) & 1) << 2);
                cx = wadd(floor_to_pow2(cx, h), (cid & 1u) ? cns : 0);
                cy = wadd(floor_to_pow2(cy, h), (cid & 2u) ? cns : 0);
                cz = wadd(floor_to_pow2(cz, h), (cid & 4u) ? cns : 0);
                last_exit = 0.0f;
            }
        }
    } while (!res.hit && h <= start_h);
    return res;
}

/* intersectVolume (raytracing.cpp:407-478). */
static void intersect_one(const uint32_t* nodes, const orc_subdag sd[8], const float* o4, const float* d4,
                          int cs, float mf, int use_tmax, const orc_hits* out, uint64_t i, uint32_t* fetches,
                          int fill_start)
{
    ray_ctx r;
    r.nodes = nodes;
    r.fill_start = fill_start;
    r.compute_surface = cs;
    r.max_footprint = mf;
    r.fetches = 0;
    r.status = ORC_RAY_OK;

    const float ox = o4[0], oy = o4[1], oz = o4[2];
    const float dx = d4[0], dy = d4[1], dz = d4[2];
    const uint32_t sbx = dx < 0.0f, sby = dy < 0.0f, sbz = dz < 0.0f;
    r.sign_bits = sbx | (sby << 1) | (sbz << 2);
    const float sx = (float)(1 - 2 * (int)sbx), sy = (float)(1 - 2 * (int)sby), sz = (float)(1 - 2 * (int)sbz);
    r.neg_sign[0] = -sx; r.neg_sign[1] = -sy; r.neg_sign[2] = -sz;
    r.o[0] = (ox + 0.5f) * sx;
    r.o[1] = (oy + 0.5f) * sy;
    r.o[2] = (oz + 0.5f) * sz;
    const float rdx = fabsf(dx), rdy = fabsf(dy), rdz = fabsf(dz);
    r.inv[0] = 1.0f / rdx;
    r.inv[1] = 1.0f / rdy;
    r.inv[2] = 1.0f / rdz;

    uint32_t oct = 0;
    float dist[3] = { (-r.o[0]) / rdx, (-r.o[1]) / rdy, (-r.o[2]) / rdz };
    if (dist[0] < 0.0f) { oct += 1; dist[0] += FLT_MAX; }
    if (dist[1] < 0.0f) { oct += 2; dist[1] += FLT_MAX; }
    if (dist[2] < 0.0f) { oct += 4; dist[2] += FLT_MAX; }

    esvo_out res;
    memset(&res, 0, sizeof(res));
    float pos[3] = { 0.0f, 0.0f, 0.0f };
    do {
        const orc_subdag* s = &sd[oct ^ r.sign_bits];
        if (s->node > 0) {
            const int32_t ns = (int32_t)(1u << s->height);
            const int32_t lx = wsub(wmul(s->lower[0], (int32_t)sx), (int32_t)sbx * ns);
            const int32_t ly = wsub(wmul(s->lower[1], (int32_t)sy), (int32_t)sby * ns);
            const int32_t lz = wsub(wmul(s->lower[2], (int32_t)sz), (int32_t)sbz * ns);
            res = esvo(&r, s->node, lx, ly, lz, s->height);
            if (r.status != ORC_RAY_OK) { memset(&res, 0, sizeof(res)); break; }
            if (res.hit) {
                const float t = res.distance;
                const float mx = dx * t, my = dy * t, mz = dz * t;
                pos[0] = ox + mx;
                pos[1] = oy + my;
                pos[2] = oz + mz;
                break;
            }
        }
        const float md = min3_ref(dist[0], dist[1], dist[2]);
        const uint32_t before = oct;
        if (dist[0] <= md) { oct += 1; dist[0] += FLT_MAX; }
        if (dist[1] <= md) { oct += 2; dist[1] += FLT_MAX; }
        if (dist[2] <= md) { oct += 4; dist[2] += FLT_MAX; }
        if (oct == before) { /* NaN distances: the reference would revisit this octant forever */
            r.status = ORC_RAY_STUCK;
            memset(&res, 0, sizeof(res));
            break;
        }
    } while (oct <= 7);

    if (use_tmax && res.hit && !(res.distance <= o4[3])) {
        memset(&res, 0, sizeof(res));
        pos[0] = pos[1] = pos[2] = 0.0f;
    }

    if (out) {
        if (out->hit) out->hit[i] = (uint8_t)res.hit;
        if (out->distance) out->distance[i] = res.distance;
        if (out->material) out->material[i] = res.material;
        if (out->position) { out->position[3 * i] = pos[0]; out->position[3 * i + 1] = pos[1]; out->position[3 * i + 2] = pos[2]; }
        if (out->normal) { out->normal[3 * i] = res.normal[0]; out->normal[3 * i + 1] = res.normal[1]; out->normal[3 * i + 2] = res.normal[2]; }
        if (out->voxel) {
            int32_t v[3] = { 0, 0, 0 };
            if (res.hit) orc_hit_voxel(pos, res.normal, v);
            out->voxel[3 * i] = v[0]; out->voxel[3 * i + 1] = v[1]; out->voxel[3 * i + 2] = v[2];
        }
        if (out->status) out->status[i] = (uint8_t)r.status;
    }
    if (fetches) fetches[i] = r.fetches;
}

/* ---- double-precision brute-force oracle ---- */

typedef struct fp64_ctx {
    const uint32_t* nodes;
    double o[3], d[3], inv[3];
    double best;
    uint32_t material;
    uint32_t sign_bits;
} fp64_ctx;

/* Exact slab test against [lo, hi]; returns 0 on a miss. */
static int slab64(const fp64_ctx* c, const double lo[3], const double hi[3], double* entry, double* exit_)
{
    double tmin = -INFINITY, tmax = INFINITY;
    for (int a = 0; a < 3; a++) {
        if (c->d[a] == 0.0) {
            if (c->o[a] < lo[a] || c->o[a] > hi[a]) return 0;
            continue;
        }
        double t0 = (lo[a] - c->o[a]) * c->inv[a];
        double t1 = (hi[a] - c->o[a]) * c->inv[a];
        if (t0 > t1) { double tt = t0; t0 = t1; t1 = tt; }
        if (t0 > tmin) tmin = t0;
        if (t1 < tmax) tmax = t1;
    }
    *entry = tmin;
    *exit_ = tmax;
    return tmax >= tmin;
}

static void fp64_visit(fp64_ctx* c, uint32_t node, int64_t lx, int64_t ly, int64_t lz, int h)
{
    const double size = (double)((int64_t)1 << h);
    const double lo[3] = { (double)lx - 0.5, (double)ly - 0.5, (double)lz - 0.5 };
    const double hi[3] = { lo[0] + size, lo[1] + size, lo[2] + size };
    double en, ex;
    if (!slab64(c, lo, hi, &en, &ex)) return;
    if (ex <= 0.0) return;
    if (en >= c->best) return;
    if (node < 256u) {
        if (node > 0u) { c->best = en; c->material = node; }
        return;
    }
    if (h == 0) return;
    const int64_t half = (int64_t)1 << (h - 1);
    for (uint32_t k = 0; k < 8; k++) {
        const uint32_t cid = k ^ c->sign_bits; /* roughly near-to-far */
        const uint32_t child = c->nodes[(uint64_t)node * 8 + cid];
        if (child == 0) continue;
        fp64_visit(c, child, lx + ((cid & 1u) ? half : 0), ly + ((cid & 2u) ? half : 0),
                   lz + ((cid & 4u) ? half : 0), h - 1);
    }
}

static void trace64_one(const uint32_t* nodes, const orc_subdag sd[8], const float* o4, const float* d4,
                        uint8_t* hit, double* distance, uint32_t* material, uint64_t i)
{
    fp64_ctx c;
    c.nodes = nodes;
    for (int a = 0; a < 3; a++) {
        c.o[a] = (double)o4[a];
        c.d[a] = (double)d4[a];
        c.inv[a] = 1.0 / c.d[a];
    }
    c.sign_bits = (d4[0] < 0.0f ? 1u : 0u) | (d4[1] < 0.0f ? 2u : 0u) | (d4[2] < 0.0f ? 4u : 0u);
    c.best = INFINITY;
    c.material = 0;
    for (int k = 0; k < 8; k++) {
        if (sd[k].node == 0) continue;
        fp64_visit(&c, sd[k].node, sd[k].lower[0], sd[k].lower[1], sd[k].lower[2], sd[k].height);
    }
    const int h = c.material != 0;
    if (hit) hit[i] = (uint8_t)h;
    if (distance) distance[i] = h ? c.best : 0.0;
    if (material) material[i] = c.material;
}

/* ---- threading ---- */

typedef struct job {
    int kind; /* 0 intersect, 1 count fetches, 2 fp64 */
    const uint32_t* nodes;
    const orc_subdag* sd;
    const float* o4;
    const float* d4;
    uint64_t n;
    int cs;
    float mf;
    int use_tmax;
    const orc_hits* out;
    uint32_t* fetches;
    uint8_t* hit;
    double* dist64;
    uint32_t* mat;
    int fill_start;
    uint64_t next; /* atomic cursor */
} job;

#define ORC_CHUNK 1024u

static void* worker(void* arg)
{
    job* j = (job*)arg;
    for (;;) {
        uint64_t b = __atomic_fetch_add(&j->next, ORC_CHUNK, __ATOMIC_RELAXED);
        if (b >= j->n) break;
        uint64_t e = b + ORC_CHUNK < j->n ? b + ORC_CHUNK : j->n;
        for (uint64_t i = b; i < e; i++) {
            if (j->kind == 2)
                trace64_one(j->nodes, j->sd, j->o4 + 4 * i, j->d4 + 4 * i, j->hit, j->dist64, j->mat, i);
            else
                intersect_one(j->nodes, j->sd, j->o4 + 4 * i, j->d4 + 4 * i, j->cs, j->mf, j->use_tmax,
                              j->kind == 0 ? j->out : NULL, i, j->fetches, j->fill_start);
        }
    }
    return NULL;
}

static int run_job(job* j, int nthreads)
{
    if (nthreads <= 0) {
        long c = sysconf(_SC_NPROCESSORS_ONLN);
        nthreads = c > 0 ? (int)c : 1;
    }
    if (nthreads > 1024) nthreads = 1024;
    j->next = 0;
    if (nthreads == 1) { worker(j); return 0; }
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    if (!th) return -1;
    int started = 0;
    for (int t = 0; t < nthreads; t++) {
        if (pthread_create(&th[t], NULL, worker, j) != 0) break;
        started++;
    }
    if (started == 0) worker(j);
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
    free(th);
    return 0;
}

static int check_nodes(const uint32_t* nodes, uint64_t node_count, const orc_subdag sd[8])
{
    if (!nodes || node_count < 256) return -1;
    for (int k = 0; k < 8; k++) {
        if (sd[k].node >= node_count || sd[k].height < 0 || sd[k].height > 31) return -2;
    }
    const uint64_t words = node_count * 8u;
    for (uint64_t w = 0; w < words; w++)
        if (nodes[w] >= node_count) return -3;
    return 0;
}

int orc_intersect_batch_ex(const uint32_t* nodes, uint64_t node_count, const orc_subdag subdags[8],
                           const float* orig4, const float* dir4, uint64_t n, int compute_surface,
                           float max_footprint, int use_tmax, const orc_hits* out, int nthreads,
                           int unwritten_slot_is_start_node)
{
    int rc = check_nodes(nodes, node_count, subdags);
    if (rc) return rc;
    job j;
    memset(&j, 0, sizeof(j));
    j.kind = 0; j.nodes = nodes; j.sd = subdags; j.o4 = orig4; j.d4 = dir4; j.n = n;
    j.cs = compute_surface; j.mf = max_footprint; j.use_tmax = use_tmax; j.out = out;
    j.fill_start = unwritten_slot_is_start_node;
    return run_job(&j, nthreads);
}

int orc_intersect_batch(const uint32_t* nodes, uint64_t node_count, const orc_subdag subdags[8],
                        const float* orig4, const float* dir4, uint64_t n, int compute_surface,
                        float max_footprint, int use_tmax, const orc_hits* out, int nthreads)
{
    return orc_intersect_batch_ex(nodes, node_count, subdags, orig4, dir4, n, compute_surface, max_footprint,
                                  use_tmax, out, nthreads, 0);
}

int orc_count_fetches(const uint32_t* nodes, uint64_t node_count, const orc_subdag subdags[8],
                      const float* orig4, const float* dir4, uint64_t n, int compute_surface,
                      float max_footprint, uint32_t* fetches_out, int nthreads)
{
    int rc = check_nodes(nodes, node_count, subdags);
    if (rc) return rc;
    job j;
    memset(&j, 0, sizeof(j));
    j.kind = 1; j.nodes = nodes; j.sd = subdags; j.o4 = orig4; j.d4 = dir4; j.n = n;
    j.cs = compute_surface; j.mf = max_footprint; j.fetches = fetches_out;
    return run_job(&j, nthreads);
}

int orc_trace_fp64_batch(const uint32_t* nodes, uint64_t node_count, const orc_subdag subdags[8],
                         const float* orig4, const float* dir4, uint64_t n, uint8_t* hit,
                         double* distance, uint32_t* material, int nthreads)
{
    int rc = check_nodes(nodes, node_count, subdags);
    if (rc) return rc;
    job j;
    memset(&j, 0, sizeof(j));
    j.kind = 2; j.nodes = nodes; j.sd = subdags; j.o4 = orig4; j.d4 = dir4; j.n = n;
    j.hit = hit; j.dist64 = distance; j.mat = material;
    return run_job(&j, nthreads);
}
