// Host-side parts of the C ABI: DAG checks, SubDAGs, .dag I/O, scene building
// and ray generation.  Compiled with -ffp-contract=off so that ray generation
// gives identical floats on x86-64 and aarch64.
#include "cbq_builder.hpp"
#include "cbq_internal.hpp"

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <new>
#include <thread>
#include <vector>

namespace cbq {

cbq_status find_subdags(const uint32_t* nodes, uint64_t node_count, uint32_t root, cbq_subdag out[8])
{
    if (!nodes || !out || node_count < kMaterialCount || root >= node_count) return CBQ_ERR_BAD_DAG;
    for (uint32_t oct = 0; oct < 8; oct++) {
        // Follow single-child chains below root child `oct` to the first node
        // with more (or fewer) than one occupied child (raytracing.cpp:43-87).
        int height = kRootHeight;
        uint32_t lb[3] = {0x80000000u, 0x80000000u, 0x80000000u};
        uint32_t only = oct;
        uint32_t next = nodes[(uint64_t)root * 8 + only];
        uint32_t node = 0;
        uint32_t count = 1;
        while (count == 1) {
            height--;
            node = next;
            if (node >= node_count) return CBQ_ERR_BAD_DAG;
            for (int a = 0; a < 3; a++) lb[a] ^= ((only >> a) & 1u) << height;
            count = 0;
            for (uint32_t i = 0; i < 8; i++) {
                const uint32_t c = nodes[(uint64_t)node * 8 + i];
                if (c > 0) { next = c; count++; only = i; }
            }
            if (height == 0 && count == 1) return CBQ_ERR_BAD_DAG;
        }
        std::memset(&out[oct], 0, sizeof(cbq_subdag));
        for (int a = 0; a < 3; a++) out[oct].lower_bound[a] = (int32_t)lb[a];
        out[oct].node_height = height;
        out[oct].node_index = node;
    }
    return CBQ_OK;
}

cbq_status validate_nodes(const uint32_t* nodes, uint64_t node_count, uint32_t root)
{
    if (!nodes || node_count < kMaterialCount) return CBQ_ERR_INVALID_ARGUMENT;
    if (node_count > (uint64_t)UINT32_MAX + 1) return CBQ_ERR_BAD_DAG;
    if (root >= node_count) return CBQ_ERR_BAD_DAG;
    for (uint32_t m = 0; m < kMaterialCount; m++)
        for (int k = 0; k < 8; k++)
            if (nodes[8ull * m + k] != m) return CBQ_ERR_BAD_DAG;
    const uint64_t words = node_count * 8;
    const uint32_t lim = (uint32_t)std::min<uint64_t>(node_count - 1, UINT32_MAX);
    for (uint64_t w = 8ull * kMaterialCount; w < words; w++)
        if (nodes[w] > lim) return CBQ_ERR_BAD_DAG;
    return CBQ_OK;
}

namespace {
std::atomic<cbq_log_fn> g_log_fn{nullptr};
std::atomic<void*> g_log_user{nullptr};
}  // namespace

void log(int level, const char* fmt, ...)
{
    cbq_log_fn fn = g_log_fn.load();
    if (!fn) return;
    char buf[512];
    va_list args;
    va_start(args, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, args);
    va_end(args);
    fn(g_log_user.load(), level, buf);
}

cbq_status validate_heights(const uint32_t* nodes, uint64_t node_count, const cbq_subdag subdags[8])
{
    // Heights (0..31) at which each internal node has been reached.
    std::vector<uint32_t> seen(node_count, 0u);
    std::vector<std::pair<uint32_t, int>> todo;
    for (int k = 0; k < 8; k++)
        if (subdags[k].node_index >= kMaterialCount) todo.emplace_back(subdags[k].node_index, subdags[k].node_height);
    while (!todo.empty()) {
        const auto [n, h] = todo.back();
        todo.pop_back();
        if (h <= 0) return CBQ_ERR_BAD_DAG;  // an internal node where only voxels can be
        if (seen[n] & (1u << h)) continue;
        seen[n] |= 1u << h;
        for (int k = 0; k < 8; k++) {
            const uint32_t c = nodes[(uint64_t)n * 8 + k];
            if (c >= kMaterialCount) todo.emplace_back(c, h - 1);
        }
    }
    return CBQ_OK;
}

cbq_status build_compact(const uint32_t* nodes, uint64_t node_count, const cbq_subdag subdags[8],
                         std::vector<uint32_t>& store, uint32_t sd_ref[8])
{
    constexpr uint32_t kUnset = 0xffffffffu;
    constexpr uint64_t kMaxUnits = 1ull << 24;
    auto mask_of = [&](uint32_t n) {
        uint32_t m = 0;
        for (int k = 0; k < 8; k++)
            if (nodes[(uint64_t)n * 8 + k] != 0u) m |= 1u << k;
        return m;
    };
    // Internal nodes reachable from the SubDAG roots, breadth first (siblings
    // and the hot upper levels end up next to each other).
    std::vector<uint32_t> offset(node_count, kUnset);
    std::vector<uint32_t> order;
    uint64_t units = 1;  // unit 0 unused: every internal reference is >= 256
    uint32_t material_root[kMaterialCount];
    for (uint32_t m = 0; m < kMaterialCount; m++) material_root[m] = kUnset;
    for (int k = 0; k < 8; k++) {
        const uint32_t r = subdags[k].node_index;
        if (r == 0u) {
            sd_ref[k] = 0u;
        } else if (r < kMaterialCount) {  // uniform octant: a node with eight children r
            if (material_root[r] == kUnset) {
                material_root[r] = (uint32_t)units;
                units += 4;
            }
            sd_ref[k] = (material_root[r] << 8) | 0xffu;
        } else if (offset[r] == kUnset) {
            offset[r] = 0;  // queued
            order.push_back(r);
        }
    }
    for (size_t i = 0; i < order.size(); i++) {
        const uint32_t n = order[i];
        for (int k = 0; k < 8; k++) {
            const uint32_t c = nodes[(uint64_t)n * 8 + k];
            if (c >= kMaterialCount && offset[c] == kUnset) {
                offset[c] = 0;
                order.push_back(c);
            }
        }
    }
    for (const uint32_t n : order) {
        if (units >= kMaxUnits) return CBQ_ERR_CAPACITY;  // offsets must fit 24 bits
        offset[n] = (uint32_t)units;
        units += (__builtin_popcount(mask_of(n)) + 1) / 2;
    }
    if (units > kMaxUnits) return CBQ_ERR_CAPACITY;
    auto ref_of = [&](uint32_t c) { return c < kMaterialCount ? c : (offset[c] << 8) | mask_of(c); };
    try {
        store.assign(units * 2, 0u);
    } catch (const std::bad_alloc&) {
        return CBQ_ERR_OUT_OF_MEMORY;
    }
    for (uint32_t m = 1; m < kMaterialCount; m++)
        if (material_root[m] != kUnset)
            for (int k = 0; k < 8; k++) store[(uint64_t)material_root[m] * 2 + k] = m;
    for (const uint32_t n : order) {
        uint64_t w = (uint64_t)offset[n] * 2;
        for (int k = 0; k < 8; k++) {
            const uint32_t c = nodes[(uint64_t)n * 8 + k];
            if (c != 0u) store[w++] = ref_of(c);
        }
    }
    for (int k = 0; k < 8; k++)
        if (subdags[k].node_index >= kMaterialCount) sd_ref[k] = ref_of(subdags[k].node_index);
    return CBQ_OK;
}

}  // namespace cbq

using namespace cbq;

extern "C" {

const char* cbq_status_string(cbq_status s)
{
    switch (s) {
    case CBQ_OK: return "ok";
    case CBQ_ERR_INVALID_ARGUMENT: return "invalid argument";
    case CBQ_ERR_BAD_DAG: return "malformed DAG";
    case CBQ_ERR_OUT_OF_MEMORY: return "out of memory";
    case CBQ_ERR_CUDA: return "CUDA error";
    case CBQ_ERR_TIMEOUT: return "timeout";
    case CBQ_ERR_IO: return "I/O error";
    case CBQ_ERR_BUSY: return "busy";
    case CBQ_ERR_NOT_FOUND: return "not found";
    case CBQ_ERR_CANCELLED: return "cancelled";
    case CBQ_ERR_CAPACITY: return "request exceeds capacity";
    case CBQ_ERR_SHUTDOWN: return "shut down";
    }
    return "unknown status";
}

int cbq_abi_version(void) { return CBQ_ABI_VERSION; }

void cbq_set_log_handler(cbq_log_fn fn, void* user)
{
    g_log_user.store(user);
    g_log_fn.store(fn);
}

cbq_status cbq_dag_validate(const uint32_t* nodes, uint64_t node_count, uint32_t root)
{
    cbq_status st = validate_nodes(nodes, node_count, root);
    if (st != CBQ_OK) return st;
    cbq_subdag sd[8];
    st = find_subdags(nodes, node_count, root, sd);
    if (st != CBQ_OK) return st;
    return validate_heights(nodes, node_count, sd);
}

cbq_status cbq_find_subdags(const uint32_t* nodes, uint64_t node_count, uint32_t root, cbq_subdag out[8])
{
    return find_subdags(nodes, node_count, root, out);
}

void cbq_free(void* p) { std::free(p); }

cbq_status cbq_compact_store(const uint32_t* nodes, uint64_t node_count, uint32_t root, uint32_t** store,
                             uint64_t* words, uint32_t subdag_refs[8])
{
    if (!store || !words || !subdag_refs) return CBQ_ERR_INVALID_ARGUMENT;
    *store = nullptr;
    *words = 0;
    cbq_status st = validate_nodes(nodes, node_count, root);
    if (st != CBQ_OK) return st;
    cbq_subdag sd[8];
    st = find_subdags(nodes, node_count, root, sd);
    if (st == CBQ_OK) st = validate_heights(nodes, node_count, sd);
    if (st != CBQ_OK) return st;
    std::vector<uint32_t> v;
    st = build_compact(nodes, node_count, sd, v, subdag_refs);
    if (st != CBQ_OK) return st;
    *store = (uint32_t*)std::malloc(v.size() * sizeof(uint32_t));
    if (!*store) return CBQ_ERR_OUT_OF_MEMORY;
    std::memcpy(*store, v.data(), v.size() * sizeof(uint32_t));
    *words = v.size();
    return CBQ_OK;
}

cbq_status cbq_dag_voxel(const uint32_t* nodes, uint64_t node_count, uint32_t root, int32_t x, int32_t y,
                         int32_t z, uint8_t* material)
{
    if (!nodes || !material || root >= node_count) return CBQ_ERR_INVALID_ARGUMENT;
    // Volume::voxel (storage.cpp:481-499): unsigned positions, one bit per level.
    uint32_t ux = (uint32_t)x + 0x80000000u, uy = (uint32_t)y + 0x80000000u, uz = (uint32_t)z + 0x80000000u;
    uint32_t node = root;
    int guard = 0;
    while (node >= kMaterialCount) {
        if (++guard > 64) return CBQ_ERR_BAD_DAG;
        const uint32_t cid = (ux >> 31) | ((uy >> 31) << 1) | ((uz >> 31) << 2);
        ux <<= 1;
        uy <<= 1;
        uz <<= 1;
        node = nodes[(uint64_t)node * 8 + cid];
        if (node >= node_count) return CBQ_ERR_BAD_DAG;
    }
    *material = (uint8_t)node;
    return CBQ_OK;
}

cbq_status cbq_dag_save(const char* path, const uint32_t* nodes, uint64_t node_count, uint32_t root)
{
    if (!path || !nodes || node_count < kMaterialCount) return CBQ_ERR_INVALID_ARGUMENT;
    if (node_count - kMaterialCount > UINT32_MAX) return CBQ_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "wb");
    if (!f) return CBQ_ERR_IO;
    const uint32_t internal = (uint32_t)(node_count - kMaterialCount);
    bool ok = std::fwrite(&root, 4, 1, f) == 1 && std::fwrite(&internal, 4, 1, f) == 1;
    if (ok && internal) ok = std::fwrite(nodes + 8ull * kMaterialCount, 32, internal, f) == internal;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? CBQ_OK : CBQ_ERR_IO;
}

cbq_status cbq_dag_load(const char* path, uint32_t** nodes_out, uint64_t* node_count_out, uint32_t* root_out)
{
    if (!path || !nodes_out || !node_count_out || !root_out) return CBQ_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "rb");
    if (!f) return CBQ_ERR_IO;
    uint32_t root = 0, internal = 0;
    if (std::fread(&root, 4, 1, f) != 1 || std::fread(&internal, 4, 1, f) != 1) {
        std::fclose(f);
        return CBQ_ERR_BAD_DAG;
    }
    const uint64_t count = (uint64_t)internal + kMaterialCount;
    uint32_t* nodes = (uint32_t*)std::malloc(count * 32);
    if (!nodes) { std::fclose(f); return CBQ_ERR_OUT_OF_MEMORY; }
    for (uint32_t m = 0; m < kMaterialCount; m++)
        for (int k = 0; k < 8; k++) nodes[8ull * m + k] = m;
    const bool ok = internal == 0 || std::fread(nodes + 8ull * kMaterialCount, 32, internal, f) == internal;
    std::fclose(f);
    if (!ok) { std::free(nodes); return CBQ_ERR_BAD_DAG; }
    // Volume::load rebases the root by sharedNodesBegin() - MaterialCount (= 0).
    cbq_status st = validate_nodes(nodes, count, root);
    if (st != CBQ_OK) { std::free(nodes); return CBQ_ERR_BAD_DAG; }
    *nodes_out = nodes;
    *node_count_out = count;
    *root_out = root;
    return CBQ_OK;
}

cbq_status cbq_dag_reorder_bfs(const uint32_t* nodes, uint64_t node_count, uint32_t root, uint32_t* out_nodes,
                               uint64_t* out_count, uint32_t* out_root)
{
    if (!nodes || !out_nodes || !out_count || !out_root) return CBQ_ERR_INVALID_ARGUMENT;
    cbq_status st = validate_nodes(nodes, node_count, root);
    if (st != CBQ_OK) return st;
    std::vector<uint32_t> newidx(node_count, UINT32_MAX);
    std::vector<uint32_t> order;
    order.reserve(node_count);
    for (uint32_t m = 0; m < kMaterialCount; m++) newidx[m] = m;
    if (root >= kMaterialCount) {
        newidx[root] = kMaterialCount;
        order.push_back(root);
    }
    for (size_t head = 0; head < order.size(); head++) {
        const uint32_t n = order[head];
        for (int k = 0; k < 8; k++) {
            const uint32_t c = nodes[(uint64_t)n * 8 + k];
            if (newidx[c] == UINT32_MAX) {
                newidx[c] = (uint32_t)(kMaterialCount + order.size());
                order.push_back(c);
            }
        }
    }
    for (uint32_t m = 0; m < kMaterialCount; m++)
        for (int k = 0; k < 8; k++) out_nodes[8ull * m + k] = m;
    for (size_t i = 0; i < order.size(); i++)
        for (int k = 0; k < 8; k++)
            out_nodes[8ull * (kMaterialCount + i) + k] = newidx[nodes[(uint64_t)order[i] * 8 + k]];
    *out_count = kMaterialCount + order.size();
    *out_root = newidx[root];
    return CBQ_OK;
}

static std::unique_ptr<Scene> make_scene(cbq_scene_kind kind, int edge_log2, uint64_t seed, int param)
{
    if (edge_log2 < 3 || edge_log2 > 16) return nullptr;
    switch (kind) {
    case CBQ_SCENE_SPHERES: return make_sphere_scene(edge_log2, param > 0 ? param : 64, seed);
    case CBQ_SCENE_TERRAIN: return make_terrain_scene(edge_log2, seed);
    case CBQ_SCENE_CITY: return edge_log2 >= 7 ? make_city_scene(edge_log2, seed) : nullptr;
    }
    return nullptr;
}

cbq_status cbq_build_scene(cbq_scene_kind kind, int edge_log2, uint64_t seed, int param, int threads,
                           uint32_t** nodes_out, uint64_t* node_count_out, uint32_t* root_out)
{
    if (!nodes_out || !node_count_out || !root_out) return CBQ_ERR_INVALID_ARGUMENT;
    try {
        std::unique_ptr<Scene> scene = make_scene(kind, edge_log2, seed, param);
        if (!scene) return CBQ_ERR_INVALID_ARGUMENT;
        const auto t0 = std::chrono::steady_clock::now();
        NodeArray arr = build_dag(*scene, threads);
        cbq::log(CBQ_LOG_INFO, "built scene kind %d edge 2^%d seed %llu: %llu nodes in %.3f s", (int)kind, edge_log2,
                 (unsigned long long)seed, (unsigned long long)arr.node_count(),
                 std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
        uint32_t* out = (uint32_t*)std::malloc(arr.words.size() * 4);
        if (!out) return CBQ_ERR_OUT_OF_MEMORY;
        std::memcpy(out, arr.words.data(), arr.words.size() * 4);
        *nodes_out = out;
        *node_count_out = arr.node_count();
        *root_out = arr.root;
        return CBQ_OK;
    } catch (const std::bad_alloc&) {
        return CBQ_ERR_OUT_OF_MEMORY;
    } catch (...) {
        return CBQ_ERR_INVALID_ARGUMENT;
    }
}

cbq_status cbq_scene_voxels(cbq_scene_kind kind, int edge_log2, uint64_t seed, int param, int32_t x0, int32_t y0,
                            int32_t z0, int32_t sx, int32_t sy, int32_t sz, uint8_t* out)
{
    if (!out || sx < 0 || sy < 0 || sz < 0) return CBQ_ERR_INVALID_ARGUMENT;
    try {
        std::unique_ptr<Scene> scene = make_scene(kind, edge_log2, seed, param);
        if (!scene) return CBQ_ERR_INVALID_ARGUMENT;
        for (int32_t z = 0; z < sz; z++)
            for (int32_t y = 0; y < sy; y++)
                for (int32_t x = 0; x < sx; x++)
                    out[((size_t)z * sy + y) * sx + x] = scene->voxel(x0 + x, y0 + y, z0 + z);
        return CBQ_OK;
    } catch (...) {
        return CBQ_ERR_OUT_OF_MEMORY;
    }
}

cbq_status cbq_gen_pinhole_rays(const double eye[3], const double target[3], double tan_half_fov, int32_t width,
                                int32_t height, float* origin_tmax, float* direction)
{
    if (!eye || !target || !origin_tmax || !direction || width <= 0 || height <= 0) return CBQ_ERR_INVALID_ARGUMENT;
    double f[3] = {target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fl > 0)) return CBQ_ERR_INVALID_ARGUMENT;
    for (double& v : f) v /= fl;
    // right = normalize(cross(f, up)), up = (0, 0, 1); camUp = cross(right, f)
    double r[3] = {f[1], -f[0], 0.0};
    double rl = std::sqrt(r[0] * r[0] + r[1] * r[1]);
    if (!(rl > 0)) return CBQ_ERR_INVALID_ARGUMENT;
    r[0] /= rl;
    r[1] /= rl;
    const double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
    const double aspect = (double)width / (double)height;
    for (int32_t py = 0; py < height; py++) {
        for (int32_t px = 0; px < width; px++) {
            const double sx = (((px + 0.5) / width) * 2.0 - 1.0) * aspect * tan_half_fov;
            const double sy = (1.0 - ((py + 0.5) / height) * 2.0) * tan_half_fov;
            double d[3];
            for (int a = 0; a < 3; a++) d[a] = f[a] + r[a] * sx + u[a] * sy;
            const double dl = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            const size_t i = (size_t)py * width + px;
            for (int a = 0; a < 3; a++) {
                origin_tmax[4 * i + a] = (float)eye[a];
                direction[4 * i + a] = (float)(d[a] / dl);
            }
            origin_tmax[4 * i + 3] = std::numeric_limits<float>::infinity();
            direction[4 * i + 3] = 0.0f;
        }
    }
    return CBQ_OK;
}

static inline uint64_t splitmix(uint64_t x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

cbq_status cbq_gen_sphere_rays(const double lo[3], const double hi[3], uint64_t n, uint64_t seed, float* origin_tmax,
                                float* direction)
{
    if (!lo || !hi || !origin_tmax || !direction) return CBQ_ERR_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < n; i++) {
        uint64_t ctr = splitmix(seed ^ splitmix(i * 0x9e3779b97f4a7c15ull + 17));
        for (int a = 0; a < 3; a++) {
            ctr = splitmix(ctr);
            const double u = (double)(ctr >> 11) * (1.0 / 9007199254740992.0);
            origin_tmax[4 * i + a] = (float)(lo[a] + (hi[a] - lo[a]) * u);
        }
        origin_tmax[4 * i + 3] = std::numeric_limits<float>::infinity();
        for (;;) {
            double q[3];
            for (int a = 0; a < 3; a++) {
                ctr = splitmix(ctr);
                q[a] = (double)(ctr >> 11) * (2.0 / 9007199254740992.0) - 1.0;
            }
            const double q2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
            if (q2 >= 1.0 || q2 < 1e-6) continue;
            const double ql = std::sqrt(q2);
            for (int a = 0; a < 3; a++) direction[4 * i + a] = (float)(q[a] / ql);
            break;
        }
        direction[4 * i + 3] = 0.0f;
    }
    return CBQ_OK;
}

cbq_status cbq_gen_bounce_rays(const float* hit_position, const float* hit_normal, uint64_t hit_count, uint64_t n,
                               uint64_t seed, float* origin_tmax, float* direction)
{
    if (!hit_position || !hit_normal || !origin_tmax || !direction || (hit_count == 0 && n > 0))
        return CBQ_ERR_INVALID_ARGUMENT;
    const int nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    auto work = [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; i++) {
            const uint64_t j = i % hit_count;
            const float* p = hit_position + 3 * j;
            const float* nm = hit_normal + 3 * j;
            // origin = position + normal * 0.01f in float (pathtracing_demo.cpp:166)
            for (int a = 0; a < 3; a++) {
                const float off = nm[a] * 0.01f;
                origin_tmax[4 * i + a] = p[a] + off;
            }
            origin_tmax[4 * i + 3] = std::numeric_limits<float>::infinity();
            // u uniform on the unit sphere: rejection-sample the ball, project.
            uint64_t ctr = splitmix(seed ^ splitmix(i));
            double d[3];
            for (;;) {
                double q[3];
                for (int a = 0; a < 3; a++) {
                    ctr = splitmix(ctr);
                    q[a] = (double)(ctr >> 11) * (2.0 / 9007199254740992.0) - 1.0;
                }
                const double q2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
                if (q2 >= 1.0 || q2 < 1e-6) continue;
                const double ql = std::sqrt(q2);
                for (int a = 0; a < 3; a++) d[a] = (double)nm[a] + q[a] / ql;
                const double dl2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                if (dl2 < 1e-12) continue;
                const double dl = std::sqrt(dl2);
                for (int a = 0; a < 3; a++) d[a] /= dl;
                break;
            }
            for (int a = 0; a < 3; a++) direction[4 * i + a] = (float)d[a];
            direction[4 * i + 3] = 0.0f;
        }
    };
    std::vector<std::thread> pool;
    const uint64_t per = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        const uint64_t b = per * t, e = std::min<uint64_t>(n, b + per);
        if (b >= e) break;
        pool.emplace_back(work, b, e);
    }
    for (auto& th : pool) th.join();
    return CBQ_OK;
}

}  // extern "C"
