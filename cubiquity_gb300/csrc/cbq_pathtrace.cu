// Wavefront pathtracer on top of the traversal (cbq_pathtrace).
//
// Restates the reference's CPU pathtracer (pathtracing_demo.cpp:81-190:
// traceSingleRayRecurse / gatherLighting) as GPU waves.  Per pass (as many
// samples per pixel as fit in kPtRaysPerPass paths, traced together):
//   camera rays -> [extension traversal -> shade -> shadow traversal -> add]
//   repeated for depth 0..bounces
// Shading follows the reference: a hit multiplies the path throughput by the
// material's colour and gathers direct light from a sun shadow ray (offset
// 0.001 along the normal, pathtracing_demo.cpp:83-97) and a sky shadow ray in
// the direction normalize(normal + random point in the unit sphere) (:99-114);
// the bounce ray starts 0.01 along the normal (:166) in the same kind of
// direction; a miss returns the background colour.  Materials may also emit.
// All traversals use the library's traversal with the LOD footprint given
// (the demo uses 0.0035, pathtracing_demo.h:84), computeSurfaceProperties on
// extension rays and off on shadow rays, exactly as the reference calls it.
// Random numbers come from a counter-based hash of (seed, pixel, sample,
// depth, purpose), so a frame is reproducible.
#include "cbq_internal.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

struct PathState {
    uint32_t pixel, sample;
    float tr, tg, tb;  // throughput
};

// Paths traced together in one pass: the samples of a pass share each wave's
// launches (fewer, larger launches; one host round trip per depth and pass).
constexpr uint64_t kPtRaysPerPass = 1ull << 24;

struct Frame {
    int width, height;
    uint32_t sample, samples;  // the pass's first sample and its sample count
    uint64_t seed;
    float ex, ey, ez;              // eye
    float fx, fy, fz;              // forward
    float rx, ry, rz;              // right
    float ux, uy, uz;              // up
    float tan_half, aspect;
};

struct Shading {
    float max_footprint;
    float sun[3], sun_colour[3], sky_colour[3], background[3];
    float albedo[256][3];
    float emission[256][3];
};

__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

__device__ __forceinline__ uint64_t rng_key(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t depth,
                                            uint32_t purpose)
{
    return mix64(seed ^ mix64(((uint64_t)pixel << 32) | ((uint64_t)sample << 8) | (depth << 4) | purpose));
}

__device__ __forceinline__ float u01(uint64_t& h)
{
    h = mix64(h + 0x9e3779b97f4a7c15ull);
    return (float)(h >> 40) * (1.0f / 16777216.0f);
}

// A point uniformly inside the unit sphere: direction from two uniforms
// (sincospif), radius from the cube root of a third.
__device__ __forceinline__ float3 in_unit_sphere(uint64_t h)
{
    const float z = 1.0f - 2.0f * u01(h);
    const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float s, c;
    sincospif(2.0f * u01(h), &s, &c);
    const float rad = cbrtf(u01(h));
    return make_float3(r * c * rad, r * s * rad, z * rad);
}

__device__ __forceinline__ float3 normalize3(float3 v)
{
    const float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return l > 0.0f ? make_float3(v.x / l, v.y / l, v.z / l) : make_float3(0.0f, 0.0f, 1.0f);
}

// Path i of a pass: pixel i % npix of sample f.sample + i / npix.
__global__ void cbq_k_pt_camera(Frame f, float4* __restrict__ o, float4* __restrict__ d, PathState* __restrict__ st)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t npix = (uint32_t)f.width * (uint32_t)f.height;
    if (i >= npix * f.samples) return;
    const uint32_t pixel = i % npix, sample = f.sample + i / npix;
    const uint32_t px = pixel % (uint32_t)f.width, py = pixel / (uint32_t)f.width;
    uint64_t h = rng_key(f.seed, pixel, sample, 0, 0);
    const float jx = u01(h), jy = u01(h);
    const float sx = (((px + jx) / f.width) * 2.0f - 1.0f) * f.aspect * f.tan_half;
    const float sy = (1.0f - ((py + jy) / f.height) * 2.0f) * f.tan_half;
    const float3 dir = normalize3(make_float3(f.fx + f.rx * sx + f.ux * sy, f.fy + f.ry * sx + f.uy * sy,
                                              f.fz + f.rz * sx + f.uz * sy));
    o[i] = make_float4(f.ex, f.ey, f.ez, __int_as_float(0x7f800000));
    d[i] = make_float4(dir.x, dir.y, dir.z, 0.0f);
    st[i] = PathState{pixel, sample, 1.0f, 1.0f, 1.0f};
}

// Contributions are never negative and the image starts at +0, so adding a zero
// changes nothing: black contributions (most materials emit nothing) are skipped.
__device__ __forceinline__ void add_pixel(float* image, uint32_t pixel, float r, float g, float b)
{
    if (r == 0.0f && g == 0.0f && b == 0.0f) return;
    atomicAdd(image + 3 * (size_t)pixel, r);
    atomicAdd(image + 3 * (size_t)pixel + 1, g);
    atomicAdd(image + 3 * (size_t)pixel + 2, b);
}

// Reserves the warp's slots in both compacted arrays with one 64-bit atomic
// (all 32 lanes call it): two shadow rays per hit in the low word of `counts`
// (the shadow count), one bounce ray per continuing path in the high word (the
// bounce count).  A lane's shadow rays are slots s0 and s0 + 1.  One atomic
// round trip per warp instead of three in a row: the kernel waits on memory.
__device__ __forceinline__ void reserve_slots(unsigned long long* counts, bool hit, bool cont, uint32_t& s0,
                                              uint32_t& b)
{
    const unsigned hm = __ballot_sync(0xffffffffu, hit), cm = __ballot_sync(0xffffffffu, cont);
    const unsigned lane = threadIdx.x & 31u, below = (1u << lane) - 1u;
    unsigned long long base = 0;
    if (lane == 0 && (hm | cm))
        base = atomicAdd(counts, 2ull * (unsigned)__popc(hm) | ((unsigned long long)(unsigned)__popc(cm) << 32));
    base = __shfl_sync(0xffffffffu, base, 0);
    s0 = (uint32_t)base + 2u * (uint32_t)__popc(hm & below);
    b = (uint32_t)(base >> 32) + (uint32_t)__popc(cm & below);
}

__global__ void cbq_k_pt_shade(const Shading* __restrict__ sh, uint32_t n, uint32_t depth, uint64_t seed, int last, const PathState* __restrict__ st,
                               const uint8_t* __restrict__ hit, const uint32_t* __restrict__ material,
                               const float* __restrict__ position, const float* __restrict__ normal,
                               float* __restrict__ image, float4* __restrict__ so, float4* __restrict__ sd,
                               float4* __restrict__ sw, unsigned long long* __restrict__ counts,
                               float4* __restrict__ no, float4* __restrict__ nd, PathState* __restrict__ nst)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    PathState p{0u, 0u, 0.0f, 0.0f, 0.0f};
    bool h = false;
    if (live) {
        p = st[i];
        h = hit[i] != 0;
        if (!h) add_pixel(image, p.pixel, p.tr * sh->background[0], p.tg * sh->background[1], p.tb * sh->background[2]);
    }
    float3 pos = make_float3(0.0f, 0.0f, 0.0f), nrm = make_float3(0.0f, 0.0f, 0.0f);
    float tr = 0.0f, tg = 0.0f, tb = 0.0f;
    uint64_t key = 0;
    if (h) {
        const uint32_t m = material[i] & 255u;
        pos = make_float3(position[3 * i], position[3 * i + 1], position[3 * i + 2]);
        nrm = make_float3(normal[3 * i], normal[3 * i + 1], normal[3 * i + 2]);
        add_pixel(image, p.pixel, p.tr * sh->emission[m][0], p.tg * sh->emission[m][1], p.tb * sh->emission[m][2]);
        tr = p.tr * sh->albedo[m][0];
        tg = p.tg * sh->albedo[m][1];
        tb = p.tb * sh->albedo[m][2];
        key = rng_key(seed, p.pixel, p.sample, depth + 1, 0);
    }
    // Two shadow rays per hit (sun and sky) and a bounce ray per continuing path.
    const bool cont = h && !last;
    uint32_t s0 = 0, b = 0;
    reserve_slots(counts, h, cont, s0, b);
    const uint32_t s1 = s0 + 1u;
    if (h) {
        const float3 off = make_float3(nrm.x * 0.001f, nrm.y * 0.001f, nrm.z * 0.001f);
        const float3 org = make_float3(pos.x + off.x, pos.y + off.y, pos.z + off.z);
        const float sdot = fmaxf(sh->sun[0] * nrm.x + sh->sun[1] * nrm.y + sh->sun[2] * nrm.z, 0.0f);
        so[s0] = make_float4(org.x, org.y, org.z, __int_as_float(0x7f800000));
        sd[s0] = make_float4(sh->sun[0], sh->sun[1], sh->sun[2], 0.0f);
        sw[s0] = make_float4(tr * sh->sun_colour[0] * sdot, tg * sh->sun_colour[1] * sdot, tb * sh->sun_colour[2] * sdot,
                             __uint_as_float(p.pixel));
        const float3 q = in_unit_sphere(mix64(key ^ 1u));
        const float3 sky = normalize3(make_float3(nrm.x + q.x, nrm.y + q.y, nrm.z + q.z));
        so[s1] = make_float4(org.x, org.y, org.z, __int_as_float(0x7f800000));
        sd[s1] = make_float4(sky.x, sky.y, sky.z, 0.0f);
        sw[s1] = make_float4(tr * sh->sky_colour[0], tg * sh->sky_colour[1], tb * sh->sky_colour[2],
                             __uint_as_float(p.pixel));
    }
    // The bounce ray.
    if (cont) {
        const float3 q = in_unit_sphere(mix64(key ^ 2u));
        const float3 dir = normalize3(make_float3(nrm.x + q.x, nrm.y + q.y, nrm.z + q.z));
        no[b] = make_float4(pos.x + nrm.x * 0.01f, pos.y + nrm.y * 0.01f, pos.z + nrm.z * 0.01f,
                            __int_as_float(0x7f800000));
        nd[b] = make_float4(dir.x, dir.y, dir.z, 0.0f);
        nst[b] = PathState{p.pixel, p.sample, tr, tg, tb};
    }
}

__global__ void cbq_k_pt_shadow_add(uint32_t n, const uint8_t* __restrict__ hit, const float4* __restrict__ sw,
                                    float* __restrict__ image)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || hit[i]) return;
    const float4 w = sw[i];
    add_pixel(image, __float_as_uint(w.w), w.x, w.y, w.z);
}

__global__ void cbq_k_pt_scale(float* image, size_t count, float scale)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) image[i] *= scale;
}

template <typename T>
T* carve(char*& p, size_t count)
{
    T* r = (T*)p;
    p += (count * sizeof(T) + 255) & ~(size_t)255;
    return r;
}

}  // namespace

extern "C" cbq_status cbq_copy_to_host(void* host_dst, const void* device_src, uint64_t bytes)
{
    if (bytes == 0) return CBQ_OK;
    if (!host_dst || !device_src) return CBQ_ERR_INVALID_ARGUMENT;
    return cudaMemcpy(host_dst, device_src, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

extern "C" cbq_status cbq_pathtrace(const cbq_dag* dag, const cbq_pt_config* cfg, float* device_image,
                                    cbq_pt_wave_fn on_wave, void* user, cbq_pt_stats* stats, cbq_stream_t cstream)
{
    if (!dag || !cfg || !device_image || !cfg->materials) return CBQ_ERR_INVALID_ARGUMENT;
    if (cfg->width <= 0 || cfg->height <= 0 || cfg->samples_per_pixel <= 0 || cfg->bounces < 0 ||
        cfg->bounces > 64)
        return CBQ_ERR_INVALID_ARGUMENT;
    const uint64_t npix = (uint64_t)cfg->width * (uint64_t)cfg->height;
    if (npix > (1u << 30)) return CBQ_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)cstream;
    const auto t_start = std::chrono::steady_clock::now();

    // Camera basis (z up), as cbq_gen_pinhole_rays.
    double f[3] = {cfg->target[0] - cfg->eye[0], cfg->target[1] - cfg->eye[1], cfg->target[2] - cfg->eye[2]};
    const double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fl > 0)) return CBQ_ERR_INVALID_ARGUMENT;
    for (double& v : f) v /= fl;
    double r[3] = {f[1], -f[0], 0.0};
    const double rl = std::sqrt(r[0] * r[0] + r[1] * r[1]);
    if (!(rl > 0)) return CBQ_ERR_INVALID_ARGUMENT;
    r[0] /= rl;
    r[1] /= rl;
    const double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};

    Shading host_sh;
    host_sh.max_footprint = cfg->max_footprint;
    for (int a = 0; a < 3; a++) {
        host_sh.sun[a] = cfg->sun_direction[a];
        host_sh.sun_colour[a] = cfg->sun_colour[a];
        host_sh.sky_colour[a] = cfg->sky_colour[a];
        host_sh.background[a] = cfg->background[a];
    }
    for (int m = 0; m < 256; m++)
        for (int a = 0; a < 3; a++) {
            host_sh.albedo[m][a] = cfg->materials[m].albedo[a];
            host_sh.emission[m][a] = cfg->materials[m].emission[a];
        }

    // Buffers for one pass: two extension sets (ping-pong) and the shadow set.
    const uint64_t per_pass = std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)cfg->samples_per_pixel, kPtRaysPerPass / npix));
    const size_t ext = npix * per_pass, sha = 2 * ext;
    const size_t per_ext = 2 * 16 + sizeof(PathState) + 1 + 4 + 12 + 12;
    const size_t bytes = 2 * (ext * per_ext) + sha * (16 * 3 + 1) + sizeof(Shading) + 32 * 256;  // + carve padding
    char* base = nullptr;
    if (cudaMalloc((void**)&base, bytes) != cudaSuccess) {
        cudaGetLastError();
        return CBQ_ERR_OUT_OF_MEMORY;
    }
    char* p = base;
    Shading* d_sh = carve<Shading>(p, 1);
    uint32_t* counters = carve<uint32_t>(p, 8);           // [0] shadow count, [1] next count (one 64-bit word)
    uint64_t* work = carve<uint64_t>(p, 4);
    struct Ext {
        float4 *o, *d;
        PathState* st;
        uint8_t* hit;
        uint32_t* material;
        float *position, *normal;
    } e[2];
    for (int k = 0; k < 2; k++) {
        e[k].o = carve<float4>(p, ext);
        e[k].d = carve<float4>(p, ext);
        e[k].st = carve<PathState>(p, ext);
        e[k].hit = carve<uint8_t>(p, ext);
        e[k].material = carve<uint32_t>(p, ext);
        e[k].position = carve<float>(p, 3 * ext);
        e[k].normal = carve<float>(p, 3 * ext);
    }
    float4* so = carve<float4>(p, sha);
    float4* sd = carve<float4>(p, sha);
    float4* sw = carve<float4>(p, sha);
    uint8_t* shit = carve<uint8_t>(p, sha);
    if ((size_t)(p - base) > bytes) {
        cudaFree(base);
        return CBQ_ERR_INVALID_ARGUMENT;
    }

    cbq_status st = CBQ_OK;
    uint64_t ext_rays = 0, shadow_rays = 0, launches = 0;
    auto fail = [&](cbq_status code) {
        st = code;
        cudaGetLastError();
    };
    if (cudaMemcpyAsync(d_sh, &host_sh, sizeof(Shading), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(device_image, 0, npix * 3 * sizeof(float), s) != cudaSuccess)
        fail(CBQ_ERR_CUDA);

    const cbq_query qext{1, cfg->max_footprint, 0u, 0u};
    const cbq_query qsh{0, cfg->max_footprint, 0u, 0u};
    // The camera wave's paths are the pass's samples' images stacked in row-major
    // order: the traversal may deal them to warps in image tiles.
    const cbq_query qcam{1, cfg->max_footprint, 0u, (uint32_t)cfg->width};
    for (int sample = 0; sample < cfg->samples_per_pixel && st == CBQ_OK; sample += (int)per_pass) {
        const uint32_t samples = (uint32_t)std::min<uint64_t>(per_pass, (uint64_t)(cfg->samples_per_pixel - sample));
        Frame fr;
        fr.width = cfg->width;
        fr.height = cfg->height;
        fr.sample = (uint32_t)sample;
        fr.samples = samples;
        fr.seed = cfg->seed;
        fr.ex = (float)cfg->eye[0];
        fr.ey = (float)cfg->eye[1];
        fr.ez = (float)cfg->eye[2];
        fr.fx = (float)f[0]; fr.fy = (float)f[1]; fr.fz = (float)f[2];
        fr.rx = (float)r[0]; fr.ry = (float)r[1]; fr.rz = (float)r[2];
        fr.ux = (float)u[0]; fr.uy = (float)u[1]; fr.uz = (float)u[2];
        fr.tan_half = (float)cfg->tan_half_fov;
        fr.aspect = (float)cfg->width / (float)cfg->height;
        const uint64_t paths = npix * samples;
        cbq_k_pt_camera<<<(unsigned)((paths + 255) / 256), 256, 0, s>>>(fr, e[0].o, e[0].d, e[0].st);
        launches++;
        uint32_t n = (uint32_t)paths;
        int cur = 0;
        for (int depth = 0; depth <= cfg->bounces && n > 0 && st == CBQ_OK; depth++) {
            Ext& E = e[cur];
            Ext& N = e[cur ^ 1];
            cbq_rays rays{(const float*)E.o, (const float*)E.d};
            cbq_hits hits{E.hit, nullptr, E.material, E.position, E.normal, nullptr, nullptr};
            const cbq_query* qe = depth == 0 ? &qcam : &qext;
            cbq_status ts = cbq_intersect_persistent(dag, &rays, n, qe, &hits, work, 0u, (cbq_stream_t)s);
            if (ts != CBQ_OK) { fail(ts); break; }
            ext_rays += n;
            launches++;
            if (on_wave) {
                if (cudaStreamSynchronize(s) != cudaSuccess) { fail(CBQ_ERR_CUDA); break; }
                on_wave(user, 0, depth, sample, (const float*)E.o, (const float*)E.d, n, &hits, qe);
            }
            if (cudaMemsetAsync(counters, 0, 8 * sizeof(uint32_t), s) != cudaSuccess) { fail(CBQ_ERR_CUDA); break; }
            const int last = depth == cfg->bounces;
            cbq_k_pt_shade<<<(n + 255) / 256, 256, 0, s>>>(d_sh, n, (uint32_t)depth, cfg->seed, last,
                                                          E.st, E.hit, E.material, E.position, E.normal, device_image,
                                                          so, sd, sw, (unsigned long long*)counters, N.o, N.d, N.st);
            launches++;
            uint32_t h_counts[2] = {0, 0};
            if (cudaMemcpyAsync(h_counts, counters, sizeof(h_counts), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess) {
                fail(CBQ_ERR_CUDA);
                break;
            }
            const uint32_t ns = h_counts[0];
            if (ns > 0) {
                cbq_rays srays{(const float*)so, (const float*)sd};
                cbq_hits shits{shit, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
                ts = cbq_intersect_persistent(dag, &srays, ns, &qsh, &shits, work + 1, 0u, (cbq_stream_t)s);
                if (ts != CBQ_OK) { fail(ts); break; }
                shadow_rays += ns;
                launches++;
                if (on_wave) {
                    if (cudaStreamSynchronize(s) != cudaSuccess) { fail(CBQ_ERR_CUDA); break; }
                    on_wave(user, 1, depth, sample, (const float*)so, (const float*)sd, ns, &shits, &qsh);
                }
                cbq_k_pt_shadow_add<<<(ns + 255) / 256, 256, 0, s>>>(ns, shit, sw, device_image);
                launches++;
            }
            n = h_counts[1];
            cur ^= 1;
        }
    }
    if (st == CBQ_OK) {
        const size_t cnt = npix * 3;
        cbq_k_pt_scale<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(device_image, cnt,
                                                                       1.0f / (float)cfg->samples_per_pixel);
        launches++;
        if (cudaStreamSynchronize(s) != cudaSuccess) fail(CBQ_ERR_CUDA);
    }
    cudaFree(base);
    if (stats) {
        stats->extension_rays = ext_rays;
        stats->shadow_rays = shadow_rays;
        stats->kernel_launches = launches;
        stats->milliseconds =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    }
    return st;
}
