// cbq_intersect_host_noalloc: the host-buffer traversal without any device
// allocation.
//
// cbq_intersect_host stages rays and hits in device buffers it allocates with
// cudaMalloc (and grows on demand).  Some callers cannot allow that: a render or
// physics thread with a frame deadline (cudaMalloc can synchronise the whole
// device and stall every stream), or a host application that owns all device
// memory through its own allocator and forbids libraries from allocating.
// This entry point keeps its staging buffers and the persistent kernel's work
// counter in one file-scope __device__ array instead, of fixed size: requests
// of more than CBQ_NOALLOC_MAX_RAYS rays are refused with CBQ_ERR_CAPACITY.
//
// The array takes device memory when the module that holds it is loaded on a
// device, which (with CUDA's lazy module loading) is the first lookup of its
// address there.  cbq_dag_create does that lookup (noalloc_prepare), so the
// array is in place before any call of this entry point can name a DAG.
#include "cbq_internal.hpp"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr uint64_t kMaxRays = CBQ_NOALLOC_MAX_RAYS;
constexpr size_t kRayBytes = 32;                                       // two float4
constexpr size_t kHitBytes = 1 + 4 + 4 + 12 + 12 + 12 + 1;             // all hit fields
constexpr size_t kScratchBytes = kMaxRays * (kRayBytes + kHitBytes) + 256;

// One array per device on which a DAG was created, held until the process
// exits.  In host code this name is only a stand-in for the device symbol: its
// device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_cbq_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_lock;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `device`, which must be current;
// looked up once per device.
cbq_status scratch_address(int device, void** out)
{
    if (device < 0 || device >= kMaxDevices) return CBQ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_setup_lock);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_cbq_noalloc_scratch) != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return CBQ_ERR_CUDA;
        }
        g_scratch_addr[device] = p;
    }
    *out = g_scratch_addr[device];
    return CBQ_OK;
}

}  // namespace

namespace cbq {

cbq_status noalloc_prepare(int device)
{
    void* p = nullptr;
    return scratch_address(device, &p);
}

}  // namespace cbq

extern "C" cbq_status cbq_intersect_host_noalloc(const cbq_dag* dag, const float* host_origin_tmax,
                                                 const float* host_direction, uint64_t n, const cbq_query* query,
                                                 const cbq_hits* host_hits)
{
    if (!dag || !host_origin_tmax || !host_direction || !host_hits) return CBQ_ERR_INVALID_ARGUMENT;
    if (n > kMaxRays) return CBQ_ERR_CAPACITY;
    if (n == 0) return CBQ_OK;
    int device = -1;
    if (cudaGetDevice(&device) != cudaSuccess) return CBQ_ERR_CUDA;
    if (device != dag->device) return CBQ_ERR_INVALID_ARGUMENT;  // the DAG lives on another device
    void* base = nullptr;
    cbq_status st = scratch_address(device, &base);  // resolved when the DAG was created
    if (st != CBQ_OK) return st;

    // Carve the array: rays, hit fields, then the work counter.  Every region
    // is fully rewritten by each call (rays by the copies, hits by the kernel
    // for all n rays), except the counter, which the launch zeroes.
    char* p = (char*)base;
    float* d_o = (float*)p;
    p += n * 16;
    float* d_d = (float*)p;
    p += n * 16;
    cbq_hits dh;
    dh.position = (float*)p; p += n * 12;
    dh.normal = (float*)p; p += n * 12;
    dh.voxel = (int32_t*)p; p += n * 12;
    dh.distance = (float*)p; p += n * 4;
    dh.material = (uint32_t*)p; p += n * 4;
    dh.hit = (uint8_t*)p; p += n;
    dh.status = (uint8_t*)p; p += n;
    uint64_t* d_counter = (uint64_t*)(((uintptr_t)p + 7u) & ~(uintptr_t)7u);

    // The calling thread's per-thread stream: it needs no creation, and it does
    // not wait for (or hold up) work on other streams the way the legacy default
    // stream would.
    const cudaStream_t s = cudaStreamPerThread;
    // Once anything is queued, every return waits for it to end first, so the
    // caller's buffers are not touched after the call returns, error or not.
    auto drain = [&](cbq_status err) {
        const bool ok = cudaStreamSynchronize(s) == cudaSuccess;
        cudaGetLastError();
        return ok ? err : CBQ_ERR_CUDA;
    };
    if (cudaMemcpyAsync(d_o, host_origin_tmax, n * 16, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return drain(CBQ_ERR_CUDA);
    if (cudaMemcpyAsync(d_d, host_direction, n * 16, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return drain(CBQ_ERR_CUDA);
    cbq_hits launch = dh;
    if (!host_hits->hit) launch.hit = nullptr;
    if (!host_hits->distance) launch.distance = nullptr;
    if (!host_hits->material) launch.material = nullptr;
    if (!host_hits->position) launch.position = nullptr;
    if (!host_hits->normal) launch.normal = nullptr;
    if (!host_hits->voxel) launch.voxel = nullptr;
    if (!host_hits->status) launch.status = nullptr;
    cbq_rays rays{d_o, d_d};
    // Always the persistent form (whatever the DAG's launch form): its work
    // counter lives in the array too.  Results are the same bits in every form.
    st = cbq_intersect_persistent(dag, &rays, n, query, &launch, d_counter, 0u, (cbq_stream_t)s);
    if (st != CBQ_OK) return drain(st);
    struct Copy { void* dst; const void* src; size_t bytes; };
    const Copy copies[] = {
        {host_hits->hit, launch.hit, n}, {host_hits->distance, launch.distance, n * 4},
        {host_hits->material, launch.material, n * 4}, {host_hits->position, launch.position, n * 12},
        {host_hits->normal, launch.normal, n * 12}, {host_hits->voxel, launch.voxel, n * 12},
        {host_hits->status, launch.status, n}};
    for (const Copy& c : copies) {
        if (!c.dst) continue;
        if (cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return drain(CBQ_ERR_CUDA);
    }
    return drain(CBQ_OK);
}
