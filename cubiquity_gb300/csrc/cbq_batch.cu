// Batched traversal: many volumes, each with its own ray batch, in one
// persistent launch, captured in a CUDA graph and replayed (cbq_batch_*).
//
// A job table in device memory holds, per job, the node store, the SubDAGs, the
// ray and hit arrays, the query and the job's first global ray index.
// Persistent warps take global ray indices from one atomic counter
// (warp-aggregated refill of idle lanes, as in the single-volume persistent
// kernel); a lane finds its job by binary search over the prefix offsets, held
// in shared memory.
#include "cbq_batch.cuh"

#include <algorithm>
#include <exception>
#include <cstring>
#include <new>
#include <vector>

namespace cbq {
namespace dev {

template <bool COMPACT>
struct BatchSrc {
    static constexpr bool kCompact = COMPACT;
    static constexpr bool kIntPos = false;  // jobs whose DAG needs integer positions run on their own
    const JobDesc* __restrict__ jobs;

    __device__ __forceinline__ const QueryParams& query(const Lane& L) const { return jobs[L.job].q; }
    __device__ __forceinline__ const uint32_t* nodes(const Lane& L) const { return L.nodes; }
    __device__ __forceinline__ const SubDag& subdag(const Lane& L, uint32_t k) const { return jobs[L.job].sd[k]; }
    // Rays are read once (from device or page-locked host memory): streaming loads.
    __device__ __forceinline__ float4 ray_origin(const Lane& L, uint64_t i) const { return __ldcs(jobs[L.job].orig + i); }
    __device__ __forceinline__ float4 ray_direction(const Lane& L, uint64_t i) const { return __ldcs(jobs[L.job].dir + i); }
    __device__ __forceinline__ void write(const Lane& L, const RayResult& r) const
    {
        write_result(jobs[L.job].out, L.ray, r);
    }
};

constexpr unsigned kFullMask = 0xffffffffu;

// Last job whose first ray is <= g, by binary search over the prefix offsets
// (prefix[lo] <= g < prefix[hi]; every job in the table has at least one ray).
__device__ __forceinline__ uint32_t job_of(const uint64_t* prefix, uint32_t njobs, uint64_t g)
{
    uint32_t lo = 0, hi = njobs;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (prefix[mid] <= g) lo = mid; else hi = mid;
    }
    return lo;
}

// `steps` ESVO steps per loop iteration.  SHARED: descent stack in shared
// memory (`stack_rows` rows after the prefix offsets, one column per thread)
// instead of a per-thread local array.  SORTED: global ray g of the launch is
// ray perm[g], a ray of the same job (launch_batch_octant_sort).  Every job of
// one launch has the node store layout COMPACT.
template <bool COMPACT, bool SHARED, bool SORTED>
__device__ __forceinline__ void batch_body(const JobDesc* __restrict__ jobs, uint32_t njobs, uint64_t total,
                                           unsigned long long* __restrict__ counter, uint32_t refill_min,
                                           uint32_t steps, const uint32_t* __restrict__ perm)
{
    extern __shared__ uint64_t prefix[];  // njobs + 1 entries, then the shared stack
    for (uint32_t j = threadIdx.x; j <= njobs; j += blockDim.x) prefix[j] = j < njobs ? jobs[j].first : total;
    __syncthreads();
    LocalStack lstack;
    SharedStack sstack;
    sstack.base = (uint32_t*)(prefix + njobs + 1) + threadIdx.x;
    sstack.stride = blockDim.x;

    BatchSrc<COMPACT> c;
    c.jobs = jobs;
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t below = (1u << lane) - 1u;
    Lane L;
    L.mode = kLaneIdle;
    L.held = 0u;
    L.job = 0;
    L.nodes = nullptr;
    bool more = true;
    for (;;) {
        if (more) {
            const uint32_t idle = __ballot_sync(kFullMask, L.mode == kLaneIdle);
            const uint32_t cnt = __popc(idle);
            if (cnt == 32u || (cnt != 0u && cnt >= refill_min)) {
                const int leader = __ffs(idle) - 1;
                unsigned long long base = 0;
                if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)cnt);
                base = __shfl_sync(kFullMask, base, leader);
                if (L.mode == kLaneIdle) {
                    uint64_t g = base + __popc(idle & below);
                    if (g < total) {
                        if (SORTED) g = __ldg(perm + g);
                        const uint32_t j = job_of(prefix, njobs, g);
                        L.job = j;
                        L.nodes = jobs[j].nodes;
                        lane_begin(L, c, g - prefix[j]);
                    }
                }
                if (base + cnt >= total) more = false;
            }
        }
        if (!__any_sync(kFullMask, L.mode != kLaneIdle)) {
            if (!more) break;
            continue;
        }
        lane_settle(L, c);
        if (SHARED)
            warp_walk_steps(L, c, sstack, steps);
        else
            warp_walk_steps(L, c, lstack, steps);
    }
}

template <bool COMPACT, bool SHARED, bool SORTED>
__global__ void __launch_bounds__(256) cbq_k_flat_batch(const JobDesc* __restrict__ jobs, uint32_t njobs,
                                                        uint64_t total, unsigned long long* __restrict__ counter,
                                                        uint32_t refill_min, uint32_t steps,
                                                        const uint32_t* __restrict__ perm)
{
    batch_body<COMPACT, SHARED, SORTED>(jobs, njobs, total, counter, refill_min, steps, perm);
}

// The local-stack form held to 56 registers per thread (more resident warps);
// a batch autotuner choice like the single-volume kernel's.
template <bool COMPACT, bool SORTED>
__global__ void __maxnreg__(56) cbq_k_flat_batch_r56(const JobDesc* __restrict__ jobs, uint32_t njobs,
                                                     uint64_t total, unsigned long long* __restrict__ counter,
                                                     uint32_t refill_min, uint32_t steps,
                                                     const uint32_t* __restrict__ perm)
{
    batch_body<COMPACT, false, SORTED>(jobs, njobs, total, counter, refill_min, steps, perm);
}

// Octant of a ray: its direction sign bits (raytracing.cpp:416-417).
__device__ __forceinline__ uint32_t batch_octant(float4 d)
{
    return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
}

// counts[8 * job + octant] += rays, warp-aggregated.
__global__ void __launch_bounds__(256) cbq_k_batch_octant_count(const JobDesc* __restrict__ jobs, uint32_t njobs,
                                                                uint64_t total, uint32_t* __restrict__ counts)
{
    extern __shared__ uint64_t prefix[];
    for (uint32_t j = threadIdx.x; j <= njobs; j += blockDim.x) prefix[j] = j < njobs ? jobs[j].first : total;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g0 = (uint64_t)blockIdx.x * blockDim.x; g0 < total; g0 += stride) {
        const uint64_t g = g0 + threadIdx.x;
        const bool valid = g < total;
        const unsigned act = __ballot_sync(kFullMask, valid);
        if (!valid) continue;
        const uint32_t j = job_of(prefix, njobs, g);
        const uint32_t key = 8u * j + batch_octant(__ldg(jobs[j].dir + (g - prefix[j])));
        const unsigned grp = __match_any_sync(act, key);
        if ((int)lane == __ffs(grp) - 1) atomicAdd(&counts[key], (uint32_t)__popc(grp));
    }
}

// perm[first(job) + (rays of lower octants in the job) + k] = g.  Every global
// index g < total is written exactly once, inside its own job's range.
__global__ void __launch_bounds__(256) cbq_k_batch_octant_scatter(const JobDesc* __restrict__ jobs, uint32_t njobs,
                                                                  uint64_t total, const uint32_t* __restrict__ counts,
                                                                  uint32_t* __restrict__ cursor,
                                                                  uint32_t* __restrict__ perm)
{
    extern __shared__ uint64_t prefix[];
    for (uint32_t j = threadIdx.x; j <= njobs; j += blockDim.x) prefix[j] = j < njobs ? jobs[j].first : total;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g0 = (uint64_t)blockIdx.x * blockDim.x; g0 < total; g0 += stride) {
        const uint64_t g = g0 + threadIdx.x;
        const bool valid = g < total;
        const unsigned act = __ballot_sync(kFullMask, valid);
        if (!valid) continue;
        const uint32_t j = job_of(prefix, njobs, g);
        const uint32_t oct = batch_octant(__ldg(jobs[j].dir + (g - prefix[j])));
        const uint32_t key = 8u * j + oct;
        const unsigned grp = __match_any_sync(act, key);
        const int leader = __ffs(grp) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&cursor[key], (uint32_t)__popc(grp));
        base = __shfl_sync(grp, base, leader);
        uint64_t start = prefix[j];
        for (uint32_t o = 0; o < oct; o++) start += counts[8u * j + o];
        perm[start + base + __popc(grp & ((1u << lane) - 1u))] = (uint32_t)g;
    }
}

}  // namespace dev

void fill_job_volume(dev::JobDesc& d, const cbq_dag* dag)
{
    d.nodes = dag->d_nodes;
    for (int k = 0; k < 8; k++) {
        const cbq_subdag& s = dag->subdags[k];
        d.sd[k].lx = s.lower_bound[0];
        d.sd[k].ly = s.lower_bound[1];
        d.sd[k].lz = s.lower_bound[2];
        d.sd[k].height = s.node_height;
        d.sd[k].node = dag->sd_ref[k];
        d.sd[k].pad[0] = d.sd[k].pad[1] = d.sd[k].pad[2] = 0;
    }
}

namespace {

template <bool COMPACT, bool SHARED, bool SORTED>
cbq_status launch_batch_variant(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint64_t* counter,
                                int device, cudaStream_t s, const BatchLaunch& bl)
{
    auto kernel = dev::cbq_k_flat_batch<COMPACT, SHARED, SORTED>;
    if constexpr (!SHARED) {
        if (bl.registers56) kernel = dev::cbq_k_flat_batch_r56<COMPACT, SORTED>;
    }
    if (cudaMemsetAsync(counter, 0, sizeof(uint64_t), s) != cudaSuccess) return CBQ_ERR_CUDA;
    // The prefix offsets, then (shared stack) one column of stack_rows slots per thread.
    const size_t smem = (size_t)(njobs + 1) * 8 + (SHARED ? (size_t)std::max(1, bl.stack_rows) * bl.block * 4 : 0);
    if (smem > 227u * 1024u) return CBQ_ERR_CAPACITY;
    if (smem > 48u * 1024u &&
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return CBQ_ERR_CUDA;
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return CBQ_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, bl.block, smem) != cudaSuccess)
        return CBQ_ERR_CUDA;
    per_sm = std::max(per_sm, 1);
    kernel<<<sms * per_sm, bl.block, smem, s>>>(d_jobs, njobs, total, (unsigned long long*)counter, bl.refill,
                                                bl.steps ? bl.steps : 1u, bl.perm);
    return cudaGetLastError() == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

template <bool COMPACT>
cbq_status launch_batch_layout(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint64_t* counter,
                               int device, cudaStream_t s, const BatchLaunch& bl)
{
    const bool sorted = bl.perm != nullptr;
    if (bl.shared_stack)
        return sorted ? launch_batch_variant<COMPACT, true, true>(d_jobs, njobs, total, counter, device, s, bl)
                      : launch_batch_variant<COMPACT, true, false>(d_jobs, njobs, total, counter, device, s, bl);
    return sorted ? launch_batch_variant<COMPACT, false, true>(d_jobs, njobs, total, counter, device, s, bl)
                  : launch_batch_variant<COMPACT, false, false>(d_jobs, njobs, total, counter, device, s, bl);
}

}  // namespace

cbq_status launch_batch_kernel(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint64_t* counter,
                               bool compact, int device, cudaStream_t s, const BatchLaunch& bl)
{
    if (total == 0 || njobs == 0) return CBQ_OK;
    return compact ? launch_batch_layout<true>(d_jobs, njobs, total, counter, device, s, bl)
                   : launch_batch_layout<false>(d_jobs, njobs, total, counter, device, s, bl);
}

cbq_status launch_batch_kernel(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint64_t* counter,
                               int block, uint32_t refill, uint32_t steps, bool compact, int device, cudaStream_t s,
                               bool registers56)
{
    BatchLaunch bl;
    bl.block = block;
    bl.refill = refill;
    bl.steps = steps;
    bl.registers56 = registers56;
    return launch_batch_kernel(d_jobs, njobs, total, counter, compact, device, s, bl);
}

cbq_status launch_batch_octant_sort(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint32_t* scratch,
                                    uint32_t* perm, int device, cudaStream_t s)
{
    if (total == 0 || njobs == 0) return CBQ_OK;
    if (total > 0xffffffffull) return CBQ_ERR_INVALID_ARGUMENT;  // perm holds 32-bit ray indices
    const size_t smem = (size_t)(njobs + 1) * 8;
    if (smem > 48u * 1024u) return CBQ_ERR_CAPACITY;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return CBQ_ERR_CUDA;
    if (cudaMemsetAsync(scratch, 0, (size_t)njobs * 16 * sizeof(uint32_t), s) != cudaSuccess) return CBQ_ERR_CUDA;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((total + 255) / 256, (uint64_t)sms * 8));
    dev::cbq_k_batch_octant_count<<<grid, 256, smem, s>>>(d_jobs, njobs, total, scratch);
    dev::cbq_k_batch_octant_scatter<<<grid, 256, smem, s>>>(d_jobs, njobs, total, scratch, scratch + 8 * njobs,
                                                            perm);
    return cudaGetLastError() == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

}  // namespace cbq

using namespace cbq;

namespace {
constexpr int kBatchBlockDefault = 128;
constexpr uint32_t kBatchRefillDefault = 8;
}  // namespace

struct cbq_batch {
    int device = 0;
    std::vector<cbq_job> jobs;              // as given (host copy)
    std::vector<int> nested_jobs;           // jobs whose DAG needs integer positions (launched on their own)
    dev::JobDesc* d_jobs = nullptr;         // reference-layout jobs, then compact-layout jobs
    uint32_t njobs = 0;                     // jobs in the device table
    uint32_t njobs_ref = 0;                 // of which reference layout (one launch per layout)
    uint64_t total = 0;
    uint64_t total_ref = 0;
    int stack_rows = 1;                     // max SubDAG height over the jobs
    uint64_t* d_counter = nullptr;
    uint32_t* d_sort = nullptr;             // octant order: 16 uint32 per job, then one index per ray
    cbq_query query{1, CBQ_MAX_FOOTPRINT_DISABLED, 0u, 0u};
    cbq_batch_config cfg{kBatchBlockDefault, kBatchRefillDefault, (int32_t)kBatchStepsDefault, 0, CBQ_STACK_LOCAL,
                         CBQ_FORM_PERSISTENT};
    cudaGraphExec_t exec = nullptr;
    // Persisting L2 window set on the graph's kernel nodes (l2_bytes 0: none).
    void* l2_base = nullptr;
    size_t l2_bytes = 0;
    float l2_hit_ratio = 0.0f;
};

namespace {

BatchLaunch batch_launch(const cbq_batch* b, const uint32_t* perm)
{
    BatchLaunch bl;
    bl.block = b->cfg.block;
    bl.refill = b->cfg.refill_min;
    bl.steps = (uint32_t)b->cfg.steps;
    bl.registers56 = b->cfg.registers == 56 && b->cfg.stack == CBQ_STACK_LOCAL;
    bl.shared_stack = b->cfg.stack == CBQ_STACK_SHARED;
    bl.stack_rows = b->stack_rows;
    bl.perm = perm;
    return bl;
}

// Device memory of the octant order, allocated when a sorted form is first
// chosen.  The sort keeps a job's first ray index per job in shared memory and
// writes 32-bit ray indices, which bounds the jobs and rays of a sorted batch.
cbq_status ensure_sort_scratch(cbq_batch* b)
{
    if ((size_t)(b->njobs + 1) * 8 > 48u * 1024u || b->total > 0xffffffffull) return CBQ_ERR_CAPACITY;
    if (b->d_sort || b->njobs == 0) return CBQ_OK;
    const size_t bytes = ((size_t)b->njobs * 16 + b->total) * sizeof(uint32_t);
    if (cudaMalloc((void**)&b->d_sort, bytes) != cudaSuccess) {
        cudaGetLastError();
        b->d_sort = nullptr;
        return CBQ_ERR_OUT_OF_MEMORY;
    }
    return CBQ_OK;
}

cbq_status enqueue_batch(cbq_batch* b, cudaStream_t s)
{
    for (int j : b->nested_jobs) {
        const cbq_job& jb = b->jobs[j];
        cbq_status st = cbq_intersect(jb.dag, &jb.rays, jb.ray_count, &b->query, &jb.hits, (cbq_stream_t)s);
        if (st != CBQ_OK) return st;
    }
    // One launch per node store layout, each with its own ray index space.
    const uint32_t njobs_c = b->njobs - b->njobs_ref;
    const uint64_t total_c = b->total - b->total_ref;
    const bool sorted = b->cfg.form == CBQ_FORM_SORTED;
    if (sorted && !b->d_sort) return CBQ_ERR_INVALID_ARGUMENT;
    uint32_t* perm_ref = sorted ? b->d_sort + 16 * (size_t)b->njobs : nullptr;
    uint32_t* perm_c = sorted ? perm_ref + b->total_ref : nullptr;
    if (sorted) {
        cbq_status st = launch_batch_octant_sort(b->d_jobs, b->njobs_ref, b->total_ref, b->d_sort, perm_ref,
                                                 b->device, s);
        if (st == CBQ_OK)
            st = launch_batch_octant_sort(b->d_jobs + b->njobs_ref, njobs_c, total_c, b->d_sort + 16 * b->njobs_ref,
                                          perm_c, b->device, s);
        if (st != CBQ_OK) return st;
    }
    cbq_status st = launch_batch_kernel(b->d_jobs, b->njobs_ref, b->total_ref, b->d_counter, false, b->device, s,
                                        batch_launch(b, perm_ref));
    if (st != CBQ_OK) return st;
    return launch_batch_kernel(b->d_jobs + b->njobs_ref, njobs_c, total_c, b->d_counter + 8, true, b->device, s,
                               batch_launch(b, perm_c));
}

void drop_graph(cbq_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
}

// Sets the batch's persisting L2 window on every kernel node of the captured
// graph (the traversal and, for sorted forms, the octant sort).
cbq_status set_kernel_node_window(const cbq_batch* b, cudaGraph_t g)
{
    size_t count = 0;
    if (cudaGraphGetNodes(g, nullptr, &count) != cudaSuccess) return CBQ_ERR_CUDA;
    std::vector<cudaGraphNode_t> nodes;
    try {
        nodes.resize(count);
    } catch (const std::exception&) {
        return CBQ_ERR_OUT_OF_MEMORY;
    }
    if (count && cudaGraphGetNodes(g, nodes.data(), &count) != cudaSuccess) return CBQ_ERR_CUDA;
    cudaKernelNodeAttrValue v;
    std::memset(&v, 0, sizeof(v));
    v.accessPolicyWindow.base_ptr = b->l2_base;
    v.accessPolicyWindow.num_bytes = b->l2_bytes;
    v.accessPolicyWindow.hitRatio = b->l2_hit_ratio;
    v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    for (cudaGraphNode_t n : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(n, &t) != cudaSuccess) return CBQ_ERR_CUDA;
        if (t != cudaGraphNodeTypeKernel) continue;
        if (cudaGraphKernelNodeSetAttribute(n, cudaKernelNodeAttributeAccessPolicyWindow, &v) != cudaSuccess)
            return CBQ_ERR_CUDA;
    }
    return CBQ_OK;
}

cbq_status capture_graph(cbq_batch* b)
{
    drop_graph(b);
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return CBQ_ERR_CUDA;
    cudaGraph_t g = nullptr;
    cbq_status st = CBQ_OK;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) st = CBQ_ERR_CUDA;
    if (st == CBQ_OK) {
        st = enqueue_batch(b, s);
        if (cudaStreamEndCapture(s, &g) != cudaSuccess) st = CBQ_ERR_CUDA;
    }
    if (st == CBQ_OK && b->l2_bytes) st = set_kernel_node_window(b, g);
    if (st == CBQ_OK && cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) st = CBQ_ERR_CUDA;
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(s);
    if (st != CBQ_OK) {
        cudaGetLastError();
        b->exec = nullptr;
    }
    return st;
}

cbq_status check_config(const cbq_batch_config& c)
{
    if (c.block < 32 || c.block > 256 || (c.block % 32) != 0) return CBQ_ERR_INVALID_ARGUMENT;
    if (c.refill_min < 1 || c.refill_min > 32 || c.steps < 1 || c.steps > 32) return CBQ_ERR_INVALID_ARGUMENT;
    if (c.registers != 0 && c.registers != 56) return CBQ_ERR_INVALID_ARGUMENT;
    if (c.stack != CBQ_STACK_LOCAL && c.stack != CBQ_STACK_SHARED) return CBQ_ERR_INVALID_ARGUMENT;
    if (c.form != CBQ_FORM_PERSISTENT && c.form != CBQ_FORM_SORTED) return CBQ_ERR_INVALID_ARGUMENT;
    return CBQ_OK;
}

}  // namespace

extern "C" {

cbq_status cbq_batch_create(const cbq_job* jobs, int32_t job_count, const cbq_query* query, cbq_batch** out)
{
    if (!out || job_count < 0 || (job_count > 0 && !jobs)) return CBQ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return CBQ_ERR_CUDA;
    std::vector<dev::JobDesc> table, compact;
    cbq_batch* b = new (std::nothrow) cbq_batch();
    if (!b) return CBQ_ERR_OUT_OF_MEMORY;
    b->device = device;
    if (query) b->query = *query;
    uint64_t first = 0, first_compact = 0;
    for (int32_t j = 0; j < job_count; j++) {
        const cbq_job& jb = jobs[j];
        if (!jb.dag || jb.dag->device != device) { delete b; return CBQ_ERR_INVALID_ARGUMENT; }
        if (jb.ray_count > 0 &&
            (!jb.rays.origin_tmax || !jb.rays.direction || ((uintptr_t)jb.rays.origin_tmax & 15u) ||
             ((uintptr_t)jb.rays.direction & 15u))) {
            delete b;
            return CBQ_ERR_INVALID_ARGUMENT;
        }
        b->jobs.push_back(jb);
        if (jb.ray_count == 0) continue;
        if (!jb.dag->flat_ok) { b->nested_jobs.push_back(j); continue; }
        b->stack_rows = std::max(b->stack_rows, (int)jb.dag->max_height);
        dev::JobDesc d;
        std::memset(&d, 0, sizeof(d));
        fill_job_volume(d, jb.dag);
        d.orig = (const float4*)jb.rays.origin_tmax;
        d.dir = (const float4*)jb.rays.direction;
        d.out.hit = jb.hits.hit;
        d.out.distance = jb.hits.distance;
        d.out.material = jb.hits.material;
        d.out.position = jb.hits.position;
        d.out.normal = jb.hits.normal;
        d.out.voxel = jb.hits.voxel;
        d.out.status = jb.hits.status;
        const bool is_compact = jb.dag->layout == CBQ_DAG_LAYOUT_COMPACT;
        d.first = is_compact ? first_compact : first;
        d.count = jb.ray_count;
        d.q.compute_surface = b->query.compute_surface;
        d.q.max_footprint = b->query.max_footprint;
        d.q.flags = b->query.flags;
        (is_compact ? compact : table).push_back(d);
        (is_compact ? first_compact : first) += jb.ray_count;
    }
    b->njobs_ref = (uint32_t)table.size();
    b->total_ref = first;
    table.insert(table.end(), compact.begin(), compact.end());
    b->njobs = (uint32_t)table.size();
    b->total = first + first_compact;
    if (cudaMalloc((void**)&b->d_counter, 256 + table.size() * sizeof(dev::JobDesc)) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return CBQ_ERR_OUT_OF_MEMORY;
    }
    b->d_jobs = (dev::JobDesc*)((char*)b->d_counter + 256);
    if (!table.empty() &&
        cudaMemcpy(b->d_jobs, table.data(), table.size() * sizeof(dev::JobDesc), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(b->d_counter);
        delete b;
        return CBQ_ERR_CUDA;
    }
    *out = b;
    return CBQ_OK;
}

cbq_status cbq_batch_set_config(cbq_batch* b, int32_t block, uint32_t refill_min)
{
    if (!b || block < 0 || block > 256 || (block % 32) != 0 || refill_min > 32) return CBQ_ERR_INVALID_ARGUMENT;
    b->cfg.block = block ? block : kBatchBlockDefault;
    b->cfg.refill_min = refill_min ? refill_min : kBatchRefillDefault;
    drop_graph(b);
    return CBQ_OK;
}

cbq_status cbq_batch_get_config(const cbq_batch* b, int32_t* block, uint32_t* refill_min, uint64_t* total_rays)
{
    if (!b) return CBQ_ERR_INVALID_ARGUMENT;
    if (block) *block = b->cfg.block;
    if (refill_min) *refill_min = b->cfg.refill_min;
    if (total_rays) *total_rays = b->total;
    return CBQ_OK;
}

cbq_status cbq_batch_set_launch_config(cbq_batch* b, const cbq_batch_config* cfg)
{
    if (!b || !cfg) return CBQ_ERR_INVALID_ARGUMENT;
    cbq_status st = check_config(*cfg);
    if (st != CBQ_OK) return st;
    if (cfg->form == CBQ_FORM_SORTED && (st = ensure_sort_scratch(b)) != CBQ_OK) return st;
    b->cfg = *cfg;
    drop_graph(b);
    return CBQ_OK;
}

cbq_status cbq_batch_get_launch_config(const cbq_batch* b, cbq_batch_config* cfg)
{
    if (!b || !cfg) return CBQ_ERR_INVALID_ARGUMENT;
    *cfg = b->cfg;
    return CBQ_OK;
}

cbq_status cbq_batch_launch(cbq_batch* b, cbq_stream_t stream)
{
    if (!b) return CBQ_ERR_INVALID_ARGUMENT;
    if (!b->exec) {
        cbq_status st = capture_graph(b);
        if (st != CBQ_OK) return st;
    }
    return cudaGraphLaunch(b->exec, (cudaStream_t)stream) == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

cbq_status cbq_batch_set_l2_persistence(cbq_batch* b, const cbq_dag* dag, float fraction)
{
    if (!b || !(fraction >= 0.0f && fraction <= 1.0f)) return CBQ_ERR_INVALID_ARGUMENT;
    if (fraction > 0.0f && (!dag || dag->device != b->device)) return CBQ_ERR_INVALID_ARGUMENT;
    drop_graph(b);  // re-captured with the new window on the next cbq_batch_launch
    if (fraction == 0.0f) {
        b->l2_base = nullptr;
        b->l2_bytes = 0;
        // Give the set-aside back to normal caching and demote persisting lines
        // (settings of the calling process's context).
        if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0) != cudaSuccess ||
            cudaCtxResetPersistingL2Cache() != cudaSuccess)
            return CBQ_ERR_CUDA;
        return CBQ_OK;
    }
    int max_window = 0, max_persist = 0;
    cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, b->device);
    cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, b->device);
    if (max_window <= 0 || max_persist <= 0) return CBQ_OK;  // not supported: caching stays as it is
    const size_t want = (size_t)((double)max_persist * fraction);
    if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) return CBQ_ERR_CUDA;
    b->l2_base = dag->d_nodes;
    b->l2_bytes = std::min<size_t>(dag->device_bytes, (size_t)max_window);
    b->l2_hit_ratio = (float)std::min(1.0, (double)want / (double)b->l2_bytes);
    return CBQ_OK;
}

cbq_status cbq_batch_launch_direct(cbq_batch* b, cbq_stream_t stream)
{
    if (!b) return CBQ_ERR_INVALID_ARGUMENT;
    return enqueue_batch(b, (cudaStream_t)stream);
}

cbq_status cbq_batch_autotune(cbq_batch* b, cbq_stream_t stream, int32_t repetitions)
{
    if (!b || repetitions <= 0) return CBQ_ERR_INVALID_ARGUMENT;
    static const int blocks[] = {64, 128, 256};
    static const uint32_t refills[] = {4, 8, 12, 16};
    static const int32_t step_counts[] = {4, 8, 16};
    // Kernel variants: local stack (64 registers), local stack held to 56
    // registers, shared-memory stack; each with the rays in the order given or
    // grouped by octant per job.
    struct Variant { int32_t registers, stack, form; };
    static const Variant variants[] = {
        {0, CBQ_STACK_LOCAL, CBQ_FORM_PERSISTENT}, {56, CBQ_STACK_LOCAL, CBQ_FORM_PERSISTENT},
        {0, CBQ_STACK_SHARED, CBQ_FORM_PERSISTENT}, {0, CBQ_STACK_LOCAL, CBQ_FORM_SORTED},
        {56, CBQ_STACK_LOCAL, CBQ_FORM_SORTED}, {0, CBQ_STACK_SHARED, CBQ_FORM_SORTED}};
    const bool can_sort = ensure_sort_scratch(b) == CBQ_OK;  // without the scratch, unsorted forms only
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return CBQ_ERR_CUDA;
    const cbq_batch_config saved = b->cfg;
    cbq_batch_config best_cfg = saved;
    float best = 1e30f;
    cbq_status st = CBQ_OK;
    for (int blk : blocks) {
        for (uint32_t rf : refills) {
            for (int32_t steps : step_counts) {
                for (const Variant& v : variants) {
                    if (v.form == CBQ_FORM_SORTED && !can_sort) continue;
                    b->cfg = cbq_batch_config{blk, rf, steps, v.registers, v.stack, v.form};
                    st = enqueue_batch(b, (cudaStream_t)stream);  // warm-up
                    if (st != CBQ_OK) break;
                    cudaEventRecord(e0, (cudaStream_t)stream);
                    for (int r = 0; r < repetitions && st == CBQ_OK; r++) st = enqueue_batch(b, (cudaStream_t)stream);
                    cudaEventRecord(e1, (cudaStream_t)stream);
                    if (st != CBQ_OK || cudaEventSynchronize(e1) != cudaSuccess) { st = CBQ_ERR_CUDA; break; }
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < best) {
                        best = ms;
                        best_cfg = b->cfg;
                    }
                }
                if (st != CBQ_OK) break;
            }
            if (st != CBQ_OK) break;
        }
        if (st != CBQ_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->cfg = st == CBQ_OK ? best_cfg : saved;
    drop_graph(b);
    if (st == CBQ_OK)
        cbq::log(CBQ_LOG_INFO,
                 "batch autotune: block %d, refill %u, %d steps per iteration, %d registers, %s stack, %s: "
                 "%.3f ms per launch",
                 best_cfg.block, best_cfg.refill_min, best_cfg.steps, best_cfg.registers ? 56 : 64,
                 best_cfg.stack == CBQ_STACK_SHARED ? "shared" : "local",
                 best_cfg.form == CBQ_FORM_SORTED ? "octant-sorted" : "rays as given", best / (float)repetitions);
    return st;
}

cbq_status cbq_batch_destroy(cbq_batch* b)
{
    if (!b) return CBQ_ERR_INVALID_ARGUMENT;
    drop_graph(b);
    if (b->d_counter) cudaFree(b->d_counter);
    if (b->d_sort) cudaFree(b->d_sort);
    delete b;
    return CBQ_OK;
}

cbq_status cbq_intersect_batch(const cbq_job* jobs, int32_t job_count, const cbq_query* query, cbq_stream_t stream)
{
    cbq_batch* b = nullptr;
    cbq_status st = cbq_batch_create(jobs, job_count, query, &b);
    if (st != CBQ_OK) return st;
    st = enqueue_batch(b, (cudaStream_t)stream);
    if (st == CBQ_OK && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) st = CBQ_ERR_CUDA;
    cbq_batch_destroy(b);
    return st;
}

}  // extern "C"
