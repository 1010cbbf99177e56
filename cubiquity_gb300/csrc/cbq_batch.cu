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
#include <cstring>
#include <new>
#include <vector>

namespace cbq {
namespace dev {

template <bool COMPACT>
struct BatchSrc {
    static constexpr bool kCompact = COMPACT;
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

// Descent stack in local memory and `steps` ESVO steps per loop iteration:
// the faster choices for the single-volume kernel on GB300.  Every job of one
// launch has the node store layout COMPACT.
template <bool COMPACT>
__device__ __forceinline__ void batch_body(const JobDesc* __restrict__ jobs, uint32_t njobs, uint64_t total,
                                           unsigned long long* __restrict__ counter, uint32_t refill_min,
                                           uint32_t steps)
{
    extern __shared__ uint64_t prefix[];  // njobs + 1 entries
    LocalStack stack;
    for (uint32_t j = threadIdx.x; j <= njobs; j += blockDim.x) prefix[j] = j < njobs ? jobs[j].first : total;
    __syncthreads();

    BatchSrc<COMPACT> c;
    c.jobs = jobs;
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t below = (1u << lane) - 1u;
    Lane L;
    L.mode = kLaneIdle;
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
                    const uint64_t g = base + __popc(idle & below);
                    if (g < total) {
                        // Last job whose first ray is <= g.  Every job in the
                        // table has at least one ray.
                        uint32_t lo = 0, hi = njobs;  // prefix[lo] <= g < prefix[hi]
                        while (hi - lo > 1u) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (prefix[mid] <= g) lo = mid; else hi = mid;
                        }
                        L.job = lo;
                        L.nodes = jobs[lo].nodes;
                        lane_begin(L, c, g - prefix[lo]);
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
        lane_walk_steps(L, c, stack, steps);
    }
}

template <bool COMPACT>
__global__ void __launch_bounds__(256) cbq_k_flat_batch(const JobDesc* __restrict__ jobs, uint32_t njobs,
                                                        uint64_t total, unsigned long long* __restrict__ counter,
                                                        uint32_t refill_min, uint32_t steps)
{
    batch_body<COMPACT>(jobs, njobs, total, counter, refill_min, steps);
}

// The same held to 56 registers per thread (more resident warps); a batch
// autotuner choice like the single-volume kernel's.
template <bool COMPACT>
__global__ void __maxnreg__(56) cbq_k_flat_batch_r56(const JobDesc* __restrict__ jobs, uint32_t njobs,
                                                     uint64_t total, unsigned long long* __restrict__ counter,
                                                     uint32_t refill_min, uint32_t steps)
{
    batch_body<COMPACT>(jobs, njobs, total, counter, refill_min, steps);
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

template <bool COMPACT>
cbq_status launch_batch_layout(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint64_t* counter,
                               int block, uint32_t refill, uint32_t steps, bool registers56, int device,
                               cudaStream_t s)
{
    const auto kernel = registers56 ? dev::cbq_k_flat_batch_r56<COMPACT> : dev::cbq_k_flat_batch<COMPACT>;
    if (cudaMemsetAsync(counter, 0, sizeof(uint64_t), s) != cudaSuccess) return CBQ_ERR_CUDA;
    const size_t smem = (size_t)(njobs + 1) * 8;  // the prefix offsets
    if (smem > 227u * 1024u) return CBQ_ERR_CAPACITY;
    if (smem > 48u * 1024u &&
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return CBQ_ERR_CUDA;
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return CBQ_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess)
        return CBQ_ERR_CUDA;
    per_sm = std::max(per_sm, 1);
    kernel<<<sms * per_sm, block, smem, s>>>(d_jobs, njobs, total, (unsigned long long*)counter, refill, steps);
    return cudaGetLastError() == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

}  // namespace

cbq_status launch_batch_kernel(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint64_t* counter,
                               int block, uint32_t refill, uint32_t steps, bool compact, int device, cudaStream_t s,
                               bool registers56)
{
    if (total == 0 || njobs == 0) return CBQ_OK;
    if (steps == 0) steps = 1;
    return compact ? launch_batch_layout<true>(d_jobs, njobs, total, counter, block, refill, steps, registers56,
                                               device, s)
                   : launch_batch_layout<false>(d_jobs, njobs, total, counter, block, refill, steps, registers56,
                                                device, s);
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
    std::vector<int> nested_jobs;           // jobs whose DAG needs the nested kernel
    dev::JobDesc* d_jobs = nullptr;         // reference-layout jobs, then compact-layout jobs
    uint32_t njobs = 0;                     // jobs in the device table
    uint32_t njobs_ref = 0;                 // of which reference layout (one launch per layout)
    uint64_t total = 0;
    uint64_t total_ref = 0;
    uint32_t steps = kBatchStepsDefault;
    bool registers56 = false;
    uint64_t* d_counter = nullptr;
    cbq_query query{1, CBQ_MAX_FOOTPRINT_DISABLED, 0u, 0u};
    int block = kBatchBlockDefault;
    uint32_t refill = kBatchRefillDefault;
    cudaGraphExec_t exec = nullptr;
};

namespace {

cbq_status enqueue_batch(cbq_batch* b, cudaStream_t s)
{
    for (int j : b->nested_jobs) {
        const cbq_job& jb = b->jobs[j];
        cbq_status st = cbq_intersect(jb.dag, &jb.rays, jb.ray_count, &b->query, &jb.hits, (cbq_stream_t)s);
        if (st != CBQ_OK) return st;
    }
    cbq_status st = launch_batch_kernel(b->d_jobs, b->njobs_ref, b->total_ref, b->d_counter, b->block, b->refill,
                                        b->steps, false, b->device, s, b->registers56);
    if (st != CBQ_OK) return st;
    return launch_batch_kernel(b->d_jobs + b->njobs_ref, b->njobs - b->njobs_ref, b->total - b->total_ref,
                               b->d_counter + 8, b->block, b->refill, b->steps, true, b->device, s, b->registers56);
}

void drop_graph(cbq_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
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
    if (st == CBQ_OK && cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) st = CBQ_ERR_CUDA;
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(s);
    if (st != CBQ_OK) {
        cudaGetLastError();
        b->exec = nullptr;
    }
    return st;
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
    b->block = block ? block : kBatchBlockDefault;
    b->refill = refill_min ? refill_min : kBatchRefillDefault;
    drop_graph(b);
    return CBQ_OK;
}

cbq_status cbq_batch_get_config(const cbq_batch* b, int32_t* block, uint32_t* refill_min, uint64_t* total_rays)
{
    if (!b) return CBQ_ERR_INVALID_ARGUMENT;
    if (block) *block = b->block;
    if (refill_min) *refill_min = b->refill;
    if (total_rays) *total_rays = b->total;
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
    static const uint32_t step_counts[] = {4, 8, 16};
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return CBQ_ERR_CUDA;
    float best = 1e30f;
    int best_block = b->block;
    uint32_t best_refill = b->refill, best_steps = b->steps;
    bool best_r56 = b->registers56;
    cbq_status st = CBQ_OK;
    for (int k = 0; k < 3 * 4 * 3 * 2 && st == CBQ_OK; k++) {
        const int blk = blocks[k / 24];
        const uint32_t rf = refills[(k / 6) % 4];
        b->block = blk;
        b->refill = rf;
        b->steps = step_counts[(k / 2) % 3];
        b->registers56 = (k & 1) != 0;
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
            best_block = blk;
            best_refill = rf;
            best_steps = b->steps;
            best_r56 = b->registers56;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->block = best_block;
    b->refill = best_refill;
    b->steps = best_steps;
    b->registers56 = best_r56;
    drop_graph(b);
    if (st == CBQ_OK)
        cbq::log(CBQ_LOG_INFO,
                 "batch autotune: block %d, refill %u, %u steps per iteration, %d registers: %.3f ms per launch",
                 best_block, best_refill, best_steps, best_r56 ? 56 : 64, best / (float)repetitions);
    return st;
}

cbq_status cbq_batch_destroy(cbq_batch* b)
{
    if (!b) return CBQ_ERR_INVALID_ARGUMENT;
    drop_graph(b);
    if (b->d_counter) cudaFree(b->d_counter);
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
