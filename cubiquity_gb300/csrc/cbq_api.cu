// Device-side C ABI: DAG upload, traversal launches (plain and persistent).
#include "cbq_flat.cuh"
#include "cbq_internal.hpp"
#include "cbq_traverse.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <exception>
#include <new>
#include <vector>

using namespace cbq;

namespace {

constexpr int kFlatBlockDefault = 128;  // GB300, terrain-4096: 64, 128 and 256 threads within 1-3%
constexpr uint32_t kRefillDefault = 8;

bool use_flat(const cbq_dag* dag)
{
    return dag->cfg.kernel != CBQ_KERNEL_NESTED || dag->layout == CBQ_DAG_LAYOUT_COMPACT;
}

int flat_block(const cbq_dag* dag) { return dag->cfg.block > 0 ? dag->cfg.block : kFlatBlockDefault; }

FlatLaunch flat_launch(const cbq_dag* dag, bool persistent, uint64_t* counter, uint32_t refill)
{
    FlatLaunch fl;
    fl.persistent = persistent;
    fl.counter = counter;
    fl.block = flat_block(dag);
    fl.refill_min = refill ? refill : (dag->cfg.refill_min ? dag->cfg.refill_min : kRefillDefault);
    fl.local_stack = dag->cfg.stack == CBQ_STACK_LOCAL;
    fl.steps = dag->cfg.steps > 0 ? (uint32_t)dag->cfg.steps : 1u;
    fl.registers56 = dag->cfg.registers == 56;
    return fl;
}

constexpr int kPlainBlock = 128;
constexpr int kPersistBlock = 256;
constexpr uint32_t kDefaultChunk = 64;

dev::DagParams make_dag_params(const cbq_dag* dag)
{
    dev::DagParams p;
    p.nodes = dag->d_nodes;
    for (int i = 0; i < 8; i++) {
        p.sd[i].lx = dag->subdags[i].lower_bound[0];
        p.sd[i].ly = dag->subdags[i].lower_bound[1];
        p.sd[i].lz = dag->subdags[i].lower_bound[2];
        p.sd[i].height = dag->subdags[i].node_height;
        p.sd[i].node = dag->sd_ref[i];
        p.sd[i].pad[0] = p.sd[i].pad[1] = p.sd[i].pad[2] = 0;
    }
    return p;
}

dev::QueryParams make_query(const cbq_query* q)
{
    dev::QueryParams p;
    p.compute_surface = q ? q->compute_surface : 1;
    p.max_footprint = q ? q->max_footprint : CBQ_MAX_FOOTPRINT_DISABLED;
    p.flags = q ? q->flags : 0u;
    p.image_width = q ? q->image_width : 0u;  // checked against each launch's ray count by launch_flat
    return p;
}

dev::HitsOut make_hits(const cbq_hits* h)
{
    dev::HitsOut o;
    o.hit = h->hit;
    o.distance = h->distance;
    o.material = h->material;
    o.position = h->position;
    o.normal = h->normal;
    o.voxel = h->voxel;
    o.status = h->status;
    return o;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// One chunk of a cbq_intersect_host call.  The call's rays are cut into blocks of
// `block` consecutive rays dealt round-robin to the chunks (block b to chunk
// b % chunks), so that every chunk samples the whole batch: a camera batch whose
// first rows are sky and whose middle rows are terrain gives chunks of equal work,
// and the copies and traversals of consecutive chunks stay balanced.  On the
// device a chunk's rays and hits are contiguous, from ray `start`; on the host its
// full blocks are the rows of a pitched array, and the batch's last, partial block
// (if this chunk has it) is copied on its own.
struct HostChunk {
    uint64_t block = 1;    // rays per block
    uint64_t start = 0;    // first ray of the chunk in the device staging
    uint64_t rows = 0;     // full blocks: host blocks k, k + chunks, ...
    uint64_t tail = 0;     // rays of the batch's partial last block, if this chunk has it
    uint64_t tail_at = 0;  // host index of that block's first ray
    uint64_t rays() const { return rows * block + tail; }
};

HostChunk host_chunk(uint64_t n, uint64_t chunks, uint64_t block, uint64_t k, uint64_t start)
{
    const uint64_t full = n / block, rem = n % block;
    HostChunk c;
    c.block = block;
    c.start = start;
    c.rows = full > k ? (full - k + chunks - 1) / chunks : 0;
    if (rem != 0 && full % chunks == k) {
        c.tail = rem;
        c.tail_at = full * block;
    }
    return c;
}

// Copies `width` bytes per ray of chunk k between the host array (every ray of the
// call) and the device array (the chunk's rays from c.start).
bool copy_chunk(void* host, void* dev, size_t width, const HostChunk& c, uint64_t k, uint64_t chunks,
                cudaMemcpyKind kind, cudaStream_t s)
{
    char* h = (char*)host;
    char* d = (char*)dev + c.start * width;
    const size_t row = c.block * width;
    const bool in = kind == cudaMemcpyHostToDevice;
    if (c.rows != 0) {
        char* hr = h + k * row;
        const cudaError_t e = in ? cudaMemcpy2DAsync(d, row, hr, chunks * row, row, c.rows, kind, s)
                                 : cudaMemcpy2DAsync(hr, chunks * row, d, row, row, c.rows, kind, s);
        if (e != cudaSuccess) return false;
    }
    if (c.tail != 0) {
        char* ht = h + c.tail_at * width;
        char* dt = d + c.rows * row;
        const cudaError_t e = in ? cudaMemcpyAsync(dt, ht, c.tail * width, kind, s)
                                 : cudaMemcpyAsync(ht, dt, c.tail * width, kind, s);
        if (e != cudaSuccess) return false;
    }
    return true;
}

// The persistent form's work counter for launches on `stream` (one per stream,
// allocated on first use), or nullptr where none can be had: the id query
// fails, or the stream is being captured (no allocation inside a capture).
uint64_t* stream_counter(const cbq_dag* cdag, cudaStream_t stream)
{
    cbq_dag* dag = const_cast<cbq_dag*>(cdag);
    // Only the capture query is legal while a capture is under way: ask it first.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &capture) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (capture != cudaStreamCaptureStatusNone) return nullptr;
    unsigned long long id = 0;
    if (cudaStreamGetId(stream, &id) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(dag->counter_lock);
    auto it = dag->stream_counters.find(id);
    if (it != dag->stream_counters.end()) return it->second;
    uint64_t* p = nullptr;
    if (cudaMalloc((void**)&p, 256) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    dag->stream_counters[id] = p;
    return p;
}

cbq_status check_rays(const cbq_rays* rays)
{
    if (!rays || !rays->origin_tmax || !rays->direction) return CBQ_ERR_INVALID_ARGUMENT;
    if (!aligned16(rays->origin_tmax) || !aligned16(rays->direction)) return CBQ_ERR_INVALID_ARGUMENT;
    return CBQ_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// One ray per thread, stack in local memory.
__global__ void __launch_bounds__(kPlainBlock) cbq_k_intersect_plain(dev::DagParams dag,
                                                                     const float4* __restrict__ orig,
                                                                     const float4* __restrict__ dir, uint64_t n,
                                                                     dev::QueryParams q, dev::HitsOut out,
                                                                     uint32_t* __restrict__ fetch_out)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dev::LocalStack stack;
    uint32_t fetches = 0;
    const dev::RayResult r = dev::intersect_volume(dag, __ldg(orig + i), __ldg(dir + i), q, stack, &fetches);
    dev::write_result(out, i, r);
    if (fetch_out) fetch_out[i] = fetches;
}

// Persistent warps: each warp takes `chunk` rays at a time from an atomic
// counter; the descent stack lives in shared memory (one column per thread).
__global__ void __launch_bounds__(kPersistBlock) cbq_k_intersect_persistent(
    dev::DagParams dag, const float4* __restrict__ orig, const float4* __restrict__ dir, uint64_t n,
    dev::QueryParams q, dev::HitsOut out, unsigned long long* __restrict__ counter, uint32_t chunk)
{
    extern __shared__ uint32_t smem_stack[];
    dev::SharedStack stack;
    stack.base = smem_stack + threadIdx.x;
    stack.stride = blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(counter, (unsigned long long)chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint64_t end = min((uint64_t)base + chunk, n);
        for (uint64_t i = base + lane; i < end; i += 32) {
            const dev::RayResult r = dev::intersect_volume(dag, __ldg(orig + i), __ldg(dir + i), q, stack,
                                                           (uint32_t*)nullptr);
            dev::write_result(out, i, r);
        }
    }
}

namespace {

cbq_status preload_nested_persistent()
{
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, cbq_k_intersect_persistent) == cudaSuccess) return CBQ_OK;
    cudaGetLastError();
    return CBQ_ERR_CUDA;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

cbq_status cbq_dag_create(const uint32_t* host_nodes, uint64_t node_count, uint32_t root, cbq_dag** out)
{
    return cbq_dag_create_ex(host_nodes, node_count, root, CBQ_DAG_LAYOUT_REFERENCE, out);
}

cbq_status cbq_dag_create_ex(const uint32_t* host_nodes, uint64_t node_count, uint32_t root, uint32_t layout,
                             cbq_dag** out)
{
    if (!out || layout > CBQ_DAG_LAYOUT_COMPACT) return CBQ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cbq_status st = validate_nodes(host_nodes, node_count, root);
    if (st != CBQ_OK) return st;
    cbq_dag* dag = new (std::nothrow) cbq_dag();
    if (!dag) return CBQ_ERR_OUT_OF_MEMORY;
    st = find_subdags(host_nodes, node_count, root, dag->subdags);
    if (st == CBQ_OK) st = validate_heights(host_nodes, node_count, dag->subdags);
    if (st != CBQ_OK) { delete dag; return st; }
    dag->node_count = node_count;
    dag->flat_ok = float_positions_exact(dag);
    dag->root = root;
    dag->max_height = 0;
    for (int i = 0; i < 8; i++)
        if (dag->subdags[i].node_index > 0) dag->max_height = std::max(dag->max_height, dag->subdags[i].node_height);
    if (cudaGetDevice(&dag->device) != cudaSuccess) { delete dag; return CBQ_ERR_CUDA; }
    // Materialise cbq_intersect_host_noalloc's fixed array, and load the persistent
    // kernels it launches, on this device now, while allocating is expected, so that
    // the no-allocation entry point never does (CUDA loads both lazily).
    if (noalloc_prepare(dag->device) != CBQ_OK || preload_persistent_kernels() != CBQ_OK ||
        preload_nested_persistent() != CBQ_OK)
        cbq::log(CBQ_LOG_WARNING, "device %d: the no-allocation staging array could not be prepared", dag->device);
    for (int i = 0; i < 8; i++) dag->sd_ref[i] = dag->subdags[i].node_index;
    const uint32_t* src = host_nodes;
    size_t bytes = (size_t)node_count * 32u;
    std::vector<uint32_t> compact;
    if (layout == CBQ_DAG_LAYOUT_COMPACT) {
        uint32_t refs[8];
        const cbq_status cst = dag->flat_ok ? build_compact(host_nodes, node_count, dag->subdags, compact, refs)
                                            : CBQ_ERR_INVALID_ARGUMENT;
        if (cst == CBQ_OK) {
            dag->layout = CBQ_DAG_LAYOUT_COMPACT;
            std::memcpy(dag->sd_ref, refs, sizeof(refs));
            src = compact.data();
            bytes = compact.size() * sizeof(uint32_t);
        } else {
            cbq::log(CBQ_LOG_WARNING, "compact layout unavailable (%s): using the reference layout",
                     dag->flat_ok ? "store beyond 128 MB" : "coordinates beyond 2^21");
        }
    }
    dag->device_bytes = bytes;
    cudaError_t e = cudaMalloc((void**)&dag->d_nodes, bytes);
    if (e != cudaSuccess) { cudaGetLastError(); delete dag; return CBQ_ERR_OUT_OF_MEMORY; }
    e = cudaMemcpy(dag->d_nodes, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cudaFree(dag->d_nodes); delete dag; return CBQ_ERR_CUDA; }
    cbq::log(CBQ_LOG_INFO,
             "DAG uploaded to device %d: %llu nodes, %s layout (%.1f MB), root %u, max sub-DAG height %d, %s kernel",
             dag->device, (unsigned long long)node_count,
             dag->layout == CBQ_DAG_LAYOUT_COMPACT ? "compact" : "reference", bytes / 1e6, root, dag->max_height,
             dag->flat_ok ? "flat (float positions)" : "flat (integer positions: coordinates beyond 2^21 or 2^29 nodes)");
    *out = dag;
    return CBQ_OK;
}

cbq_status cbq_dag_destroy(cbq_dag* dag)
{
    if (!dag) return CBQ_ERR_INVALID_ARGUMENT;
    cudaFree(dag->d_nodes);
    for (auto& kv : dag->stream_counters) cudaFree(kv.second);
    for (auto& hs : dag->stages) {
        if (hs->d_stage) cudaFree(hs->d_stage);
        for (cudaStream_t& st : hs->pipe)
            if (st) cudaStreamDestroy(st);
        for (cudaEvent_t& ev : hs->pipe_ev)
            if (ev) cudaEventDestroy(ev);
    }
    delete dag;
    return CBQ_OK;
}

cbq_status cbq_dag_get_info(const cbq_dag* dag, cbq_dag_info* info)
{
    if (!dag || !info) return CBQ_ERR_INVALID_ARGUMENT;
    info->node_count = dag->node_count;
    info->bytes = dag->node_count * 32u;
    info->root = dag->root;
    info->max_subdag_height = dag->max_height;
    std::memcpy(info->subdags, dag->subdags, sizeof(dag->subdags));
    info->device_nodes = dag->d_nodes;
    info->layout = dag->layout;
    info->device_bytes = dag->device_bytes;
    return CBQ_OK;
}

cbq_status cbq_dag_set_l2_persistence(const cbq_dag* dag, cbq_stream_t stream, float fraction)
{
    if (!dag || fraction < 0.0f || fraction > 1.0f) return CBQ_ERR_INVALID_ARGUMENT;
    cudaStreamAttrValue attr;
    std::memset(&attr, 0, sizeof(attr));
    if (fraction > 0.0f) {
        int max_window = 0, max_persist = 0;
        cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, dag->device);
        cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, dag->device);
        if (max_window <= 0 || max_persist <= 0) return CBQ_OK;  // not supported: leave caching as is
        const size_t want = (size_t)((double)max_persist * fraction);
        if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) return CBQ_ERR_CUDA;
        const size_t window = std::min<size_t>(dag->device_bytes, (size_t)max_window);
        attr.accessPolicyWindow.base_ptr = dag->d_nodes;
        attr.accessPolicyWindow.num_bytes = window;
        attr.accessPolicyWindow.hitRatio = (float)std::min(1.0, (double)want / (double)window);
        attr.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    }
    if (cudaStreamSetAttribute((cudaStream_t)stream, cudaStreamAttributeAccessPolicyWindow, &attr) != cudaSuccess)
        return CBQ_ERR_CUDA;
    if (fraction == 0.0f) {
        // Give the set-aside back to normal caching, and demote lines already marked
        // persisting (both settings belong to this process's context).
        if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0) != cudaSuccess ||
            cudaCtxResetPersistingL2Cache() != cudaSuccess)
            return CBQ_ERR_CUDA;
    }
    return CBQ_OK;
}

cbq_status cbq_intersect(const cbq_dag* dag, const cbq_rays* rays, uint64_t n, const cbq_query* query,
                         const cbq_hits* hits, cbq_stream_t stream)
{
    if (!dag || !hits) return CBQ_ERR_INVALID_ARGUMENT;
    if (!rays) return CBQ_ERR_INVALID_ARGUMENT;
    if (n == 0) return CBQ_OK;  // an empty batch may carry NULL buffers
    cbq_status st = check_rays(rays);
    if (st != CBQ_OK) return st;
    if (use_flat(dag)) {
        // The DAG's form: persistent (the default, with this stream's work counter) or plain.
        uint64_t* counter = dag->cfg.form != CBQ_FORM_PLAIN ? stream_counter(dag, (cudaStream_t)stream) : nullptr;
        const FlatLaunch fl = counter ? flat_launch(dag, true, counter, 0u) : flat_launch(dag, false, nullptr, 0u);
        return launch_flat(dag, make_dag_params(dag), make_query(query), make_hits(hits),
                           (const float4*)rays->origin_tmax, (const float4*)rays->direction, n, nullptr, fl,
                           (cudaStream_t)stream);
    }
    const uint64_t blocks = (n + kPlainBlock - 1) / kPlainBlock;
    if (blocks > 0x7fffffffull) return CBQ_ERR_INVALID_ARGUMENT;
    cbq_k_intersect_plain<<<(unsigned)blocks, kPlainBlock, 0, (cudaStream_t)stream>>>(
        make_dag_params(dag), (const float4*)rays->origin_tmax, (const float4*)rays->direction, n,
        make_query(query), make_hits(hits), nullptr);
    return cudaGetLastError() == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

cbq_status cbq_dag_set_launch_config(cbq_dag* dag, const cbq_launch_config* cfg)
{
    if (!dag || !cfg) return CBQ_ERR_INVALID_ARGUMENT;
    if (cfg->kernel < CBQ_KERNEL_AUTO || cfg->kernel > CBQ_KERNEL_FLAT) return CBQ_ERR_INVALID_ARGUMENT;
    if (cfg->block < 0 || cfg->block > 256 || (cfg->block % 32) != 0) return CBQ_ERR_INVALID_ARGUMENT;
    if (cfg->refill_min > 32) return CBQ_ERR_INVALID_ARGUMENT;
    if (cfg->stack != CBQ_STACK_SHARED && cfg->stack != CBQ_STACK_LOCAL) return CBQ_ERR_INVALID_ARGUMENT;
    if (cfg->form < CBQ_FORM_PLAIN || cfg->form > CBQ_FORM_SORTED) return CBQ_ERR_INVALID_ARGUMENT;
    if (cfg->steps < 0 || cfg->steps > 32) return CBQ_ERR_INVALID_ARGUMENT;
    if (cfg->registers != 0 && cfg->registers != 56) return CBQ_ERR_INVALID_ARGUMENT;
    if (cfg->kernel == CBQ_KERNEL_NESTED && dag->layout == CBQ_DAG_LAYOUT_COMPACT) return CBQ_ERR_INVALID_ARGUMENT;
    dag->cfg = *cfg;
    return CBQ_OK;
}

uint64_t cbq_scratch_bytes(uint64_t n) { return 256 + 4 * n; }

cbq_status cbq_intersect_auto(const cbq_dag* dag, const cbq_rays* rays, uint64_t n, const cbq_query* query,
                              const cbq_hits* hits, void* scratch, uint64_t scratch_bytes, cbq_stream_t stream)
{
    if (!dag || !hits || !rays) return CBQ_ERR_INVALID_ARGUMENT;
    if (n == 0) return CBQ_OK;
    if (!scratch || scratch_bytes < cbq_scratch_bytes(n) || ((uintptr_t)scratch & 15u))
        return CBQ_ERR_INVALID_ARGUMENT;
    cbq_status st = check_rays(rays);
    if (st != CBQ_OK) return st;
    // Scratch: [0, 8) work counter | [64, 128) octant counts and cursors | [256, 256 + 4n) permutation
    uint64_t* counter = (uint64_t*)scratch;
    uint32_t* counts = (uint32_t*)((char*)scratch + 64);
    uint32_t* perm = (uint32_t*)((char*)scratch + 256);
    const int form = dag->cfg.form;
    if (form == CBQ_FORM_PLAIN || !use_flat(dag)) {
        if (form == CBQ_FORM_PLAIN) return cbq_intersect(dag, rays, n, query, hits, stream);
        return cbq_intersect_persistent(dag, rays, n, query, hits, counter, 0u, stream);
    }
    FlatLaunch fl = flat_launch(dag, true, counter, 0u);
    if (form == CBQ_FORM_SORTED) {
        st = launch_octant_sort((const float4*)rays->direction, n, counts, perm, dag->device, (cudaStream_t)stream);
        if (st != CBQ_OK) return st;
        fl.perm = perm;
    }
    return launch_flat(dag, make_dag_params(dag), make_query(query), make_hits(hits),
                       (const float4*)rays->origin_tmax, (const float4*)rays->direction, n, nullptr, fl,
                       (cudaStream_t)stream);
}

cbq_status cbq_autotune(cbq_dag* dag, const cbq_rays* rays, uint64_t n, const cbq_query* query,
                        const cbq_hits* hits, void* scratch, uint64_t scratch_bytes, int32_t repetitions,
                        cbq_launch_config* best, float* best_ms, cbq_stream_t stream)
{
    if (!dag || repetitions <= 0 || n == 0) return CBQ_ERR_INVALID_ARGUMENT;
    if (!scratch || scratch_bytes < cbq_scratch_bytes(n)) return CBQ_ERR_INVALID_ARGUMENT;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return CBQ_ERR_CUDA;
    const cbq_launch_config saved = dag->cfg;
    cbq_launch_config winner = saved;
    float win_ms = 1e30f;
    cbq_status st = CBQ_OK;
    static const int blocks[] = {64, 128, 256};
    static const uint32_t refills[] = {4, 8, 16};
    static const int stacks[] = {CBQ_STACK_SHARED, CBQ_STACK_LOCAL};
    static const int step_counts[] = {2, 4, 8, 16, 32};
    constexpr int kSteps = 5;
    for (int form = CBQ_FORM_PLAIN; form <= CBQ_FORM_SORTED && st == CBQ_OK; form++) {
        for (int blk : blocks) {
            for (uint32_t rf : refills) {
                if (form == CBQ_FORM_PLAIN && rf != refills[0]) continue;  // refill unused
                // stack x steps, plus the 56-register kernel for the persistent local-stack form
                for (int v = 0; v < 3 * kSteps; v++) {
                    const int stk = v < 2 * kSteps ? stacks[v & 1] : CBQ_STACK_LOCAL;
                    const int regs = v < 2 * kSteps ? 0 : 56;
                    if (regs && form == CBQ_FORM_PLAIN) continue;
                    cbq_launch_config c = saved;
                    c.kernel = CBQ_KERNEL_FLAT;
                    c.block = blk;
                    c.refill_min = rf;
                    c.stack = stk;
                    c.form = form;
                    c.steps = v < 2 * kSteps ? step_counts[v >> 1] : step_counts[v - 2 * kSteps];
                    c.registers = regs;
                    dag->cfg = c;
                    st = cbq_intersect_auto(dag, rays, n, query, hits, scratch, scratch_bytes, stream);  // warm-up
                    if (st != CBQ_OK) break;
                    cudaEventRecord(e0, (cudaStream_t)stream);
                    for (int r = 0; r < repetitions && st == CBQ_OK; r++)
                        st = cbq_intersect_auto(dag, rays, n, query, hits, scratch, scratch_bytes, stream);
                    cudaEventRecord(e1, (cudaStream_t)stream);
                    if (st != CBQ_OK || cudaEventSynchronize(e1) != cudaSuccess) { st = CBQ_ERR_CUDA; break; }
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    ms /= (float)repetitions;
                    if (ms < win_ms) { win_ms = ms; winner = c; }
                }
                if (st != CBQ_OK) break;
            }
            if (st != CBQ_OK) break;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dag->cfg = st == CBQ_OK ? winner : saved;
    if (st == CBQ_OK)
        cbq::log(CBQ_LOG_INFO,
                 "autotune over %llu rays: form %d, block %d, refill %u, stack %s, steps %d, registers %d: %.3f ms",
                 (unsigned long long)n, winner.form, winner.block, winner.refill_min,
                 winner.stack == CBQ_STACK_LOCAL ? "local" : "shared", winner.steps, winner.registers, win_ms);
    if (best) *best = dag->cfg;
    if (best_ms) *best_ms = st == CBQ_OK ? win_ms : 0.0f;
    return st;
}

cbq_status cbq_dag_get_launch_config(const cbq_dag* dag, cbq_launch_config* cfg)
{
    if (!dag || !cfg) return CBQ_ERR_INVALID_ARGUMENT;
    *cfg = dag->cfg;
    if (cfg->kernel == CBQ_KERNEL_AUTO) cfg->kernel = CBQ_KERNEL_FLAT;
    if (cfg->block == 0) cfg->block = use_flat(dag) ? kFlatBlockDefault : kPlainBlock;
    if (cfg->chunk == 0) cfg->chunk = kDefaultChunk;
    if (cfg->refill_min == 0) cfg->refill_min = kRefillDefault;
    return CBQ_OK;
}

cbq_status cbq_count_fetches(const cbq_dag* dag, const cbq_rays* rays, uint64_t n, const cbq_query* query,
                             uint32_t* fetches, cbq_stream_t stream)
{
    if (!dag || !fetches) return CBQ_ERR_INVALID_ARGUMENT;
    if (!rays) return CBQ_ERR_INVALID_ARGUMENT;
    if (n == 0) return CBQ_OK;  // an empty batch may carry NULL buffers
    cbq_status st = check_rays(rays);
    if (st != CBQ_OK) return st;
    dev::HitsOut none;
    std::memset(&none, 0, sizeof(none));
    if (use_flat(dag))
        return launch_flat(dag, make_dag_params(dag), make_query(query), none, (const float4*)rays->origin_tmax,
                           (const float4*)rays->direction, n, fetches, flat_launch(dag, false, nullptr, 0u),
                           (cudaStream_t)stream);
    const uint64_t blocks = (n + kPlainBlock - 1) / kPlainBlock;
    cbq_k_intersect_plain<<<(unsigned)blocks, kPlainBlock, 0, (cudaStream_t)stream>>>(
        make_dag_params(dag), (const float4*)rays->origin_tmax, (const float4*)rays->direction, n,
        make_query(query), none, fetches);
    return cudaGetLastError() == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

cbq_status cbq_intersect_persistent(const cbq_dag* dag, const cbq_rays* rays, uint64_t n, const cbq_query* query,
                                    const cbq_hits* hits, uint64_t* work_counter, uint32_t chunk,
                                    cbq_stream_t stream)
{
    if (!dag || !hits || !work_counter) return CBQ_ERR_INVALID_ARGUMENT;
    if (!rays) return CBQ_ERR_INVALID_ARGUMENT;
    if (n == 0) return CBQ_OK;  // an empty batch may carry NULL buffers
    cbq_status st = check_rays(rays);
    if (st != CBQ_OK) return st;
    if (use_flat(dag))
        return launch_flat(dag, make_dag_params(dag), make_query(query), make_hits(hits),
                           (const float4*)rays->origin_tmax, (const float4*)rays->direction, n, nullptr,
                           flat_launch(dag, true, work_counter, std::min<uint32_t>(chunk, 32u)),
                           (cudaStream_t)stream);
    if (chunk == 0) chunk = dag->cfg.chunk ? dag->cfg.chunk : kDefaultChunk;
    const int stack_h = std::max(1, (int)dag->max_height);
    const size_t smem = (size_t)stack_h * kPersistBlock * sizeof(uint32_t);
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dag->device) != cudaSuccess) return CBQ_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cbq_k_intersect_persistent, kPersistBlock, smem) !=
        cudaSuccess)
        return CBQ_ERR_CUDA;
    per_sm = std::max(per_sm, 1);
    if (cudaMemsetAsync(work_counter, 0, sizeof(uint64_t), (cudaStream_t)stream) != cudaSuccess) return CBQ_ERR_CUDA;
    cbq_k_intersect_persistent<<<sms * per_sm, kPersistBlock, smem, (cudaStream_t)stream>>>(
        make_dag_params(dag), (const float4*)rays->origin_tmax, (const float4*)rays->direction, n,
        make_query(query), make_hits(hits), (unsigned long long*)work_counter, chunk);
    return cudaGetLastError() == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

}  // extern "C"

namespace {

// cbq_intersect_host calls in flight in this process (any DAG).
std::atomic<int> g_host_calls{0};
struct HostCallCount {
    HostCallCount() { g_host_calls.fetch_add(1, std::memory_order_relaxed); }
    ~HostCallCount() { g_host_calls.fetch_sub(1, std::memory_order_relaxed); }
};

// Takes a staging set of `dag` for one call, locked: a free one, else a new
// one while fewer than kHostStagesMax exist, else the first (waiting for it).
std::unique_lock<std::mutex> take_stage(cbq_dag* dag, HostStage** out)
{
    std::unique_lock<std::mutex> pool(dag->stages_lock);
    for (auto& hs : dag->stages) {
        std::unique_lock<std::mutex> lk(hs->lock, std::try_to_lock);
        if (lk.owns_lock()) {
            *out = hs.get();
            return lk;
        }
    }
    if ((int)dag->stages.size() < kHostStagesMax) {
        HostStage* hs = new (std::nothrow) HostStage();
        if (hs) {
            try {
                dag->stages.emplace_back(hs);
            } catch (const std::exception&) {  // nothing may throw across the C ABI
                delete hs;
                hs = nullptr;
            }
        }
        if (hs) {
            *out = hs;
            return std::unique_lock<std::mutex>(hs->lock);
        }
        if (dag->stages.empty()) {
            *out = nullptr;
            return std::unique_lock<std::mutex>();
        }
    }
    HostStage* hs = dag->stages.front().get();
    pool.unlock();
    *out = hs;
    return std::unique_lock<std::mutex>(hs->lock);
}

}  // namespace

extern "C" cbq_status cbq_intersect_host(const cbq_dag* cdag, const float* host_origin_tmax,
                                         const float* host_direction, uint64_t n, const cbq_query* query,
                                         const cbq_hits* host_hits)
{
    if (!cdag || !host_origin_tmax || !host_direction || !host_hits) return CBQ_ERR_INVALID_ARGUMENT;
    if (n == 0) return CBQ_OK;
    const HostCallCount in_flight;
    cbq_dag* dag = const_cast<cbq_dag*>(cdag);
    HostStage* hs = nullptr;
    std::unique_lock<std::mutex> lock = take_stage(dag, &hs);
    if (!hs) return CBQ_ERR_OUT_OF_MEMORY;
    // Staging: rays (32 B), hit fields (46 B) per ray, then one work counter per chunk.
    const size_t per_ray = 32 + 1 + 4 + 4 + 12 + 12 + 12 + 1;
    const size_t tail = 256 + kHostChunksMax * 64;
    if (n > hs->capacity) {
        if (hs->d_stage) cudaFree(hs->d_stage);
        hs->d_stage = nullptr;
        hs->capacity = 0;
        if (cudaMalloc(&hs->d_stage, (size_t)n * per_ray + tail) != cudaSuccess) {
            cudaGetLastError();
            return CBQ_ERR_OUT_OF_MEMORY;
        }
        hs->capacity = n;
    }
    if (!hs->pipe[0]) {  // created all together, or not at all
        bool ok = true;
        for (int k = 0; k < 4 && ok; k++)
            ok = cudaStreamCreateWithFlags(&hs->pipe[k], cudaStreamNonBlocking) == cudaSuccess;
        for (uint64_t k = 0; k < 2 * kHostChunksMax && ok; k++)
            ok = cudaEventCreateWithFlags(&hs->pipe_ev[k], cudaEventDisableTiming) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            for (cudaStream_t& st : hs->pipe)
                if (st) { cudaStreamDestroy(st); st = nullptr; }
            for (cudaEvent_t& ev : hs->pipe_ev)
                if (ev) { cudaEventDestroy(ev); ev = nullptr; }
            return CBQ_ERR_CUDA;
        }
    }
    char* p = (char*)hs->d_stage;
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
    dh.status = (uint8_t*)p;
    p += n;
    // Work counters, one 64-byte line per chunk.
    uint64_t* d_counters = (uint64_t*)(((uintptr_t)p + 255u) & ~(uintptr_t)255u);
    // Chunks pipeline the copies with the traversal: while chunk k is traversed, chunk k + 1 is
    // copied in and chunk k - 1 copied out.  Consecutive chunks are traversed on alternating
    // streams, so the next chunk's blocks fill the SMs while the previous launch drains (a
    // persistent launch ends with a tail of few busy warps).  Events order each chunk's copy in,
    // traversal and copy out.  Chunks interleave blocks of the batch (HostChunk).  Measured on
    // terrain-4096 (primary and bounce calls, 4 Mi rays each): alone, 8 chunks per call (3.0
    // Grays/s end to end; 2.9 with 4); with the two batches' calls from two threads, 4 chunks
    // (4.25 against 3.9 with 8).
    const uint64_t cmax =
        g_host_calls.load(std::memory_order_relaxed) > 1 ? kHostChunksConcurrent : kHostChunksMax;
    const uint64_t chunks = std::min<uint64_t>(cmax, std::max<uint64_t>(1, n / kHostChunkMin));
    cudaStream_t s_in = hs->pipe[0], s_out = hs->pipe[1];
    // Every queued copy and launch ends before the call returns (the staging buffers are reused).
    auto drain = [&](cbq_status st) {
        bool ok = true;
        for (cudaStream_t s : hs->pipe) ok = cudaStreamSynchronize(s) == cudaSuccess && ok;
        return ok ? st : CBQ_ERR_CUDA;
    };
    const uint64_t block = std::max<uint64_t>(kHostBlockMin, n / (chunks * kHostBlocksPerChunk));
    uint64_t start = 0;
    for (uint64_t k = 0; k < chunks; k++) {
        const HostChunk hc = host_chunk(n, chunks, block, k, start);
        const uint64_t a = start, m = hc.rays();
        start += m;
        if (m == 0) continue;
        cudaStream_t s_run = hs->pipe[2 + (k & 1)];
        cudaEvent_t copied = hs->pipe_ev[2 * k], traversed = hs->pipe_ev[2 * k + 1];
        if (!copy_chunk((void*)host_origin_tmax, d_o, 16, hc, k, chunks, cudaMemcpyHostToDevice, s_in) ||
            !copy_chunk((void*)host_direction, d_d, 16, hc, k, chunks, cudaMemcpyHostToDevice, s_in) ||
            cudaEventRecord(copied, s_in) != cudaSuccess || cudaStreamWaitEvent(s_run, copied, 0) != cudaSuccess)
            return drain(CBQ_ERR_CUDA);
        cbq_hits launch;
        launch.hit = host_hits->hit ? dh.hit + a : nullptr;
        launch.distance = host_hits->distance ? dh.distance + a : nullptr;
        launch.material = host_hits->material ? dh.material + a : nullptr;
        launch.position = host_hits->position ? dh.position + 3 * a : nullptr;
        launch.normal = host_hits->normal ? dh.normal + 3 * a : nullptr;
        launch.voxel = host_hits->voxel ? dh.voxel + 3 * a : nullptr;
        launch.status = host_hits->status ? dh.status + a : nullptr;
        cbq_rays rays{d_o + 4 * a, d_d + 4 * a};
        // Persistent form; each chunk's counter is private to this call (its staging set is held).
        cbq_status st = cbq_intersect_persistent(dag, &rays, m, query, &launch, d_counters + 8 * k, 0u,
                                                 (cbq_stream_t)s_run);
        if (st != CBQ_OK) return drain(st);
        if (cudaEventRecord(traversed, s_run) != cudaSuccess || cudaStreamWaitEvent(s_out, traversed, 0) != cudaSuccess)
            return drain(CBQ_ERR_CUDA);
        struct Copy {
            void* host;
            void* dev;
            size_t width;
        };
        const Copy copies[] = {{host_hits->hit, dh.hit, 1},           {host_hits->distance, dh.distance, 4},
                               {host_hits->material, dh.material, 4}, {host_hits->position, dh.position, 12},
                               {host_hits->normal, dh.normal, 12},    {host_hits->voxel, dh.voxel, 12},
                               {host_hits->status, dh.status, 1}};
        for (const Copy& c : copies) {
            if (!c.host) continue;
            if (!copy_chunk(c.host, c.dev, c.width, hc, k, chunks, cudaMemcpyDeviceToHost, s_out))
                return drain(CBQ_ERR_CUDA);
        }
    }
    return drain(CBQ_OK);
}
