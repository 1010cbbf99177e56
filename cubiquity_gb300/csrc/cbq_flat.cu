// Kernels of the flat traversal (cbq_flat.cuh), the octant sort, and their
// launchers.
#include "cbq_flat.cuh"
#include "cbq_internal.hpp"

#include <cuda_runtime.h>

#include <algorithm>

namespace cbq {
namespace dev {

constexpr unsigned kFull = 0xffffffffu;

// PERSISTENT = false: one ray per thread (the drop-in form).
// PERSISTENT = true : an SM-sized grid; when at least `refill_min` lanes of a
//                     warp are idle, the warp takes that many new rays from
//                     `counter` with one atomic and the idle lanes start them.
// SHARED: descent stack in shared memory (one column per thread) or in a
//         per-thread local array.
// SORTED: ray g of the launch is ray perm[g] of the input (octant order).
// Ctx: FlatCtxT of the node store layout.
template <bool PERSISTENT, bool SHARED, bool SORTED, typename Ctx>
__device__ __forceinline__ void flat_body(const Ctx& c, uint64_t n, unsigned long long* __restrict__ counter,
                                          uint32_t refill_min, const uint32_t* __restrict__ perm, uint32_t steps)
{
    extern __shared__ uint32_t smem_stack[];
    SharedStack sstack;
    sstack.base = smem_stack + threadIdx.x;
    sstack.stride = blockDim.x;
    LocalStack lstack;
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t below = (1u << lane) - 1u;

    Lane L;
    L.mode = kLaneIdle;
    L.held = 0u;
    bool more = PERSISTENT;  // warp-uniform: the queue may still hold rays
    if (!PERSISTENT) {
        const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i < n) lane_begin(L, c, SORTED ? (uint64_t)__ldg(perm + i) : c.ray_slot(i));
    }
    for (;;) {
        if (PERSISTENT && more) {
            const uint32_t idle = __ballot_sync(kFull, L.mode == kLaneIdle);
            const uint32_t cnt = __popc(idle);
            if (cnt == 32u || (cnt != 0u && cnt >= refill_min)) {
                const int leader = __ffs(idle) - 1;
                unsigned long long base = 0;
                if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)cnt);
                base = __shfl_sync(kFull, base, leader);
                if (L.mode == kLaneIdle) {
                    const uint64_t i = base + __popc(idle & below);
                    if (i < n) lane_begin(L, c, SORTED ? (uint64_t)__ldg(perm + i) : c.ray_slot(i));
                }
                if (base + cnt >= n) more = false;
            }
        }
        if (!__any_sync(kFull, L.mode != kLaneIdle)) {
            if (!more) break;
            continue;
        }
        lane_settle(L, c);
        // Up to `steps` ESVO steps per outer iteration: amortises the refill
        // ballot and the settle check over several node fetches.
        if (SHARED)
            warp_walk_steps(L, c, sstack, steps);
        else
            warp_walk_steps(L, c, lstack, steps);
    }
}

template <bool PERSISTENT, bool SHARED, bool SORTED, typename Ctx>
__global__ void __launch_bounds__(256) cbq_k_flat(Ctx c, uint64_t n, unsigned long long* __restrict__ counter,
                                                  uint32_t refill_min, const uint32_t* __restrict__ perm,
                                                  uint32_t steps)
{
    flat_body<PERSISTENT, SHARED, SORTED>(c, n, counter, refill_min, perm, steps);
}

// The persistent local-stack form held to 56 registers per thread: 36 resident
// warps per SM instead of 32 with blocks of 64 or 128 threads.  Measured on
// GB300 it is the faster choice for incoherent (bounce) rays, so the tuner
// tries it (launch config `registers` = 56).
template <bool SORTED, typename Ctx>
__global__ void __maxnreg__(56) cbq_k_flat_r56(Ctx c, uint64_t n, unsigned long long* __restrict__ counter,
                                               uint32_t refill_min, const uint32_t* __restrict__ perm,
                                               uint32_t steps)
{
    flat_body<true, false, SORTED>(c, n, counter, refill_min, perm, steps);
}

// Octant of a ray: its direction sign bits (raytracing.cpp:416-417).
__device__ __forceinline__ uint32_t octant_of(float4 d)
{
    return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
}

// counts[8] += rays per octant.
__global__ void __launch_bounds__(256) cbq_k_octant_count(const float4* __restrict__ dir, uint32_t n,
                                                          uint32_t* __restrict__ counts)
{
    __shared__ uint32_t c[8];
    if (threadIdx.x < 8) c[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&c[octant_of(__ldg(dir + i))], 1u);
    __syncthreads();
    if (threadIdx.x < 8 && c[threadIdx.x]) atomicAdd(&counts[threadIdx.x], c[threadIdx.x]);
}

// perm[start(octant) + k] = i: rays grouped by octant (order within a group
// follows the atomics).  Every index i < n is written exactly once.
__global__ void __launch_bounds__(256) cbq_k_octant_scatter(const float4* __restrict__ dir, uint32_t n,
                                                            const uint32_t* __restrict__ counts,
                                                            uint32_t* __restrict__ cursor, uint32_t* __restrict__ perm)
{
    __shared__ uint32_t start[8];
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int b = 0; b < 8; b++) {
            start[b] = s;
            s += counts[b];
        }
    }
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        const uint32_t i = i0 + threadIdx.x;
        const bool valid = i < n;
        const unsigned act = __ballot_sync(kFull, valid);
        if (!valid) continue;
        const uint32_t b = octant_of(__ldg(dir + i));
        const unsigned grp = __match_any_sync(act, b);
        const int leader = __ffs(grp) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&cursor[b], (uint32_t)__popc(grp));
        base = __shfl_sync(grp, base, leader);
        perm[start[b] + base + __popc(grp & ((1u << lane) - 1u))] = i;
    }
}

}  // namespace dev

// True when every occupied SubDAG's reflected coordinates stay within
// +-2^21 (heights at most 21), so the flat kernel's float positions are exact
// and their biased bit patterns carry the integer bits its pop reads, and the
// store has fewer than 2^29 nodes, so its word offsets fit 32 bits.
bool float_positions_exact(const cbq_dag* dag)
{
    if (dag->node_count > dev::kFlatMaxNodes) return false;  // 32-bit node word offsets
    const int64_t lim = (int64_t)1 << 21;
    for (int i = 0; i < 8; i++) {
        const cbq_subdag& s = dag->subdags[i];
        if (s.node_index == 0) continue;
        if (s.node_height > 21) return false;
        const int64_t size = (int64_t)1 << s.node_height;
        for (int a = 0; a < 3; a++) {
            const int64_t lo = s.lower_bound[a], hi = lo + size;
            if (lo < -lim || hi > lim) return false;
        }
    }
    return true;
}

namespace {

template <typename Ctx>
bool query_persistent_kernels()
{
    cudaFuncAttributes a;
    return cudaFuncGetAttributes(&a, dev::cbq_k_flat<true, false, false, Ctx>) == cudaSuccess &&
           cudaFuncGetAttributes(&a, dev::cbq_k_flat<true, false, true, Ctx>) == cudaSuccess &&
           cudaFuncGetAttributes(&a, dev::cbq_k_flat<true, true, false, Ctx>) == cudaSuccess &&
           cudaFuncGetAttributes(&a, dev::cbq_k_flat<true, true, true, Ctx>) == cudaSuccess &&
           cudaFuncGetAttributes(&a, dev::cbq_k_flat_r56<false, Ctx>) == cudaSuccess &&
           cudaFuncGetAttributes(&a, dev::cbq_k_flat_r56<true, Ctx>) == cudaSuccess;
}

}  // namespace

// Querying a kernel's attributes loads it on the current device (CUDA loads
// modules and kernels lazily, on first use, and that load can take device
// memory).  Done for every persistent traversal kernel when a DAG is created.
cbq_status preload_persistent_kernels()
{
    const bool ok = query_persistent_kernels<dev::FlatCtxT<false>>() && query_persistent_kernels<dev::FlatCtxT<true>>() &&
                    query_persistent_kernels<dev::FlatCtxT<false, false, true>>();
    if (!ok) cudaGetLastError();
    return ok ? CBQ_OK : CBQ_ERR_CUDA;
}

namespace {

template <bool P, bool S, bool O, typename Ctx>
cbq_status launch_variant(const Ctx& c, uint64_t n, const FlatLaunch& fl, int rows, cudaStream_t stream,
                          int device)
{
    const size_t smem = S ? (size_t)rows * fl.block * sizeof(uint32_t) : 0;
    if (!P) {
        const uint64_t blocks = (n + fl.block - 1) / fl.block;
        if (blocks > 0x7fffffffull) return CBQ_ERR_INVALID_ARGUMENT;
        dev::cbq_k_flat<false, S, O, Ctx><<<(unsigned)blocks, fl.block, smem, stream>>>(c, n, nullptr, 0u, fl.perm,
                                                                                     fl.steps ? fl.steps : 1u);
    } else {
        int sms = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return CBQ_ERR_CUDA;
        auto kernel = dev::cbq_k_flat<true, S, O, Ctx>;
        if constexpr (!S) {
            if (fl.registers56) kernel = dev::cbq_k_flat_r56<O, Ctx>;
        }
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, fl.block, smem) != cudaSuccess)
            return CBQ_ERR_CUDA;
        per_sm = std::max(per_sm, 1);
        if (cudaMemsetAsync(fl.counter, 0, sizeof(uint64_t), stream) != cudaSuccess) return CBQ_ERR_CUDA;
        kernel<<<sms * per_sm, fl.block, smem, stream>>>(c, n, (unsigned long long*)fl.counter, fl.refill_min,
                                                          fl.perm, fl.steps ? fl.steps : 1u);
    }
    return cudaGetLastError() == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

}  // namespace

cbq_status launch_octant_sort(const float4* dir, uint64_t n, uint32_t* counts16, uint32_t* perm, int device,
                              cudaStream_t stream)
{
    if (n >= 0xffffffffull) return CBQ_ERR_INVALID_ARGUMENT;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return CBQ_ERR_CUDA;
    if (cudaMemsetAsync(counts16, 0, 16 * sizeof(uint32_t), stream) != cudaSuccess) return CBQ_ERR_CUDA;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8));
    dev::cbq_k_octant_count<<<grid, 256, 0, stream>>>(dir, (uint32_t)n, counts16);
    dev::cbq_k_octant_scatter<<<grid, 256, 0, stream>>>(dir, (uint32_t)n, counts16, counts16 + 8, perm);
    return cudaGetLastError() == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

// The eight launch shapes of one context type.
template <typename Ctx>
cbq_status launch_ctx(const Ctx& c, uint64_t n, const FlatLaunch& fl, int rows, cudaStream_t stream, int dv)
{
    const bool sorted = fl.perm != nullptr;
    if (fl.persistent) {
        if (fl.local_stack)
            return sorted ? launch_variant<true, false, true>(c, n, fl, rows, stream, dv)
                          : launch_variant<true, false, false>(c, n, fl, rows, stream, dv);
        return sorted ? launch_variant<true, true, true>(c, n, fl, rows, stream, dv)
                      : launch_variant<true, true, false>(c, n, fl, rows, stream, dv);
    }
    if (fl.local_stack)
        return sorted ? launch_variant<false, false, true>(c, n, fl, rows, stream, dv)
                      : launch_variant<false, false, false>(c, n, fl, rows, stream, dv);
    return sorted ? launch_variant<false, true, true>(c, n, fl, rows, stream, dv)
                  : launch_variant<false, true, false>(c, n, fl, rows, stream, dv);
}

template <typename Ctx>
Ctx make_ctx(const dev::DagParams& dp, const dev::QueryParams& q, const dev::HitsOut& out, const float4* orig,
             const float4* dir, uint32_t* fetch_out)
{
    Ctx c;
    c.dag = dp;
    c.q = q;
    c.out = out;
    c.orig = orig;
    c.dir = dir;
    c.fetch_out = fetch_out;
    return c;
}

cbq_status launch_flat(const cbq_dag* dag, const dev::DagParams& dp, const dev::QueryParams& query,
                       const dev::HitsOut& out, const float4* orig, const float4* dir, uint64_t n,
                       uint32_t* fetch_out, const FlatLaunch& fl, cudaStream_t stream)
{
    // The image order applies where it is a bijection of this launch's rays:
    // whole 8-row bands of a width that is a multiple of 4, 32-bit indices.
    dev::QueryParams q = query;
    const uint64_t band = 8ull * q.image_width;
    if (q.image_width && ((q.image_width & 3u) || n >= (1ull << 32) || n % band != 0 || fl.perm))
        q.image_width = 0u;
    if (fl.persistent && !fl.counter) return CBQ_ERR_INVALID_ARGUMENT;
    if (fl.perm && n >= 0xffffffffull) return CBQ_ERR_INVALID_ARGUMENT;
    const int rows = std::max(1, (int)dag->max_height);
    const int dv = dag->device;
    if (fetch_out) {  // fetch / load counting: its own instantiation, one shape
        FlatLaunch one = fl;
        one.persistent = false;
        one.local_stack = true;
        one.perm = nullptr;
        if (dag->layout == CBQ_DAG_LAYOUT_COMPACT)
            return launch_variant<false, false, false>(
                make_ctx<dev::FlatCtxT<true, true>>(dp, q, out, orig, dir, fetch_out), n, one, rows, stream, dv);
        if (!dag->flat_ok)
            return launch_variant<false, false, false>(
                make_ctx<dev::FlatCtxT<false, true, true>>(dp, q, out, orig, dir, fetch_out), n, one, rows, stream,
                dv);
        return launch_variant<false, false, false>(
            make_ctx<dev::FlatCtxT<false, true>>(dp, q, out, orig, dir, fetch_out), n, one, rows, stream, dv);
    }
    if (dag->layout == CBQ_DAG_LAYOUT_COMPACT)
        return launch_ctx(make_ctx<dev::FlatCtxT<true>>(dp, q, out, orig, dir, nullptr), n, fl, rows, stream, dv);
    if (!dag->flat_ok)  // coordinates beyond +-2^21 or 2^29 nodes or more: integer positions
        return launch_ctx(make_ctx<dev::FlatCtxT<false, false, true>>(dp, q, out, orig, dir, nullptr), n, fl, rows,
                          stream, dv);
    return launch_ctx(make_ctx<dev::FlatCtxT<false>>(dp, q, out, orig, dir, nullptr), n, fl, rows, stream, dv);
}

}  // namespace cbq
