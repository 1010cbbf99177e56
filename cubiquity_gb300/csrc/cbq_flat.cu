// Kernels of the flat traversal (cbq_flat.cuh) and their launchers.
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
template <bool PERSISTENT>
__global__ void __launch_bounds__(256) cbq_k_flat(FlatCtx c, uint64_t n, unsigned long long* __restrict__ counter,
                                                  uint32_t refill_min)
{
    extern __shared__ uint32_t smem_stack[];
    SharedStack stack;
    stack.base = smem_stack + threadIdx.x;
    stack.stride = blockDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t below = (1u << lane) - 1u;

    Lane L;
    L.mode = kLaneIdle;
    bool more = PERSISTENT;  // warp-uniform: the queue may still hold rays
    if (!PERSISTENT) {
        const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i < n) lane_begin(L, c, i);
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
                    if (i < n) lane_begin(L, c, i);
                }
                if (base + cnt >= n) more = false;
            }
        }
        if (!__any_sync(kFull, L.mode != kLaneIdle)) {
            if (!more) break;
            continue;
        }
        lane_settle(L, c);
        if (L.mode == kLaneWalk) lane_walk(L, c, stack);
    }
}

template __global__ void cbq_k_flat<false>(FlatCtx, uint64_t, unsigned long long*, uint32_t);
template __global__ void cbq_k_flat<true>(FlatCtx, uint64_t, unsigned long long*, uint32_t);

}  // namespace dev

// True when every occupied SubDAG's reflected coordinates stay within
// +-2^24, so the flat kernel's float positions are exact.
bool float_positions_exact(const cbq_dag* dag)
{
    const int64_t lim = (int64_t)1 << 24;
    for (int i = 0; i < 8; i++) {
        const cbq_subdag& s = dag->subdags[i];
        if (s.node_index == 0) continue;
        const int64_t size = (int64_t)1 << s.node_height;
        for (int a = 0; a < 3; a++) {
            const int64_t lo = s.lower_bound[a], hi = lo + size;
            if (lo < -lim || hi > lim) return false;
        }
    }
    return true;
}

cbq_status launch_flat(const cbq_dag* dag, const dev::DagParams& dp, const dev::QueryParams& q,
                       const dev::HitsOut& out, const float4* orig, const float4* dir, uint64_t n,
                       uint32_t* fetch_out, bool persistent, uint64_t* counter, int block, uint32_t refill_min,
                       cudaStream_t stream)
{
    dev::FlatCtx c;
    c.dag = dp;
    c.q = q;
    c.out = out;
    c.orig = orig;
    c.dir = dir;
    c.fetch_out = fetch_out;
    const int rows = std::max(1, (int)dag->max_height);
    const size_t smem = (size_t)rows * block * sizeof(uint32_t);
    if (!persistent) {
        const uint64_t blocks = (n + block - 1) / block;
        if (blocks > 0x7fffffffull) return CBQ_ERR_INVALID_ARGUMENT;
        dev::cbq_k_flat<false><<<(unsigned)blocks, block, smem, stream>>>(c, n, nullptr, 0u);
    } else {
        if (!counter) return CBQ_ERR_INVALID_ARGUMENT;
        int sms = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dag->device) != cudaSuccess)
            return CBQ_ERR_CUDA;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::cbq_k_flat<true>, block, smem) != cudaSuccess)
            return CBQ_ERR_CUDA;
        per_sm = std::max(per_sm, 1);
        if (cudaMemsetAsync(counter, 0, sizeof(uint64_t), stream) != cudaSuccess) return CBQ_ERR_CUDA;
        dev::cbq_k_flat<true><<<sms * per_sm, block, smem, stream>>>(c, n, (unsigned long long*)counter,
                                                                     refill_min);
    }
    return cudaGetLastError() == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

}  // namespace cbq
