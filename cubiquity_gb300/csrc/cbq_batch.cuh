// Job table of the multi-volume traversal kernel, shared by the batch API
// (cbq_batch.cu) and the request server (cbq_server.cu).
#pragma once

#include "cbq_flat.cuh"
#include "cbq_internal.hpp"

#include <cuda_runtime.h>

namespace cbq {
namespace dev {

// One job: a volume, its rays, its outputs and its query.  Jobs with rays are
// stored back to back in global ray index space starting at `first`.
struct JobDesc {
    const uint32_t* nodes;
    const float4* orig;
    const float4* dir;
    HitsOut out;
    uint64_t first;
    uint64_t count;
    QueryParams q;
    uint32_t pad;
    SubDag sd[8];
};

}  // namespace dev

// Fills the parts of a JobDesc that come from the volume.
void fill_job_volume(dev::JobDesc& d, const cbq_dag* dag);

// Launch shape of the multi-volume kernel.
struct BatchLaunch {
    int block = 128;
    uint32_t refill = 8;             // idle lanes that trigger a warp's refill
    uint32_t steps = 8;              // ESVO steps per loop iteration
    bool registers56 = false;        // local-stack kernel held to 56 registers
    bool shared_stack = false;       // descent stack in shared memory (stack_rows rows) instead of local
    int stack_rows = 0;              // max SubDAG height over the jobs
    const uint32_t* perm = nullptr;  // octant order (launch_batch_octant_sort), or null
};

// Launches the persistent multi-volume kernel over `njobs` device-resident job
// descriptors holding `total` rays; all jobs' volumes have the compact layout,
// or none.  `counter` is zeroed on `stream` first.
cbq_status launch_batch_kernel(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint64_t* counter,
                               bool compact, int device, cudaStream_t stream, const BatchLaunch& bl);

// The same with the default shape but for block, refill, steps and register cap.
cbq_status launch_batch_kernel(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint64_t* counter,
                               int block, uint32_t refill, uint32_t steps, bool compact, int device,
                               cudaStream_t stream, bool registers56 = false);

// Groups each job's rays by octant (direction sign bits): perm[g] for g in a
// job's range [first, first + count) is a ray of the same job, all of its
// octant-0 rays first, then octant 1, and so on.  `scratch` holds 16 uint32
// per job (counts and cursors, zeroed here).
cbq_status launch_batch_octant_sort(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint32_t* scratch,
                                    uint32_t* perm, int device, cudaStream_t stream);

constexpr uint32_t kBatchStepsDefault = 8;

}  // namespace cbq
