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

// Launches the persistent multi-volume kernel over `njobs` device-resident job
// descriptors holding `total` rays, `steps` ESVO steps per loop iteration; all
// jobs' volumes have the compact layout, or none.  `counter` is zeroed on
// `stream` first.
cbq_status launch_batch_kernel(const dev::JobDesc* d_jobs, uint32_t njobs, uint64_t total, uint64_t* counter,
                               int block, uint32_t refill, uint32_t steps, bool compact, int device,
                               cudaStream_t stream, bool registers56 = false);

constexpr uint32_t kBatchStepsDefault = 8;

}  // namespace cbq
