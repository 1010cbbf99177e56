// Internal declarations shared by the host (.cpp) and device (.cu) parts of
// libcbq.  Not part of the public ABI.
#pragma once

#include "../../include/cubiquity_gb300.h"

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

namespace cbq {

// Host-side findSubDAGs (raytracing.cpp:43-97).  Returns CBQ_ERR_BAD_DAG if a
// followed index is out of range.
cbq_status find_subdags(const uint32_t* nodes, uint64_t node_count, uint32_t root, cbq_subdag out[8]);

// Full structural check of a host node array.
cbq_status validate_nodes(const uint32_t* nodes, uint64_t node_count, uint32_t root);

// printf-style message to the registered log handler (no-op without one).
void log(int level, const char* fmt, ...)
#if defined(__GNUC__)
    __attribute__((format(printf, 2, 3)))
#endif
    ;

// Checks that no internal node is reachable from a SubDAG root at height 0
// (which also excludes cycles), so a traversal never descends below the leaves.
cbq_status validate_heights(const uint32_t* nodes, uint64_t node_count, const cbq_subdag subdags[8]);

// Compact node store (CBQ_DAG_LAYOUT_COMPACT).  Every internal node reachable
// from a SubDAG root keeps only its occupied children, packed in slot order.  A
// reference to an internal node is (offset << 8) | occupancy mask, the offset
// counted in 8-byte units from the start of the store; unit 0 is unused, so
// every such reference is >= 256, above the material values, which children
// keep as they are.  A SubDAG rooted at a material m becomes a node with eight
// children m.  sd_ref[k] is SubDAG k's root reference (0 if empty).
// CBQ_ERR_CAPACITY when the store would exceed 2^24 units (128 MB).
cbq_status build_compact(const uint32_t* nodes, uint64_t node_count, const cbq_subdag subdags[8],
                         std::vector<uint32_t>& store, uint32_t sd_ref[8]);

// Resolves, on the current device, the device address of the fixed staging
// array of cbq_intersect_host_noalloc.  The lookup loads the module that holds
// the array, which is when the array takes its device memory; cbq_dag_create
// calls this so that the allocation happens there, never inside a
// cbq_intersect_host_noalloc call.
cbq_status noalloc_prepare(int device);

// Calls of cbq_intersect_host on one DAG that overlap in time (from several
// host threads) each take their own staging set, up to kHostStagesMax of them;
// beyond that they queue for one.
constexpr int kHostStagesMax = 4;

// cbq_intersect_host splits a call into at most kHostChunksMax chunks of at
// least kHostChunkMin rays; kHostChunksConcurrent while another call is in
// flight in the process (its copies and traversals fill the gaps that smaller
// chunks would, so fewer persistent-launch tails pay more).
constexpr uint64_t kHostChunksMax = 8;
constexpr uint64_t kHostChunksConcurrent = 4;
constexpr uint64_t kHostChunkMin = 1ull << 18;
// ... each made of about kHostBlocksPerChunk blocks of consecutive rays (at least
// kHostBlockMin) dealt round-robin.
constexpr uint64_t kHostBlocksPerChunk = 4;
constexpr uint64_t kHostBlockMin = 4096;

// Device staging and streams of one cbq_intersect_host call at a time: rays and
// hits, copied in and out in chunks on four streams (copy in, copy out, two for
// traversal) so that copies overlap the traversal.
struct HostStage {
    std::mutex lock;               // held by the call using this set
    void* d_stage = nullptr;
    uint64_t capacity = 0;         // rays
    struct CUstream_st* pipe[4] = {};  // cudaStream_t (this header is also compiled without CUDA)
    struct CUevent_st* pipe_ev[2 * kHostChunksMax] = {};  // cudaEvent_t
};

}  // namespace cbq

// The opaque DAG handle.
struct cbq_dag {
    uint32_t* d_nodes = nullptr;   // device: node_count * 8 words, or the compact store
    uint32_t layout = CBQ_DAG_LAYOUT_REFERENCE;
    uint64_t device_bytes = 0;     // size of the device node store
    uint32_t sd_ref[8] = {};       // SubDAG roots as the device store refers to them
    uint64_t node_count = 0;
    uint32_t root = 0;
    cbq_subdag subdags[8];
    int32_t max_height = 0;        // max SubDAG height (stack depth)
    int device = 0;
    bool flat_ok = false;          // float-position flat kernel applies (coordinates within +-2^21,
                                   // under 2^29 nodes); otherwise the integer-position form
    // Defaults from GB300 sweeps of untuned shapes on terrain-4096 (primary and bounce
    // rays) and the city pathtracer: persistent refill (block 128, 8 idle lanes), stack in
    // shared memory, 16 ESVO steps per loop iteration; against the 56-register
    // local-stack kernel at 8 steps: primary 6.47 vs 6.05, bounce 3.65 vs 3.55 Grays/s,
    // city frame 42.5 vs 43.0 ms.
    cbq_launch_config cfg{CBQ_KERNEL_AUTO, 0, 0, 0, CBQ_STACK_SHARED, CBQ_FORM_PERSISTENT, 16, 0};

    // Staging sets of cbq_intersect_host, created as concurrent calls need them.
    std::mutex stages_lock;
    std::vector<std::unique_ptr<cbq::HostStage>> stages;
    // Work counters of cbq_intersect's persistent form, one per stream id (ids are unique
    // for the context's lifetime, so launches sharing a counter are ordered by their stream).
    std::mutex counter_lock;
    std::map<unsigned long long, uint64_t*> stream_counters;
};
