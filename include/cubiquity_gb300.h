/*
 * cubiquity_gb300 — GB300 (sm_103a) sparse-voxel-DAG ray traversal, C ABI.
 *
 * A drop-in for Cubiquity's ray cast (src/library/raytracing.h:48-81): the same
 * flat node store, the same eight SubDAG virtual roots, the same ray -> hit
 * semantics (hit flag, distance, material, position, normal), bit-exact, plus an
 * integer hit voxel.  All entry points return a cbq_status and never throw.
 *
 * Conventions
 *   - "device" pointers are CUDA global-memory pointers on the current device;
 *     "host" pointers are CPU memory (pinned memory is faster but not required).
 *   - Rays are two arrays of float4 (16-byte aligned, 16 bytes per ray):
 *       origin_tmax[i] = (ox, oy, oz, tmax)   direction[i] = (dx, dy, dz, unused)
 *     tmax is read only when CBQ_QUERY_TMAX is set in cbq_query.flags.
 *   - Outputs are per-field arrays; any pointer may be NULL to skip that field.
 *     position / normal / voxel hold three values per ray (x, y, z interleaved).
 *   - Launching calls are stream-ordered and asynchronous on `stream`
 *     (a cudaStream_t; NULL = legacy default stream).
 *   - A cbq_dag's node store is immutable once created; the handle may be used
 *     from several host threads and streams at once.  Its launch configuration
 *     (cbq_dag_set_launch_config, cbq_autotune) is the one mutable part: change
 *     it while no other thread launches on the handle.
 */
#ifndef CUBIQUITY_GB300_H
#define CUBIQUITY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CBQ_ABI_VERSION 1

typedef struct CUstream_st* cbq_stream_t; /* identical to cudaStream_t */

typedef enum cbq_status {
    CBQ_OK = 0,
    CBQ_ERR_INVALID_ARGUMENT = 1,
    CBQ_ERR_BAD_DAG = 2,          /* child index out of range, bad root, bad file */
    CBQ_ERR_OUT_OF_MEMORY = 3,
    CBQ_ERR_CUDA = 4,
    CBQ_ERR_TIMEOUT = 5,
    CBQ_ERR_IO = 6,
    CBQ_ERR_BUSY = 7,
    CBQ_ERR_NOT_FOUND = 8,
    CBQ_ERR_CANCELLED = 9,
    CBQ_ERR_CAPACITY = 10,        /* request larger than the server can ever admit */
    CBQ_ERR_SHUTDOWN = 11
} cbq_status;

/* Per-ray status values written to cbq_hits.status. */
#define CBQ_RAY_OK 0u
#define CBQ_RAY_ITER_LIMIT 1u  /* more than CBQ_MAX_RAY_FETCHES node fetches: reported as a miss */
#define CBQ_RAY_STUCK 2u       /* an advance step that moved nowhere (NaN slab): reported as a miss */
#define CBQ_MAX_RAY_FETCHES (1u << 17)

#define CBQ_MATERIAL_COUNT 256u
#define CBQ_MAX_FOOTPRINT_DISABLED (-1.0f) /* raytracing.h:71 */

/* Same 32-byte layout as the reference's SubDAG (raytracing.h:57-65) and its
 * std430 GLSL twin (pathtracing.frag SSBO 1). */
typedef struct cbq_subdag {
    int32_t lower_bound[3];
    int32_t node_height;
    uint32_t padding0;
    uint32_t node_index;
    uint32_t padding1, padding2;
} cbq_subdag;

typedef struct cbq_rays {
    const float* origin_tmax; /* 4 floats per ray */
    const float* direction;   /* 4 floats per ray */
} cbq_rays;

typedef struct cbq_hits {
    uint8_t* hit;
    float* distance;          /* FP32; the reference widens the same value to double */
    uint32_t* material;
    float* position;          /* 3 per ray */
    float* normal;            /* 3 per ray */
    int32_t* voxel;           /* 3 per ray: floor(position - 0.5*normal + 0.5) */
    uint8_t* status;          /* CBQ_RAY_* */
} cbq_hits;

#define CBQ_QUERY_TMAX 0x1u   /* a hit with distance > tmax is reported as a miss */

typedef struct cbq_query {
    int32_t compute_surface;  /* intersectVolume's computeSurfaceProperties */
    float max_footprint;      /* intersectVolume's maxFootprint (LOD); -1 disables */
    uint32_t flags;           /* CBQ_QUERY_* */
    uint32_t image_width;     /* 0, or: the call's rays are the pixels of a row-major
                                 image this many rays wide (a camera's rays; samples
                                 stacked as further rows).  The flat kernels then
                                 deal them to warps in tiles of 4 x 8 pixels, whose
                                 rays stay together through the DAG longer (same
                                 results; ~9% faster on terrain-4096's camera rays).
                                 Used by a launch whose width is a multiple of 4 and
                                 whose ray count is a multiple of 8 rows and below
                                 2^32, outside the octant-sorted form; ignored
                                 otherwise and by the batch, server and nested
                                 kernels. */
} cbq_query;

typedef struct cbq_dag cbq_dag;

/* Device layouts of the node store.  REFERENCE is the reference's array as
 * given (storage.h:51-116).  COMPACT keeps only occupied children, packed, and
 * carries each internal node's 8-bit occupancy mask in the reference to it, so
 * an empty child is known without a load; traversal decisions and results are
 * identical. */
#define CBQ_DAG_LAYOUT_REFERENCE 0u
#define CBQ_DAG_LAYOUT_COMPACT 1u

typedef struct cbq_dag_info {
    uint64_t node_count;      /* including the 256 material slots */
    uint64_t bytes;           /* node_count * 32 */
    uint32_t root;
    int32_t max_subdag_height;
    cbq_subdag subdags[8];
    const uint32_t* device_nodes;
    uint32_t layout;          /* CBQ_DAG_LAYOUT_* in use */
    uint64_t device_bytes;    /* bytes of the device node store */
} cbq_dag_info;

/* ---------------------------------------------------------------- basics */

const char* cbq_status_string(cbq_status s);
int cbq_abi_version(void);

/* Diagnostics callback, in the spirit of the reference's set_debug_handler /
 * set_warning_handler (base.h:102-107): the library reports DAG uploads, scene
 * builds, autotuner choices and server events.  NULL disables.  The callback
 * may run on library threads (the server's). */
#define CBQ_LOG_DEBUG 0
#define CBQ_LOG_INFO 1
#define CBQ_LOG_WARNING 2
typedef void (*cbq_log_fn)(void* user, int32_t level, const char* message);
void cbq_set_log_handler(cbq_log_fn fn, void* user);

/* Checks that every child index (and the root) is < node_count and that slots
 * 0..255 are material nodes.  Host memory. */
cbq_status cbq_dag_validate(const uint32_t* nodes, uint64_t node_count, uint32_t root);

/* findSubDAGs (raytracing.h:69 / raytracing.cpp:89-97) on a host node array. */
cbq_status cbq_find_subdags(const uint32_t* nodes, uint64_t node_count, uint32_t root,
                            cbq_subdag out[8]);

/* ------------------------------------------------------------ DAG store */

/* Validates, computes the SubDAGs and uploads the node store to the current
 * device as one flat uint32 array (the buffer the reference binds as SSBO 0,
 * gpu_pathtracing_viewer.cpp:43-57).  Replaces Volume + findSubDAGs for the
 * device path.  Synchronous. */
cbq_status cbq_dag_create(const uint32_t* host_nodes, uint64_t node_count, uint32_t root,
                          cbq_dag** out);
/* cbq_dag_create with a device layout (CBQ_DAG_LAYOUT_*; no reference
 * counterpart).  COMPACT falls back to REFERENCE, with a log message, when the
 * DAG needs integer positions (coordinates beyond +-2^21, or 2^29 nodes or
 * more) or the compact store would exceed 128 MB; cbq_dag_get_info reports the
 * layout in use. */
cbq_status cbq_dag_create_ex(const uint32_t* host_nodes, uint64_t node_count, uint32_t root,
                             uint32_t layout, cbq_dag** out);
cbq_status cbq_dag_destroy(cbq_dag* dag);
cbq_status cbq_dag_get_info(const cbq_dag* dag, cbq_dag_info* info);

/* Kernel selection and launch shape (chosen by the autotuner; 0 = default).
 *   CBQ_KERNEL_FLAT    one ray per thread, the ESVO loops flattened into one
 *                      per-lane state machine (lanes reconverge every step);
 *                      child positions as exact floats where the DAG's
 *                      coordinates lie within +-2^21 and it has fewer than
 *                      2^29 nodes, else as wrapping i32 (any DAG); the default
 *   CBQ_KERNEL_NESTED  one ray per thread, the reference's nested loops as
 *                      written (any DAG; kept as a second restatement)
 * For cbq_intersect_persistent, `refill_min` (flat) is the number of idle lanes
 * at which a warp takes new rays and `chunk` (nested) the rays per warp grab. */
typedef enum cbq_kernel {
    CBQ_KERNEL_AUTO = 0,
    CBQ_KERNEL_NESTED = 1,
    CBQ_KERNEL_FLAT = 2
} cbq_kernel;

#define CBQ_STACK_SHARED 0    /* descent stack in shared memory, one column per thread */
#define CBQ_STACK_LOCAL 1     /* descent stack in a per-thread local array (L1) */

#define CBQ_FORM_PLAIN 0      /* cbq_intersect_auto: one thread per ray */
#define CBQ_FORM_PERSISTENT 1 /* persistent grid refilling idle lanes */
#define CBQ_FORM_SORTED 2     /* rays grouped by octant first, then persistent */

typedef struct cbq_launch_config {
    int32_t kernel;           /* cbq_kernel */
    int32_t block;            /* threads per block (multiple of 32, <= 256), 0 = default */
    uint32_t chunk;           /* nested persistent: rays per warp grab, 0 = default */
    uint32_t refill_min;      /* flat persistent: idle lanes that trigger a refill, 0 = default */
    int32_t stack;            /* CBQ_STACK_* (flat kernel; shared by default) */
    int32_t form;             /* CBQ_FORM_*, used by cbq_intersect_auto */
    int32_t steps;            /* flat kernel: ESVO steps per loop iteration (1..32, 16 by
                                 default), 0 = 1 */
    int32_t registers;        /* 0 (the default), or 56: the persistent local-stack
                                 kernel held to 56 registers per thread (more
                                 resident warps); other forms ignore it */
} cbq_launch_config;

cbq_status cbq_dag_set_launch_config(cbq_dag* dag, const cbq_launch_config* cfg);
cbq_status cbq_dag_get_launch_config(const cbq_dag* dag, cbq_launch_config* cfg);

/* Device scratch cbq_intersect_auto needs for n rays (work counter, octant
 * histogram and, for the sorted form, a uint32 permutation): 256 + 4n bytes. */
uint64_t cbq_scratch_bytes(uint64_t n);

/* Traverses with the form and launch shape in the DAG's launch config
 * (CBQ_FORM_*), using caller-owned device scratch of cbq_scratch_bytes(n)
 * bytes.  Results equal cbq_intersect's for every form. */
cbq_status cbq_intersect_auto(const cbq_dag* dag, const cbq_rays* rays, uint64_t n, const cbq_query* query,
                              const cbq_hits* hits, void* scratch, uint64_t scratch_bytes, cbq_stream_t stream);

/* Autotuner: times every form x block {64,128,256} x refill {4,8,16} x stack
 * {shared, local} x steps {2,4,8,16,32}, and the 56-register persistent
 * local-stack kernel, on these rays (synchronous; `repetitions` launches each),
 * stores the fastest in the DAG's launch config and returns it with its time. */
cbq_status cbq_autotune(cbq_dag* dag, const cbq_rays* rays, uint64_t n, const cbq_query* query,
                        const cbq_hits* hits, void* scratch, uint64_t scratch_bytes, int32_t repetitions,
                        cbq_launch_config* best, float* best_ms, cbq_stream_t stream);

/* Sets a persisting-L2 access-policy window over the node store on `stream`
 * (fraction of the device's persisting-L2 limit to reserve; 0 removes the window,
 * releases the set-aside and demotes persisting lines).  The set-aside is a
 * setting of the calling process's context.  Measured on GB300 it does not
 * help: a DAG that fits in L2 already stays there, and the set-aside shrinks
 * the cache left for the streamed rays and hits (terrain-4096: -2% primary,
 * -5% bounce at fraction 1). */
cbq_status cbq_dag_set_l2_persistence(const cbq_dag* dag, cbq_stream_t stream, float fraction);

/* ------------------------------------------------------------ traversal */

/* intersectVolume (raytracing.h:72-76 / raytracing.cpp:397-478) for n rays:
 * one launch, device rays in, device hits out, stream-ordered.  It runs in the
 * DAG's launch form: persistent by default, with a work counter the DAG keeps
 * per stream (allocated on the first call on a stream, so launches sharing it
 * are ordered by that stream), or one thread per ray for CBQ_FORM_PLAIN and
 * while the stream is being captured into a graph. */
cbq_status cbq_intersect(const cbq_dag* dag, const cbq_rays* rays, uint64_t n,
                         const cbq_query* query, const cbq_hits* hits, cbq_stream_t stream);

/* As cbq_intersect, with HOST rays and HOST hits: copies in, traverses, copies
 * out, and waits for completion.  Calls of 2^19 rays or more are split into up
 * to 8 chunks whose copies overlap the traversal of their neighbours (own
 * streams; page-locked host buffers copy fastest); each chunk takes every k-th
 * of about 4k blocks of consecutive rays, so chunks carry even work.  Allocates
 * and caches device staging buffers and streams per dag.  Calls on one dag from
 * several host threads run concurrently, each with its own staging set (up to
 * four sets per dag, created as needed; further calls wait for one), so one
 * call's copies and traversal overlap another's.  On an error every copy and
 * launch it queued has ended before it returns. */
cbq_status cbq_intersect_host(const cbq_dag* dag, const float* host_origin_tmax,
                              const float* host_direction, uint64_t n, const cbq_query* query,
                              const cbq_hits* host_hits);

/* No counterpart in the reference.  As cbq_intersect_host, but without any
 * device allocation, for callers that must not call cudaMalloc: a render or
 * physics thread with a frame deadline (cudaMalloc can synchronise the device
 * and stall every stream), or a host application whose own allocator owns all
 * device memory.  Rays and hits are staged, and the persistent kernel's work
 * counter kept, in one fixed array compiled into the library
 * (CBQ_NOALLOC_MAX_RAYS * 78 bytes + 256, about 5 MB per device).
 *   - The array takes its device memory when cbq_dag_create first runs on a
 *     device: it loads the array's module there and looks up its address
 *     (cudaGetSymbolAddress).  It is held until the process exits.  A call of
 *     this entry point needs a DAG, so its array is always in place already;
 *     the call itself allocates nothing, not even on its first use.
 *   - n > CBQ_NOALLOC_MAX_RAYS returns CBQ_ERR_CAPACITY; nothing is launched.
 *   - The current device must be the DAG's device.
 *   - Copies and the launch go on the calling thread's per-thread stream
 *     (cudaStreamPerThread), so the call neither waits for nor holds up other
 *     streams.  It always runs the persistent form (same results as every
 *     other form, whatever the DAG's launch configuration says).
 *   - Every call on a device shares the array and leaves its contents behind;
 *     each call rewrites what it reads (rays, hits) and zeroes the counter.
 *     Calls that overlap on the GPU (for instance from several host threads)
 *     race on the array: callers must serialise them.
 *   - Synchronous, like cbq_intersect_host: whether it succeeds or fails,
 *     every copy and launch it queued has ended when it returns. */
#define CBQ_NOALLOC_MAX_RAYS 65536u
cbq_status cbq_intersect_host_noalloc(const cbq_dag* dag, const float* host_origin_tmax,
                                      const float* host_direction, uint64_t n, const cbq_query* query,
                                      const cbq_hits* host_hits);

/* Persistent form: a grid sized to the device's SMs whose warps pull rays from
 * an atomic work counter.  `work_counter` is caller-owned device scratch (one
 * uint64, zeroed by this call on `stream`).  With the flat kernel a warp takes
 * new rays whenever `chunk` (<= 32) of its lanes are idle; with the nested one
 * it takes `chunk` rays at a time.  chunk = 0 selects the tuned default. */
cbq_status cbq_intersect_persistent(const cbq_dag* dag, const cbq_rays* rays, uint64_t n,
                                    const cbq_query* query, const cbq_hits* hits,
                                    uint64_t* work_counter, uint32_t chunk, cbq_stream_t stream);

/* ------------------------------------------------------- batched form */

/* One volume and its ray batch (device buffers). */
typedef struct cbq_job {
    const cbq_dag* dag;
    cbq_rays rays;
    uint64_t ray_count;
    cbq_hits hits;
} cbq_job;

/* A prepared batch: many volumes of uneven size and ray batches of uneven
 * length traversed by ONE persistent launch (a job table in device memory;
 * warps refill idle lanes from a single work counter), captured in a CUDA
 * graph on first launch and replayed after.  Results equal cbq_intersect on
 * each job alone.  The job arrays must stay valid while the batch exists. */
typedef struct cbq_batch cbq_batch;

cbq_status cbq_batch_create(const cbq_job* jobs, int32_t job_count, const cbq_query* query, cbq_batch** out);
/* block: threads per block (32..256, 0 = default); refill_min: idle lanes that
 * trigger a warp's refill (1..32, 0 = default).  Re-captures on next launch. */
cbq_status cbq_batch_set_config(cbq_batch* b, int32_t block, uint32_t refill_min);
cbq_status cbq_batch_get_config(const cbq_batch* b, int32_t* block, uint32_t* refill_min, uint64_t* total_rays);

/* The batch's full launch configuration.  Every choice gives the same results. */
typedef struct cbq_batch_config {
    int32_t block;            /* threads per block: 32..256, a multiple of 32 */
    uint32_t refill_min;      /* idle lanes that trigger a warp's refill: 1..32 */
    int32_t steps;            /* ESVO steps per loop iteration: 1..32 */
    int32_t registers;        /* 0, or 56: the local-stack kernel held to 56 registers */
    int32_t stack;            /* CBQ_STACK_LOCAL or CBQ_STACK_SHARED (descent stack placement) */
    int32_t form;             /* CBQ_FORM_PERSISTENT: rays in the order given; CBQ_FORM_SORTED: each
                                 job's rays grouped by octant first (two small kernels per launch;
                                 4 bytes of device memory per ray, allocated when first chosen) */
} cbq_batch_config;
cbq_status cbq_batch_set_launch_config(cbq_batch* b, const cbq_batch_config* cfg);
cbq_status cbq_batch_get_launch_config(const cbq_batch* b, cbq_batch_config* cfg);

/* Autotuner of the batched form: times block {64,128,256} x refill
 * {4,8,12,16} x steps {4,8,16} x {local stack, local stack at 56 registers,
 * shared-memory stack} x {rays as given, octant-sorted} on this batch
 * (synchronous; `repetitions` launches each) and keeps the fastest. */
cbq_status cbq_batch_autotune(cbq_batch* b, cbq_stream_t stream, int32_t repetitions);
/* Replays the captured graph on `stream` (captures it first if needed). */
cbq_status cbq_batch_launch(cbq_batch* b, cbq_stream_t stream);
/* Pins one DAG's node store in L2 for the batch's graph launches: a persisting
 * access-policy window over `dag`'s store, set on every kernel node of the
 * graph (re-captured on the next cbq_batch_launch), reserving `fraction` of the
 * device's persisting-L2 limit (a setting of the calling process's context);
 * 0 removes the window, releases the set-aside and demotes persisting lines.
 * Direct launches (cbq_batch_launch_direct) carry no window.  Measured on a
 * 64-volume batch it does not help: the stores' L2 misses are first touches. */
cbq_status cbq_batch_set_l2_persistence(cbq_batch* b, const cbq_dag* dag, float fraction);
/* The same work launched directly, without the graph. */
cbq_status cbq_batch_launch_direct(cbq_batch* b, cbq_stream_t stream);
cbq_status cbq_batch_destroy(cbq_batch* b);
/* One-shot: create, launch on `stream`, wait, destroy. */
cbq_status cbq_intersect_batch(const cbq_job* jobs, int32_t job_count, const cbq_query* query,
                               cbq_stream_t stream);

/* ------------------------------------------------------- serving */

/* A request: host rays in, host hits out, against a resident DAG.  The host
 * buffers must stay valid until the request has completed (cbq_server_wait). */
typedef struct cbq_request {
    const cbq_dag* dag;
    const float* host_origin_tmax;  /* 4 floats per ray */
    const float* host_direction;    /* 4 floats per ray */
    uint64_t ray_count;
    cbq_query query;                /* per request (e.g. CBQ_QUERY_TMAX for collision rays) */
    cbq_hits host_hits;             /* host arrays; NULL fields are not copied back */
} cbq_request;

typedef struct cbq_server_config {
    uint64_t device_memory_budget;  /* bytes for in-flight ray and hit buffers (0 = 1 GiB);
                                       a request needs about 78 bytes per ray */
    int32_t max_inflight_launches;  /* launches on the device at once (0 = 4) */
    int32_t max_batch_requests;     /* requests per launch (0 = 256) */
    uint64_t max_batch_rays;        /* rays per launch (0 = 4 Mi) */
    int32_t block;                  /* threads per block (0 = 128) */
    uint32_t refill_min;            /* idle lanes that trigger a refill (0 = 8) */
    uint32_t flags;                 /* CBQ_SERVER_* */
} cbq_server_config;

/* By default every request is staged: rays copied into the device memory
 * budget, hits copied back.  With CBQ_SERVER_IN_PLACE, a request whose ray and
 * hit buffers are all device-accessible host memory (page-locked by
 * cudaHostAlloc / cudaHostRegister, or managed) and whose rays are 16-byte
 * aligned is served in place instead: the kernel reads its rays and writes its
 * hits in host memory, it takes no room in the budget and no copy is issued.
 * Hit stores across the host link are narrow, so in-place traversal runs at
 * about half the staged rate; it suits small requests and clients that cannot
 * spare device memory. */
#define CBQ_SERVER_IN_PLACE 0x1u

typedef struct cbq_server_stats {
    uint64_t submitted, completed, rays_completed, launches;
    uint64_t queued, inflight_launches;
    double mean_requests_per_launch;
    double latency_p50_us, latency_p99_us, latency_max_us, latency_mean_us; /* submit -> hits on host */
    double busy_seconds;            /* first submit -> last completion */
    uint64_t direct_requests;       /* completed requests served in place (CBQ_SERVER_IN_PLACE) */
} cbq_server_stats;

/* Continuous batching: requests are admitted in arrival order while the memory
 * budget and a launch slot allow, grouped into one persistent multi-volume
 * launch per group, and launched while earlier groups still run; launches are
 * completed in the order they finish.  Each result equals cbq_intersect_host
 * on that request alone.  A server runs two threads: a scheduler, asleep
 * unless requests queue, and a completion thread that polls the events of the
 * launches in flight (yielding between rounds), so it keeps one host core busy
 * while the GPU has work from the server and sleeps otherwise. */
typedef struct cbq_server cbq_server;

cbq_status cbq_server_create(const cbq_server_config* cfg, cbq_server** out);
/* Queues a request; returns at once with a ticket.  CBQ_ERR_CAPACITY if the
 * request could never fit in the memory budget; CBQ_ERR_SHUTDOWN while the
 * server is being destroyed. */
cbq_status cbq_server_submit(cbq_server* s, const cbq_request* r, uint64_t* ticket);
/* Waits for a ticket (timeout_us < 0: no limit) and returns the request's
 * status; CBQ_ERR_TIMEOUT if it is still running, CBQ_ERR_NOT_FOUND for an
 * unknown or already-waited ticket. */
cbq_status cbq_server_wait(cbq_server* s, uint64_t ticket, int64_t timeout_us);
cbq_status cbq_server_poll(cbq_server* s, uint64_t ticket, int32_t* done);
/* Withdraws a request that has not been launched yet: its wait then returns
 * CBQ_ERR_CANCELLED and its buffers are never touched again.  CBQ_ERR_BUSY if it
 * is already on the device (it will complete), CBQ_ERR_NOT_FOUND if unknown. */
cbq_status cbq_server_cancel(cbq_server* s, uint64_t ticket);
cbq_status cbq_server_get_stats(cbq_server* s, cbq_server_stats* out);
cbq_status cbq_server_reset_stats(cbq_server* s);
/* Finishes every queued and running request, then stops. */
cbq_status cbq_server_destroy(cbq_server* s);

/* Open-loop load driver (no reference counterpart): replays a request trace
 * against the server from native threads, so that a serving measurement is
 * not shaped by the client.  The calling thread submits requests[k] at
 * arrival_s[k] seconds (non-decreasing) after the call starts, sleeping while
 * an arrival is far off and spinning for the last 200 us; a second thread
 * waits for the tickets in order.  Requests k and k + max_outstanding may
 * share host buffers: request k is submitted only once request
 * k - max_outstanding has completed (counted in `backpressure`).  Latency per
 * request is the server's own (cbq_server_get_stats); lateness_us[k]
 * (optional, count entries) receives how late request k was submitted against
 * its arrival time.  Returns when every submitted request has completed, or
 * the first submission error. */
typedef struct cbq_replay_result {
    double wall_seconds;            /* call start -> last completion */
    uint64_t submitted, failed, backpressure;
    double lateness_p50_us, lateness_p99_us, lateness_max_us;
    double submit_p99_us, submit_max_us;   /* time spent inside cbq_server_submit */
} cbq_replay_result;
cbq_status cbq_server_replay(cbq_server* s, const cbq_request* requests, const double* arrival_s, uint64_t count,
                             uint32_t max_outstanding, double* lateness_us, cbq_replay_result* result);

/* ------------------------------------------------------- pathtracer */

/* Wavefront restatement of the reference's CPU pathtracer
 * (pathtracing_demo.cpp:81-190) on top of the traversal: per sample pass,
 * camera rays, then for each depth an extension traversal (surface properties
 * on), shading (material colour, emission, a sun and a sky shadow ray, a
 * cosine bounce ray) and a shadow traversal (surface properties off), all with
 * the LOD footprint `max_footprint`.  Counter-based random numbers (seed,
 * pixel, sample, depth): a frame is reproducible. */
typedef struct cbq_pt_material {
    float albedo[3];
    float emission[3];
} cbq_pt_material;

typedef struct cbq_pt_config {
    int32_t width, height, samples_per_pixel, bounces;
    double eye[3], target[3];
    double tan_half_fov;
    float max_footprint;            /* the demo uses 0.0035 (pathtracing_demo.h:84) */
    float sun_direction[3], sun_colour[3], sky_colour[3], background[3];
    uint64_t seed;
    const cbq_pt_material* materials; /* 256 entries, host memory */
} cbq_pt_config;

typedef struct cbq_pt_stats {
    uint64_t extension_rays, shadow_rays;
    double milliseconds;
    uint64_t kernel_launches;       /* kernels of this library launched for the frame */
} cbq_pt_stats;

/* Called after every traversal wave with device pointers to its rays and hits
 * (kind 0: extension rays, 1: shadow rays); the stream has been synchronised.
 * A wave holds the paths of one pass: `sample` is the pass's first sample (a
 * pass traces as many samples per pixel together as fit in 2^24 paths). */
typedef void (*cbq_pt_wave_fn)(void* user, int32_t kind, int32_t depth, int32_t sample, const float* origin_tmax,
                               const float* direction, uint64_t n, const cbq_hits* hits, const cbq_query* query);

/* Convenience for wave callbacks in languages without a CUDA binding: a
 * synchronous device-to-host copy. */
cbq_status cbq_copy_to_host(void* host_dst, const void* device_src, uint64_t bytes);

/* Renders into device_image (width * height * 3 floats, the mean over samples).
 * Synchronous; allocates its wave buffers for the call. */
cbq_status cbq_pathtrace(const cbq_dag* dag, const cbq_pt_config* cfg, float* device_image,
                         cbq_pt_wave_fn on_wave, void* user, cbq_pt_stats* stats, cbq_stream_t stream);

/* Statistics form of cbq_intersect: writes only the number of node fetches
 * (dependent child loads) each ray performed to the device array `fetches`. */
cbq_status cbq_count_fetches(const cbq_dag* dag, const cbq_rays* rays, uint64_t n,
                             const cbq_query* query, uint32_t* fetches, cbq_stream_t stream);

/* Diagnostic (no reference counterpart): on the current device, measures the
 * streaming read bandwidth of an L2-resident buffer of about working_set_bytes
 * (GB/s) and the rate of independent random 32-byte-sector reads within it
 * (Gsectors/s), each the fastest of three timed launches after a warm-up pass.
 * These are the roofline denominators of the traversal, whose node fetches are
 * L2 sectors.  Synchronous. */
cbq_status cbq_measure_l2(uint64_t working_set_bytes, int iterations, double* stream_gbs,
                          double* random_gsectors_per_s);

/* ---------------------------------------------------- workload generators */

typedef enum cbq_scene_kind {
    CBQ_SCENE_SPHERES = 0, /* param = sphere count */
    CBQ_SCENE_TERRAIN = 1,
    CBQ_SCENE_CITY = 2
} cbq_scene_kind;

/* Builds the canonical DAG of a seeded scene of edge 2^edge_log2 at the origin
 * (the same DAG Volume::setVoxel + bake would reach).  *nodes_out is malloc'd;
 * release with cbq_free.  threads <= 0 uses all cores. */
cbq_status cbq_build_scene(cbq_scene_kind kind, int edge_log2, uint64_t seed, int param, int threads,
                           uint32_t** nodes_out, uint64_t* node_count_out, uint32_t* root_out);

/* Evaluates the scene's voxels over the box [x0, x0+sx) x [y0, y0+sy) x [z0, z0+sz)
 * into out (x fastest). */
cbq_status cbq_scene_voxels(cbq_scene_kind kind, int edge_log2, uint64_t seed, int param,
                            int32_t x0, int32_t y0, int32_t z0, int32_t sx, int32_t sy, int32_t sz,
                            uint8_t* out);

void cbq_free(void* p);

/* The compact node store that CBQ_DAG_LAYOUT_COMPACT uploads (host only, for
 * inspection and tests): *store (release with cbq_free) holds *words uint32;
 * subdag_refs[k] is SubDAG k's root reference in it. */
cbq_status cbq_compact_store(const uint32_t* nodes, uint64_t node_count, uint32_t root, uint32_t** store,
                             uint64_t* words, uint32_t subdag_refs[8]);

/* Volume::voxel (storage.cpp:481-499) on a host node array. */
cbq_status cbq_dag_voxel(const uint32_t* nodes, uint64_t node_count, uint32_t root, int32_t x,
                         int32_t y, int32_t z, uint8_t* material);

/* The reference .dag format (storage.cpp:192-206, 505-542):
 * u32 root | u32 internal_count | internal_count * 32 bytes (material slots omitted). */
cbq_status cbq_dag_save(const char* path, const uint32_t* nodes, uint64_t node_count, uint32_t root);
cbq_status cbq_dag_load(const char* path, uint32_t** nodes_out, uint64_t* node_count_out,
                        uint32_t* root_out);

/* Renumbers the reachable internal nodes in breadth-first order from the root
 * (material slots keep 0..255); the graph is unchanged.  out_nodes must hold
 * node_count * 8 words; *out_count receives the reachable count. */
cbq_status cbq_dag_reorder_bfs(const uint32_t* nodes, uint64_t node_count, uint32_t root,
                               uint32_t* out_nodes, uint64_t* out_count, uint32_t* out_root);

/* Pinhole camera rays in scanline order, computed in double precision with
 * + - * / sqrt only (identical on every platform) and rounded to float.
 * tan_half_fov = tan(vertical fov / 2); z is up. */
cbq_status cbq_gen_pinhole_rays(const double eye[3], const double target[3], double tan_half_fov,
                                int32_t width, int32_t height, float* origin_tmax, float* direction);

/* Rays with origins uniform in the box [lo, hi] and directions uniform on the
 * unit sphere, from a counter-based hash of (seed, i); same floats everywhere. */
cbq_status cbq_gen_sphere_rays(const double lo[3], const double hi[3], uint64_t n, uint64_t seed,
                               float* origin_tmax, float* direction);

/* Cosine-weighted bounce rays: ray i starts at hit (i mod hit_count) at
 * position + 0.01 * normal (pathtracing_demo.cpp:166) with direction
 * normalize(normal + u), u uniform on the unit sphere from a counter-based hash
 * of (seed, i). */
cbq_status cbq_gen_bounce_rays(const float* hit_position, const float* hit_normal, uint64_t hit_count,
                               uint64_t n, uint64_t seed, float* origin_tmax, float* direction);

#ifdef __cplusplus
}
#endif

#endif /* CUBIQUITY_GB300_H */
