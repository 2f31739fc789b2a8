/*
 * meshopt_gb300.h - C ABI of the GB300 (sm_103a) edge-collapse simplifier.
 *
 * The first group of entry points keeps the exact signatures of meshoptimizer.h, so a
 * program linked against libmeshopt_gb300.so instead of libmeshoptimizer gets the same
 * results (bit-identical index buffers) computed on the GPU. Pointers are HOST pointers,
 * caller-owned, with the reference's rules for strides, aliasing and result_error == NULL.
 *
 * Errors: the reference has no error return (invalid input is an assert). Here a call that
 * cannot run (unsupported option, CUDA error, invalid index) writes the input indices
 * unchanged to destination, returns index_count, prints one line to stderr and records a
 * nonzero status, queryable per thread with meshoptgpu_getLastStatus(). It never aborts
 * the process and never falls back to a CPU implementation.
 */
#ifndef MESHOPT_GB300_H
#define MESHOPT_GB300_H

#include <stddef.h>

#ifndef MESHOPTGPU_API
#define MESHOPTGPU_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C"
{
#endif

/* The option and vertex_lock enumerators below are meshoptimizer.h's own (same names and values).
 * A translation unit that mixes CPU and GPU calls includes meshoptimizer.h first and this header
 * after it; this header then leaves the enumerators to meshoptimizer.h (its version macro
 * MESHOPTIMIZER_VERSION marks it as included) and only adds the GPU entry points. */
#ifndef MESHOPTIMIZER_VERSION

/* Option bits: same values as meshoptimizer.h:466-482. */
enum
{
	meshopt_SimplifyLockBorder = 1 << 0,
	meshopt_SimplifySparse = 1 << 1,
	meshopt_SimplifyErrorAbsolute = 1 << 2,
	meshopt_SimplifyPrune = 1 << 3,
	meshopt_SimplifyRegularize = 1 << 4,
	meshopt_SimplifyPermissive = 1 << 5,
	meshopt_SimplifyRegularizeLight = 1 << 6,
};

/* vertex_lock flags: same values as meshoptimizer.h:488-495. */
enum
{
	meshopt_SimplifyVertex_Lock = 1 << 0,
	meshopt_SimplifyVertex_Protect = 1 << 1,
	meshopt_SimplifyVertex_Priority = 1 << 2,
};

#endif /* MESHOPTIMIZER_VERSION */

/* Replaces meshopt_simplify, meshoptimizer.h:513 (implementation src/simplifier.cpp:2628). */
MESHOPTGPU_API size_t meshopt_simplify(unsigned int* destination, const unsigned int* indices, size_t index_count, const float* vertex_positions,
    size_t vertex_count, size_t vertex_positions_stride, size_t target_index_count, float target_error, unsigned int options, float* result_error);

/* Replaces meshopt_simplifyWithAttributes, meshoptimizer.h:537 (src/simplifier.cpp:2635). */
MESHOPTGPU_API size_t meshopt_simplifyWithAttributes(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride, const float* vertex_attributes,
    size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count, const unsigned char* vertex_lock,
    size_t target_index_count, float target_error, unsigned int options, float* result_error);

/* Replaces meshopt_simplifyScale, meshoptimizer.h:611 (src/simplifier.cpp:2938). */
MESHOPTGPU_API float meshopt_simplifyScale(const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride);

/* ---- additions with no counterpart in meshoptimizer.h ---- */

enum
{
	meshoptgpu_StatusOk = 0,
	meshoptgpu_StatusUnsupported = 1, /* an option the GPU path does not implement */
	meshoptgpu_StatusInvalidArgument = 2,
	meshoptgpu_StatusCudaError = 3,
	meshoptgpu_StatusOutOfMemory = 4,
	meshoptgpu_StatusInternal = 5, /* a bound the GPU path keeps was exceeded (a defect: please report) */
};

/* Status and message of the calling thread's last simplifier call. */
MESHOPTGPU_API int meshoptgpu_getLastStatus(void);
MESHOPTGPU_API const char* meshoptgpu_getLastMessage(void);

/* Per-pass counters of the calling thread's last call: the quantities the reference
 * prints under TRACE (src/simplifier.cpp:1625-1633). stop: 0 out of collapses,
 * 1 error limit, 2 count limit, 3 error goal. rounds: decision rounds of the pass;
 * active: candidates processed by the decision rounds, summed over its rounds; windows:
 * sorted-order windows decided before the stop cut was found. */
typedef struct meshoptgpu_PassStats
{
	unsigned int triangles, candidates, evaluated, done, skipped, invalid, stop, rounds, active, windows;
} meshoptgpu_PassStats;

/* Copies up to max_passes entries; returns the number of passes of the last call. */
MESHOPTGPU_API int meshoptgpu_getLastPassStats(meshoptgpu_PassStats* out, int max_passes);

/* Device time (ms) of the phases of the calling thread's last call. The first 8 values are
 * CUDA-event times, filled when timing was enabled with meshoptgpu_setTiming(1): setup,
 * adjacency, pick, rank, sort, perform, apply, total. The next 8 split the cooperative pass
 * kernel by phase, summed over passes (SM clock of one block): init, window marks, decision
 * rounds, stop rules, apply, loop remap + counts, count scan, compaction emit.
 * Returns the number of values written (16). */
MESHOPTGPU_API void meshoptgpu_setTiming(int enabled);

/* Decision rounds of the calling thread's last call on the single-mesh path, in order (at most
 * 512): candidates processed by the round and its duration in microseconds (SM clock of one
 * block). Returns the number of rounds recorded. */
MESHOPTGPU_API int meshoptgpu_getLastRoundTrace(unsigned int* active, float* micros, int max_rounds);
MESHOPTGPU_API int meshoptgpu_getLastPhaseTimes(float* out16);

/* With timing enabled, the CUDA-event time (ms) of each pass of the calling thread's last
 * single-mesh call, five values per pass: adjacency, pick, rank, sort, perform. Copies up to
 * max_passes rows; returns the number of passes recorded. */
MESHOPTGPU_API int meshoptgpu_getLastPassPhaseTimes(float* out, int max_passes);

/* meshoptimizer.h:560 (src/simplifier.cpp:2642): simplifies indices in place and writes the
 * optimal positions (and attributes) of the vertices the result uses back into the caller's
 * buffers. Same results as the reference, for every option bit (Prune and the internal debug
 * bit included). */
MESHOPTGPU_API size_t meshopt_simplifyWithUpdate(unsigned int* indices, size_t index_count, float* vertex_positions, size_t vertex_count,
    size_t vertex_positions_stride, float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options, float* result_error);

/* Device-resident form of meshopt_simplifyWithUpdate: indices, positions, attributes and
 * vertex_lock are DEVICE pointers (updated in place), attribute_weights is host; work on
 * `stream`, returning once the result count is known. */
MESHOPTGPU_API size_t meshoptgpu_simplifyWithUpdateDevice(unsigned int* indices, size_t index_count, float* vertex_positions, size_t vertex_count,
    size_t vertex_positions_stride, float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options, float* result_error, void* stream);

/* Device-resident form of meshopt_simplifyWithAttributes: every array pointer is a DEVICE
 * pointer on the current device, except attribute_weights (host, at most 32 floats).
 * destination must hold index_count indices and may alias indices. Work is queued on
 * `stream` (a cudaStream_t, or NULL for the legacy default stream) and the call returns
 * once the result count is known. */
MESHOPTGPU_API size_t meshoptgpu_simplifyDevice(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride, const float* vertex_attributes,
    size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count, const unsigned char* vertex_lock,
    size_t target_index_count, float target_error, unsigned int options, float* result_error, void* stream);

/* ---- batched simplification: many meshes in one persistent launch ---- */

/* One mesh of a batch: meshopt_simplifyWithAttributes' arguments plus its output buffer,
 * which must hold index_count indices. The fields after `destination` are optional (zero /
 * NULL: positions only, no vertex_lock), so a zero-initialised struct with the first nine
 * fields set is a meshopt_simplify call. With meshopt_SimplifySparse, any number of meshes
 * may share one vertex buffer (and attribute and lock arrays) and index subsets of it, as a
 * cluster-LOD builder's groups do; each is simplified as a separate sparse call would. */
typedef struct meshoptgpu_BatchMesh
{
	const unsigned int* indices;
	size_t index_count;
	const float* vertex_positions;
	size_t vertex_count;
	size_t vertex_positions_stride;
	size_t target_index_count;
	float target_error;
	unsigned int options; /* every meshopt_Simplify* option except Prune and InternalDebug
	                         (the server accepts those too and runs them on the single-mesh path) */
	unsigned int* destination;
	const float* vertex_attributes;
	size_t vertex_attributes_stride;
	const float* attribute_weights; /* HOST memory, attribute_count floats (read during the call) */
	size_t attribute_count;
	const unsigned char* vertex_lock;
} meshoptgpu_BatchMesh;

/* Simplifies every mesh of the batch in one launch of a persistent kernel: each CTA takes
 * meshes from a device work queue and runs the whole simplifier for one mesh at a time, in
 * shared memory when the mesh fits. Results are the same as mesh_count separate
 * meshopt_simplify calls. All pointers inside meshes[] are DEVICE pointers; the meshes[]
 * array itself and the result arrays are host memory. Returns a meshoptgpu_Status* value. */
MESHOPTGPU_API int meshoptgpu_simplifyBatch(const meshoptgpu_BatchMesh* meshes, size_t mesh_count, size_t* result_index_counts, float* result_errors,
    void* stream);

/* The same with HOST pointers inside meshes[]: inputs are packed into one device buffer and
 * copied once, results copied back once. */
MESHOPTGPU_API int meshoptgpu_simplifyBatchHost(const meshoptgpu_BatchMesh* meshes, size_t mesh_count, size_t* result_index_counts, float* result_errors);

/* One level of a cluster-LOD build on device data: the boundary locks between groups
 * (lockBoundary, demo/clusterlod.h:372-418), then every group simplified in one batch
 * launch as clusterlod's simplify() does (demo/clusterlod.h:455-479). No counterpart in the
 * library itself: it replaces the demo's per-level loop body (demo/clusterlod.h:642-690)
 * up to re-clusterization.
 *   indices            group g's merged cluster indices are indices[group_offsets[g] ..
 *                      group_offsets[g+1]) (device; group_offsets is host, group_count + 1)
 *   destination        group g's result at the same offsets (device; may alias indices)
 *   position_remap     meshopt_generatePositionRemap of the vertex buffer (device), e.g. from
 *                      meshoptgpu_generatePositionRemapDevice
 *   locks              vertex_count bytes (device), kept by the caller across levels: on entry
 *                      its Protect bits (seams to keep in permissive mode) are kept; on return it
 *                      holds this level's locks (Lock where a position is used by two or more
 *                      groups, | Protect, | vertex_lock), as clusterlod's locks array does
 *   vertex_lock        optional user locks (device), ORed in
 *   attribute_weights  host; target_index_counts host, one per group
 * options are ORed with meshopt_SimplifySparse (groups address a shared vertex buffer); Prune is
 * not supported. Results per group go to result_index_counts / result_errors (host). Returns a
 * meshoptgpu_Status* value. */
MESHOPTGPU_API int meshoptgpu_simplifyGroups(unsigned int* destination, const unsigned int* indices, const size_t* group_offsets, size_t group_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride, const float* vertex_attributes, size_t vertex_attributes_stride,
    const float* attribute_weights, size_t attribute_count, const unsigned int* position_remap, unsigned char* locks, const unsigned char* vertex_lock,
    const size_t* target_index_counts, float target_error, unsigned int options, size_t* result_index_counts, float* result_errors, void* stream);

/* Re-clusterization of a cluster-LOD level, on device data: meshopt_buildMeshletsFlex
 * (src/clusterizer.cpp:1035; the clusterize step of demo/clusterlod.h:266-296) for every group,
 * one warp per group, each group's result equal to a separate call's on its indices.
 *   indices            group g is indices[group_offsets[g] .. group_offsets[g+1]) (device;
 *                      group_offsets host, group_count + 1 entries); each count a multiple of 3
 *   meshlets           {vertex_offset, triangle_offset, vertex_count, triangle_count} rows
 *                      (meshopt_Meshlet, device); group g's start at row meshlet_offsets[g] (host,
 *                      group_count + 1) and have room for at least
 *                      meshopt_buildMeshletsBound(index_count, max_vertices, min_triangles) rows;
 *                      offsets inside the rows are relative to the group's own arrays
 *   meshlet_vertices   group g's at group_offsets[g] (device; index_count entries each)
 *   meshlet_triangles  group g's at group_offsets[g] (device; index_count bytes each)
 *   meshlet_counts     meshlets per group (host, out)
 *   optimize_level     0..9: meshopt_optimizeMeshletLevel (src/meshletutils.cpp:366) on every meshlet
 *                      afterwards, as clusterize does with its optimize_clusters_level; -1: none
 * The other arguments are meshopt_buildMeshletsFlex's. Returns a meshoptgpu_Status* value. */
MESHOPTGPU_API int meshoptgpu_buildMeshletsFlexGroups(unsigned int* meshlets, unsigned int* meshlet_vertices, unsigned char* meshlet_triangles,
    const size_t* meshlet_offsets, size_t* meshlet_counts, const unsigned int* indices, const size_t* group_offsets, size_t group_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride, size_t max_vertices, size_t min_triangles, size_t max_triangles,
    float cone_weight, float split_factor, int optimize_level, void* stream);

/* Batch launch shape: threads per CTA (128, 256 or 512; 0 = autotune, the default) and the
 * shared-memory budget per CTA in bytes (0 = autotune, the default). The autotuner times every
 * open pair of thread count and budget (64, 104 and 160 KiB) on the first batch of a size class
 * and keeps the fastest for that class. */
MESHOPTGPU_API void meshoptgpu_setBatchConfig(int threads, unsigned int smem_bytes);

/* Drop-in calls (meshopt_simplify, meshopt_simplifyWithAttributes, meshoptgpu_simplifyDevice)
 * on meshes with at most max_index_count indices run on the batch kernel as a batch of one,
 * where one CTA does the whole simplification: for small meshes that is faster than the
 * multi-CTA pass loop, whose cost per call is fixed by its launches. Results are identical
 * either way. Such calls record no pass statistics, phase times or round trace
 * (meshoptgpu_setTiming(1) keeps every call on the single-mesh path). Per calling thread.
 * The default, (size_t)-1, leaves the route to the autotuner: up to 3000 indices the batch
 * kernel, above 98304 the single-mesh path, and in between whichever the first repeatable call
 * of the size class timed faster on its own mesh. 0 sends every call to the single-mesh path.
 *
 * The single-mesh path's launch shape (pass-kernel blocks per SM, the pass sort's tile) is
 * autotuned the same way, per size class of the mesh: the first repeatable call (destination
 * not aliasing indices, no update mode, Prune or debug bit) times the candidates on its own
 * mesh. MESHOPTGPU_AUTOTUNE=0 in the environment turns both tuners off (fixed defaults). */
MESHOPTGPU_API void meshoptgpu_setDropinBatchLimit(size_t max_index_count);

/* The autotuner's choices for meshes of index_count indices (with attributes or not), on the
 * current device: out4[0] pass-kernel blocks per SM, out4[1] pass sort candidates per thread
 * (0: chosen by count), out4[2] drop-in route (1 batch kernel, 0 single-mesh path, -1 not
 * tuned), out4[3] the batch kernel's shared-memory budget (KiB) for the largest size class
 * tuned so far (0: none). Returns 1 if the single-mesh shape is tuned for that size class. */
MESHOPTGPU_API int meshoptgpu_getTuning(size_t index_count, size_t attribute_count, int* out4);

/* The single-mesh path runs its pass loop (src/simplifier.cpp:2493-2541) on the device: one
 * pass is recorded into a CUDA graph as the body of a WHILE conditional node and replayed
 * until the loop ends, with no host round trip between passes. enabled = 0 switches the
 * calling thread to the host-driven loop (one host read per pass), which per-launch kernel
 * timing (meshoptgpu_setKernelProfile) needs. Pruning, the debug bit and
 * meshoptgpu_setTiming(1) always use the host loop. Results are identical. Returns a
 * meshoptgpu_Status* value. */
MESHOPTGPU_API int meshoptgpu_setDeviceLoop(int enabled);
MESHOPTGPU_API int meshoptgpu_getBatchThreads(void);

/* Failure-path check of the cooperative kernels' grid barriers (no reference counterpart):
 * launches `blocks` blocks (2 .. the resident limit) where one block never arrives at the
 * barrier (once != 0: the single-use barrier of the one-launch scans), so the others' bounded
 * waits run out after wait_limit polls (1 .. 2^20, about 32 ns or more each) and record the
 * error flag the pass kernel's host reads as "grid barrier wait limit reached". *timed_out
 * receives that flag (1 expected). Nothing faults or hangs; the context stays usable.
 * Returns a meshoptgpu_Status* value. */
MESHOPTGPU_API int meshoptgpu_probeBarrierWait(int once, unsigned int blocks, unsigned int wait_limit, unsigned int* timed_out);

/* ---- serving: continuous batching of simplify requests ---- */

typedef struct meshoptgpu_Server meshoptgpu_Server;

typedef struct meshoptgpu_ServerConfig
{
	size_t memory_budget;     /* device bytes the server may hold for admitted requests (0: 40 GB) */
	int batch_workers;        /* concurrent batch launches, one stream each (0: 8) */
	int large_workers;        /* concurrent single-mesh simplifications, one stream each (0: 8) */
	size_t large_index_count; /* requests with more indices take the multi-CTA single-mesh path, the
	                             others the batch kernel (0: 30000, i.e. 10k triangles; measured best
	                             p99 under Poisson load: larger meshes on one CTA take too long) */
	int max_batch;            /* requests per batch launch at most (0: 2048) */
	int batch_threads;        /* threads per CTA of the batch kernel (0: 256) */
	int plain;                /* 1: no batching, one request at a time on the single-mesh path */
	int perform_blocks;       /* cap on the cooperative pass kernel's grid per single-mesh request, so
	                             that concurrent requests share the GPU (0: 64; plain mode: no cap) */
} meshoptgpu_ServerConfig;

/* Creates a server on the current device. Requests are admitted while their device scratch
 * fits the memory budget; when a worker frees up it takes every request that has arrived in
 * the meantime (up to max_batch) as one launch, so work that arrives while other requests are
 * on the GPU overlaps with them. Returns NULL on failure (see meshoptgpu_getLastStatus). */
MESHOPTGPU_API meshoptgpu_Server* meshoptgpu_serverCreate(const meshoptgpu_ServerConfig* config);

/* Waits for all admitted requests, stops the workers and frees the server. */
MESHOPTGPU_API void meshoptgpu_serverDestroy(meshoptgpu_Server* server);

/* Submits one request without blocking. Pointers in mesh are DEVICE pointers that must stay
 * valid until the request completes, except attribute_weights (host memory, copied before
 * the call returns); every option meshopt_simplifyWithAttributes takes is accepted. Returns a
 * ticket (>= 0) or a negative meshoptgpu_Status* value. */
MESHOPTGPU_API long long meshoptgpu_serverSubmit(meshoptgpu_Server* server, const meshoptgpu_BatchMesh* mesh);

/* Blocks until the request completes; fills the result index count and error, and the
 * request's latency from submission to completion in milliseconds. Returns its status. */
MESHOPTGPU_API int meshoptgpu_serverWait(meshoptgpu_Server* server, long long ticket, size_t* result_index_count, float* result_error,
    double* latency_ms);

/* Server counters: requests completed, batch launches, single-mesh launches, peak device
 * bytes reserved, peak requests in flight. */
MESHOPTGPU_API void meshoptgpu_serverStats(meshoptgpu_Server* server, unsigned long long* out5);

/* Kernel launch accounting for the calling thread: the number of kernels this library has
 * launched, and optional CUDA-event timing of every launch of one kernel (selected by its
 * name prefix, e.g. "kDecide"; NULL disables). The events are recorded on the launching
 * stream and read after each call's final synchronisation. */
MESHOPTGPU_API unsigned long long meshoptgpu_getLaunchCount(void);
MESHOPTGPU_API void meshoptgpu_setKernelProfile(const char* kernel_name);
MESHOPTGPU_API void meshoptgpu_getKernelProfile(unsigned long long* launches, double* total_ms);

/* Bytes of device scratch one call on a mesh of this shape needs (for admission control). */
MESHOPTGPU_API size_t meshoptgpu_workspaceBytes(size_t index_count, size_t vertex_count, size_t attribute_count);

/* ---- compaction after simplification, on device data ---- */

/* Device forms of meshopt_optimizeVertexFetchRemap, meshopt_optimizeVertexFetch
 * (meshoptimizer.h; src/vfetchoptimizer.cpp:7-71) and meshopt_generatePositionRemap
 * (src/indexgenerator.cpp:555-578), for callers that keep the simplified mesh in HBM: every
 * buffer is a DEVICE pointer, the work is queued on `stream` (a cudaStream_t or NULL) and the
 * call returns once the result is known. Results equal the reference's. The fetch functions
 * return the number of used vertices; on invalid input (an index >= vertex_count, a
 * vertex_size outside 1..256) or a CUDA error they return 0 and set the status read by
 * meshoptgpu_getLastStatus. optimizeVertexFetch allows destination == vertices (other
 * overlaps are not supported) and rewrites indices in place. */
MESHOPTGPU_API size_t meshoptgpu_optimizeVertexFetchRemapDevice(unsigned int* destination, const unsigned int* indices, size_t index_count,
    size_t vertex_count, void* stream);
MESHOPTGPU_API size_t meshoptgpu_optimizeVertexFetchDevice(void* destination, unsigned int* indices, size_t index_count, const void* vertices,
    size_t vertex_count, size_t vertex_size, void* stream);
MESHOPTGPU_API int meshoptgpu_generatePositionRemapDevice(unsigned int* destination, const float* vertex_positions, size_t vertex_count,
    size_t vertex_positions_stride, void* stream);

/* Allocation-free mesh extent. No counterpart in the reference: it is the device-pointer
 * form of meshopt_simplifyScale for callers that must not allocate device memory while they
 * run: a renderer's frame loop whose device-memory budget is fixed up front, or a plugin whose
 * host application owns every device allocation. It writes the extent (the value
 * meshopt_simplifyScale returns) to the device float *extent, reading positions that are
 * already on the device, enqueued on `stream` without synchronising; it calls no
 * cudaMalloc/cudaFree and no allocating library routine.
 * Its scratch is a fixed 1 MiB device array inside the library (held on every GPU that
 * loads it until exit), which limits vertex_count to 67,108,864; larger counts return
 * meshoptgpu_StatusInvalidArgument. The first call on each device looks up that array's
 * device address: make it before any stream capture. All calls share the array, so calls
 * that overlap on the GPU race; order them (e.g. one stream). Returns a meshoptgpu_Status*
 * value (this call does not update meshoptgpu_getLastStatus). */
MESHOPTGPU_API int meshoptgpu_simplifyScaleNoAlloc(float* extent, const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    void* stream);

/* Releases the calling thread's device scratch and streams. */
MESHOPTGPU_API void meshoptgpu_releaseThreadResources(void);

#ifdef __cplusplus
}
#endif

#endif
