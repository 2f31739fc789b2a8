/*
 * mo_oracle.h - CPU oracle for the quadric edge-collapse simplifier.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of meshoptimizer's
 * edge-collapse simplifier (src/simplifier.cpp, meshopt_simplifyEdge :2344-2626)
 * used to check the CUDA path and to time a CPU baseline. The product library
 * (meshoptimizer_gb300/) never links, loads or calls it.
 *
 * Build with -ffp-contract=off: the reference's output depends on whether
 * a*b+c is contracted to an FMA, and this restatement mirrors its FP32
 * operation order exactly.
 */
#ifndef MO_ORACLE_H
#define MO_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* option bits, same values as meshoptimizer.h:466-482 */
enum
{
	MO_LockBorder = 1 << 0,
	MO_Sparse = 1 << 1,
	MO_ErrorAbsolute = 1 << 2,
	MO_Prune = 1 << 3,
	MO_Regularize = 1 << 4,
	MO_Permissive = 1 << 5,
	MO_RegularizeLight = 1 << 6,
	MO_InternalSolve = 1 << 29,  /* meshopt_simplifyWithUpdate's mode (src/simplifier.cpp:2340) */
	MO_InternalDebug = 1 << 30,
};

/* vertex_lock flag bits, same values as meshoptimizer.h:488-495 */
enum
{
	MO_Vertex_Lock = 1 << 0,
	MO_Vertex_Protect = 1 << 1,
	MO_Vertex_Priority = 1 << 2,
};

#define MO_MAX_PASSES 128

/* Per-pass counters, the same quantities the reference prints under TRACE
 * (src/simplifier.cpp:1625-1633). stop: 0 out of collapses, 1 error limit,
 * 2 count limit, 3 error goal. */
typedef struct mo_stats
{
	unsigned int passes;
	unsigned int tri[MO_MAX_PASSES];       /* triangles at pass start */
	unsigned int cand[MO_MAX_PASSES];      /* collapse candidates picked */
	unsigned int evaluated[MO_MAX_PASSES]; /* candidates reached before the stop */
	unsigned int done[MO_MAX_PASSES];      /* committed collapses */
	unsigned int skipped[MO_MAX_PASSES];   /* rejected: endpoint already locked */
	unsigned int invalid[MO_MAX_PASSES];   /* rejected: triangle flip */
	unsigned int stop[MO_MAX_PASSES];
	float result_error_sq;                 /* internal (squared, rescaled) error */
	float error_limit;                     /* target_error^2 / error_scale^2 */
} mo_stats;

/* Optional intermediate arrays after setup (before the first pass), caller-owned,
 * each sized for the (dense) vertex count; any pointer may be NULL. */
typedef struct mo_setup_dump
{
	unsigned int* remap;
	unsigned int* wedge;
	unsigned char* kind;
	unsigned int* loop;
	unsigned int* loopback;
	float* positions;          /* 3 floats per vertex, rescaled */
	float* quadrics;           /* 11 floats per vertex */
	float* attr_quadrics;      /* 11 floats per vertex */
	float* attr_gradients;     /* 4*attribute_count floats per vertex */
	size_t capacity;           /* boundEdgeCollapses result */
	float scale;
} mo_setup_dump;

/* Full driver, same contract as meshopt_simplifyEdge (src/simplifier.cpp:2344). */
size_t mo_simplify_edge(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options,
    float* result_error, mo_stats* stats, mo_setup_dump* dump);

/* Same signatures as meshoptimizer.h:513 and :537, routed to the restatement. */
size_t mo_simplify(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    size_t target_index_count, float target_error, unsigned int options, float* result_error);

size_t mo_simplifyWithAttributes(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options, float* result_error);

/* meshoptimizer.h:560: simplifies indices in place and writes the optimal positions (and
 * attributes) of the vertices the result uses back into the caller's buffers */
size_t mo_simplifyWithUpdate(unsigned int* indices, size_t index_count, float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count, const unsigned char* vertex_lock,
    size_t target_index_count, float target_error, unsigned int options, float* result_error);

/* meshoptimizer.h:611 */
float mo_simplifyScale(const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride);

/* FP64 oracle: the same driver with every quadric, position and error held in
 * double (the sort key is still taken from the error rounded to float). Its
 * result_error is the reference point against which the FP32 path's error is
 * stated; its index buffer is not expected to match bit for bit. */
size_t mo_simplify_edge_f64(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options,
    double* result_error, mo_stats* stats);

/* The compaction step after the simplifier in its callers: same signatures as
 * meshoptimizer.h's meshopt_optimizeVertexFetchRemap, meshopt_optimizeVertexFetch and
 * meshopt_generatePositionRemap. */
size_t mo_optimizeVertexFetchRemap(unsigned int* destination, const unsigned int* indices, size_t index_count, size_t vertex_count);
size_t mo_optimizeVertexFetch(void* destination, unsigned int* indices, size_t index_count, const void* vertices, size_t vertex_count, size_t vertex_size);
void mo_generatePositionRemap(unsigned int* destination, const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride);

/* Re-clusterization after a cluster-LOD level's simplify (mo_meshlet.c): same signatures as
 * meshoptimizer.h's meshopt_buildMeshletsBound and meshopt_buildMeshletsFlex; `meshlets` holds
 * {vertex_offset, triangle_offset, vertex_count, triangle_count} per meshlet. */
size_t mo_buildMeshletsBound(size_t index_count, size_t max_vertices, size_t max_triangles);
size_t mo_buildMeshletsFlex(unsigned int* meshlets, unsigned int* meshlet_vertices, unsigned char* meshlet_triangles, const unsigned int* indices,
    size_t index_count, const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride, size_t max_vertices, size_t min_triangles,
    size_t max_triangles, float cone_weight, float split_factor);
/* meshopt_optimizeMeshletLevel (src/meshletutils.cpp:366), same signature */
void mo_optimizeMeshletLevel(unsigned int* meshlet_vertices, size_t vertex_count, unsigned char* meshlet_triangles, size_t triangle_count, int level);
/* mo_optimizeMeshletLevel on each of meshlet_count {vertex_offset, triangle_offset, vertex_count, triangle_count} rows */
void mo_optimizeMeshlets(const unsigned int* meshlets, size_t meshlet_count, unsigned int* meshlet_vertices, unsigned char* meshlet_triangles, int level);

#ifdef __cplusplus
}
#endif

#endif
