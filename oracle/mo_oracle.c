/*
 * mo_oracle.c - CPU oracle for the quadric edge-collapse simplifier.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of meshoptimizer's
 * meshopt_simplifyEdge (src/simplifier.cpp:2344-2626) and its phase functions,
 * used by the tests and by bench.py's CPU-baseline leg to check and time the
 * CUDA path. The product library never links or calls it.
 *
 * mo_core.inc is compiled twice: with float (bit-exact with the reference when
 * built with -ffp-contract=off) and with double (the FP64 oracle).
 */
#include "mo_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define REAL float
#define SQRT sqrtf
#define FABS fabsf
#define FN(name) name##_f32
#include "mo_core.inc"
#undef REAL
#undef SQRT
#undef FABS
#undef FN

#define REAL double
#define SQRT sqrt
#define FABS fabs
#define FN(name) name##_f64
#include "mo_core.inc"
#undef REAL
#undef SQRT
#undef FABS
#undef FN

size_t mo_simplify_edge(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options,
    float* result_error, mo_stats* stats, mo_setup_dump* dump)
{
	return simplify_edge_f32(destination, indices, index_count, vertex_positions, vertex_count, vertex_positions_stride,
	    vertex_attributes, vertex_attributes_stride, attribute_weights, attribute_count, vertex_lock,
	    target_index_count, target_error, options, result_error, stats, dump);
}

size_t mo_simplify_edge_f64(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options,
    double* result_error, mo_stats* stats)
{
	return simplify_edge_f64(destination, indices, index_count, vertex_positions, vertex_count, vertex_positions_stride,
	    vertex_attributes, vertex_attributes_stride, attribute_weights, attribute_count, vertex_lock,
	    target_index_count, target_error, options, result_error, stats, NULL);
}

size_t mo_simplify(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    size_t target_index_count, float target_error, unsigned int options, float* result_error)
{
	return simplify_edge_f32(destination, indices, index_count, vertex_positions, vertex_count, vertex_positions_stride,
	    NULL, 0, NULL, 0, NULL, target_index_count, target_error, options, result_error, NULL, NULL);
}

size_t mo_simplifyWithAttributes(unsigned int* destination, const unsigned int* indices, size_t index_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options, float* result_error)
{
	return simplify_edge_f32(destination, indices, index_count, vertex_positions, vertex_count, vertex_positions_stride,
	    vertex_attributes, vertex_attributes_stride, attribute_weights, attribute_count, vertex_lock,
	    target_index_count, target_error, options, result_error, NULL, NULL);
}

size_t mo_simplifyWithUpdate(unsigned int* indices, size_t index_count, float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count, const unsigned char* vertex_lock,
    size_t target_index_count, float target_error, unsigned int options, float* result_error)
{
	return simplify_edge_f32(indices, indices, index_count, vertex_positions, vertex_count, vertex_positions_stride, vertex_attributes,
	    vertex_attributes_stride, attribute_weights, attribute_count, vertex_lock, target_index_count, target_error, options | MO_InternalSolve,
	    result_error, NULL, NULL);
}

float mo_simplifyScale(const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride)
{
	return rescale_positions_f32(NULL, vertex_positions, vertex_count, vertex_positions_stride / sizeof(float), NULL, NULL);
}

/* ---- the step after the simplifier in its callers (compaction of the vertex buffer) ---- */

/* meshopt_optimizeVertexFetchRemap (src/vfetchoptimizer.cpp:7-26): each vertex's new index in
 * order of first use by the index buffer, ~0u for unused vertices; returns the used count */
size_t mo_optimizeVertexFetchRemap(unsigned int* destination, const unsigned int* indices, size_t index_count, size_t vertex_count)
{
	unsigned int used = 0;
	memset(destination, 0xff, vertex_count * sizeof(unsigned int));
	for (size_t i = 0; i < index_count; ++i)
	{
		unsigned int* slot = &destination[indices[i]];
		if (*slot == ~0u)
			*slot = used++;
	}
	return used;
}

/* meshopt_optimizeVertexFetch (src/vfetchoptimizer.cpp:28-71): vertices copied in order of first
 * use, indices rewritten in place; destination may be vertices */
size_t mo_optimizeVertexFetch(void* destination, unsigned int* indices, size_t index_count, const void* vertices, size_t vertex_count, size_t vertex_size)
{
	unsigned char* copy = NULL;
	if (destination == vertices)
	{
		copy = (unsigned char*)malloc(vertex_count * vertex_size + 1);
		memcpy(copy, vertices, vertex_count * vertex_size);
		vertices = copy;
	}
	unsigned int* order = (unsigned int*)malloc((vertex_count ? vertex_count : 1) * sizeof(unsigned int));
	size_t used = mo_optimizeVertexFetchRemap(order, indices, index_count, vertex_count);
	for (size_t v = 0; v < vertex_count; ++v)
		if (order[v] != ~0u)
			memcpy((unsigned char*)destination + (size_t)order[v] * vertex_size, (const unsigned char*)vertices + v * vertex_size, vertex_size);
	for (size_t i = 0; i < index_count; ++i)
		indices[i] = order[indices[i]];
	free(order);
	free(copy);
	return used;
}

/* meshopt_generatePositionRemap (src/indexgenerator.cpp:555-578): the smallest vertex index
 * whose position compares equal (float ==) to each vertex's; the remap half of the
 * simplifier's position remap */
void mo_generatePositionRemap(unsigned int* destination, const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride)
{
	unsigned int* wedge = (unsigned int*)malloc((vertex_count ? vertex_count : 1) * sizeof(unsigned int));
	mo_position_remap(destination, wedge, vertex_positions, vertex_count, vertex_positions_stride / sizeof(float), NULL);
	free(wedge);
}
