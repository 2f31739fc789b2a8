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

float mo_simplifyScale(const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride)
{
	return rescale_positions_f32(NULL, vertex_positions, vertex_count, vertex_positions_stride / sizeof(float), NULL);
}
