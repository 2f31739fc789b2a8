// mo_meshlets.cuh - re-clusterization of simplified groups on device data:
// meshopt_buildMeshletsFlex (src/clusterizer.cpp:1035-1224) for many index subsets of one vertex
// buffer, one warp per subset, each result equal to a separate call's.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace mogpu
{

struct MeshletBatch
{
	// group g is indices[offsets[g] .. offsets[g + 1]) (device, 64-bit offsets)
	const unsigned int* indices;
	const unsigned long long* offsets;
	unsigned int groups;
	const float* positions; // first 3 floats of every stride_f-float vertex
	unsigned int stride_f;
	unsigned int vertex_count;
	unsigned int max_vertices, min_triangles, max_triangles;
	float cone_weight, split_factor;
	// group g's meshlets start at row meshlet_base[g] of `meshlets` ({vertex_offset,
	// triangle_offset, vertex_count, triangle_count} per row, offsets relative to the group);
	// its meshlet vertices and triangles at offsets[g] of mverts / mtris
	unsigned int* meshlets;
	const unsigned long long* meshlet_base;
	unsigned int* mverts;
	unsigned char* mtris;
	unsigned int* counts; // meshlets per group
	char* scratch;        // group g's at scratch_off[g] (meshletScratchBytes of its index count)
	const unsigned long long* scratch_off;
	unsigned int* error; // nonzero: an index out of range, or a bound the algorithm keeps was exceeded
	// shared memory per warp (at most 48 KiB) for the arrays the greedy loop reads at every step,
	// placed while they fit; 0: all in global scratch
	unsigned int pool_bytes;
	int optimize_level; // meshopt_optimizeMeshletLevel level run on every meshlet after the build, -1: none
	unsigned long long rows; // meshlet rows of the batch (meshlet_base[groups])
};

// meshopt_buildMeshletsBound (src/clusterizer.cpp:1017-1033)
size_t meshletBound(size_t index_count, size_t max_vertices, size_t max_triangles);

// device scratch bytes for one group of index_count indices (a multiple of 256)
size_t meshletScratchBytes(size_t index_count);

void buildMeshletsBatch(const MeshletBatch& b, cudaStream_t stream);

} // namespace mogpu
