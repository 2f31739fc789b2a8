// mo_vfetch.cuh - vertex-buffer compaction after simplification, on device data
// (src/vfetchoptimizer.cpp:7-71, src/indexgenerator.cpp:555-578).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace mogpu
{

// scratch words vertexOrder needs
size_t vertexOrderScratchWords(size_t index_count, size_t vertex_count);

// order[v] = new index of vertex v in order of first use by indices, ~0u if unused.
// counters (2 device words): [0] = used vertex count, [1] = nonzero if an index is out of range.
void vertexOrder(unsigned int* order, const unsigned int* indices, size_t index_count, size_t vertex_count, unsigned int* scratch, unsigned int* counters,
    cudaStream_t stream);

// indices[i] = order[indices[i]]
void rewriteIndices(unsigned int* indices, size_t index_count, const unsigned int* order, cudaStream_t stream);

// destination[order[v]] = vertices[v] for used vertices (vertex_size bytes each); the buffers
// must not overlap
void moveVertices(void* destination, const void* vertices, size_t vertex_count, size_t vertex_size, const unsigned int* order, cudaStream_t stream);

// scratch words positionRemap needs
size_t positionRemapScratchWords(size_t vertex_count);

// remap[i] = smallest vertex index whose position (the first 3 floats of each stride_f-float
// vertex) compares equal to vertex i's. counters: [1] nonzero if the table overflowed.
void positionRemap(unsigned int* remap, const float* positions, size_t vertex_count, size_t stride_f, unsigned int* scratch, unsigned int* counters,
    cudaStream_t stream);

} // namespace mogpu
