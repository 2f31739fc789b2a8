// mo_batch.cuh - persistent multi-mesh simplification (one CTA per mesh, device work queue).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace mogpu
{

// attributes with weight > 0 of a batched mesh (rescaleAttributes :605-621, :2410-2421): source
// column and weight of each used attribute
struct BatchAttr
{
	unsigned int src[32];
	float weight[32];
};

// one mesh of a batch; device pointers
struct BatchDesc
{
	const unsigned int* indices;
	const float* positions;
	unsigned int* out;
	unsigned int index_count;
	unsigned int vertex_count; // of the vertex buffer the indices address
	unsigned int stride_f;     // position stride in floats
	unsigned int target_index_count;
	float target_error;
	unsigned int options;
	const float* attributes;   // nullptr: positions only
	const unsigned char* lock; // vertex_lock, nullptr: none
	const BatchAttr* amap;     // used attributes (ac of them)
	unsigned int attr_stride_f;
	unsigned int ac;
};

struct BatchResult
{
	unsigned int index_count;
	float result_error;
	unsigned int passes;
	unsigned int status; // 0 ok, 2 invalid index, 3 a decision round made no progress
};

// scratch bytes one mesh needs: without the decision-round state (rounds = false) in shared
// memory, where it runs when that size fits the launch's budget, else with it in a global slab.
// A sparse mesh has at most min(index_count, vertex_count) vertices of its own.
size_t batchWorkspaceBytes(size_t index_count, size_t vertex_count, size_t ac, bool sparse, bool rounds);

// whether a mesh needs the full-option kernel: a sparse subset (option bit 1), attributes,
// vertex_lock or Permissive (option bit 5)
inline bool batchNeedsFull(const BatchDesc& d)
{
	return d.ac || d.lock || (d.options & ((1u << 1) | (1u << 5)));
}

// resident CTAs per SM for a thread count, dynamic shared memory size and kernel form
int batchBlocksPerSM(int threads, unsigned int smem_bytes, bool full);

// full: the instantiation with every option; otherwise the positions-only one
void launchBatch(const BatchDesc* d_descs, unsigned int count, unsigned int* d_ticket, BatchResult* d_results, char* d_slabs, size_t slab_bytes,
    unsigned int smem_bytes, unsigned int blocks, int threads, bool full, cudaStream_t stream);

} // namespace mogpu
