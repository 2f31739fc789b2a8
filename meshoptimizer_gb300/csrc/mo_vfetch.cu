// mo_vfetch.cu - the compaction step that follows the simplifier in its callers, on device data:
// meshopt_optimizeVertexFetchRemap / meshopt_optimizeVertexFetch (src/vfetchoptimizer.cpp:7-71)
// and meshopt_generatePositionRemap (src/indexgenerator.cpp:555-578).
//
// The reference walks the index buffer once and numbers vertices as they are first seen. Here
// the same order comes from three data-parallel steps: the first index position of every
// vertex (atomicMin), a flag at every index position that is a first use, and an exclusive
// scan of the flags, whose value at a first use is that vertex's new index. The position remap
// is an open-addressing table keyed by position in which the smallest vertex index of each
// position wins (atomicMin), which is the vertex the reference's sequential insertion keeps.
#include "mo_vfetch.cuh"
#include "mo_common.cuh"
#include "mo_prims.cuh"
#include "mo_probe.cuh"

namespace mogpu
{

namespace
{

constexpr int kThreads = 256;

__device__ __forceinline__ size_t gtidv()
{
	return (size_t)blockIdx.x * blockDim.x + threadIdx.x;
}

__global__ void kClearWords(unsigned int* p, size_t n, unsigned int value)
{
	size_t i = gtidv();
	if (i < n)
		p[i] = value;
}

// first[v] = smallest index position that references v; out-of-range indices raise *bad
__global__ void kFirstPosition(const unsigned int* __restrict__ idx, size_t n, size_t vcount, unsigned int* first, unsigned int* bad)
{
	size_t p = gtidv();
	if (p >= n)
		return;
	unsigned int v = idx[p];
	if (v >= vcount)
	{
		atomicOr(bad, 1u);
		return;
	}
	atomicMin(&first[v], (unsigned int)p);
}

__global__ void kFirstFlag(const unsigned int* __restrict__ idx, size_t n, size_t vcount, const unsigned int* __restrict__ first, unsigned int* __restrict__ flags)
{
	size_t p = gtidv();
	if (p >= n)
		return;
	unsigned int v = idx[p];
	flags[p] = (v < vcount && first[v] == (unsigned int)p) ? 1u : 0u;
}

// new index of each vertex: the rank of its first use, ~0u when unused
__global__ void kVertexOrder(const unsigned int* __restrict__ first, const unsigned int* __restrict__ rank, size_t vcount, unsigned int* __restrict__ order)
{
	size_t v = gtidv();
	if (v >= vcount)
		return;
	unsigned int f = first[v];
	order[v] = f == ~0u ? ~0u : rank[f];
}

__global__ void kRewriteIndices(unsigned int* idx, size_t n, const unsigned int* __restrict__ order)
{
	size_t p = gtidv();
	if (p < n)
		idx[p] = order[idx[p]];
}

// vertices to their new slots: one thread per 4-byte word (vertex_size a multiple of 4 and
// both buffers 4-byte aligned) or per byte otherwise
__global__ void kMoveVertexWords(const unsigned int* __restrict__ src, size_t vcount, size_t words, const unsigned int* __restrict__ order, unsigned int* __restrict__ dst)
{
	size_t t = gtidv();
	if (t >= vcount * words)
		return;
	size_t v = t / words, w = t - v * words;
	unsigned int o = order[v];
	if (o != ~0u)
		dst[(size_t)o * words + w] = src[t];
}

__global__ void kMoveVertexBytes(const unsigned char* __restrict__ src, size_t vcount, size_t size, const unsigned int* __restrict__ order, unsigned char* __restrict__ dst)
{
	size_t t = gtidv();
	if (t >= vcount * size)
		return;
	size_t v = t / size, b = t - v * size;
	unsigned int o = order[v];
	if (o != ~0u)
		dst[(size_t)o * size + b] = src[t];
}

__device__ __forceinline__ unsigned int keyBits(float f)
{
	unsigned int u = __float_as_uint(f);
	return u == 0x80000000u ? 0u : u; // -0 hashes as +0 (they compare equal)
}

__device__ __forceinline__ unsigned int mixBits(unsigned int h)
{
	h ^= h >> 16;
	h *= 0x7feb352du;
	h ^= h >> 15;
	h *= 0x846ca68bu;
	h ^= h >> 16;
	return h;
}

// position table: a vertex claims an empty slot or, finding a slot whose vertex has an equal
// position, lowers it to its own index if smaller; slot[i] records where vertex i landed
__global__ void kPositionInsert(const float* __restrict__ pos, size_t stride_f, size_t n, unsigned int* table, unsigned int mask, unsigned int* __restrict__ slot,
    unsigned int* fail)
{
	size_t vi = gtidv();
	if (vi >= n)
		return;
	unsigned int i = (unsigned int)vi;
	const float* p = pos + vi * stride_f;
	float x = p[0], y = p[1], z = p[2];
	unsigned int h = mixBits(keyBits(x) * 0x9e3779b1u ^ mixBits(keyBits(y) + 0x85ebca6bu) ^ mixBits(keyBits(z) * 0xc2b2ae35u + 1u));
	unsigned int b = h & mask;
	for (unsigned int probe = 0; probe <= mask; ++probe)
	{
		unsigned int cur = table[b];
		if (cur == ~0u)
		{
			unsigned int prev = atomicCAS(&table[b], ~0u, i);
			if (prev == ~0u)
			{
				slot[i] = b;
				return;
			}
			cur = prev;
		}
		const float* q = pos + (size_t)cur * stride_f;
		if (q[0] == x && q[1] == y && q[2] == z)
		{
			atomicMin(&table[b], i);
			slot[i] = b;
			return;
		}
		b = (b + probe + 1) & mask;
	}
	atomicOr(fail, 1u);
	slot[i] = ~0u;
}

__global__ void kPositionRemap(const unsigned int* __restrict__ table, const unsigned int* __restrict__ slot, size_t n, unsigned int* __restrict__ remap)
{
	size_t i = gtidv();
	if (i >= n)
		return;
	unsigned int s = slot[i];
	remap[i] = s == ~0u ? (unsigned int)i : table[s];
}

size_t alignWords(size_t n)
{
	return (n + 63) & ~size_t(63);
}

} // namespace

size_t vertexOrderScratchWords(size_t index_count, size_t vertex_count)
{
	return alignWords(vertex_count) + alignWords(index_count) + alignWords(scanScratchWords(index_count)) + 64;
}

void vertexOrder(unsigned int* order, const unsigned int* indices, size_t index_count, size_t vertex_count, unsigned int* scratch, unsigned int* counters,
    cudaStream_t stream)
{
	unsigned int* first = scratch;
	unsigned int* flags = first + alignWords(vertex_count);
	unsigned int* sscratch = flags + alignWords(index_count);
	MO_CUDA_CHECK(cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned int), stream));
	if (vertex_count)
		MO_LAUNCH(kClearWords, gridFor(vertex_count, kThreads), kThreads, 0, stream, first, vertex_count, ~0u);
	if (index_count)
	{
		MO_LAUNCH(kFirstPosition, gridFor(index_count, kThreads), kThreads, 0, stream, indices, index_count, vertex_count, first, &counters[1]);
		MO_LAUNCH(kFirstFlag, gridFor(index_count, kThreads), kThreads, 0, stream, indices, index_count, vertex_count, first, flags);
		scanExclusive(flags, flags, index_count, &counters[0], sscratch, stream);
	}
	if (vertex_count)
		MO_LAUNCH(kVertexOrder, gridFor(vertex_count, kThreads), kThreads, 0, stream, first, flags, vertex_count, order);
}

void rewriteIndices(unsigned int* indices, size_t index_count, const unsigned int* order, cudaStream_t stream)
{
	if (index_count)
		MO_LAUNCH(kRewriteIndices, gridFor(index_count, kThreads), kThreads, 0, stream, indices, index_count, order);
}

void moveVertices(void* destination, const void* vertices, size_t vertex_count, size_t vertex_size, const unsigned int* order, cudaStream_t stream)
{
	if (!vertex_count)
		return;
	bool words = vertex_size % 4 == 0 && reinterpret_cast<uintptr_t>(destination) % 4 == 0 && reinterpret_cast<uintptr_t>(vertices) % 4 == 0;
	if (words)
		MO_LAUNCH(kMoveVertexWords, gridFor(vertex_count * (vertex_size / 4), kThreads), kThreads, 0, stream, static_cast<const unsigned int*>(vertices),
		    vertex_count, vertex_size / 4, order, static_cast<unsigned int*>(destination));
	else
		MO_LAUNCH(kMoveVertexBytes, gridFor(vertex_count * vertex_size, kThreads), kThreads, 0, stream, static_cast<const unsigned char*>(vertices),
		    vertex_count, vertex_size, order, static_cast<unsigned char*>(destination));
}

size_t positionRemapScratchWords(size_t vertex_count)
{
	size_t buckets = 1;
	while (buckets < vertex_count + vertex_count / 4)
		buckets *= 2;
	return alignWords(buckets) + alignWords(vertex_count) + 64;
}

void positionRemap(unsigned int* remap, const float* positions, size_t vertex_count, size_t stride_f, unsigned int* scratch, unsigned int* counters,
    cudaStream_t stream)
{
	size_t buckets = 1;
	while (buckets < vertex_count + vertex_count / 4)
		buckets *= 2;
	unsigned int* table = scratch;
	unsigned int* slot = table + alignWords(buckets);
	MO_CUDA_CHECK(cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned int), stream));
	if (!vertex_count)
		return;
	MO_CUDA_CHECK(cudaMemsetAsync(table, 0xFF, buckets * sizeof(unsigned int), stream));
	MO_LAUNCH(kPositionInsert, gridFor(vertex_count, kThreads), kThreads, 0, stream, positions, stride_f, vertex_count, table, unsigned(buckets - 1), slot,
	    &counters[1]);
	MO_LAUNCH(kPositionRemap, gridFor(vertex_count, kThreads), kThreads, 0, stream, table, slot, vertex_count, remap);
}

} // namespace mogpu
