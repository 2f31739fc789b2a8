// mo_groups.cu - the boundary locks of one cluster-LOD level on device data.
//
// A cluster-LOD builder simplifies groups of clusters that share one vertex buffer; before it
// does, it locks every position that more than one group uses, so that neighbouring groups
// keep a common border (lockBoundary, demo/clusterlod.h:372-418). The reference walks the
// groups in order and locks a position when an earlier group has seen it; that is the same
// set as "used by at least two groups", which one pass over all groups' indices finds here:
// each position records the first group that claims it (atomicCAS) and is marked shared when
// a different group finds it claimed.
#include "mo_groups.cuh"
#include "mo_common.cuh"
#include "mo_prims.cuh"
#include "mo_probe.cuh"

namespace mogpu
{

namespace
{

constexpr int kThreads = 256;

__global__ void kClearOwners(unsigned int* owner, unsigned char* shared, size_t n)
{
	size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n)
	{
		owner[i] = ~0u;
		shared[i] = 0;
	}
}

// one block per group: claim the position of every index of the group
__global__ void kClaimPositions(const unsigned int* __restrict__ indices, const unsigned long long* __restrict__ offsets, const unsigned int* __restrict__ remap,
    size_t vertex_count, unsigned int* owner, unsigned char* shared, unsigned int* bad)
{
	const unsigned int g = blockIdx.x;
	const unsigned long long b = offsets[g], e = offsets[g + 1];
	for (unsigned long long p = b + threadIdx.x; p < e; p += blockDim.x)
	{
		unsigned int v = indices[p];
		if (v >= vertex_count)
		{
			atomicOr(bad, 1u);
			continue;
		}
		unsigned int r = remap[v];
		if (r >= vertex_count)
		{
			atomicOr(bad, 1u);
			continue;
		}
		unsigned int prev = atomicCAS(&owner[r], ~0u, g);
		if (prev != ~0u && prev != g)
			shared[r] = 1;
	}
}

// locks[i] = lock bit | the vertex's own Protect bit | vertex_lock[i]. The reference rewrites
// locks in vertex order and reads locks[r] (r = remap[i] <= i) after it was rewritten, so the
// lock bit of every vertex at a position also carries vertex_lock[r]'s Lock bit
__global__ void kLevelLocks(const unsigned int* __restrict__ remap, const unsigned char* __restrict__ shared, const unsigned char* __restrict__ vertex_lock,
    size_t n, unsigned char* locks, unsigned int* bad)
{
	size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	unsigned int r = remap[i];
	if (r >= n)
	{
		atomicOr(bad, 1u);
		return;
	}
	bool lock = shared[r] || (vertex_lock && (vertex_lock[r] & kVertexLock));
	unsigned char l = (unsigned char)((lock ? kVertexLock : 0) | (locks[i] & kVertexProtect));
	if (vertex_lock)
		l |= vertex_lock[i];
	locks[i] = l;
}

} // namespace

size_t groupLockScratchBytes(size_t vertex_count, size_t group_count)
{
	return ((vertex_count * 4 + 255) & ~size_t(255)) + ((vertex_count + 255) & ~size_t(255)) + (group_count + 1) * 8 + 256;
}

void groupLocks(unsigned char* locks, const unsigned int* indices, const unsigned long long* d_offsets, size_t group_count, const unsigned int* remap,
    const unsigned char* vertex_lock, size_t vertex_count, void* scratch, unsigned int* bad, cudaStream_t stream)
{
	unsigned int* owner = static_cast<unsigned int*>(scratch);
	unsigned char* shared = reinterpret_cast<unsigned char*>(owner) + ((vertex_count * 4 + 255) & ~size_t(255));
	MO_CUDA_CHECK(cudaMemsetAsync(bad, 0, sizeof(unsigned int), stream));
	if (!vertex_count)
		return;
	MO_LAUNCH(kClearOwners, gridFor(vertex_count, kThreads), kThreads, 0, stream, owner, shared, vertex_count);
	if (group_count)
		MO_LAUNCH(kClaimPositions, unsigned(group_count), kThreads, 0, stream, indices, d_offsets, remap, vertex_count, owner, shared, bad);
	MO_LAUNCH(kLevelLocks, gridFor(vertex_count, kThreads), kThreads, 0, stream, remap, shared, vertex_lock, vertex_count, locks, bad);
}

} // namespace mogpu
