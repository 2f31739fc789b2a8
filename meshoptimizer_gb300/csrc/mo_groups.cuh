// mo_groups.cuh - boundary locks of one cluster-LOD level (demo/clusterlod.h:372-418).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace mogpu
{

// device scratch bytes groupLocks needs
size_t groupLockScratchBytes(size_t vertex_count, size_t group_count);

// locks[i] = kVertexLock if the position of vertex i (remap[i] <= i, as generatePositionRemap
// gives) is used by two or more groups or vertex_lock[remap[i]] has the Lock bit, | the Protect
// bit locks[i] held before, | vertex_lock[i] (nullptr: none). Groups are
// indices[d_offsets[g] .. d_offsets[g+1]) (device offsets). *bad (device) becomes nonzero when
// an index or a remap entry is out of range.
void groupLocks(unsigned char* locks, const unsigned int* indices, const unsigned long long* d_offsets, size_t group_count, const unsigned int* remap,
    const unsigned char* vertex_lock, size_t vertex_count, void* scratch, unsigned int* bad, cudaStream_t stream);

} // namespace mogpu
