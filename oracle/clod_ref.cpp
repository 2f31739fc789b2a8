// Test harness (TEST INFRASTRUCTURE ONLY): exposes the reference cluster-LOD builder's per-level
// boundary lock computation (lockBoundary, demo/clusterlod.h:372-418) through a C entry point so
// the oracle's restatement and the GPU path can be checked against it. Built by oracle/Makefile
// (`make clod-ref`) from the reference's own header and sources where they lie; every group is
// passed as one cluster, which is how the builder's groups reach lockBoundary (each group's
// clusters' indices in order).
#define CLUSTERLOD_IMPLEMENTATION
#include "meshoptimizer.h"
#include "clusterlod.h"

#include <vector>

extern "C" void clod_ref_lock_boundary(unsigned char* locks, size_t vertex_count, const unsigned int* indices, const size_t* group_offsets,
    size_t group_count, const unsigned int* remap, const unsigned char* vertex_lock)
{
	std::vector<unsigned char> l(locks, locks + vertex_count);
	std::vector<clod::Cluster> clusters(group_count);
	std::vector<std::vector<int> > groups(group_count);
	for (size_t g = 0; g < group_count; ++g)
	{
		clusters[g].indices.assign(indices + group_offsets[g], indices + group_offsets[g + 1]);
		groups[g].push_back(int(g));
	}
	std::vector<unsigned int> r(remap, remap + vertex_count);
	clod::lockBoundary(l, groups, clusters, r, vertex_lock);
	for (size_t i = 0; i < vertex_count; ++i)
		locks[i] = l[i];
}
