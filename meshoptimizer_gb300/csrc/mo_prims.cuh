// mo_prims.cuh - integer primitives for the simplifier: block scans, a device-wide
// exclusive scan, and a stable LSD radix sort of (key, value) pairs.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <stdexcept>
#include <string>

namespace mogpu
{

struct CudaError : std::runtime_error
{
	cudaError_t code;
	CudaError(cudaError_t e, const char* expr, const char* file, int line)
	    : std::runtime_error(std::string(cudaGetErrorString(e)) + " at " + file + ":" + std::to_string(line) + " (" + expr + ")"), code(e)
	{
	}
};

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;                               // one uint4 per thread
constexpr int kScanTile = kScanThreads * kScanItems;        // 1024 elements per block

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;        // 2048 pairs per block
constexpr int kSortBins = 256;

__device__ __forceinline__ unsigned int laneId()
{
	return threadIdx.x & 31;
}

__device__ __forceinline__ unsigned int warpInclusiveScan(unsigned int v)
{
#pragma unroll
	for (int o = 1; o < 32; o <<= 1)
	{
		unsigned int n = __shfl_up_sync(0xffffffffu, v, o);
		if (laneId() >= (unsigned)o)
			v += n;
	}
	return v;
}

// Exclusive scan of one value per thread across a block of NT threads (NT multiple of 32,
// at most 1024). Returns the exclusive prefix; *total receives the block sum. Uses `smem`
// (NT/32 words) and synchronises the block twice.
template <int NT>
__device__ __forceinline__ unsigned int blockExclusiveScan(unsigned int v, unsigned int* smem, unsigned int* total)
{
	const int warps = NT / 32;
	unsigned int inc = warpInclusiveScan(v);
	unsigned int w = threadIdx.x >> 5;
	if (laneId() == 31)
		smem[w] = inc;
	__syncthreads();
	if (w == 0)
	{
		unsigned int s = laneId() < (unsigned)warps ? smem[laneId()] : 0;
		unsigned int si = warpInclusiveScan(s);
		if (laneId() < (unsigned)warps)
			smem[laneId()] = si - s;
		if (laneId() == warps - 1)
			smem[warps] = si;
	}
	__syncthreads();
	unsigned int r = smem[w] + inc - v;
	*total = smem[warps];
	return r;
}

// scratch words needed by scanExclusive for n elements
size_t scanScratchWords(size_t n);

// Single-launch mode of scanExclusive (and of radixSortPairs' histogram scans): a scan over
// more than one tile runs as one cooperative kernel (reduce, one grid barrier, apply) instead
// of a reduce and an apply launch per level. bar: two device words, zero before the first
// scan, which every scan leaves zero; err: set to 1 if the barrier's bounded wait gave up.
// A caller gives each stream that scans concurrently words of its own.
struct ScanSync
{
	unsigned int* bar = nullptr;
	unsigned int* err = nullptr;
	unsigned int max_blocks = 0; // at most this many blocks (0: as many as are resident at once), so
	                             // concurrent callers on other streams can be resident beside it
	const unsigned int* n_dev = nullptr; // optional: the live element count on the device (at most n),
	                                     // read by the kernels; needs the single-launch mode
};

// Runs the grid barrier (once != 0: the single-use one) with one of `blocks` blocks never
// arriving and a wait limit of `limit` polls; returns the error flag the waiting blocks set
// (1 when the bounded wait ran out, as it must). For tests of the failure path.
unsigned int probeBarrierWait(int once, unsigned int blocks, unsigned int limit, cudaStream_t stream);

// Blocks a single-launch scan may use on the current device (all resident at once); queried
// once per device and cached. Call it outside stream capture before the first such scan.
unsigned int coopScanCapacity();

// out[i] = sum(in[0..i)) for i < n; if total != nullptr, *total (device) = sum(in[0..n)).
// in and out may alias. scratch: scanScratchWords(n) words of device memory.
void scanExclusive(const unsigned int* in, unsigned int* out, size_t n, unsigned int* total, unsigned int* scratch, cudaStream_t stream,
    ScanSync sync = ScanSync());

// scratch words needed by radixSortPairs for n pairs
size_t radixScratchWords(size_t n);

// Stable LSD radix sort of (keys, vals) on key bits [0, bits); vals_in == nullptr means
// the values 0..n-1. Sorted result ends in
// (keys_out, vals_out); keys_tmp/vals_tmp are ping-pong buffers of n elements. Input
// arrays are left unchanged only when the pass count is even; callers treat them as scratch.
// n_dev (optional): the live count on the device (<= n), read by the kernels, so that the
// launches can be recorded once and replayed for any count up to n. Up to 4,096 pairs with a
// host count sort in one single-block launch instead of the digit passes (the same order).
// The outputs must not alias the inputs.
void radixSortPairs(const unsigned int* keys_in, const unsigned int* vals_in, unsigned int* keys_out, unsigned int* vals_out,
    unsigned int* keys_tmp, unsigned int* vals_tmp, size_t n, int bits, unsigned int* scratch, cudaStream_t stream,
    const unsigned int* n_dev = nullptr, ScanSync sync = ScanSync());

inline unsigned int gridFor(size_t n, int threads)
{
	size_t g = (n + threads - 1) / threads;
	return unsigned(g ? g : 1);
}

} // namespace mogpu
