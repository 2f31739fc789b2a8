// mo_grid.cuh - grid-wide barrier for kernels launched cooperatively.
//
// cudaLaunchCooperativeKernel guarantees that all blocks are resident, so the wait below
// always ends; it still carries an iteration limit: past it the block records an error flag
// and leaves the barrier, and the kernel's caller turns the flag into an error status.
#pragma once

#include <cuda_runtime.h>

namespace mogpu
{

#ifndef MO_BARRIER_SLEEP_NS
#define MO_BARRIER_SLEEP_NS 32
#endif
constexpr unsigned int kBarrierSpinLimit = 1u << 25; // x >= 32 ns sleep (or an L2 round trip): seconds, never reached in a normal run
constexpr unsigned int kBarrierSleepNs = MO_BARRIER_SLEEP_NS; // between polls

// an arrival that publishes everything the block wrote before it (the block barrier ahead of it
// orders the other threads' writes before this thread's release)
__device__ __forceinline__ unsigned int arriveRelease(unsigned int* p)
{
	unsigned int old;
	asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
	return old;
}

// a poll that, once it sees the last arrival, makes the other blocks' writes visible to this
// block (the block barrier after it passes them on to the other threads)
__device__ __forceinline__ unsigned int pollAcquire(const unsigned int* p)
{
	unsigned int v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

// bar[0] counts the arrivals of all barriers of the launch and is zero before it. Barrier i ends
// when the count reaches (i + 1) * gridDim.x: no block can arrive at barrier i + 1 before every
// block has arrived at barrier i, so an arrival that reads old = n belongs to barrier n / G.
// Waiting blocks poll the count itself, so the last arrival releases them with its own add.
__device__ __forceinline__ void gridBarrier(unsigned int* bar, unsigned int* err, unsigned int limit = kBarrierSpinLimit)
{
	__syncthreads();
	if (threadIdx.x == 0)
	{
		const unsigned int old = arriveRelease(bar);
		const unsigned int target = (old / gridDim.x + 1) * gridDim.x;
		unsigned int spins = 0;
		while ((int)(pollAcquire(bar) - target) < 0)
		{
			if (++spins > limit)
			{
				atomicOr(err, 1u);
				break;
			}
			if (kBarrierSleepNs)
				__nanosleep(kBarrierSleepNs);
		}
	}
	__syncthreads();
}

// A grid barrier that a cooperative launch passes once, leaving its two words zero for the next
// launch: bar[0] counts arrivals, bar[1] departures, and the last block to depart clears both
// (by then no block polls bar[0] any more). A launch whose wait ran out leaves them nonzero: the
// owner clears them before it uses them again (the simplifier clears its words, with the rest of
// its scalars, at the start of every call, and a call whose barrier ran out reports an error).
__device__ __forceinline__ void gridBarrierOnce(unsigned int* bar, unsigned int* err, unsigned int limit = kBarrierSpinLimit)
{
	__syncthreads();
	if (threadIdx.x == 0)
	{
		arriveRelease(bar);
		unsigned int spins = 0;
		while (pollAcquire(bar) < gridDim.x)
		{
			if (++spins > limit)
			{
				atomicOr(err, 1u);
				break;
			}
			if (kBarrierSleepNs)
				__nanosleep(kBarrierSleepNs);
		}
		if (atomicAdd(bar + 1, 1u) == gridDim.x - 1)
		{
			atomicExch(bar, 0u);
			atomicExch(bar + 1, 0u);
		}
	}
	__syncthreads();
}

} // namespace mogpu
