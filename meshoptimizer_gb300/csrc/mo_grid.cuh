// mo_grid.cuh - grid-wide barrier for kernels launched cooperatively.
//
// cudaLaunchCooperativeKernel guarantees that all blocks are resident, so the wait below
// always ends; it still carries an iteration limit: past it the block records an error flag
// and leaves the barrier, and the kernel's caller turns the flag into an error status.
#pragma once

#include <cuda_runtime.h>

namespace mogpu
{

constexpr unsigned int kBarrierSpinLimit = 1u << 25; // x ~64 ns sleep: seconds, never reached in a normal run

// bar[0]: arrivals, bar[1]: generation. Both zero before the launch.
__device__ __forceinline__ void gridBarrier(unsigned int* bar, unsigned int* err)
{
	__syncthreads();
	if (threadIdx.x == 0)
	{
		volatile unsigned int* gen = bar + 1;
		unsigned int g = *gen;
		__threadfence();
		unsigned int arrived = atomicAdd(bar, 1u);
		if (arrived == gridDim.x - 1)
		{
			atomicExch(bar, 0u);
			__threadfence();
			atomicAdd(bar + 1, 1u);
		}
		else
		{
			unsigned int spins = 0;
			while (*gen == g)
			{
				if (++spins > kBarrierSpinLimit)
				{
					atomicOr(err, 1u);
					break;
				}
				__nanosleep(64);
			}
		}
		__threadfence();
	}
	__syncthreads();
}

} // namespace mogpu
