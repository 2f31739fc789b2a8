// mo_noalloc.cu - meshoptgpu_simplifyScaleNoAlloc: the mesh extent (what meshopt_simplifyScale
// returns) computed on device data without allocating anything.
//
// Who needs this: code that must not call cudaMalloc/cudaFree while it runs, e.g. a renderer's
// frame loop whose device-memory budget is fixed up front, or a plugin whose host application
// owns all device allocations. meshopt_simplifyScale stages the positions in
// device scratch that it allocates on first use; this entry point instead reads positions the
// caller already has on the device and keeps its only scratch, the per-block partial extents,
// in a fixed file-scope device array.
//
// The scratch array is shared by every call in the process on a given device and keeps the
// last call's contents. Its ticket word must start at zero; each call clears it on its stream
// before the launch. Two calls whose kernels overlap on the GPU (different streams, no ordering
// between them) race on the array and produce garbage: callers order them, e.g. on one stream.
#include "../../include/meshopt_gb300.h"

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdio>
#include <mutex>

namespace
{

constexpr int kThreads = 256;
constexpr int kPerThread = 8;
constexpr size_t kPerBlock = size_t(kThreads) * kPerThread;        // 2048 vertices per block
constexpr size_t kMaxBlocks = 32768;
constexpr size_t kMaxVertices = kMaxBlocks * kPerBlock;           // 67,108,864 vertices
constexpr size_t kTicketWord = kMaxBlocks * 8;                     // after the partials
constexpr size_t kScratchWords = kTicketWord + 64;                 // 1 MiB + 256 B

// per block: min xyz, max xyz (as float bits) at [8 * block]; the finished-block ticket at kTicketWord
static __device__ __align__(256) unsigned int g_scale_scratch[kScratchWords];

// min/max with the comparison form of the reference's rescalePositions (src/simplifier.cpp:551-567):
// the leftmost of values that compare equal wins and NaN is skipped, so folding left to right
// in any tree gives the sequential result bit for bit
__device__ __forceinline__ float foldMin(float l, float r)
{
	return l > r ? r : l;
}

__device__ __forceinline__ float foldMax(float l, float r)
{
	return l < r ? r : l;
}

// folds the six running values of this thread with the lanes to its right, then the warps of
// the block, in index order; the result is valid in thread 0
__device__ void blockFold(float (&v)[6], float (*sm)[6])
{
#pragma unroll
	for (int o = 1; o < 32; o <<= 1)
	{
#pragma unroll
		for (int j = 0; j < 6; ++j)
		{
			float x = __shfl_down_sync(0xffffffffu, v[j], o);
			if ((threadIdx.x & 31) + o < 32 && ((threadIdx.x & (2 * o - 1)) == 0))
				v[j] = j < 3 ? foldMin(v[j], x) : foldMax(v[j], x);
		}
	}
	if ((threadIdx.x & 31) == 0)
		for (int j = 0; j < 6; ++j)
			sm[threadIdx.x >> 5][j] = v[j];
	__syncthreads();
	if (threadIdx.x == 0)
		for (int q = 1; q < kThreads / 32; ++q)
			for (int j = 0; j < 6; ++j)
				v[j] = j < 3 ? foldMin(v[j], sm[q][j]) : foldMax(v[j], sm[q][j]);
}

// One launch: every block folds 2048 vertices into its partial; the last block to finish
// (ticket) folds the partials in block order and writes the extent. A block first copies the
// positions of its vertices into shared memory with consecutive threads on consecutive words
// (coalesced whatever the stride), then each thread folds its 8 consecutive vertices from there
// in index order.
__global__ void __launch_bounds__(kThreads) kScaleNoAlloc(const float* __restrict__ pos, size_t stride_f, size_t n, unsigned int* scratch, float* out)
{
	__shared__ float sm[kThreads / 32][6];
	__shared__ float sp[kPerBlock * 3];
	__shared__ bool last;
	float v[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
	const size_t base = blockIdx.x * kPerBlock;
	const unsigned int count = unsigned(n - base < kPerBlock ? n - base : kPerBlock);
	for (unsigned int w = threadIdx.x; w < count * 3; w += kThreads)
	{
		const unsigned int i = w / 3, c = w - i * 3;
		sp[w] = __ldg(pos + (base + i) * stride_f + c);
	}
	__syncthreads();
	const unsigned int begin = threadIdx.x * kPerThread;
	const unsigned int end = begin + kPerThread < count ? begin + kPerThread : count;
	for (unsigned int i = begin; i < end; ++i)
	{
		const float* p = sp + i * 3;
		for (int j = 0; j < 3; ++j)
		{
			v[j] = v[j] > p[j] ? p[j] : v[j];
			v[3 + j] = v[3 + j] < p[j] ? p[j] : v[3 + j];
		}
	}
	blockFold(v, sm);
	if (threadIdx.x == 0)
	{
		for (int j = 0; j < 6; ++j)
			scratch[blockIdx.x * 8 + j] = __float_as_uint(v[j]);
		__threadfence();
		last = atomicAdd(&scratch[kTicketWord], 1u) == gridDim.x - 1;
	}
	__syncthreads();
	if (!last)
		return;

	// the last block: partials of blocks [t*per, (t+1)*per) per thread, then the ordered tree
	for (int j = 0; j < 6; ++j)
		v[j] = j < 3 ? FLT_MAX : -FLT_MAX;
	unsigned int per = (gridDim.x + kThreads - 1) / kThreads;
	unsigned int b0 = threadIdx.x * per, b1 = min(b0 + per, gridDim.x);
	for (unsigned int b = b0; b < b1; ++b)
		for (int j = 0; j < 6; ++j)
		{
			float x = __uint_as_float(__ldcg(&scratch[b * 8 + j]));
			v[j] = j < 3 ? foldMin(v[j], x) : foldMax(v[j], x);
		}
	__syncthreads();
	blockFold(v, sm);
	if (threadIdx.x == 0)
	{
		float extent = 0.f;
		extent = (v[3] - v[0]) < extent ? extent : (v[3] - v[0]);
		extent = (v[4] - v[1]) < extent ? extent : (v[4] - v[1]);
		extent = (v[5] - v[2]) < extent ? extent : (v[5] - v[2]);
		*out = extent;
		scratch[kTicketWord] = 0;
	}
}

// Device address of g_scale_scratch per device, resolved once per device (first call).
std::mutex g_lock;
unsigned int* g_scratch_ptr[128];
bool g_scratch_ready[128];

int scratchFor(int device, unsigned int** out)
{
	if (device < 0 || device >= 128)
		return meshoptgpu_StatusInvalidArgument;
	std::lock_guard<std::mutex> guard(g_lock);
	if (!g_scratch_ready[device])
	{
		// host code sees g_scale_scratch as a host-side stand-in; the kernel needs its device address
		void* ptr = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&ptr, g_scale_scratch);
		if (e != cudaSuccess)
		{
			fprintf(stderr, "meshopt_gb300: cudaGetSymbolAddress for the no-alloc scratch failed: %s\n", cudaGetErrorString(e));
			return meshoptgpu_StatusCudaError;
		}
		g_scratch_ptr[device] = static_cast<unsigned int*>(ptr);
		g_scratch_ready[device] = true;
	}
	*out = g_scratch_ptr[device];
	return meshoptgpu_StatusOk;
}

} // namespace

extern "C" int meshoptgpu_simplifyScaleNoAlloc(float* extent, const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    void* stream)
{
	if (vertex_positions_stride < 12 || vertex_positions_stride > 256 || vertex_positions_stride % 4 != 0)
	{
		fprintf(stderr, "meshopt_gb300: meshoptgpu_simplifyScaleNoAlloc: vertex_positions_stride must be in [12, 256] and a multiple of 4\n");
		return meshoptgpu_StatusInvalidArgument;
	}
	if (vertex_count > kMaxVertices)
	{
		fprintf(stderr, "meshopt_gb300: meshoptgpu_simplifyScaleNoAlloc: vertex_count %zu exceeds the no-alloc limit of %zu vertices\n", vertex_count,
		    kMaxVertices);
		return meshoptgpu_StatusInvalidArgument;
	}
	if (!extent || (vertex_count && !vertex_positions))
		return meshoptgpu_StatusInvalidArgument;
	int device = 0;
	if (cudaGetDevice(&device) != cudaSuccess)
		return meshoptgpu_StatusCudaError;
	unsigned int* scratch = nullptr;
	int st = scratchFor(device, &scratch);
	if (st != meshoptgpu_StatusOk)
		return st;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	if (cudaMemsetAsync(scratch + kTicketWord, 0, sizeof(unsigned int), s) != cudaSuccess)
		return meshoptgpu_StatusCudaError;
	unsigned int blocks = unsigned((vertex_count + kPerBlock - 1) / kPerBlock);
	blocks = blocks ? blocks : 1;
	kScaleNoAlloc<<<blocks, kThreads, 0, s>>>(vertex_positions, vertex_positions_stride / 4, vertex_count, scratch, extent);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess)
	{
		fprintf(stderr, "meshopt_gb300: meshoptgpu_simplifyScaleNoAlloc launch failed: %s\n", cudaGetErrorString(e));
		return meshoptgpu_StatusCudaError;
	}
	return meshoptgpu_StatusOk;
}
