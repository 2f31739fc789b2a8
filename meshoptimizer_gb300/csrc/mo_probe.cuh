// mo_probe.cuh - launch counting and optional CUDA-event timing of one named kernel.
//
// Every kernel launch of the library goes through MO_LAUNCH, which counts it in the
// calling thread's probe and, when that kernel's name was selected, brackets it with CUDA
// events recorded on the launching stream. The events are read after the run's final
// stream synchronisation, so timing adds no host synchronisation.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace mogpu
{

struct LaunchProbe
{
	unsigned long long launches = 0;
	std::string selected;
	std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
	std::vector<cudaEvent_t> pool;
	unsigned long long timed_launches = 0;
	double timed_ms = 0;
	bool capturing = false; // launches are being recorded into a graph: count them, record no events

	~LaunchProbe();
	cudaEvent_t take();
	void collect(); // call after the stream that ran the timed launches has been synchronised
};

LaunchProbe& probe();

inline cudaEvent_t probeBegin(const char* name, cudaStream_t stream)
{
	LaunchProbe& p = probe();
	p.launches++;
	while (*name == '(' || *name == ' ') // template kernels are passed parenthesised
		++name;
	if (p.capturing || p.selected.empty() || p.selected.compare(0, p.selected.size(), name, 0, p.selected.size()) != 0)
		return nullptr;
	cudaEvent_t e = p.take();
	cudaEventRecord(e, stream);
	return e;
}

inline void probeEnd(cudaEvent_t e0, cudaStream_t stream)
{
	if (!e0)
		return;
	LaunchProbe& p = probe();
	cudaEvent_t e1 = p.take();
	cudaEventRecord(e1, stream);
	p.pending.emplace_back(e0, e1);
}

} // namespace mogpu

#define MO_LAUNCH(kernel, grid, block, smem, stream, ...)                      \
	do                                                                         \
	{                                                                          \
		cudaEvent_t mo_e0_ = mogpu::probeBegin(#kernel, stream);               \
		kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);            \
		mogpu::probeEnd(mo_e0_, stream);                                       \
	} while (0)
