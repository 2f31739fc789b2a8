// mo_capi.cu - the C ABI (include/meshopt_gb300.h): drop-in entry points with the
// signatures of meshoptimizer.h, plus device-resident and diagnostic additions.
//
// Each calling thread owns one Simplifier (device scratch arena) and one CUDA stream, so
// concurrent callers do not share mutable state (the reference is reentrant too,
// meshoptimizer.h:1206-1210).
#include "../../include/meshopt_gb300.h"

#include "mo_common.cuh"
#include "mo_probe.cuh"
#include "mo_simplify.cuh"

#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>

namespace
{

using namespace mogpu;

struct HostStaging
{
	void* ptr = nullptr;
	size_t cap = 0;
	~HostStaging()
	{
		if (ptr)
			cudaFreeHost(ptr);
	}
};

struct DeviceBuffer
{
	void* ptr = nullptr;
	size_t cap = 0;
	~DeviceBuffer()
	{
		if (ptr)
			cudaFree(ptr);
	}
	void* ensure(size_t bytes)
	{
		if (bytes <= cap)
			return ptr;
		if (ptr)
			cudaFree(ptr);
		ptr = nullptr;
		cap = 0;
		size_t want = bytes + bytes / 4 + 256;
		MO_CUDA_CHECK(cudaMalloc(&ptr, want));
		cap = want;
		return ptr;
	}
};

struct ThreadState
{
	int status = meshoptgpu_StatusOk;
	std::string message;
	int device = -1;
	cudaStream_t stream = nullptr;
	std::unique_ptr<Simplifier> simplifier;
	DeviceBuffer inputs;
	RunResult last;
	PhaseTimes times;
	bool timing = false;

	~ThreadState()
	{
		simplifier.reset();
		if (stream)
			cudaStreamDestroy(stream);
	}

	void ensure()
	{
		int dev = 0;
		MO_CUDA_CHECK(cudaGetDevice(&dev));
		if (simplifier && device == dev)
			return;
		simplifier.reset();
		if (stream)
			cudaStreamDestroy(stream);
		stream = nullptr;
		device = dev;
		MO_CUDA_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
		simplifier.reset(new Simplifier(dev));
	}
};

thread_local ThreadState* tls = nullptr;

ThreadState& state()
{
	if (!tls)
		tls = new ThreadState();
	return *tls;
}

void setStatus(int status, const std::string& msg)
{
	ThreadState& s = state();
	s.status = status;
	s.message = msg;
	if (status != meshoptgpu_StatusOk)
		fprintf(stderr, "meshopt_gb300: %s\n", msg.c_str());
}

const unsigned int kSupportedOptions = kOptLockBorder | kOptErrorAbsolute | kOptRegularize | kOptRegularizeLight;

// argument checks of meshopt_simplifyEdge (:2348-2357); returns an error message or empty
std::string checkArgs(size_t index_count, size_t vertex_positions_stride, size_t target_index_count, float target_error,
    size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count, unsigned int options)
{
	if (index_count % 3 != 0)
		return "index_count must be a multiple of 3";
	if (vertex_positions_stride < 12 || vertex_positions_stride > 256 || vertex_positions_stride % 4 != 0)
		return "vertex_positions_stride must be in [12, 256] and a multiple of 4";
	if (target_index_count > index_count)
		return "target_index_count must not exceed index_count";
	if (!(target_error >= 0))
		return "target_error must be >= 0";
	if (attribute_count > (size_t)kMaxAttributes)
		return "attribute_count must be <= 32";
	if (attribute_count && (vertex_attributes_stride < attribute_count * 4 || vertex_attributes_stride > 256 || vertex_attributes_stride % 4 != 0))
		return "vertex_attributes_stride must be in [4*attribute_count, 256] and a multiple of 4";
	for (size_t i = 0; i < attribute_count; ++i)
		if (!(attribute_weights[i] >= 0))
			return "attribute weights must be >= 0";
	if (options & ~kSupportedOptions)
		return "option bits 0x" + [](unsigned v) {
			char b[16];
			snprintf(b, sizeof(b), "%x", v);
			return std::string(b);
		}(options & ~kSupportedOptions) + " are not implemented on the GPU path";
	return std::string();
}

int statusOf(const std::exception& e)
{
	if (auto ce = dynamic_cast<const CudaError*>(&e))
		return ce->code == cudaErrorMemoryAllocation ? meshoptgpu_StatusOutOfMemory : meshoptgpu_StatusCudaError;
	if (dynamic_cast<const std::invalid_argument*>(&e))
		return meshoptgpu_StatusInvalidArgument;
	if (dynamic_cast<const std::bad_alloc*>(&e))
		return meshoptgpu_StatusOutOfMemory;
	return meshoptgpu_StatusCudaError;
}

size_t failHost(unsigned int* destination, const unsigned int* indices, size_t index_count, float* result_error, int status, const std::string& msg)
{
	setStatus(status, msg);
	if (destination && indices && destination != indices)
		memmove(destination, indices, index_count * sizeof(unsigned int));
	if (result_error)
		*result_error = 0.f;
	return index_count;
}

size_t align256(size_t v)
{
	return (v + 255) & ~size_t(255);
}

size_t simplifyHost(unsigned int* destination, const unsigned int* indices, size_t index_count, const float* vertex_positions, size_t vertex_count,
    size_t vertex_positions_stride, const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options, float* result_error)
{
	std::string bad = checkArgs(index_count, vertex_positions_stride, target_index_count, target_error, vertex_attributes_stride, attribute_weights,
	    attribute_count, options);
	if (!bad.empty())
		return failHost(destination, indices, index_count, result_error,
		    (options & ~kSupportedOptions) ? meshoptgpu_StatusUnsupported : meshoptgpu_StatusInvalidArgument, bad);
	try
	{
		ThreadState& s = state();
		s.ensure();
		// device copies of the inputs, laid out back to back in one buffer
		size_t b_idx = align256(index_count * 4), b_pos = align256(vertex_count * vertex_positions_stride);
		size_t b_attr = attribute_count ? align256(vertex_count * vertex_attributes_stride) : 0;
		size_t b_lock = vertex_lock ? align256(vertex_count) : 0;
		size_t b_out = align256(index_count * 4);
		char* base = static_cast<char*>(s.inputs.ensure(b_idx + b_pos + b_attr + b_lock + b_out + 256));
		unsigned int* d_idx = reinterpret_cast<unsigned int*>(base);
		float* d_pos = reinterpret_cast<float*>(base + b_idx);
		float* d_attr = attribute_count ? reinterpret_cast<float*>(base + b_idx + b_pos) : nullptr;
		unsigned char* d_lock = vertex_lock ? reinterpret_cast<unsigned char*>(base + b_idx + b_pos + b_attr) : nullptr;
		unsigned int* d_out = reinterpret_cast<unsigned int*>(base + b_idx + b_pos + b_attr + b_lock);
		cudaStream_t st = s.stream;
		if (index_count)
			MO_CUDA_CHECK(cudaMemcpyAsync(d_idx, indices, index_count * 4, cudaMemcpyHostToDevice, st));
		if (vertex_count)
			MO_CUDA_CHECK(cudaMemcpyAsync(d_pos, vertex_positions, vertex_count * vertex_positions_stride, cudaMemcpyHostToDevice, st));
		if (d_attr)
			MO_CUDA_CHECK(cudaMemcpyAsync(d_attr, vertex_attributes, vertex_count * vertex_attributes_stride, cudaMemcpyHostToDevice, st));
		if (d_lock)
			MO_CUDA_CHECK(cudaMemcpyAsync(d_lock, vertex_lock, vertex_count, cudaMemcpyHostToDevice, st));

		MeshDesc m;
		m.indices = d_idx;
		m.index_count = index_count;
		m.positions = d_pos;
		m.vertex_count = vertex_count;
		m.positions_stride = vertex_positions_stride;
		m.attributes = d_attr;
		m.attributes_stride = vertex_attributes_stride;
		m.weights = attribute_weights;
		m.attribute_count = attribute_count;
		m.lock = d_lock;
		m.target_index_count = target_index_count;
		m.target_error = target_error;
		m.options = options;
		s.last = s.simplifier->run(m, d_out, st, s.timing ? &s.times : nullptr);
		if (s.last.index_count)
			MO_CUDA_CHECK(cudaMemcpyAsync(destination, d_out, s.last.index_count * 4, cudaMemcpyDeviceToHost, st));
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		if (result_error)
			*result_error = s.last.result_error;
		setStatus(meshoptgpu_StatusOk, "");
		return s.last.index_count;
	}
	catch (const std::exception& e)
	{
		return failHost(destination, indices, index_count, result_error, statusOf(e), e.what());
	}
}

} // namespace

extern "C" {

size_t meshopt_simplify(unsigned int* destination, const unsigned int* indices, size_t index_count, const float* vertex_positions, size_t vertex_count,
    size_t vertex_positions_stride, size_t target_index_count, float target_error, unsigned int options, float* result_error)
{
	return simplifyHost(destination, indices, index_count, vertex_positions, vertex_count, vertex_positions_stride, nullptr, 0, nullptr, 0, nullptr,
	    target_index_count, target_error, options, result_error);
}

size_t meshopt_simplifyWithAttributes(unsigned int* destination, const unsigned int* indices, size_t index_count, const float* vertex_positions,
    size_t vertex_count, size_t vertex_positions_stride, const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights,
    size_t attribute_count, const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options, float* result_error)
{
	return simplifyHost(destination, indices, index_count, vertex_positions, vertex_count, vertex_positions_stride, vertex_attributes,
	    vertex_attributes_stride, attribute_weights, attribute_count, vertex_lock, target_index_count, target_error, options, result_error);
}

float meshopt_simplifyScale(const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride)
{
	if (vertex_positions_stride < 12 || vertex_positions_stride > 256 || vertex_positions_stride % 4 != 0)
	{
		setStatus(meshoptgpu_StatusInvalidArgument, "vertex_positions_stride must be in [12, 256] and a multiple of 4");
		return 0.f;
	}
	try
	{
		ThreadState& s = state();
		s.ensure();
		float* d_pos = static_cast<float*>(s.inputs.ensure(align256(vertex_count * vertex_positions_stride) + 256));
		if (vertex_count)
			MO_CUDA_CHECK(cudaMemcpyAsync(d_pos, vertex_positions, vertex_count * vertex_positions_stride, cudaMemcpyHostToDevice, s.stream));
		float r = s.simplifier->scale(d_pos, vertex_count, vertex_positions_stride, s.stream);
		setStatus(meshoptgpu_StatusOk, "");
		return r;
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return 0.f;
	}
}

int meshoptgpu_getLastStatus(void)
{
	return state().status;
}

const char* meshoptgpu_getLastMessage(void)
{
	return state().message.c_str();
}

int meshoptgpu_getLastPassStats(meshoptgpu_PassStats* out, int max_passes)
{
	ThreadState& s = state();
	int n = s.last.passes < kMaxPassStats ? s.last.passes : kMaxPassStats;
	for (int i = 0; i < n && i < max_passes; ++i)
	{
		const PassStats& p = s.last.pass[i];
		out[i] = meshoptgpu_PassStats{p.triangles, p.candidates, p.evaluated, p.done, p.skipped, p.invalid, p.stop, p.rounds, p.active, p.windows};
	}
	return s.last.passes;
}

void meshoptgpu_setTiming(int enabled)
{
	state().timing = enabled != 0;
}

int meshoptgpu_getLastPhaseTimes(float* out16)
{
	const PhaseTimes& t = state().times;
	float v[8] = {t.setup, t.adjacency, t.pick, t.rank, t.sort, t.perform, t.apply, t.total};
	memcpy(out16, v, sizeof(v));
	memcpy(out16 + 8, state().last.perform_phase_ms, sizeof(v));
	return 16;
}

size_t meshoptgpu_simplifyDevice(unsigned int* destination, const unsigned int* indices, size_t index_count, const float* vertex_positions,
    size_t vertex_count, size_t vertex_positions_stride, const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights,
    size_t attribute_count, const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options, float* result_error,
    void* stream)
{
	std::string bad = checkArgs(index_count, vertex_positions_stride, target_index_count, target_error, vertex_attributes_stride, attribute_weights,
	    attribute_count, options);
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	auto fail = [&](int status, const std::string& msg) {
		setStatus(status, msg);
		if (destination != indices && index_count)
			cudaMemcpyAsync(destination, indices, index_count * 4, cudaMemcpyDeviceToDevice, st);
		if (result_error)
			*result_error = 0.f;
		return index_count;
	};
	if (!bad.empty())
		return fail((options & ~kSupportedOptions) ? meshoptgpu_StatusUnsupported : meshoptgpu_StatusInvalidArgument, bad);
	try
	{
		ThreadState& s = state();
		s.ensure();
		MeshDesc m;
		m.indices = indices;
		m.index_count = index_count;
		m.positions = vertex_positions;
		m.vertex_count = vertex_count;
		m.positions_stride = vertex_positions_stride;
		m.attributes = vertex_attributes;
		m.attributes_stride = vertex_attributes_stride;
		m.weights = attribute_weights;
		m.attribute_count = attribute_count;
		m.lock = vertex_lock;
		m.target_index_count = target_index_count;
		m.target_error = target_error;
		m.options = options;
		s.last = s.simplifier->run(m, destination, st, s.timing ? &s.times : nullptr);
		if (result_error)
			*result_error = s.last.result_error;
		setStatus(meshoptgpu_StatusOk, "");
		return s.last.index_count;
	}
	catch (const std::exception& e)
	{
		return fail(statusOf(e), e.what());
	}
}

void meshoptgpu_setKernelProfile(const char* kernel_name)
{
	LaunchProbe& p = probe();
	p.selected = kernel_name ? kernel_name : "";
	p.timed_launches = 0;
	p.timed_ms = 0;
}

void meshoptgpu_getKernelProfile(unsigned long long* launches, double* total_ms)
{
	LaunchProbe& p = probe();
	if (launches)
		*launches = p.timed_launches;
	if (total_ms)
		*total_ms = p.timed_ms;
}

unsigned long long meshoptgpu_getLaunchCount(void)
{
	return probe().launches;
}

size_t meshoptgpu_workspaceBytes(size_t index_count, size_t vertex_count, size_t attribute_count)
{
	return Simplifier::workspaceBytes(index_count, vertex_count, attribute_count);
}

void meshoptgpu_releaseThreadResources(void)
{
	delete tls;
	tls = nullptr;
}

} // extern "C"
