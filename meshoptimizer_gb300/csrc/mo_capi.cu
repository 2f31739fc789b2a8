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
#include "mo_batch.cuh"
#include "mo_vfetch.cuh"
#include "mo_groups.cuh"
#include "mo_meshlets.cuh"

#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <thread>
#include <tuple>
#include <memory>
#include <mutex>
#include <numeric>
#include <vector>
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
	void* ensure(size_t bytes)
	{
		if (bytes <= cap)
			return ptr;
		if (ptr)
			cudaFreeHost(ptr);
		ptr = nullptr;
		cap = 0;
		size_t want = bytes + bytes / 4 + 4096;
		MO_CUDA_CHECK(cudaMallocHost(&ptr, want));
		cap = want;
		return ptr;
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
	// batched path
	DeviceBuffer batch_meta, batch_slabs, batch_io, compact_scratch, group_scratch, update_io, meshlet_scratch;
	HostStaging batch_host, batch_meta_host;
	int batch_threads = 0;          // 0: autotune
	int sms = 1;                    // the device's SM count
	unsigned int batch_smem = 0;    // 0: default budget
	// drop-in calls with at most this many indices run on the batch kernel as a batch of one;
	// (size_t)-1: the autotuner picks the route per size class (see routeAndRun)
	size_t dropin_batch_limit = ~size_t(0);
	bool autotune = true; // the single-mesh path's launch shape and the drop-in route are timed per size class
	// drop-in copies on a stream of their own, in the order the setup first reads them:
	// positions, indices, attributes (one stream takes the whole host link, so a second one would
	// only slow the first inputs down). Events: positions, attributes, indices copied.
	cudaStream_t copy_stream = nullptr;
	cudaEvent_t copy_done[3] = {nullptr, nullptr, nullptr};

	void ensureCopyStreams()
	{
		if (!copy_stream)
			MO_CUDA_CHECK(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
		for (int i = 0; i < 3; ++i)
			if (!copy_done[i])
				MO_CUDA_CHECK(cudaEventCreateWithFlags(&copy_done[i], cudaEventDisableTiming));
	}

	void releaseCopyStreams()
	{
		for (int i = 0; i < 3; ++i)
		{
			if (copy_done[i])
				cudaEventDestroy(copy_done[i]);
			copy_done[i] = nullptr;
		}
		if (copy_stream)
			cudaStreamDestroy(copy_stream);
		copy_stream = nullptr;
	}

	~ThreadState()
	{
		simplifier.reset();
		releaseCopyStreams();
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
		releaseCopyStreams();
		if (stream)
			cudaStreamDestroy(stream);
		stream = nullptr;
		device = dev;
		MO_CUDA_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
		MO_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
		simplifier.reset(new Simplifier(dev));
		const char* at = getenv("MESHOPTGPU_AUTOTUNE");
		autotune = !(at && atoi(at) == 0) && !getenv("MESHOPTGPU_PERFORM_BLOCKS_PER_SM");
	}
};

// per-thread state, freed when the thread exits (server workers) or on request
thread_local std::unique_ptr<ThreadState> tls;

ThreadState& state()
{
	if (!tls)
		tls.reset(new ThreadState());
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

const unsigned int kSupportedOptions =
    kOptLockBorder | kOptErrorAbsolute | kOptRegularize | kOptRegularizeLight | kOptSparse | kOptPermissive | kOptPrune | kOptInternalDebug;
// the one-CTA-per-mesh batch kernel implements every option but the component pruning and the
// debug output
const unsigned int kBatchOptions = kOptLockBorder | kOptErrorAbsolute | kOptRegularize | kOptRegularizeLight | kOptSparse | kOptPermissive;

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

// host bytes of `count` records of `stride` bytes of which the first `used` are read: the last
// record ends after its used bytes, as the reference reads it (an interleaved array may end
// there, and a copy of whole strides would read, or write back, past the caller's buffer)
size_t stridedExtent(size_t count, size_t stride, size_t used)
{
	return count ? (count - 1) * stride + used : 0;
}

struct HostCopy
{
	void* dst;
	const void* src;
	size_t bytes;
};

// Host threads for the batch path's packing and scattering copies (memory-bound host loops),
// started on first use and kept for the process (never joined: the threads only ever wait for
// the next job). One job at a time: a caller that finds the pool busy copies on its own thread.
class CopyPool
{
public:
	static CopyPool& get()
	{
		static CopyPool* pool = new CopyPool(); // left to the process: no teardown order at exit
		return *pool;
	}

	// copies[0, n) in `parts` contiguous runs given by cut (cut[0] = 0, cut[parts] = n); the calling
	// thread takes the last run. False when the pool is busy (nothing copied).
	bool run(const HostCopy* copies, const std::vector<size_t>& cut)
	{
		std::unique_lock<std::mutex> own(busy_, std::try_to_lock);
		if (!own.owns_lock())
			return false;
		const size_t parts = cut.size() - 1;
		{
			std::lock_guard<std::mutex> g(m_);
			while (workers_.size() + 1 < parts)
			{
				const size_t id = workers_.size();
				workers_.emplace_back([this, id]() { work(id); });
				workers_.back().detach();
			}
			copies_ = copies;
			cut_ = cut;
			pending_ = parts - 1;
			++generation_;
		}
		cv_.notify_all();
		copyRun(copies, cut[parts - 1], cut[parts]);
		std::unique_lock<std::mutex> g(m_);
		done_.wait(g, [&]() { return pending_ == 0; });
		return true;
	}

	static void copyRun(const HostCopy* copies, size_t b, size_t e)
	{
		for (size_t i = b; i < e; ++i)
			memcpy(copies[i].dst, copies[i].src, copies[i].bytes);
	}

private:
	void work(size_t id)
	{
		size_t seen = 0;
		for (;;)
		{
			const HostCopy* copies;
			size_t b, e;
			{
				std::unique_lock<std::mutex> g(m_);
				cv_.wait(g, [&]() { return generation_ != seen; });
				seen = generation_;
				if (id + 1 >= cut_.size() - 1)
					continue; // this job has fewer runs than workers
				copies = copies_;
				b = cut_[id];
				e = cut_[id + 1];
			}
			copyRun(copies, b, e);
			std::lock_guard<std::mutex> g(m_);
			if (--pending_ == 0)
				done_.notify_one();
		}
	}

	std::mutex busy_, m_;
	std::condition_variable cv_, done_;
	std::vector<std::thread> workers_;
	const HostCopy* copies_ = nullptr;
	std::vector<size_t> cut_;
	size_t generation_ = 0, pending_ = 0;
};

// Host memcpy of many pieces, spread over up to 16 threads in contiguous runs of about equal
// bytes when there is enough to copy (one thread per 256 KiB at least: one host thread copies
// about 10 GB/s, the link to the GPU takes 200).
void parallelCopies(const HostCopy* copies, size_t n)
{
	size_t total = 0;
	for (size_t i = 0; i < n; ++i)
		total += copies[i].bytes;
	const unsigned int hw = std::max(1u, std::thread::hardware_concurrency());
	const size_t threads = std::min<size_t>(std::min<size_t>(16, hw), total >> 18);
	if (threads <= 1)
	{
		CopyPool::copyRun(copies, 0, n);
		return;
	}
	std::vector<size_t> cut(1, 0);
	size_t acc = 0;
	const size_t share = total / threads;
	for (size_t i = 0; i < n && cut.size() < threads; ++i)
	{
		acc += copies[i].bytes;
		if (acc >= share * cut.size())
			cut.push_back(i + 1);
	}
	cut.push_back(n);
	if (!CopyPool::get().run(copies, cut))
		CopyPool::copyRun(copies, 0, n);
}

void parallelCopies(const std::vector<HostCopy>& copies)
{
	parallelCopies(copies.data(), copies.size());
}

// Offsets of distinct (pointer, bytes) keys in insertion order: an open-addressing table over a
// flat array (no allocation per key), for packing the arrays that meshes of a batch share once.
class PieceTable
{
public:
	explicit PieceTable(size_t keys)
	{
		size_t cap = 16;
		while (cap < 2 * keys)
			cap <<= 1;
		slots_.assign(cap, Slot{nullptr, 0, 0});
	}
	// the offset stored for (p, bytes), or ~0 after storing `at` for it
	size_t findOrInsert(const void* p, size_t bytes, size_t at)
	{
		const size_t mask = slots_.size() - 1;
		size_t h = (reinterpret_cast<uintptr_t>(p) * 0x9E3779B97F4A7C15ull ^ bytes * 0xC2B2AE3D27D4EB4Full) >> 17;
		for (;; ++h)
		{
			Slot& sl = slots_[h & mask];
			if (!sl.p)
			{
				sl = Slot{p, bytes, at};
				return ~size_t(0);
			}
			if (sl.p == p && sl.bytes == bytes)
				return sl.at;
		}
	}

private:
	struct Slot
	{
		const void* p;
		size_t bytes, at;
	};
	std::vector<Slot> slots_;
};

// Runs a small mesh (device pointers) on the batch kernel when the mesh's options allow; returns
// false to leave it to the single-mesh path.
bool smallMeshOnBatch(ThreadState& s, const MeshDesc& m, unsigned int* d_out, cudaStream_t st);

// A drop-in or device call's simplification (device pointers): on the batch kernel or the
// single-mesh path, as the calling thread's drop-in limit or the autotuner decides; the result
// in d_out and s.last.
void routeAndRun(ThreadState& s, const MeshDesc& m, unsigned int* d_out, cudaStream_t st, bool allow_batch);

// the index count above which routeAndRun sends every drop-in call to the single-mesh path
size_t singlePathAbove(const ThreadState& s);

size_t simplifyHost(unsigned int* destination, const unsigned int* indices, size_t index_count, const float* vertex_positions, size_t vertex_count,
    size_t vertex_positions_stride, const float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options, float* result_error)
{
	std::string bad = checkArgs(index_count, vertex_positions_stride, target_index_count, target_error, vertex_attributes_stride, attribute_weights,
	    attribute_count, options);
	if (!bad.empty())
		return failHost(destination, indices, index_count, result_error,
		    (options & ~kSupportedOptions) ? meshoptgpu_StatusUnsupported : meshoptgpu_StatusInvalidArgument, bad);
	bool split = false; // inputs copied on the copy streams too
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
		// large meshes on the single-mesh path: the copies on the copy stream, positions first (the
		// setup's first kernels read only them), then indices, then attributes; the setup waits for
		// each where it first reads it
		const size_t pos_bytes = stridedExtent(vertex_count, vertex_positions_stride, 12);
		const size_t attr_bytes = d_attr ? stridedExtent(vertex_count, vertex_attributes_stride, attribute_count * 4) : 0;
		split = index_count * 4 + pos_bytes + attr_bytes >= (size_t(1) << 20) && index_count > singlePathAbove(s);
		if (split)
		{
			s.ensureCopyStreams();
			if (vertex_count)
				MO_CUDA_CHECK(cudaMemcpyAsync(d_pos, vertex_positions, pos_bytes, cudaMemcpyHostToDevice, s.copy_stream));
			MO_CUDA_CHECK(cudaEventRecord(s.copy_done[0], s.copy_stream));
			if (index_count)
				MO_CUDA_CHECK(cudaMemcpyAsync(d_idx, indices, index_count * 4, cudaMemcpyHostToDevice, s.copy_stream));
			MO_CUDA_CHECK(cudaEventRecord(s.copy_done[2], s.copy_stream));
			if (d_attr)
				MO_CUDA_CHECK(cudaMemcpyAsync(d_attr, vertex_attributes, attr_bytes, cudaMemcpyHostToDevice, s.copy_stream));
			MO_CUDA_CHECK(cudaEventRecord(s.copy_done[1], s.copy_stream));
			MO_CUDA_CHECK(cudaStreamWaitEvent(st, s.copy_done[0], 0));
		}
		else
		{
			if (index_count)
				MO_CUDA_CHECK(cudaMemcpyAsync(d_idx, indices, index_count * 4, cudaMemcpyHostToDevice, st));
			if (vertex_count)
				MO_CUDA_CHECK(cudaMemcpyAsync(d_pos, vertex_positions, pos_bytes, cudaMemcpyHostToDevice, st));
			if (d_attr)
				MO_CUDA_CHECK(cudaMemcpyAsync(d_attr, vertex_attributes, attr_bytes, cudaMemcpyHostToDevice, st));
		}
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
		m.attributes_ready = split ? s.copy_done[1] : nullptr;
		m.indices_ready = split ? s.copy_done[2] : nullptr;
		routeAndRun(s, m, d_out, st, !split);
		if (s.last.index_count)
			MO_CUDA_CHECK(cudaMemcpyAsync(destination, d_out, s.last.index_count * 4, cudaMemcpyDeviceToHost, st));
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		if (split) // the caller's index and attribute buffers are read to the end before returning
		{
			MO_CUDA_CHECK(cudaEventSynchronize(s.copy_done[1]));
			MO_CUDA_CHECK(cudaEventSynchronize(s.copy_done[2]));
		}
		if (result_error)
			*result_error = s.last.result_error;
		setStatus(meshoptgpu_StatusOk, "");
		return s.last.index_count;
	}
	catch (const std::exception& e)
	{
		if (split)
		{
			ThreadState& s = state();
			cudaEventSynchronize(s.copy_done[0]);
			cudaEventSynchronize(s.copy_done[1]);
			cudaEventSynchronize(s.copy_done[2]);
		}
		return failHost(destination, indices, index_count, result_error, statusOf(e), e.what());
	}
}

// ---------------------------------------------------------------- the update mode

// meshopt_simplifyWithUpdate on host buffers. The vertex data goes to the device as one region
// when positions and attributes overlap (one interleaved buffer, as the reference's tests pass
// it) or as two, and comes back the same way after the write-back.
size_t updateHost(unsigned int* indices, size_t index_count, float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count, const unsigned char* vertex_lock,
    size_t target_index_count, float target_error, unsigned int options, float* result_error)
{
	std::string bad = checkArgs(index_count, vertex_positions_stride, target_index_count, target_error, vertex_attributes_stride, attribute_weights,
	    attribute_count, options);
	if (!bad.empty())
		return failHost(indices, indices, index_count, result_error,
		    (options & ~kSupportedOptions) ? meshoptgpu_StatusUnsupported : meshoptgpu_StatusInvalidArgument, bad);
	try
	{
		ThreadState& s = state();
		s.ensure();
		const size_t pbytes = stridedExtent(vertex_count, vertex_positions_stride, 12);
		const size_t abytes = attribute_count ? stridedExtent(vertex_count, vertex_attributes_stride, attribute_count * 4) : 0;
		const char* P = reinterpret_cast<const char*>(vertex_positions);
		const char* A = reinterpret_cast<const char*>(vertex_attributes);
		const bool joint = abytes && A < P + pbytes && P < A + abytes;
		const char* lo = joint ? std::min(P, A) : P;
		const size_t span = joint ? size_t(std::max(P + pbytes, A + abytes) - lo) : pbytes;
		size_t b_idx = align256(index_count * 4), b_v = align256(span), b_a = joint ? 0 : align256(abytes), b_lock = vertex_lock ? align256(vertex_count) : 0;
		char* base = static_cast<char*>(s.update_io.ensure(b_idx + b_v + b_a + b_lock + 256));
		unsigned int* d_idx = reinterpret_cast<unsigned int*>(base);
		char* d_v = base + b_idx;
		float* d_pos = reinterpret_cast<float*>(d_v + (P - lo));
		float* d_attr = abytes ? (joint ? reinterpret_cast<float*>(d_v + (A - lo)) : reinterpret_cast<float*>(base + b_idx + b_v)) : nullptr;
		unsigned char* d_lock = vertex_lock ? reinterpret_cast<unsigned char*>(base + b_idx + b_v + b_a) : nullptr;
		cudaStream_t st = s.stream;
		if (index_count)
			MO_CUDA_CHECK(cudaMemcpyAsync(d_idx, indices, index_count * 4, cudaMemcpyHostToDevice, st));
		if (span)
			MO_CUDA_CHECK(cudaMemcpyAsync(d_v, lo, span, cudaMemcpyHostToDevice, st));
		if (abytes && !joint)
			MO_CUDA_CHECK(cudaMemcpyAsync(d_attr, A, abytes, cudaMemcpyHostToDevice, st));
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
		m.options = options | kOptInternalSolve;
		m.update_positions = d_pos;
		m.update_attributes = d_attr;
		s.last = s.simplifier->run(m, d_idx, st, s.timing ? &s.times : nullptr);
		if (s.last.index_count)
			MO_CUDA_CHECK(cudaMemcpyAsync(indices, d_idx, s.last.index_count * 4, cudaMemcpyDeviceToHost, st));
		if (span)
			MO_CUDA_CHECK(cudaMemcpyAsync(const_cast<char*>(lo), d_v, span, cudaMemcpyDeviceToHost, st));
		if (abytes && !joint)
			MO_CUDA_CHECK(cudaMemcpyAsync(vertex_attributes, d_attr, abytes, cudaMemcpyDeviceToHost, st));
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		if (result_error)
			*result_error = s.last.result_error;
		setStatus(meshoptgpu_StatusOk, "");
		return s.last.index_count;
	}
	catch (const std::exception& e)
	{
		return failHost(indices, indices, index_count, result_error, statusOf(e), e.what());
	}
}

// ---------------------------------------------------------------- batched path

const size_t kBatchSmemDefault = 104 * 1024;    // shared-memory budget per CTA (two CTAs per SM)
const unsigned int kMeshletPoolDefault = 0;      // re-clusterization: all per-group arrays in global scratch
const size_t kBatchSlabTotal = size_t(16) << 30; // global slabs for meshes beyond the budget

struct BatchTuner
{
	std::mutex lock;
	std::map<int, std::pair<int, size_t>> shape; // size class -> fastest (threads per CTA, shared-memory budget per CTA)
} g_tuner;

// the shared-memory budgets the batch autotuner times (two, two and one CTAs of 256 threads per SM)
const size_t kBatchSmemBudgets[3] = {64 * 1024, kBatchSmemDefault, 160 * 1024};

int sizeClass(size_t max_index_count)
{
	int c = 0;
	while ((size_t(1) << c) < max_index_count)
		++c;
	return c;
}

// The used attributes (weight > 0, :2410-2421) of a batched mesh, deduplicated across the
// batch: meshes with the same weights share one map in device memory.
struct AttrMaps
{
	std::vector<BatchAttr> maps;
	std::map<std::string, int> index;

	// returns the map's index (or -1 when no attribute has a positive weight); ac = used count
	int add(const float* weights, size_t count, unsigned int& ac)
	{
		BatchAttr a;
		memset(&a, 0, sizeof(a));
		ac = 0;
		for (size_t k = 0; k < count; ++k)
			if (weights[k] > 0)
			{
				a.src[ac] = unsigned(k);
				a.weight[ac] = weights[k];
				ac++;
			}
		if (ac == 0)
			return -1;
		std::string key(reinterpret_cast<const char*>(&a), sizeof(a));
		auto it = index.find(key);
		if (it != index.end())
			return it->second;
		maps.push_back(a);
		index.emplace(key, int(maps.size()) - 1);
		return int(maps.size()) - 1;
	}
};

// The kernel descriptor of one batched mesh (device pointers); amap is patched by runBatch.
BatchDesc makeDesc(const meshoptgpu_BatchMesh& m, const unsigned int* indices, const float* positions, const float* attributes,
    const unsigned char* lock, unsigned int* out, AttrMaps& maps, int& attr_index)
{
	BatchDesc d{};
	d.indices = indices;
	d.positions = positions;
	d.out = out;
	d.index_count = unsigned(m.index_count);
	d.vertex_count = unsigned(m.vertex_count);
	d.stride_f = unsigned(m.vertex_positions_stride / 4);
	d.target_index_count = unsigned(m.target_index_count);
	d.target_error = m.target_error;
	d.options = m.options;
	d.lock = lock;
	unsigned int ac = 0;
	attr_index = m.attribute_count ? maps.add(m.attribute_weights, m.attribute_count, ac) : -1;
	d.attributes = ac ? attributes : nullptr;
	d.attr_stride_f = ac ? unsigned(m.vertex_attributes_stride / 4) : 0;
	d.ac = ac;
	d.amap = nullptr;
	return d;
}

// workspace of a batched mesh in shared memory (serial perform) and in a global slab (rounds)
size_t descWorkspace(const BatchDesc& d, bool rounds)
{
	return batchWorkspaceBytes(d.index_count, d.vertex_count, d.ac, (d.options & kOptSparse) != 0, rounds);
}

// Runs descs (device pointers) through the persistent kernel; results in the same order.
// attr_of[i] indexes maps.maps for descs[i] (-1: none).
void runBatch(ThreadState& s, std::vector<BatchDesc>& descs, const AttrMaps& maps, const std::vector<int>& attr_of, std::vector<BatchResult>& results,
    cudaStream_t st)
{
	const size_t n = descs.size();
	results.assign(n, BatchResult{0, 0.f, 0, 0});
	if (n == 0)
		return;
	// largest meshes first so the queue's tail is short; results are mapped back below
	std::vector<unsigned int> perm(n);
	std::iota(perm.begin(), perm.end(), 0u);
	std::stable_sort(perm.begin(), perm.end(), [&](unsigned int a, unsigned int b) { return descs[a].index_count > descs[b].index_count; });
	std::vector<BatchDesc> ordered(n);
	size_t maxidx = 0;
	for (size_t i = 0; i < n; ++i)
	{
		ordered[i] = descs[perm[i]];
		maxidx = std::max<size_t>(maxidx, ordered[i].index_count);
	}
	// a budget's dynamic shared memory (the largest mesh that fits it) and slab size (the largest
	// that does not): meshes whose workspace fits the launch's shared memory run there
	auto footprint = [&](size_t budget, unsigned int& smem, size_t& maxslab) {
		size_t maxfit = 0;
		maxslab = 0;
		for (const BatchDesc& d : ordered)
		{
			const size_t ws = descWorkspace(d, false);
			if (ws <= budget)
				maxfit = std::max(maxfit, ws);
			else
				maxslab = std::max(maxslab, descWorkspace(d, true));
		}
		smem = unsigned((maxfit + 15) & ~size_t(15));
	};
	const int sms = s.sms;

	// device metadata: descriptors, results, the ticket, the attribute maps; descriptors and
	// maps go up in one copy from pinned staging
	const size_t nm = maps.maps.size();
	const size_t off_res = align256(n * sizeof(BatchDesc)), off_ticket = off_res + align256(n * sizeof(BatchResult));
	const size_t off_maps = off_ticket + 256;
	size_t meta = off_maps + align256(nm * sizeof(BatchAttr));
	char* mbase = static_cast<char*>(s.batch_meta.ensure(meta));
	BatchDesc* d_descs = reinterpret_cast<BatchDesc*>(mbase);
	BatchResult* d_res = reinterpret_cast<BatchResult*>(mbase + off_res);
	unsigned int* d_ticket = reinterpret_cast<unsigned int*>(mbase + off_ticket);
	BatchAttr* d_maps = reinterpret_cast<BatchAttr*>(mbase + off_maps);
	for (size_t i = 0; i < n; ++i)
		ordered[i].amap = attr_of[perm[i]] >= 0 ? d_maps + attr_of[perm[i]] : nullptr;
	char* hmeta = static_cast<char*>(s.batch_meta_host.ensure(meta));
	memcpy(hmeta, ordered.data(), n * sizeof(BatchDesc));
	if (nm)
		memcpy(hmeta + off_maps, maps.maps.data(), nm * sizeof(BatchAttr));
	MO_CUDA_CHECK(cudaMemcpyAsync(d_descs, hmeta, n * sizeof(BatchDesc), cudaMemcpyHostToDevice, st));
	if (nm)
		MO_CUDA_CHECK(cudaMemcpyAsync(d_maps, hmeta + off_maps, nm * sizeof(BatchAttr), cudaMemcpyHostToDevice, st));

	bool full = false;
	for (const BatchDesc& d : ordered)
		full = full || batchNeedsFull(d);
	auto launch = [&](int threads, size_t budget) {
		unsigned int smem = 0;
		size_t maxslab = 0;
		footprint(budget, smem, maxslab);
		int per_sm = std::max(1, batchBlocksPerSM(threads, smem, full));
		unsigned int blocks = unsigned(std::min<size_t>(size_t(per_sm) * sms, n));
		if (maxslab)
			blocks = unsigned(std::max<size_t>(1, std::min<size_t>(blocks, kBatchSlabTotal / maxslab)));
		char* slabs = maxslab ? static_cast<char*>(s.batch_slabs.ensure(size_t(blocks) * maxslab)) : nullptr;
		launchBatch(d_descs, unsigned(n), d_ticket, d_res, slabs, maxslab, smem, blocks, threads, full, st);
	};

	int threads = s.batch_threads;
	size_t budget = s.batch_smem ? s.batch_smem : kBatchSmemDefault;
	if (threads == 0 || s.batch_smem == 0)
	{
		// the block size and the shared-memory budget the caller left open are autotuned per size
		// class: the first batch of a class times every candidate pair on its own meshes
		// (identical results) and keeps the fastest
		int cls = sizeClass(maxidx);
		bool known = false;
		{
			std::lock_guard<std::mutex> g(g_tuner.lock);
			auto it = g_tuner.shape.find(cls);
			if (it != g_tuner.shape.end())
			{
				threads = threads ? threads : it->second.first;
				budget = s.batch_smem ? budget : it->second.second;
				known = true;
			}
		}
		if (!known)
		{
			cudaEvent_t e0, e1;
			MO_CUDA_CHECK(cudaEventCreate(&e0));
			MO_CUDA_CHECK(cudaEventCreate(&e1));
			float best = 1e30f;
			int best_t = threads ? threads : 256;
			size_t best_b = budget;
			for (int t : {128, 256, 512})
			{
				if (threads && t != threads)
					continue;
				for (size_t b : kBatchSmemBudgets)
				{
					if (s.batch_smem && b != s.batch_smem)
						continue;
					MO_CUDA_CHECK(cudaEventRecord(e0, st));
					launch(t, b);
					MO_CUDA_CHECK(cudaEventRecord(e1, st));
					MO_CUDA_CHECK(cudaEventSynchronize(e1));
					float ms = 0;
					MO_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
					if (ms < best)
						best = ms, best_t = t, best_b = b;
				}
			}
			cudaEventDestroy(e0);
			cudaEventDestroy(e1);
			threads = best_t;
			budget = best_b;
			std::lock_guard<std::mutex> g(g_tuner.lock);
			g_tuner.shape[cls] = std::make_pair(threads, budget);
		}
	}
	launch(threads, budget);
	std::vector<BatchResult> tmp(n);
	MO_CUDA_CHECK(cudaMemcpyAsync(tmp.data(), d_res, n * sizeof(BatchResult), cudaMemcpyDeviceToHost, st));
	MO_CUDA_CHECK(cudaStreamSynchronize(st));
	probe().collect();
	for (size_t i = 0; i < n; ++i)
		results[perm[i]] = tmp[i];
}

// argument checks of a batched mesh: those of meshopt_simplifyEdge (:2348-2357), then the
// batch kernel's option set unless the mesh may take the single-mesh path
bool smallMeshOnBatch(ThreadState& s, const MeshDesc& m, unsigned int* d_out, cudaStream_t st)
{
	if (s.timing || m.index_count == 0 || (m.options & ~kBatchOptions) || m.vertex_count >= (size_t(1) << 32))
		return false;
	meshoptgpu_BatchMesh bm{};
	bm.index_count = m.index_count;
	bm.vertex_count = m.vertex_count;
	bm.vertex_positions_stride = m.positions_stride;
	bm.target_index_count = m.target_index_count;
	bm.target_error = m.target_error;
	bm.options = m.options;
	bm.vertex_attributes_stride = m.attributes_stride;
	bm.attribute_weights = m.weights;
	bm.attribute_count = m.attribute_count;
	AttrMaps maps;
	std::vector<int> attr_of(1);
	std::vector<BatchDesc> descs{makeDesc(bm, m.indices, m.positions, m.attributes, m.lock, d_out, maps, attr_of[0])};
	std::vector<BatchResult> res;
	runBatch(s, descs, maps, attr_of, res, st);
	if (res[0].status == 2)
		throw std::invalid_argument("index out of range of vertex_count");
	if (res[0].status == 3)
		throw std::runtime_error("collapse decision round made no progress");
	s.last = RunResult();
	s.last.index_count = res[0].index_count;
	s.last.result_error = res[0].result_error;
	return true;
}

// ---------------------------------------------------------------- autotuning of the single-mesh path
//
// Per size class of the mesh (its index count's bit length, and whether it has attributes), the
// first call that can be repeated (its destination does not alias its indices, no update mode,
// Prune or debug bit) times the candidates on the call's own mesh and keeps the fastest for the
// class; the results are identical whatever the choice, so the call returns the last candidate's.
// Later calls of the class take the choice. Tuned:
//  * the pass kernels' launch shape: pass-kernel blocks per SM (the resident maximum and one and
//    two fewer), then the pass sort's tile (4, 8 or 16 candidates per thread) at the best;
//  * the drop-in route for meshes between kDropinBatchAlways and kDropinSingleAlways indices: the
//    batch kernel (one CTA does the whole mesh) or the single-mesh path (multi-CTA pass loop).
constexpr size_t kTuneMinIndices = 3000;       // below: the default shape (nothing to gain)
constexpr size_t kDropinBatchAlways = 3000;    // up to here drop-in calls take the batch kernel
constexpr size_t kDropinSingleAlways = 98304;  // above here the single-mesh path
constexpr size_t kDropinDefault = 15000;       // the route of calls that cannot be timed

struct ShapeTuner
{
	std::mutex lock;
	std::map<std::tuple<int, int, int>, std::pair<int, unsigned int>> shape; // -> (blocks per SM, sort items)
	std::map<std::tuple<int, int, int>, bool> batch;                         // -> batch kernel faster
} g_shapes;

std::tuple<int, int, int> shapeKey(const ThreadState& s, const MeshDesc& m)
{
	return std::make_tuple(s.device, sizeClass(m.index_count), m.attribute_count ? 1 : 0);
}

bool repeatable(const ThreadState& s, const MeshDesc& m, const unsigned int* d_out)
{
	return s.autotune && !s.timing && static_cast<const void*>(d_out) != static_cast<const void*>(m.indices) &&
	       !(m.options & (kOptPrune | kOptInternalDebug | kOptInternalSolve)) && m.index_count > m.target_index_count;
}

float timedMs(cudaStream_t st, const std::function<void()>& f, int reps)
{
	cudaEvent_t e0, e1;
	MO_CUDA_CHECK(cudaEventCreate(&e0));
	MO_CUDA_CHECK(cudaEventCreate(&e1));
	float best = 1e30f;
	for (int r = 0; r < reps; ++r)
	{
		MO_CUDA_CHECK(cudaEventRecord(e0, st));
		f();
		MO_CUDA_CHECK(cudaEventRecord(e1, st));
		MO_CUDA_CHECK(cudaEventSynchronize(e1));
		float ms = 0;
		MO_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
		best = std::min(best, ms);
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return best;
}

// the single-mesh path with its size class's tuned launch shape (tuning it first if it has none)
void runSingle(ThreadState& s, const MeshDesc& m, unsigned int* d_out, cudaStream_t st)
{
	Simplifier& sp = *s.simplifier;
	if (!s.autotune)
	{
		s.last = sp.run(m, d_out, st, s.timing ? &s.times : nullptr);
		return;
	}
	const auto key = shapeKey(s, m);
	{
		std::lock_guard<std::mutex> g(g_shapes.lock);
		auto it = g_shapes.shape.find(key);
		if (it != g_shapes.shape.end())
		{
			sp.setPassShape(it->second.first, it->second.second);
			s.last = sp.run(m, d_out, st, s.timing ? &s.times : nullptr);
			return;
		}
	}
	const int top = std::max(1, sp.performBlocksPerSMMax());
	if (!repeatable(s, m, d_out) || m.index_count < kTuneMinIndices)
	{
		sp.setPassShape(top, 0);
		s.last = sp.run(m, d_out, st, s.timing ? &s.times : nullptr);
		return;
	}
	const int reps = 2; // the faster of two runs per candidate
	auto trial = [&](int bps, unsigned int items) {
		sp.setPassShape(bps, items);
		return timedMs(st, [&]() { s.last = sp.run(m, d_out, st); }, reps);
	};
	int best_bps = top;
	float best = 1e30f;
	for (int bps = top; bps >= std::max(1, top - 2); --bps)
	{
		const float ms = trial(bps, 0);
		if (ms < best)
			best = ms, best_bps = bps;
	}
	unsigned int best_items = 0;
	for (unsigned int items : {4u, 8u, 16u})
	{
		const float ms = trial(best_bps, items);
		if (ms < best)
			best = ms, best_items = items;
	}
	sp.setPassShape(best_bps, best_items);
	std::lock_guard<std::mutex> g(g_shapes.lock);
	g_shapes.shape[key] = std::make_pair(best_bps, best_items);
}

size_t singlePathAbove(const ThreadState& s)
{
	if (s.dropin_batch_limit != ~size_t(0))
		return s.dropin_batch_limit;
	return s.autotune ? kDropinSingleAlways : kDropinDefault;
}

void routeAndRun(ThreadState& s, const MeshDesc& m, unsigned int* d_out, cudaStream_t st, bool allow_batch)
{
	const bool batchable = allow_batch && !s.timing && m.index_count && !(m.options & ~kBatchOptions) && m.vertex_count < (size_t(1) << 32);
	if (!batchable)
	{
		runSingle(s, m, d_out, st);
		return;
	}
	if (s.dropin_batch_limit != ~size_t(0) || !s.autotune)
	{
		// a fixed limit: the caller's (meshoptgpu_setDropinBatchLimit), or the default
		const size_t limit = s.dropin_batch_limit != ~size_t(0) ? s.dropin_batch_limit : kDropinDefault;
		if (m.index_count > limit || !smallMeshOnBatch(s, m, d_out, st))
			runSingle(s, m, d_out, st);
		return;
	}
	if (m.index_count <= kDropinBatchAlways && smallMeshOnBatch(s, m, d_out, st))
		return;
	if (m.index_count > kDropinSingleAlways)
	{
		runSingle(s, m, d_out, st);
		return;
	}
	const auto key = shapeKey(s, m);
	int route = -1; // 1: batch kernel, 0: single-mesh path
	{
		std::lock_guard<std::mutex> g(g_shapes.lock);
		auto it = g_shapes.batch.find(key);
		if (it != g_shapes.batch.end())
			route = it->second ? 1 : 0;
	}
	if (route < 0 && !repeatable(s, m, d_out))
		route = m.index_count <= kDropinDefault ? 1 : 0;
	if (route < 0)
	{
		// each route once untimed (its own first-call tuning), then each timed
		smallMeshOnBatch(s, m, d_out, st);
		runSingle(s, m, d_out, st);
		const float tb = timedMs(st, [&]() { smallMeshOnBatch(s, m, d_out, st); }, 2);
		const float ts = timedMs(st, [&]() { runSingle(s, m, d_out, st); }, 2);
		std::lock_guard<std::mutex> g(g_shapes.lock);
		g_shapes.batch[key] = tb < ts;
		return; // d_out and s.last hold the single-mesh path's result, identical to the batch kernel's
	}
	if (route == 1 && smallMeshOnBatch(s, m, d_out, st))
		return;
	runSingle(s, m, d_out, st);
}

std::string checkBatchMesh(const meshoptgpu_BatchMesh& m, bool any_option = false)
{
	if (m.attribute_count && (!m.vertex_attributes || !m.attribute_weights))
		return "vertex_attributes and attribute_weights are required when attribute_count > 0";
	std::string bad = checkArgs(m.index_count, m.vertex_positions_stride, m.target_index_count, m.target_error, m.vertex_attributes_stride,
	    m.attribute_weights, m.attribute_count, m.options);
	if (!bad.empty())
		return bad;
	if (!any_option && (m.options & ~kBatchOptions))
		return "batched meshes support every option but Prune and InternalDebug";
	if (m.index_count >= (size_t(1) << 32) || m.vertex_count >= (size_t(1) << 32))
		return "batched meshes must have fewer than 2^32 indices and vertices";
	return std::string();
}

int batchCheckStatus(const meshoptgpu_BatchMesh& m, bool any_option = false)
{
	return (m.options & ~(any_option ? kSupportedOptions : kBatchOptions)) ? meshoptgpu_StatusUnsupported : meshoptgpu_StatusInvalidArgument;
}

int finishBatch(const std::vector<BatchResult>& res, size_t* counts, float* errors)
{
	int status = meshoptgpu_StatusOk;
	for (size_t i = 0; i < res.size(); ++i)
	{
		if (counts)
			counts[i] = res[i].index_count;
		if (errors)
			errors[i] = res[i].result_error;
		if (res[i].status)
			status = res[i].status == 3 ? meshoptgpu_StatusCudaError : meshoptgpu_StatusInvalidArgument;
	}
	if (status == meshoptgpu_StatusInvalidArgument)
		setStatus(status, "a batched mesh has an index out of range of its vertex_count");
	else if (status != meshoptgpu_StatusOk)
		setStatus(status, "a batched mesh's decision round made no progress");
	else
		setStatus(meshoptgpu_StatusOk, "");
	return status;
}

// ---------------------------------------------------------------- serving

struct ServerRequest
{
	BatchDesc desc;
	std::vector<float> weights; // attribute weights, copied at submission
	size_t index_count = 0, vertex_count = 0;
	size_t reserve = 0;
	std::chrono::steady_clock::time_point submitted, completed;
	bool done = false;
	int status = meshoptgpu_StatusOk;
	size_t result_count = 0;
	float result_error = 0.f;
};

struct ServerImpl
{
	meshoptgpu_ServerConfig cfg;
	int device = 0;
	int sms = 1;
	std::mutex m;
	std::condition_variable cv_work, cv_done;
	std::deque<ServerRequest*> small_q, large_q;
	std::vector<std::unique_ptr<ServerRequest>> reqs; // index = ticket
	size_t reserved = 0, peak_reserved = 0;
	unsigned long long completed = 0, batches = 0, singles = 0, inflight = 0, peak_inflight = 0;
	bool stop = false;
	std::vector<std::thread> threads;
};

const size_t kServerBudgetDefault = size_t(40) << 30;

// device bytes a request holds while it runs on the batch path (its global slab; meshes that
// fit shared memory hold none) or on the single-mesh path (its arena)
size_t batchReserve(const ServerRequest& r)
{
	return descWorkspace(r.desc, false) <= kBatchSmemDefault ? 4096 : descWorkspace(r.desc, true);
}

void publish(ServerImpl& S, std::vector<ServerRequest*>& done_reqs, size_t release)
{
	std::lock_guard<std::mutex> g(S.m);
	auto now = std::chrono::steady_clock::now();
	for (ServerRequest* r : done_reqs)
	{
		r->done = true;
		r->completed = now;
	}
	S.completed += done_reqs.size();
	S.inflight -= done_reqs.size();
	S.reserved -= release;
	S.cv_done.notify_all();
	S.cv_work.notify_all();
}

void batchWorker(ServerImpl* S)
{
	cudaSetDevice(S->device);
	ThreadState& ts = state();
	ts.batch_threads = S->cfg.batch_threads;
	for (;;)
	{
		std::vector<ServerRequest*> take;
		size_t reserve = 0;
		{
			std::unique_lock<std::mutex> lk(S->m);
			S->cv_work.wait(lk, [&] {
				if (S->stop)
					return true;
				return !S->small_q.empty() && S->reserved + batchReserve(*S->small_q.front()) <= S->cfg.memory_budget;
			});
			if (S->stop && S->small_q.empty())
				return;
			// continuous batching: everything that arrived since this worker last launched, in
			// arrival order, while the memory budget and the batch limit allow
			size_t maxslab = 0;
			while (!S->small_q.empty() && take.size() < size_t(S->cfg.max_batch))
			{
				ServerRequest* r = S->small_q.front();
				size_t slab = batchReserve(*r) > 4096 ? batchReserve(*r) : 0;
				size_t nm = std::max(maxslab, slab);
				size_t blocks = std::min<size_t>(take.size() + 1, size_t(S->sms) * 4);
				size_t need = blocks * nm + 4096 * (take.size() + 1);
				if (S->reserved + need > S->cfg.memory_budget && !take.empty())
					break;
				maxslab = nm;
				reserve = need;
				take.push_back(r);
				S->small_q.pop_front();
			}
			S->reserved += reserve;
			S->peak_reserved = std::max(S->peak_reserved, S->reserved);
			S->inflight += take.size();
			S->peak_inflight = std::max(S->peak_inflight, S->inflight);
			S->batches++;
		}
		std::vector<BatchDesc> descs(take.size());
		std::vector<int> attr_of(take.size(), -1);
		AttrMaps maps;
		for (size_t i = 0; i < take.size(); ++i)
		{
			descs[i] = take[i]->desc;
			unsigned int ac = 0;
			if (!take[i]->weights.empty())
				attr_of[i] = maps.add(take[i]->weights.data(), take[i]->weights.size(), ac);
		}
		std::vector<BatchResult> res;
		try
		{
			ts.ensure();
			runBatch(ts, descs, maps, attr_of, res, ts.stream);
			for (size_t i = 0; i < take.size(); ++i)
			{
				take[i]->result_count = res[i].index_count;
				take[i]->result_error = res[i].result_error;
				take[i]->status = res[i].status ? meshoptgpu_StatusInvalidArgument : meshoptgpu_StatusOk;
			}
		}
		catch (const std::exception& e)
		{
			for (ServerRequest* r : take)
				r->status = statusOf(e);
			fprintf(stderr, "meshopt_gb300: server batch failed: %s\n", e.what());
		}
		publish(*S, take, reserve);
	}
}

void largeWorker(ServerImpl* S)
{
	cudaSetDevice(S->device);
	ThreadState& ts = state();
	try
	{
		ts.ensure();
		Tuning t = ts.simplifier->tuning();
		t.perform_grid_cap = S->cfg.perform_blocks;
		// requests come in every shape, so a recorded pass graph is never replayed for a second
		// request, and concurrent workers instantiating graphs contend in the driver: the
		// single-mesh workers drive their pass loops from the host
		t.device_loop = false;
		ts.simplifier->setTuning(t);
	}
	catch (const std::exception& e)
	{
		fprintf(stderr, "meshopt_gb300: server worker setup failed: %s\n", e.what());
	}
	for (;;)
	{
		ServerRequest* r = nullptr;
		{
			std::unique_lock<std::mutex> lk(S->m);
			S->cv_work.wait(lk, [&] {
				if (S->stop)
					return true;
				return !S->large_q.empty() && S->reserved + S->large_q.front()->reserve <= S->cfg.memory_budget;
			});
			if (S->stop && S->large_q.empty())
				return;
			r = S->large_q.front();
			S->large_q.pop_front();
			S->reserved += r->reserve;
			S->peak_reserved = std::max(S->peak_reserved, S->reserved);
			S->inflight++;
			S->peak_inflight = std::max(S->peak_inflight, S->inflight);
			S->singles++;
		}
		try
		{
			ts.ensure();
			MeshDesc m;
			m.indices = r->desc.indices;
			m.index_count = r->index_count;
			m.positions = r->desc.positions;
			m.vertex_count = r->vertex_count;
			m.positions_stride = size_t(r->desc.stride_f) * 4;
			m.target_index_count = r->desc.target_index_count;
			m.target_error = r->desc.target_error;
			m.options = r->desc.options;
			m.lock = r->desc.lock;
			if (!r->weights.empty())
			{
				m.attributes = r->desc.attributes;
				m.attributes_stride = size_t(r->desc.attr_stride_f) * 4;
				m.weights = r->weights.data();
				m.attribute_count = r->weights.size();
			}
			RunResult rr = ts.simplifier->run(m, r->desc.out, ts.stream);
			r->result_count = rr.index_count;
			r->result_error = rr.result_error;
			r->status = meshoptgpu_StatusOk;
		}
		catch (const std::exception& e)
		{
			r->status = statusOf(e);
			fprintf(stderr, "meshopt_gb300: server request failed: %s\n", e.what());
		}
		std::vector<ServerRequest*> one{r};
		publish(*S, one, r->reserve);
	}
}

} // namespace

extern "C" {

size_t meshopt_simplifyWithUpdate(unsigned int* indices, size_t index_count, float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count, const unsigned char* vertex_lock,
    size_t target_index_count, float target_error, unsigned int options, float* result_error)
{
	return updateHost(indices, index_count, vertex_positions, vertex_count, vertex_positions_stride, vertex_attributes, vertex_attributes_stride,
	    attribute_weights, attribute_count, vertex_lock, target_index_count, target_error, options, result_error);
}

size_t meshoptgpu_simplifyWithUpdateDevice(unsigned int* indices, size_t index_count, float* vertex_positions, size_t vertex_count,
    size_t vertex_positions_stride, float* vertex_attributes, size_t vertex_attributes_stride, const float* attribute_weights, size_t attribute_count,
    const unsigned char* vertex_lock, size_t target_index_count, float target_error, unsigned int options, float* result_error, void* stream)
{
	std::string bad = checkArgs(index_count, vertex_positions_stride, target_index_count, target_error, vertex_attributes_stride, attribute_weights,
	    attribute_count, options);
	if (!bad.empty())
	{
		setStatus((options & ~kSupportedOptions) ? meshoptgpu_StatusUnsupported : meshoptgpu_StatusInvalidArgument, bad);
		if (result_error)
			*result_error = 0.f;
		return index_count;
	}
	try
	{
		ThreadState& s = state();
		s.ensure();
		cudaStream_t st = static_cast<cudaStream_t>(stream);
		MeshDesc m;
		m.indices = indices;
		m.index_count = index_count;
		m.positions = vertex_positions;
		m.vertex_count = vertex_count;
		m.positions_stride = vertex_positions_stride;
		m.attributes = attribute_count ? vertex_attributes : nullptr;
		m.attributes_stride = vertex_attributes_stride;
		m.weights = attribute_weights;
		m.attribute_count = attribute_count;
		m.lock = vertex_lock;
		m.target_index_count = target_index_count;
		m.target_error = target_error;
		m.options = options | kOptInternalSolve;
		m.update_positions = vertex_positions;
		m.update_attributes = attribute_count ? vertex_attributes : nullptr;
		s.last = s.simplifier->run(m, indices, st, s.timing ? &s.times : nullptr);
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		if (result_error)
			*result_error = s.last.result_error;
		setStatus(meshoptgpu_StatusOk, "");
		return s.last.index_count;
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		if (result_error)
			*result_error = 0.f;
		return index_count;
	}
}

int meshoptgpu_simplifyBatch(const meshoptgpu_BatchMesh* meshes, size_t mesh_count, size_t* result_index_counts, float* result_errors, void* stream)
{
	for (size_t i = 0; i < mesh_count; ++i)
	{
		std::string bad = checkBatchMesh(meshes[i]);
		if (!bad.empty())
		{
			int st = batchCheckStatus(meshes[i]);
			setStatus(st, "mesh " + std::to_string(i) + ": " + bad);
			return st;
		}
	}
	try
	{
		ThreadState& s = state();
		s.ensure();
		std::vector<BatchDesc> descs(mesh_count);
		std::vector<int> attr_of(mesh_count);
		AttrMaps maps;
		for (size_t i = 0; i < mesh_count; ++i)
		{
			const meshoptgpu_BatchMesh& m = meshes[i];
			descs[i] = makeDesc(m, m.indices, m.vertex_positions, m.vertex_attributes, m.vertex_lock, m.destination, maps, attr_of[i]);
		}
		std::vector<BatchResult> res;
		runBatch(s, descs, maps, attr_of, res, static_cast<cudaStream_t>(stream));
		return finishBatch(res, result_index_counts, result_errors);
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return statusOf(e);
	}
}

int meshoptgpu_simplifyBatchHost(const meshoptgpu_BatchMesh* meshes, size_t mesh_count, size_t* result_index_counts, float* result_errors)
{
	for (size_t i = 0; i < mesh_count; ++i)
	{
		std::string bad = checkBatchMesh(meshes[i]);
		if (!bad.empty())
		{
			int st = batchCheckStatus(meshes[i]);
			setStatus(st, "mesh " + std::to_string(i) + ": " + bad);
			return st;
		}
	}
	try
	{
		ThreadState& s = state();
		s.ensure();
		// pack inputs into one pinned buffer (16-byte aligned pieces): per mesh its indices, and
		// every distinct vertex, attribute and lock array once (meshes of a sparse group share
		// them); outputs follow all inputs on the device
		size_t in_bytes = 0, out_words = 0;
		PieceTable shared(3 * mesh_count);
		std::vector<std::pair<const void*, size_t>> pieces; // (source, bytes) in pack order
		pieces.reserve(2 * mesh_count);
		auto place = [&](const void* p, size_t bytes, bool dedupe) -> size_t {
			if (!p || !bytes)
				return ~size_t(0);
			const size_t at = in_bytes;
			if (dedupe)
			{
				const size_t seen = shared.findOrInsert(p, bytes, at);
				if (seen != ~size_t(0))
					return seen;
			}
			in_bytes = (in_bytes + bytes + 15) & ~size_t(15);
			pieces.push_back({p, bytes});
			return at;
		};
		std::vector<size_t> off_idx(mesh_count), off_pos(mesh_count), off_attr(mesh_count), off_lock(mesh_count), off_out(mesh_count);
		for (size_t i = 0; i < mesh_count; ++i)
		{
			const meshoptgpu_BatchMesh& m = meshes[i];
			off_idx[i] = place(m.indices, m.index_count * 4, false);
			off_pos[i] = place(m.vertex_positions, stridedExtent(m.vertex_count, m.vertex_positions_stride, 12), true);
			off_attr[i] = m.attribute_count ? place(m.vertex_attributes, stridedExtent(m.vertex_count, m.vertex_attributes_stride, m.attribute_count * 4), true)
			                                : ~size_t(0);
			off_lock[i] = place(m.vertex_lock, m.vertex_count, true);
			off_out[i] = out_words;
			out_words += m.index_count;
		}
		char* h = static_cast<char*>(s.batch_host.ensure(in_bytes + 16));
		char* d = static_cast<char*>(s.batch_io.ensure(align256(in_bytes) + out_words * 4 + 256));
		unsigned int* d_out = reinterpret_cast<unsigned int*>(d + align256(in_bytes));
		cudaStream_t st = s.stream;
		{
			// packed and uploaded in chunks of about a quarter of the bytes (4 MiB at least): the
			// upload of one chunk runs while the next one is packed
			std::vector<HostCopy> copies;
			copies.reserve(pieces.size());
			size_t at = 0;
			for (auto& pc : pieces)
			{
				copies.push_back(HostCopy{h + at, pc.first, pc.second});
				at = (at + pc.second + 15) & ~size_t(15);
			}
			const size_t chunk = std::max<size_t>(size_t(4) << 20, in_bytes / 4);
			for (size_t b = 0; b < copies.size();)
			{
				size_t e = b, bytes = 0;
				while (e < copies.size() && (e == b || bytes < chunk))
					bytes += copies[e++].bytes;
				parallelCopies(copies.data() + b, e - b);
				const size_t lo = static_cast<size_t>(static_cast<char*>(copies[b].dst) - h);
				const size_t hi = e < copies.size() ? static_cast<size_t>(static_cast<char*>(copies[e].dst) - h) : in_bytes;
				MO_CUDA_CHECK(cudaMemcpyAsync(d + lo, h + lo, hi - lo, cudaMemcpyHostToDevice, st));
				b = e;
			}
		}
		std::vector<BatchDesc> descs(mesh_count);
		std::vector<int> attr_of(mesh_count);
		AttrMaps maps;
		auto at = [&](size_t off) { return off == ~size_t(0) ? nullptr : d + off; };
		for (size_t i = 0; i < mesh_count; ++i)
			descs[i] = makeDesc(meshes[i], reinterpret_cast<const unsigned int*>(at(off_idx[i])), reinterpret_cast<const float*>(at(off_pos[i])),
			    reinterpret_cast<const float*>(at(off_attr[i])), reinterpret_cast<const unsigned char*>(at(off_lock[i])), d_out + off_out[i], maps,
			    attr_of[i]);
		std::vector<BatchResult> res;
		runBatch(s, descs, maps, attr_of, res, st);
		// results back in one copy (the packed outputs), then scattered to the callers' buffers
		unsigned int* hout = static_cast<unsigned int*>(s.batch_host.ensure(std::max(in_bytes + 16, out_words * 4 + 16)));
		MO_CUDA_CHECK(cudaMemcpyAsync(hout, d_out, out_words * 4, cudaMemcpyDeviceToHost, st));
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		std::vector<HostCopy> copies(mesh_count);
		for (size_t i = 0; i < mesh_count; ++i)
			copies[i] = HostCopy{meshes[i].destination, hout + off_out[i], size_t(res[i].index_count) * 4};
		parallelCopies(copies);
		return finishBatch(res, result_index_counts, result_errors);
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return statusOf(e);
	}
}

int meshoptgpu_simplifyGroups(unsigned int* destination, const unsigned int* indices, const size_t* group_offsets, size_t group_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride, const float* vertex_attributes, size_t vertex_attributes_stride,
    const float* attribute_weights, size_t attribute_count, const unsigned int* position_remap, unsigned char* locks, const unsigned char* vertex_lock,
    const size_t* target_index_counts, float target_error, unsigned int options, size_t* result_index_counts, float* result_errors, void* stream)
{
	if (!position_remap || !locks || (group_count && (!group_offsets || !target_index_counts)))
	{
		setStatus(meshoptgpu_StatusInvalidArgument, "position_remap, locks, group_offsets and target_index_counts are required");
		return meshoptgpu_StatusInvalidArgument;
	}
	std::vector<meshoptgpu_BatchMesh> meshes(group_count);
	for (size_t g = 0; g < group_count; ++g)
	{
		meshoptgpu_BatchMesh& m = meshes[g];
		m = meshoptgpu_BatchMesh{};
		if (group_offsets[g + 1] < group_offsets[g])
		{
			setStatus(meshoptgpu_StatusInvalidArgument, "group_offsets must not decrease");
			return meshoptgpu_StatusInvalidArgument;
		}
		m.indices = indices + group_offsets[g];
		m.index_count = group_offsets[g + 1] - group_offsets[g];
		m.vertex_positions = vertex_positions;
		m.vertex_count = vertex_count;
		m.vertex_positions_stride = vertex_positions_stride;
		m.target_index_count = target_index_counts[g];
		m.target_error = target_error;
		m.options = options | kOptSparse;
		m.destination = destination + group_offsets[g];
		m.vertex_attributes = vertex_attributes;
		m.vertex_attributes_stride = vertex_attributes_stride;
		m.attribute_weights = attribute_weights;
		m.attribute_count = attribute_count;
		m.vertex_lock = locks;
		std::string bad = checkBatchMesh(m);
		if (!bad.empty())
		{
			int st = batchCheckStatus(m);
			setStatus(st, "group " + std::to_string(g) + ": " + bad);
			return st;
		}
	}
	try
	{
		ThreadState& s = state();
		s.ensure();
		cudaStream_t st = static_cast<cudaStream_t>(stream);
		// offsets (device, 64-bit), the claim tables, the error word
		const size_t lock_bytes = groupLockScratchBytes(vertex_count, group_count);
		char* base = static_cast<char*>(s.group_scratch.ensure(lock_bytes + (group_count + 1) * 8 + 512));
		unsigned long long* d_off = reinterpret_cast<unsigned long long*>(base + lock_bytes);
		unsigned int* d_bad = reinterpret_cast<unsigned int*>(base + lock_bytes + ((group_count + 1) * 8 + 255) / 256 * 256);
		std::vector<unsigned long long> off(group_offsets, group_offsets + group_count + 1);
		unsigned long long* h_off = static_cast<unsigned long long*>(s.batch_host.ensure(off.size() * 8));
		memcpy(h_off, off.data(), off.size() * 8);
		MO_CUDA_CHECK(cudaMemcpyAsync(d_off, h_off, off.size() * 8, cudaMemcpyHostToDevice, st));
		groupLocks(locks, indices, d_off, group_count, position_remap, vertex_lock, vertex_count, base, d_bad, st);
		std::vector<BatchDesc> descs(group_count);
		std::vector<int> attr_of(group_count);
		AttrMaps maps;
		for (size_t g = 0; g < group_count; ++g)
		{
			const meshoptgpu_BatchMesh& m = meshes[g];
			descs[g] = makeDesc(m, m.indices, m.vertex_positions, m.vertex_attributes, m.vertex_lock, m.destination, maps, attr_of[g]);
		}
		std::vector<BatchResult> res;
		runBatch(s, descs, maps, attr_of, res, st);
		unsigned int hbad = 0;
		MO_CUDA_CHECK(cudaMemcpyAsync(h_off, d_bad, 4, cudaMemcpyDeviceToHost, st));
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		memcpy(&hbad, h_off, 4);
		if (hbad)
		{
			setStatus(meshoptgpu_StatusInvalidArgument, "an index or a position_remap entry is out of range of vertex_count");
			return meshoptgpu_StatusInvalidArgument;
		}
		return finishBatch(res, result_index_counts, result_errors);
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return statusOf(e);
	}
}

// shared memory per warp of the re-clusterization kernel (MESHOPTGPU_MESHLET_POOL bytes, at
// most 48 KiB; default below)
static unsigned int meshletPoolBytes()
{
	static const unsigned int bytes = [] {
		const char* v = getenv("MESHOPTGPU_MESHLET_POOL");
		long n = v ? atol(v) : long(kMeshletPoolDefault);
		return unsigned(std::min(std::max(n, 0L), 48L * 1024) & ~15L);
	}();
	return bytes;
}

int meshoptgpu_buildMeshletsFlexGroups(unsigned int* meshlets, unsigned int* meshlet_vertices, unsigned char* meshlet_triangles,
    const size_t* meshlet_offsets, size_t* meshlet_counts, const unsigned int* indices, const size_t* group_offsets, size_t group_count,
    const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride, size_t max_vertices, size_t min_triangles, size_t max_triangles,
    float cone_weight, float split_factor, int optimize_level, void* stream)
{
	// the reference's argument checks (src/clusterizer.cpp:1039-1049), as errors
	std::string bad;
	if (group_count && (!group_offsets || !meshlet_offsets || !meshlet_counts))
		bad = "group_offsets, meshlet_offsets and meshlet_counts are required";
	else if (vertex_positions_stride < 12 || vertex_positions_stride > 256 || vertex_positions_stride % 4)
		bad = "vertex_positions_stride must be 12..256 and a multiple of 4";
	else if (max_vertices < 3 || max_vertices > 256)
		bad = "max_vertices must be 3..256";
	else if (min_triangles < 1 || min_triangles > max_triangles || max_triangles > 512)
		bad = "need 1 <= min_triangles <= max_triangles <= 512";
	else if (!(cone_weight >= 0.f && cone_weight <= 1.f))
		bad = "cone_weight must be in [0, 1]";
	else if (!(split_factor >= 0.f))
		bad = "split_factor must be >= 0";
	else if (vertex_count >= (size_t(1) << 32))
		bad = "vertex_count must be below 2^32";
	else if (optimize_level < -1 || optimize_level > 9)
		bad = "optimize_level must be -1 (none) or 0..9";
	for (size_t g = 0; bad.empty() && g < group_count; ++g)
	{
		const size_t n = group_offsets[g + 1] - group_offsets[g];
		if (group_offsets[g + 1] < group_offsets[g] || n % 3)
			bad = "group " + std::to_string(g) + ": index counts must be multiples of 3 and offsets must not decrease";
		else if (meshlet_offsets[g + 1] < meshlet_offsets[g] || meshlet_offsets[g + 1] - meshlet_offsets[g] < meshletBound(n, max_vertices, min_triangles))
			bad = "group " + std::to_string(g) + ": fewer meshlet rows than meshopt_buildMeshletsBound(index_count, max_vertices, min_triangles)";
		else if (n >= (size_t(1) << 31))
			bad = "group " + std::to_string(g) + ": index count must be below 2^31";
	}
	if (!bad.empty())
	{
		setStatus(meshoptgpu_StatusInvalidArgument, bad);
		return meshoptgpu_StatusInvalidArgument;
	}
	if (!group_count)
	{
		setStatus(meshoptgpu_StatusOk, "");
		return meshoptgpu_StatusOk;
	}
	try
	{
		ThreadState& s = state();
		s.ensure();
		cudaStream_t st = static_cast<cudaStream_t>(stream);
		// per group: index offsets, meshlet rows, scratch offsets (64-bit, device); counts and the error word
		const size_t G = group_count;
		std::vector<unsigned long long> host((G + 1) * 3, 0);
		unsigned long long scratch = 0;
		for (size_t g = 0; g <= G; ++g)
		{
			host[g] = group_offsets[g];
			host[(G + 1) + g] = meshlet_offsets[g];
			host[2 * (G + 1) + g] = scratch;
			if (g < G)
				scratch += meshletScratchBytes(group_offsets[g + 1] - group_offsets[g]);
		}
		const size_t meta = ((host.size() * 8 + 255) / 256) * 256, words = ((G + 1) * 4 + 255) / 256 * 256;
		char* base = static_cast<char*>(s.meshlet_scratch.ensure(meta + words + scratch + 256));
		unsigned long long* d_meta = reinterpret_cast<unsigned long long*>(base);
		unsigned int* d_counts = reinterpret_cast<unsigned int*>(base + meta);
		unsigned int* d_err = d_counts + G;
		char* d_scratch = base + meta + words;
		void* h = s.batch_host.ensure(host.size() * 8 + (G + 1) * 4);
		memcpy(h, host.data(), host.size() * 8);
		MO_CUDA_CHECK(cudaMemcpyAsync(d_meta, h, host.size() * 8, cudaMemcpyHostToDevice, st));
		MO_CUDA_CHECK(cudaMemsetAsync(d_err, 0, 4, st));
		MeshletBatch b;
		b.indices = indices;
		b.offsets = d_meta;
		b.groups = unsigned(G);
		b.positions = vertex_positions;
		b.stride_f = unsigned(vertex_positions_stride / 4);
		b.vertex_count = unsigned(vertex_count);
		b.max_vertices = unsigned(max_vertices);
		b.min_triangles = unsigned(min_triangles);
		b.max_triangles = unsigned(max_triangles);
		b.cone_weight = cone_weight;
		b.split_factor = split_factor;
		b.meshlets = meshlets;
		b.meshlet_base = d_meta + (G + 1);
		b.mverts = meshlet_vertices;
		b.mtris = meshlet_triangles;
		b.counts = d_counts;
		b.scratch = d_scratch;
		b.scratch_off = d_meta + 2 * (G + 1);
		b.error = d_err;
		b.pool_bytes = meshletPoolBytes();
		b.optimize_level = optimize_level;
		b.rows = meshlet_offsets[G];
		buildMeshletsBatch(b, st);
		unsigned int* hc = reinterpret_cast<unsigned int*>(static_cast<char*>(h) + host.size() * 8);
		MO_CUDA_CHECK(cudaMemcpyAsync(hc, d_counts, (G + 1) * 4, cudaMemcpyDeviceToHost, st));
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		if (hc[G] & 1u)
		{
			setStatus(meshoptgpu_StatusInvalidArgument, "an index is out of range of vertex_count");
			return meshoptgpu_StatusInvalidArgument;
		}
		if (hc[G])
		{
			setStatus(meshoptgpu_StatusInternal, "meshlet construction exceeded a bound it keeps (tree depth or output size)");
			return meshoptgpu_StatusInternal;
		}
		for (size_t g = 0; g < G; ++g)
			meshlet_counts[g] = hc[g];
		setStatus(meshoptgpu_StatusOk, "");
		return meshoptgpu_StatusOk;
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return statusOf(e);
	}
}

size_t meshoptgpu_optimizeVertexFetchRemapDevice(unsigned int* destination, const unsigned int* indices, size_t index_count, size_t vertex_count,
    void* stream)
{
	try
	{
		if (vertex_count && !destination)
			throw std::invalid_argument("destination is required");
		if (vertex_count >= (size_t(1) << 32) || index_count >= (size_t(1) << 32))
			throw std::invalid_argument("counts must be below 2^32");
		ThreadState& s = state();
		cudaStream_t st = static_cast<cudaStream_t>(stream);
		unsigned int* scratch = static_cast<unsigned int*>(s.compact_scratch.ensure((vertexOrderScratchWords(index_count, vertex_count) + 64) * 4));
		unsigned int* counters = scratch + vertexOrderScratchWords(index_count, vertex_count);
		vertexOrder(destination, indices, index_count, vertex_count, scratch, counters, st);
		unsigned int h[2];
		MO_CUDA_CHECK(cudaMemcpyAsync(h, counters, sizeof(h), cudaMemcpyDeviceToHost, st));
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		probe().collect();
		if (h[1])
			throw std::invalid_argument("an index is out of range of vertex_count");
		setStatus(meshoptgpu_StatusOk, "");
		return h[0];
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return 0;
	}
}

size_t meshoptgpu_optimizeVertexFetchDevice(void* destination, unsigned int* indices, size_t index_count, const void* vertices, size_t vertex_count,
    size_t vertex_size, void* stream)
{
	try
	{
		if (vertex_size == 0 || vertex_size > 256)
			throw std::invalid_argument("vertex_size must be in [1, 256]");
		if (vertex_count >= (size_t(1) << 32) || index_count >= (size_t(1) << 32))
			throw std::invalid_argument("counts must be below 2^32");
		ThreadState& s = state();
		cudaStream_t st = static_cast<cudaStream_t>(stream);
		// scratch: the order table, the vertex-order scratch, counters, and for an in-place call
		// a copy of the vertices
		const size_t ow = (vertex_count + 63) & ~size_t(63), sw = vertexOrderScratchWords(index_count, vertex_count);
		const size_t copy_bytes = destination == vertices ? vertex_count * vertex_size : 0;
		char* base = static_cast<char*>(s.compact_scratch.ensure((ow + sw + 64) * 4 + copy_bytes + 256));
		unsigned int* order = reinterpret_cast<unsigned int*>(base);
		unsigned int* scratch = order + ow;
		unsigned int* counters = scratch + sw;
		const void* src = vertices;
		if (copy_bytes)
		{
			void* copy = base + (ow + sw + 64) * 4;
			MO_CUDA_CHECK(cudaMemcpyAsync(copy, vertices, copy_bytes, cudaMemcpyDeviceToDevice, st));
			src = copy;
		}
		vertexOrder(order, indices, index_count, vertex_count, scratch, counters, st);
		unsigned int h[2];
		MO_CUDA_CHECK(cudaMemcpyAsync(h, counters, sizeof(h), cudaMemcpyDeviceToHost, st));
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		if (h[1])
		{
			probe().collect();
			throw std::invalid_argument("an index is out of range of vertex_count");
		}
		moveVertices(destination, src, vertex_count, vertex_size, order, st);
		rewriteIndices(indices, index_count, order, st);
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		probe().collect();
		setStatus(meshoptgpu_StatusOk, "");
		return h[0];
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return 0;
	}
}

int meshoptgpu_generatePositionRemapDevice(unsigned int* destination, const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride,
    void* stream)
{
	try
	{
		if (vertex_positions_stride < 12 || vertex_positions_stride > 256 || vertex_positions_stride % 4 != 0)
			throw std::invalid_argument("vertex_positions_stride must be in [12, 256] and a multiple of 4");
		if (vertex_count >= (size_t(1) << 32))
			throw std::invalid_argument("vertex_count must be below 2^32");
		ThreadState& s = state();
		cudaStream_t st = static_cast<cudaStream_t>(stream);
		const size_t sw = positionRemapScratchWords(vertex_count);
		unsigned int* scratch = static_cast<unsigned int*>(s.compact_scratch.ensure((sw + 64) * 4));
		unsigned int* counters = scratch + sw;
		positionRemap(destination, vertex_positions, vertex_count, vertex_positions_stride / 4, scratch, counters, st);
		unsigned int h[2];
		MO_CUDA_CHECK(cudaMemcpyAsync(h, counters, sizeof(h), cudaMemcpyDeviceToHost, st));
		MO_CUDA_CHECK(cudaStreamSynchronize(st));
		probe().collect();
		if (h[1])
			throw std::runtime_error("position table overflow");
		setStatus(meshoptgpu_StatusOk, "");
		return meshoptgpu_StatusOk;
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return statusOf(e);
	}
}

meshoptgpu_Server* meshoptgpu_serverCreate(const meshoptgpu_ServerConfig* config)
{
	try
	{
		std::unique_ptr<ServerImpl> S(new ServerImpl());
		meshoptgpu_ServerConfig c = config ? *config : meshoptgpu_ServerConfig{};
		c.memory_budget = c.memory_budget ? c.memory_budget : kServerBudgetDefault;
		c.batch_workers = c.batch_workers > 0 ? c.batch_workers : 8;
		c.large_workers = c.large_workers > 0 ? c.large_workers : 8;
		c.large_index_count = c.large_index_count ? c.large_index_count : 30000;
		c.max_batch = c.max_batch > 0 ? c.max_batch : 2048;
		c.batch_threads = (c.batch_threads == 128 || c.batch_threads == 256 || c.batch_threads == 512) ? c.batch_threads : 256;
		c.perform_blocks = c.plain ? 0 : (c.perform_blocks > 0 ? c.perform_blocks : 64);
		S->cfg = c;
		MO_CUDA_CHECK(cudaGetDevice(&S->device));
		MO_CUDA_CHECK(cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, S->device));
		ServerImpl* raw = S.get();
		if (!c.plain)
			for (int i = 0; i < c.batch_workers; ++i)
				S->threads.emplace_back(batchWorker, raw);
		for (int i = 0; i < (c.plain ? 1 : c.large_workers); ++i)
			S->threads.emplace_back(largeWorker, raw);
		setStatus(meshoptgpu_StatusOk, "");
		return reinterpret_cast<meshoptgpu_Server*>(S.release());
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return nullptr;
	}
}

void meshoptgpu_serverDestroy(meshoptgpu_Server* server)
{
	if (!server)
		return;
	ServerImpl* S = reinterpret_cast<ServerImpl*>(server);
	{
		std::unique_lock<std::mutex> lk(S->m);
		S->cv_done.wait(lk, [&] { return S->small_q.empty() && S->large_q.empty() && S->inflight == 0; });
		S->stop = true;
		S->cv_work.notify_all();
	}
	for (std::thread& t : S->threads)
		t.join();
	delete S;
}

long long meshoptgpu_serverSubmit(meshoptgpu_Server* server, const meshoptgpu_BatchMesh* mesh)
{
	if (!server || !mesh)
		return -meshoptgpu_StatusInvalidArgument;
	ServerImpl* S = reinterpret_cast<ServerImpl*>(server);
	std::string bad = checkBatchMesh(*mesh, true);
	if (!bad.empty())
	{
		int st = batchCheckStatus(*mesh, true);
		setStatus(st, bad);
		return -st;
	}
	std::unique_ptr<ServerRequest> r(new ServerRequest());
	AttrMaps unused;
	int attr_index = -1;
	r->desc = makeDesc(*mesh, mesh->indices, mesh->vertex_positions, mesh->vertex_attributes, mesh->vertex_lock, mesh->destination, unused, attr_index);
	if (r->desc.ac)
		r->weights.assign(mesh->attribute_weights, mesh->attribute_weights + mesh->attribute_count);
	r->index_count = mesh->index_count;
	r->vertex_count = mesh->vertex_count;
	// meshes up to large_index_count indices go to the batch kernel (one CTA per mesh, shared
	// memory or a global slab); larger ones, and the options the batch kernel does not have,
	// take the multi-CTA single-mesh path
	bool large = S->cfg.plain || mesh->index_count > S->cfg.large_index_count || (mesh->options & ~kBatchOptions);
	r->reserve = large ? Simplifier::workspaceBytes(mesh->index_count, mesh->vertex_count, r->desc.ac) : batchReserve(*r);
	if (r->reserve > S->cfg.memory_budget)
	{
		setStatus(meshoptgpu_StatusOutOfMemory, "request needs more device scratch than the server's memory budget");
		return -meshoptgpu_StatusOutOfMemory;
	}
	r->submitted = std::chrono::steady_clock::now();
	std::lock_guard<std::mutex> g(S->m);
	long long ticket = (long long)S->reqs.size();
	(large ? S->large_q : S->small_q).push_back(r.get());
	S->reqs.push_back(std::move(r));
	S->cv_work.notify_all();
	return ticket;
}

int meshoptgpu_serverWait(meshoptgpu_Server* server, long long ticket, size_t* result_index_count, float* result_error, double* latency_ms)
{
	if (!server)
		return meshoptgpu_StatusInvalidArgument;
	ServerImpl* S = reinterpret_cast<ServerImpl*>(server);
	std::unique_lock<std::mutex> lk(S->m);
	if (ticket < 0 || ticket >= (long long)S->reqs.size())
		return meshoptgpu_StatusInvalidArgument;
	ServerRequest* r = S->reqs[size_t(ticket)].get();
	S->cv_done.wait(lk, [&] { return r->done; });
	if (result_index_count)
		*result_index_count = r->result_count;
	if (result_error)
		*result_error = r->result_error;
	if (latency_ms)
		*latency_ms = std::chrono::duration<double, std::milli>(r->completed - r->submitted).count();
	return r->status;
}

void meshoptgpu_serverStats(meshoptgpu_Server* server, unsigned long long* out5)
{
	ServerImpl* S = reinterpret_cast<ServerImpl*>(server);
	std::lock_guard<std::mutex> g(S->m);
	out5[0] = S->completed;
	out5[1] = S->batches;
	out5[2] = S->singles;
	out5[3] = S->peak_reserved;
	out5[4] = S->peak_inflight;
}

void meshoptgpu_setBatchConfig(int threads, unsigned int smem_bytes)
{
	ThreadState& s = state();
	s.batch_threads = (threads == 128 || threads == 256 || threads == 512) ? threads : 0;
	s.batch_smem = smem_bytes;
}

void meshoptgpu_setDropinBatchLimit(size_t max_index_count)
{
	state().dropin_batch_limit = max_index_count;
}

int meshoptgpu_setDeviceLoop(int enabled)
{
	try
	{
		ThreadState& s = state();
		s.ensure();
		Tuning t = s.simplifier->tuning();
		t.device_loop = enabled != 0;
		s.simplifier->setTuning(t);
		return meshoptgpu_StatusOk;
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return statusOf(e);
	}
}

int meshoptgpu_probeBarrierWait(int once, unsigned int blocks, unsigned int wait_limit, unsigned int* timed_out)
{
	try
	{
		ThreadState& s = state();
		s.ensure();
		if (blocks < 2 || blocks > coopScanCapacity() || wait_limit == 0 || wait_limit > (1u << 20) || !timed_out)
			throw std::invalid_argument("probeBarrierWait: blocks must be 2..resident blocks, wait_limit 1..2^20, timed_out non-null");
		*timed_out = probeBarrierWait(once, blocks, wait_limit, s.stream);
		setStatus(meshoptgpu_StatusOk, "");
		return meshoptgpu_StatusOk;
	}
	catch (const std::exception& e)
	{
		setStatus(statusOf(e), e.what());
		return statusOf(e);
	}
}

int meshoptgpu_getBatchThreads(void)
{
	ThreadState& s = state();
	if (s.batch_threads)
		return s.batch_threads;
	std::lock_guard<std::mutex> g(g_tuner.lock);
	return g_tuner.shape.empty() ? 0 : g_tuner.shape.rbegin()->second.first;
}

int meshoptgpu_getTuning(size_t index_count, size_t attribute_count, int* out4)
{
	if (!out4)
		return 0;
	int dev = 0;
	cudaGetDevice(&dev);
	const auto key = std::make_tuple(dev, sizeClass(index_count), attribute_count ? 1 : 0);
	int found = 0;
	out4[0] = out4[1] = 0;
	out4[2] = -1;
	out4[3] = 0;
	{
		std::lock_guard<std::mutex> g(g_shapes.lock);
		auto it = g_shapes.shape.find(key);
		if (it != g_shapes.shape.end())
		{
			out4[0] = it->second.first;
			out4[1] = int(it->second.second);
			found = 1;
		}
		auto jt = g_shapes.batch.find(key);
		if (jt != g_shapes.batch.end())
			out4[2] = jt->second ? 1 : 0;
	}
	{
		std::lock_guard<std::mutex> g(g_tuner.lock);
		if (!g_tuner.shape.empty())
			out4[3] = int(g_tuner.shape.rbegin()->second.second / 1024);
	}
	return found;
}

} // extern "C"

namespace
{

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
			MO_CUDA_CHECK(cudaMemcpyAsync(d_pos, vertex_positions, stridedExtent(vertex_count, vertex_positions_stride, 12), cudaMemcpyHostToDevice, s.stream));
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

int meshoptgpu_getLastRoundTrace(unsigned int* active, float* micros, int max_rounds)
{
	const RunResult& r = state().last;
	int n = int(r.round_trace.size());
	for (int i = 0; i < n && i < max_rounds; ++i)
	{
		active[i] = r.round_trace[i].first;
		micros[i] = r.round_trace[i].second;
	}
	return n;
}

int meshoptgpu_getLastPassPhaseTimes(float* out, int max_passes)
{
	const RunResult& r = state().last;
	int n = int(r.pass_phase_ms.size());
	for (int i = 0; i < n && i < max_passes; ++i)
		memcpy(out + 5 * i, r.pass_phase_ms[i].data(), 5 * sizeof(float));
	return n;
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
		routeAndRun(s, m, destination, st, true);
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
	tls.reset();
}

} // extern "C"
