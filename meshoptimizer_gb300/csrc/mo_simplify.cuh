// mo_simplify.cuh - host interface of the device-resident edge-collapse simplifier.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include <algorithm>
#include <array>
#include <vector>

#include "mo_prims.cuh"

namespace mogpu
{

constexpr int kMaxAttributes = 32;   // src/simplifier.cpp:665
constexpr int kMaxPassStats = 128;

// One mesh to simplify; all array pointers are DEVICE pointers (except weights, which
// live on the host: at most 32 floats, folded into kernel arguments).
struct MeshDesc
{
	const unsigned int* indices = nullptr;
	size_t index_count = 0;
	const float* positions = nullptr;
	size_t vertex_count = 0;
	size_t positions_stride = 12; // bytes
	const float* attributes = nullptr;
	size_t attributes_stride = 0; // bytes
	const float* weights = nullptr; // host
	size_t attribute_count = 0;
	const unsigned char* lock = nullptr;
	size_t target_index_count = 0;
	float target_error = 0.f;
	unsigned int options = 0;
	// the update mode (options with kOptInternalSolve): the buffers the solved positions and
	// attributes are written back to, same layout as positions / attributes (may be the same
	// device buffers)
	float* update_positions = nullptr;
	float* update_attributes = nullptr;
	// when set, the attributes are still arriving: the stream waits for this event before it
	// first reads them (their copy overlaps the setup that does not need them)
	cudaEvent_t attributes_ready = nullptr;
	// the same for the indices (their copy overlaps the setup's position-only kernels)
	cudaEvent_t indices_ready = nullptr;
};

// Per-pass counters, the same quantities the reference prints under TRACE
// (src/simplifier.cpp:1625-1633). stop: 0 out of collapses, 1 error limit, 2 count
// limit, 3 error goal.
struct PassStats
{
	unsigned int triangles;
	unsigned int candidates;
	unsigned int evaluated;
	unsigned int done;
	unsigned int skipped;
	unsigned int invalid;
	unsigned int stop;
	unsigned int rounds;
	unsigned int active; // candidates processed by the decision kernels, summed over rounds
	unsigned int windows; // sorted-order windows decided before the stop cut was found
};

struct RunResult
{
	size_t index_count = 0;
	float result_error = 0.f;   // linear, scaled like the reference's *result_error
	float result_error_sq = 0.f;
	float scale = 0.f;
	int passes = 0;
	PassStats pass[kMaxPassStats];
	// time inside the cooperative pass kernel by phase (block 0's SM clock): init, window marks,
	// decision rounds, stop rules, apply, loop remap + counts, count scan, compaction emit
	float perform_phase_ms[8] = {};
	// decision rounds of the run in order: active candidates and duration (microseconds)
	std::vector<std::pair<unsigned int, float>> round_trace;
	// with timing on: CUDA-event times (ms) of each pass's adjacency, pick, rank, sort and perform
	std::vector<std::array<float, 5>> pass_phase_ms;
};

// Device timings of the phases of one run (milliseconds, from CUDA events).
struct PhaseTimes
{
	float setup = 0, adjacency = 0, pick = 0, rank = 0, sort = 0, perform = 0, apply = 0, total = 0;
};

// Debug copies of setup arrays (device -> host) for per-phase comparison with the oracle.
struct SetupDump
{
	std::vector<unsigned int> remap, wedge, loop, loopback;
	std::vector<unsigned char> kind;
	std::vector<float> positions; // 3 per vertex
	std::vector<float> quadrics;  // 11 per vertex
	std::vector<float> attr_quadrics, attr_gradients;
	size_t capacity = 0;
	float scale = 0;
};

// Grow-only device arena; one per Simplifier.
class DeviceArena
{
public:
	~DeviceArena();
	void reserve(size_t bytes);
	char* base() const { return base_; }
	size_t capacity() const { return cap_; }
	void release();

private:
	char* base_ = nullptr;
	size_t cap_ = 0;
};

// Launch-shape parameters (picked by the autotuner, or set with environment variables
// MESHOPTGPU_PERFORM_BLOCKS_PER_SM, MESHOPTGPU_WINDOW_FACTOR and MESHOPTGPU_DEVICE_LOOP).
struct Tuning
{
	int perform_blocks_per_sm = 4;  // resident blocks per SM of the cooperative pass kernel
	double window_factor = 2.0;     // first decision window = factor * (triangle goal / 2) + 4096
	int perform_grid_cap = 0;       // at most this many blocks for the pass kernel (0: no cap); lets
	                                // concurrent simplifications share the GPU
	bool device_loop = true;        // run the pass loop as a device-resident CUDA graph (off: one host
	                                // round trip per pass, needed for per-kernel event timing)
	static Tuning fromEnvironment();
};

class Simplifier
{
public:
	explicit Simplifier(int device);
	~Simplifier();

	// Simplifies `mesh` on `stream`, writing the result index buffer to d_out (device,
	// room for mesh.index_count indices). Blocks until the result count is known.
	RunResult run(const MeshDesc& mesh, unsigned int* d_out, cudaStream_t stream, PhaseTimes* times = nullptr, SetupDump* dump = nullptr);

	// meshopt_simplifyScale on device positions
	float scale(const float* d_positions, size_t vertex_count, size_t stride, cudaStream_t stream);

	int device() const { return device_; }
	size_t arenaBytes() const { return arena_.capacity(); }

	// Bytes of device scratch a run on this mesh shape needs (used by admission control).
	static size_t workspaceBytes(size_t index_count, size_t vertex_count, size_t attribute_count);

private:
	RunResult runSparse(const MeshDesc& mesh, unsigned int* d_out, cudaStream_t stream, PhaseTimes* times, SetupDump* dump);

	int device_;
	DeviceArena arena_;
	DeviceArena sparse_arena_; // compact copy of a sparse subset
	unsigned int* pinned_ = nullptr; // small pinned readback buffer
	cudaStream_t capture2_ = nullptr; // records the pass body's second branch (the pick)
	cudaEvent_t fork_ = nullptr, join_ = nullptr; // the branch's fork and join while recording
	cudaStream_t capture_ = nullptr; // records the device-resident pass loop (the caller's stream may be
	                                 // the legacy default stream, which cannot capture)
	unsigned int coop_blocks_ = 1;   // resident blocks of the cooperative pass kernel (occupancy)
	unsigned int perform_blocks_ = 1;
	unsigned int sort_items_ = 0;    // candidates per thread of the pass sort's tiles (0: by count)
	int sms_ = 1;
	int solve_per_sm_ = 1; // resident blocks of the position solve kernel per SM
	int clock_khz_ = 0;    // SM clock for the phase counters (queried once: the query costs ~0.6 ms)
	Tuning tuning_;
	// The device-resident pass loop's executable graph, kept for the next run of the same shape:
	// the graph holds workspace pointers (fixed by the arena base and the layout's sizes) and
	// grid sizes; everything else it reads (targets, counts, the error limit) is on the device.
	struct LoopGraph
	{
		const void* base = nullptr;
		size_t I = 0, V = 0;
		int ac = 0;
		bool solve = false;
		unsigned int blocks = 0;
		unsigned int sort_items = 0;
		unsigned int scan_blocks = 0;         // the one-launch scans' grid cap recorded in the body (0: none)
		unsigned long long body_launches = 0; // kernels one replay of the body launches
		cudaGraph_t graph = nullptr;
		cudaGraphExec_t exec = nullptr;
	} loop_;
	void dropLoopGraph();

public:
	void setTuning(const Tuning& t)
	{
		tuning_ = t;
		perform_blocks_ = std::min(coop_blocks_, unsigned(std::max(1, sms_ * t.perform_blocks_per_sm)));
	}
	// The launch shape of the pass kernels an autotuner picks: pass-kernel blocks per SM, and the
	// pass sort's candidates per thread (4, 8 or 16; 0: chosen by the candidate count). Results do
	// not depend on either.
	void setPassShape(int perform_blocks_per_sm, unsigned int sort_items)
	{
		Tuning t = tuning_;
		t.perform_blocks_per_sm = perform_blocks_per_sm;
		setTuning(t);
		sort_items_ = (sort_items == 4 || sort_items == 8 || sort_items == 16) ? sort_items : 0;
	}
	int performBlocksPerSM() const { return tuning_.perform_blocks_per_sm; }
	// resident blocks per SM of the pass kernel at most (its register count)
	int performBlocksPerSMMax() const { return int(coop_blocks_ / unsigned(std::max(1, sms_))); }
	unsigned int sortItems() const { return sort_items_; }
	const Tuning& tuning() const { return tuning_; }
};

} // namespace mogpu
