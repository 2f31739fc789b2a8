// mo_simplify.cu - device-resident quadric edge-collapse simplifier for GB300 (sm_103a).
//
// Restates meshopt_simplifyEdge (meshoptimizer src/simplifier.cpp:2344-2626) as integer
// sort/scan/compaction kernels plus FP32 quadric kernels whose operation order follows the
// reference, so that the output index buffer is bit-identical to the CPU library.
//
// Where the reference is sequential and order-dependent, the GPU form is chosen so that the
// order no longer matters or is reproduced exactly:
//  * vertex -> face lists are built by a stable radix sort of (vertex, corner) pairs, so each
//    vertex folds its face quadrics in face order (fillFaceQuadrics :1057-1082) with no float
//    atomics;
//  * open-edge classification (classifyVertices :364-414) is computed per vertex from its own
//    half-edge list: half-edge u->v is stored in both u's list (next = v) and v's list
//    (prev = u), so "is there an opposite edge" is a local question;
//  * the greedy collapse loop (performEdgeCollapses :1498-1636) is decided in deterministic
//    rounds: a candidate is resolved once every earlier candidate (in sorted order) that shares
//    an endpoint, or moves a vertex of its one-ring, is resolved, which reproduces the serial
//    decisions; the stop rules are then applied as a prefix scan over sorted order.
#include "mo_common.cuh"
#include "mo_prims.cuh"
#include "mo_probe.cuh"
#include "mo_grid.cuh"
#include "mo_simplify.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace mogpu
{

namespace
{

constexpr int kThreads = 256;
constexpr int kStopTile = 1024; // sorted candidates per block in the stop-rule scan
constexpr size_t kPinnedBytes = 16384; // host readback buffer of the scalars block
#ifndef MO_STAGE_CHUNK
#define MO_STAGE_CHUNK 2048
#endif
#ifndef MO_STAGE_ITEMS
#define MO_STAGE_ITEMS 2
#endif
constexpr unsigned int kStageChunk = MO_STAGE_CHUNK; // candidates of a block taken through the decision stages at a time
constexpr unsigned int kStageItems = MO_STAGE_ITEMS; // candidates per thread in the first decision stage

// State of the device-resident pass loop: the counts each pass's kernels read instead of
// launch parameters, so that one recorded pass can be replayed until the loop ends.
struct PassLive
{
	const unsigned int* res;  // current index buffer
	unsigned int* res_next;   // the next pass's
	unsigned int indices;     // current index count
	unsigned int tris;
	unsigned int count;       // candidates of the pass
	unsigned int stop;        // nonzero: the loop has ended; the pass's kernels return at once
	unsigned long long goal;  // triangle goal of the pass
	unsigned int first_window;
	unsigned int round_base;
	unsigned int passes;
	unsigned int iterations;
	unsigned int target;      // target_index_count
	unsigned int sort_items;  // candidates per thread of the sort's tiles
	unsigned int sort_cells;  // cells of the pass's live sort histogram matrix
	float error_limit;        // squared, in the rescaled space (:2489-2491)
	double window_factor;     // this pass's first decision window, in units of the triangle goal / 2
	double window_base;       // its smallest value
};

// The sorted positions a pass decides before its stop rules cut grow from pass to pass relative to
// its triangle goal; the next pass's first window is this much larger than the last pass needed,
// so that it rarely needs a second window (a second window costs a full set of decision rounds).
#ifndef MO_WINDOW_MARGIN
#define MO_WINDOW_MARGIN 1.5
#endif
constexpr double kWindowMargin = MO_WINDOW_MARGIN;

__host__ __device__ inline double nextWindowFactor(double base, unsigned long long goal, unsigned long long evaluated)
{
	const double half = double(goal / 2 ? goal / 2 : 1);
	const double f = kWindowMargin * double(evaluated) / half;
	return f > base ? f : base;
}

struct Scalars
{
	float minv[3];
	float maxv[3];
	float extent;
	float scale;
	unsigned int bad_index;
	unsigned int probe_fail;
	unsigned int dup_count;
	unsigned int capacity;
	unsigned long long dual;
	unsigned int pick_total;
	unsigned int pick_trunc;
	unsigned int active_count;
	unsigned int tri_total;
	unsigned long long cut;
	unsigned int done;
	unsigned int skipped;
	unsigned int invalid;
	unsigned int result_error_bits;
	unsigned int vertex_error_bits;
	unsigned int bar[2];          // grid barrier (arrivals, generation)
	unsigned int grid_error;      // a grid barrier gave up waiting
	unsigned int rounds;          // decision rounds of the last pass
	unsigned int act_count[3];    // appended candidates, rotating by round (round r appends to [(r+1)%3])
	unsigned long long active_sum; // candidates processed by the rounds of the last pass
	unsigned int carry[3];        // stop-rule prefix (triangles, flips, max error) after a window
	unsigned int windows;         // sorted-order windows the last pass needed
	unsigned long long phase_cycles[8]; // kPerform phases, SM cycles of block 0, summed over the run
	unsigned int trace_count;           // decision rounds traced so far in the run
	unsigned int trace[2 * 512];        // per round: active candidates, SM cycles / 16
	PassLive live;                      // device-resident pass loop
	PassStats pstats[kMaxPassStats];    // its per-pass counters
	unsigned int solve_pending[3];      // update mode: position-solve candidates left, rotating by round
	unsigned int solve_rounds;
	unsigned int max_degree;            // corners of the busiest vertex
	unsigned int scan_bar[2];           // the single-launch scans' barrier words (left zero by each scan)
	unsigned int scan_bar2[2];          // those of the scans on the pass loop's second branch (the pick)
	unsigned int scan_error;            // a single-launch scan's barrier gave up waiting
};

static_assert(sizeof(Scalars) <= kPinnedBytes, "the scalars block must fit the pinned readback buffer");

__device__ __forceinline__ size_t gtid()
{
	return (size_t)blockIdx.x * blockDim.x + threadIdx.x;
}

// ---------------------------------------------------------------- setup: positions

__global__ void kGatherPositions(const float* __restrict__ data, size_t stride_f, size_t n, float4* __restrict__ out)
{
	size_t i = gtid();
	if (i >= n)
		return;
	const float* v = data + i * stride_f;
	out[i] = make_float4(v[0], v[1], v[2], 0.f);
}

__global__ void kValidateIndices(const unsigned int* __restrict__ idx, size_t n, size_t vcount, unsigned int* bad)
{
	size_t i = gtid();
	if (i < n && idx[i] >= vcount)
		atomicOr(bad, 1u);
}

// min/max fold with the reference's comparison form (rescalePositions :551-567): the
// sequential fold keeps the leftmost extreme among values that compare equal (matters only
// for the sign of zero) and skips NaN. "combine(left, right)" keeps that semantics.
__device__ __forceinline__ float foldMin(float l, float r)
{
	return l > r ? r : l;
}

__device__ __forceinline__ float foldMax(float l, float r)
{
	return l < r ? r : l;
}

constexpr int kMinMaxThreads = 256;
constexpr size_t kMinMaxMaxThreads = 152 * 4 * kMinMaxThreads; // threads of the partial pass, at most

__global__ void __launch_bounds__(kMinMaxThreads) kMinMaxPartial(const float4* __restrict__ pos, size_t n, size_t per_thread, float* __restrict__ partial)
{
	float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
	float mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
	size_t begin = gtid() * per_thread;
	size_t end = min(begin + per_thread, n);
	for (size_t i = begin; i < end; ++i)
	{
		float4 p = pos[i];
		float v[3] = {p.x, p.y, p.z};
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			mn[j] = mn[j] > v[j] ? v[j] : mn[j];
			mx[j] = mx[j] < v[j] ? v[j] : mx[j];
		}
	}
	// combine lanes left to right: lane l holds a lower index range than lane l+o
#pragma unroll
	for (int o = 1; o < 32; o <<= 1)
	{
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			float a = __shfl_down_sync(0xffffffffu, mn[j], o);
			float b = __shfl_down_sync(0xffffffffu, mx[j], o);
			if ((threadIdx.x & 31) + o < 32 && ((threadIdx.x & (2 * o - 1)) == 0))
			{
				mn[j] = foldMin(mn[j], a);
				mx[j] = foldMax(mx[j], b);
			}
		}
	}
	__shared__ float sm[kMinMaxThreads / 32][6];
	int w = threadIdx.x >> 5;
	if ((threadIdx.x & 31) == 0)
		for (int j = 0; j < 3; ++j)
			sm[w][j] = mn[j], sm[w][3 + j] = mx[j];
	__syncthreads();
	if (threadIdx.x == 0)
	{
		for (int q = 1; q < kMinMaxThreads / 32; ++q)
			for (int j = 0; j < 3; ++j)
			{
				sm[0][j] = foldMin(sm[0][j], sm[q][j]);
				sm[0][3 + j] = foldMax(sm[0][3 + j], sm[q][3 + j]);
			}
		for (int j = 0; j < 6; ++j)
			partial[blockIdx.x * 6 + j] = sm[0][j];
	}
}

// folds the per-block partials in block order: thread t takes a contiguous run of blocks,
// then lanes and warps are combined left to right as in kMinMaxPartial
__global__ void __launch_bounds__(kMinMaxThreads) kMinMaxFinal(const float* __restrict__ partial, int blocks, Scalars* sc)
{
	float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
	float mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
	int per = (blocks + kMinMaxThreads - 1) / kMinMaxThreads;
	int b0 = threadIdx.x * per, b1 = min(b0 + per, blocks);
	for (int b = b0; b < b1; ++b)
		for (int j = 0; j < 3; ++j)
		{
			mn[j] = foldMin(mn[j], partial[b * 6 + j]);
			mx[j] = foldMax(mx[j], partial[b * 6 + 3 + j]);
		}
#pragma unroll
	for (int o = 1; o < 32; o <<= 1)
	{
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			float a = __shfl_down_sync(0xffffffffu, mn[j], o);
			float b = __shfl_down_sync(0xffffffffu, mx[j], o);
			if ((threadIdx.x & 31) + o < 32 && ((threadIdx.x & (2 * o - 1)) == 0))
			{
				mn[j] = foldMin(mn[j], a);
				mx[j] = foldMax(mx[j], b);
			}
		}
	}
	__shared__ float sm[kMinMaxThreads / 32][6];
	int w = threadIdx.x >> 5;
	if ((threadIdx.x & 31) == 0)
		for (int j = 0; j < 3; ++j)
			sm[w][j] = mn[j], sm[w][3 + j] = mx[j];
	__syncthreads();
	if (threadIdx.x != 0)
		return;
	for (int q = 1; q < kMinMaxThreads / 32; ++q)
		for (int j = 0; j < 3; ++j)
		{
			sm[0][j] = foldMin(sm[0][j], sm[q][j]);
			sm[0][3 + j] = foldMax(sm[0][3 + j], sm[q][3 + j]);
		}
	float extent = 0.f;
	extent = (sm[0][3] - sm[0][0]) < extent ? extent : (sm[0][3] - sm[0][0]);
	extent = (sm[0][4] - sm[0][1]) < extent ? extent : (sm[0][4] - sm[0][1]);
	extent = (sm[0][5] - sm[0][2]) < extent ? extent : (sm[0][5] - sm[0][2]);
	for (int j = 0; j < 3; ++j)
		sc->minv[j] = sm[0][j], sc->maxv[j] = sm[0][3 + j];
	sc->extent = extent;
	sc->scale = extent == 0 ? 0.f : 1.f / extent;
}

__global__ void kRescale(const float4* __restrict__ raw, size_t n, const Scalars* __restrict__ sc, float4* __restrict__ out)
{
	size_t i = gtid();
	if (i >= n)
		return;
	float4 p = raw[i];
	float s = sc->scale;
	out[i] = make_float4((p.x - sc->minv[0]) * s, (p.y - sc->minv[1]) * s, (p.z - sc->minv[2]) * s, 0.f);
}

// ---------------------------------------------------------------- setup: position remap

__device__ __forceinline__ unsigned int mix32(unsigned int h)
{
	h ^= h >> 16;
	h *= 0x7feb352du;
	h ^= h >> 15;
	h *= 0x846ca68bu;
	h ^= h >> 16;
	return h;
}

__device__ __forceinline__ unsigned int posBits(float f)
{
	unsigned int u = __float_as_uint(f);
	return u == 0x80000000u ? 0u : u; // -0 and +0 compare equal
}

// Concurrent open addressing: the first vertex to claim a slot stores its index, every
// vertex whose position compares equal (float ==, so NaN never matches) joins that slot and
// lowers it to the smallest index with atomicMin. Equal positions hash alike and follow the
// same probe sequence, and slots are never freed, so all members of a class meet in one slot.
// Result: remap[i] = smallest index with an equal position (buildPositionRemap :195-214).
__global__ void kHashInsert(const float4* __restrict__ pos, size_t n, unsigned int* table, unsigned int mask, unsigned int* __restrict__ slot_of, unsigned int* fail)
{
	size_t i = gtid();
	if (i >= n)
		return;
	float4 p = pos[i];
	unsigned int h = mix32(posBits(p.x) * 0x9e3779b1u ^ mix32(posBits(p.y) + 0x85ebca6bu) ^ mix32(posBits(p.z) * 0xc2b2ae35u + 1u));
	unsigned int b = h & mask;
	for (unsigned int probe = 0; probe <= mask; ++probe)
	{
		unsigned int cur = table[b];
		if (cur == ~0u)
		{
			unsigned int prev = atomicCAS(&table[b], ~0u, (unsigned int)i);
			if (prev == ~0u)
			{
				slot_of[i] = b;
				return;
			}
			cur = prev;
		}
		float4 q = pos[cur];
		if (q.x == p.x && q.y == p.y && q.z == p.z)
		{
			atomicMin(&table[b], (unsigned int)i);
			slot_of[i] = b;
			return;
		}
		b = (b + probe + 1) & mask;
	}
	atomicOr(fail, 1u);
	slot_of[i] = ~0u;
}

__global__ void kHashRemap(const unsigned int* __restrict__ table, const unsigned int* __restrict__ slot_of, size_t n, unsigned int* __restrict__ remap,
    unsigned int* __restrict__ wedge, unsigned int* __restrict__ dupflag)
{
	size_t i = gtid();
	if (i >= n)
		return;
	unsigned int s = slot_of[i];
	unsigned int r = s == ~0u ? (unsigned int)i : table[s];
	remap[i] = r;
	wedge[i] = (unsigned int)i;
	dupflag[i] = r != i;
}

// dup vertices sorted by (class, index): wedge[i] = previous member of the class (the
// primary for the smallest duplicate) and wedge[primary] = largest duplicate, the cycle
// buildPositionRemap builds at :229-239.
__global__ void kWedgeLink(const unsigned int* __restrict__ keys, const unsigned int* __restrict__ vals, size_t n, unsigned int* __restrict__ wedge)
{
	size_t q = gtid();
	if (q >= n)
		return;
	unsigned int r = keys[q], i = vals[q];
	wedge[i] = (q > 0 && keys[q - 1] == r) ? vals[q - 1] : r;
	if (q + 1 == n || keys[q + 1] != r)
		wedge[r] = i;
}

__global__ void kCompactFlagged(const unsigned int* __restrict__ flags, const unsigned int* __restrict__ offs, const unsigned int* __restrict__ remap, size_t n,
    unsigned int* __restrict__ keys, unsigned int* __restrict__ vals)
{
	size_t i = gtid();
	if (i >= n || !flags[i])
		return;
	unsigned int o = offs[i];
	keys[o] = remap[i];
	vals[o] = (unsigned int)i;
}

// ---------------------------------------------------------------- setup: CSR

__global__ void kCountKeys(const unsigned int* __restrict__ idx, const unsigned int* __restrict__ remap, size_t n, unsigned int* __restrict__ cnt)
{
	size_t i = gtid();
	if (i >= n)
		return;
	unsigned int v = idx[i];
	if (remap)
		v = remap[v];
	atomicAdd(&cnt[v], 1u);
}

// the corners of every vertex, each corner keeping its slot in its vertex's list; an index of
// vcount or more is not counted and sets bad. The indices are copied to res on the way (the
// first pass's index buffer).
__global__ void kCountCornerLists(const unsigned int* __restrict__ idx, size_t n, size_t vcount, unsigned int* __restrict__ cnt,
    unsigned int* __restrict__ slot, unsigned int* bad, unsigned int* __restrict__ res)
{
	const size_t i = gtid();
	if (i - (threadIdx.x & 31) >= n)
		return; // the whole warp is past the corners
	// corners of one vertex among the warp's 32 take their slots with one atomic add (the lists
	// are sorted afterwards, so the order the slots give is arbitrary)
	const unsigned int lane = threadIdx.x & 31;
	unsigned int v = i < n ? idx[i] : ~0u;
	if (i < n)
		res[i] = v;
	if (i < n && v >= vcount)
		atomicOr(bad, 1u);
	const bool valid = v < vcount;
	// lanes without a valid corner share a key and are masked out of every group (a vertex id
	// equal to that key stays correct)
	const unsigned int peers = __match_any_sync(0xffffffffu, valid ? v : ~0u) & __ballot_sync(0xffffffffu, valid);
	const unsigned int leader = __ffs(peers) - 1;
	unsigned int base = 0;
	if (valid && lane == leader)
		base = atomicAdd(&cnt[v], __popc(peers));
	base = __shfl_sync(0xffffffffu, base, leader);
	if (valid)
		slot[i] = base + __popc(peers & ((1u << lane) - 1u));
}

// the largest count of corners[v] = off[v+1] - off[v]
__global__ void kMaxDegree(const unsigned int* __restrict__ off, size_t n, unsigned int* out)
{
	__shared__ unsigned int wmax[32];
	size_t i = gtid();
	unsigned int d = i < n ? off[i + 1] - off[i] : 0u;
	for (int o = 16; o > 0; o >>= 1)
		d = max(d, __shfl_down_sync(0xffffffffu, d, o));
	if ((threadIdx.x & 31) == 0)
		wmax[threadIdx.x >> 5] = d;
	__syncthreads();
	if (threadIdx.x < 32)
	{
		d = threadIdx.x < blockDim.x / 32 ? wmax[threadIdx.x] : 0u;
		for (int o = 16; o > 0; o >>= 1)
			d = max(d, __shfl_down_sync(0xffffffffu, d, o));
		if (threadIdx.x == 0 && d)
			atomicMax(out, d); // one atomic per block
	}
}

// vertex -> corner lists: every corner into its vertex's range at the slot its count gave it
// (arbitrary order within the range), then each range sorted by corner index, which is the
// order a stable sort by vertex gives
__global__ void kCornerFill(const unsigned int* __restrict__ idx, const unsigned int* __restrict__ remap, size_t n, const unsigned int* __restrict__ off,
    const unsigned int* __restrict__ slot, unsigned int* __restrict__ csr)
{
	size_t p = gtid();
	if (p >= n)
		return;
	unsigned int v = idx[p];
	if (remap)
		v = remap[v];
	csr[off[v] + slot[p]] = (unsigned int)p;
}

// insertion sort of each vertex's corners (only used when no vertex has more than
// kCornerSortMax corners)
constexpr unsigned int kCornerSortMax = 64;
constexpr unsigned int kCornerRegs = 16; // lists up to this long are sorted in registers

__global__ void kCornerSort(const unsigned int* __restrict__ off, size_t n, unsigned int* csr)
{
	size_t v = gtid();
	if (v >= n)
		return;
	const unsigned int b = off[v], e = off[v + 1];
	if (e - b <= kCornerRegs)
	{
		// in registers: corner indices are distinct, so each one's rank is the count of smaller ones
		const unsigned int d = e - b;
		unsigned int c[kCornerRegs];
#pragma unroll
		for (unsigned int q = 0; q < kCornerRegs; ++q)
			c[q] = q < d ? csr[b + q] : ~0u;
#pragma unroll
		for (unsigned int q = 0; q < kCornerRegs; ++q)
			if (q < d)
			{
				unsigned int r = 0;
#pragma unroll
				for (unsigned int p = 0; p < kCornerRegs; ++p)
					r += c[p] < c[q];
				csr[b + r] = c[q];
			}
		return;
	}
	for (unsigned int j = b + 1; j < e; ++j)
	{
		unsigned int x = csr[j];
		unsigned int q = j;
		while (q > b && csr[q - 1] > x)
		{
			csr[q] = csr[q - 1];
			--q;
		}
		csr[q] = x;
	}
}

__global__ void kIota(unsigned int* __restrict__ out, size_t n)
{
	size_t i = gtid();
	if (i < n)
		out[i] = (unsigned int)i;
}

__device__ __forceinline__ void cornerNeighbours(const unsigned int* __restrict__ idx, unsigned int p, unsigned int& next, unsigned int& prev)
{
	unsigned int f = p / 3, c = p - f * 3;
	unsigned int b = f * 3;
	next = idx[b + (c == 2 ? 0 : c + 1)];
	prev = idx[b + (c == 0 ? 2 : c - 1)];
}

// ---------------------------------------------------------------- setup: classification

constexpr unsigned int kOpenEdgesRegs = 12; // vertices with at most this many corners search in registers
#ifndef MO_FILL_BATCH
#define MO_FILL_BATCH 2
#endif
constexpr unsigned int kFillBatch = MO_FILL_BATCH; // corners whose loads kFillQuadrics issues together

// openout (stored in loop) and openinc (stored in loopback) of classifyVertices :370-396,
// from the vertex's own raw half-edge list: ~0u for none, the unique open neighbour, or the
// vertex itself for several / a degenerate triangle.
__global__ void kOpenEdges(const unsigned int* __restrict__ idx, const unsigned int* __restrict__ off, const unsigned int* __restrict__ csr, size_t n,
    unsigned int* __restrict__ loop, unsigned int* __restrict__ loopback)
{
	size_t vi = gtid();
	if (vi >= n)
		return;
	unsigned int v = (unsigned int)vi;
	unsigned int b = off[v], e = off[v + 1];
	if (e - b <= kOpenEdgesRegs)
	{
		// the corners' neighbours in registers (all loads issued together), then the same
		// search over them
		unsigned int nxs[kOpenEdgesRegs], pvs[kOpenEdgesRegs];
		const unsigned int d = e - b;
#pragma unroll
		for (unsigned int q = 0; q < kOpenEdgesRegs; ++q)
			nxs[q] = q < d ? csr[b + q] : 0u;
#pragma unroll
		for (unsigned int q = 0; q < kOpenEdgesRegs; ++q)
		{
			if (q < d)
				cornerNeighbours(idx, nxs[q], nxs[q], pvs[q]);
			else
				nxs[q] = pvs[q] = ~0u;
		}
		bool degen = false;
#pragma unroll
		for (unsigned int q = 0; q < kOpenEdgesRegs; ++q)
			degen |= q < d && nxs[q] == v;
		unsigned int outc = 0, outt = ~0u, inc = 0, ins = ~0u;
#pragma unroll
		for (unsigned int j = 0; j < kOpenEdgesRegs; ++j)
		{
			if (j >= d)
				break;
			bool has_back = false, has_fwd = false;
#pragma unroll
			for (unsigned int q = 0; q < kOpenEdgesRegs; ++q)
			{
				has_back |= q < d && pvs[q] == nxs[j];
				has_fwd |= q < d && nxs[q] == pvs[j];
			}
			if (!has_back)
				outc++, outt = nxs[j];
			if (!has_fwd)
				inc++, ins = pvs[j];
		}
		loop[v] = degen ? v : (outc == 0 ? ~0u : (outc == 1 ? outt : v));
		loopback[v] = degen ? v : (inc == 0 ? ~0u : (inc == 1 ? ins : v));
		return;
	}
	bool degen = false;
	for (unsigned int j = b; j < e; ++j)
	{
		unsigned int nx, pv;
		cornerNeighbours(idx, csr[j], nx, pv);
		degen |= nx == v;
	}
	unsigned int outc = 0, outt = ~0u, inc = 0, ins = ~0u;
	if (!degen)
		for (unsigned int j = b; j < e; ++j)
		{
			unsigned int nx, pv;
			cornerNeighbours(idx, csr[j], nx, pv);
			bool has_back = false, has_fwd = false;
			for (unsigned int q = b; q < e; ++q)
			{
				unsigned int nq, pq;
				cornerNeighbours(idx, csr[q], nq, pq);
				has_back |= pq == nx; // half-edge nx -> v exists
				has_fwd |= nq == pv;  // half-edge v -> pv exists
			}
			if (!has_back)
				outc++, outt = nx;
			if (!has_fwd)
				inc++, ins = pv;
		}
	loop[v] = degen ? v : (outc == 0 ? ~0u : (outc == 1 ? outt : v));
	loopback[v] = degen ? v : (inc == 0 ? ~0u : (inc == 1 ? ins : v));
}

// classifyVertices :405-471 for the primary vertex i
__device__ unsigned char classifyPrimary(unsigned int i, const unsigned int* __restrict__ remap, const unsigned int* __restrict__ wedge,
    const unsigned int* __restrict__ openout, const unsigned int* __restrict__ openinc)
{
	unsigned int w = wedge[i];
	if (w == i)
	{
		unsigned int openi = openinc[i], openo = openout[i];
		if (openi == ~0u && openo == ~0u)
			return kManifold;
		if (openi != ~0u && openo != ~0u && remap[openi] == remap[openo] && openi != i)
			return kSeam;
		if (openi != i && openo != i)
			return kBorder;
		return kLocked;
	}
	if (wedge[w] == i)
	{
		unsigned int openiv = openinc[i], openov = openout[i];
		unsigned int openiw = openinc[w], openow = openout[w];
		if (openiv != ~0u && openiv != i && openov != ~0u && openov != i && openiw != ~0u && openiw != w && openow != ~0u && openow != w)
		{
			if (remap[openiv] == remap[openow] && remap[openov] == remap[openiw] && remap[openiv] != remap[openov])
				return kSeam;
			return kLocked;
		}
		return kLocked;
	}
	return kLocked;
}

__global__ void kClassify(size_t n, const unsigned int* __restrict__ remap, const unsigned int* __restrict__ wedge, const unsigned int* __restrict__ loop,
    const unsigned int* __restrict__ loopback, unsigned char* __restrict__ kind)
{
	size_t i = gtid();
	if (i < n)
		kind[i] = classifyPrimary(remap[i], remap, wedge, loop, loopback);
}

__global__ void kLockMark(size_t n, const unsigned char* __restrict__ lock, const unsigned int* __restrict__ remap, unsigned char* kind)
{
	size_t i = gtid();
	if (i < n && (lock[i] & kVertexLock))
		kind[remap[i]] = kLocked;
}

__global__ void kLockSpread(size_t n, const unsigned int* __restrict__ remap, unsigned char* kind)
{
	size_t i = gtid();
	if (i < n && kind[remap[i]] == kLocked)
		kind[i] = kLocked;
}

__global__ void kLockBorder(size_t n, unsigned char* kind)
{
	size_t i = gtid();
	if (i < n && kind[i] == kBorder)
		kind[i] = kLocked;
}

// Permissive mode (classifyVertices :481-515): a seam or locked primary becomes Complex unless
// one of its wedges is protected by vertex_lock or has a half-edge without an opposite edge in
// position space (hasEdge with remap/wedge, :345-362). `off/csr` is the raw corner list.
__device__ bool hasEdgeWedged(unsigned int a, unsigned int b, const unsigned int* __restrict__ idx, const unsigned int* __restrict__ off,
    const unsigned int* __restrict__ csr, const unsigned int* __restrict__ remap, const unsigned int* __restrict__ wedge)
{
	unsigned int rb = remap[b];
	unsigned int v = a;
	do
	{
		for (unsigned int j = off[v]; j < off[v + 1]; ++j)
		{
			unsigned int nx, pv;
			cornerNeighbours(idx, csr[j], nx, pv);
			if (remap[nx] == rb)
				return true;
		}
		v = wedge[v];
	} while (v != a);
	return false;
}

__global__ void kPermissivePrimary(size_t n, const unsigned int* __restrict__ idx, const unsigned int* __restrict__ off, const unsigned int* __restrict__ csr,
    const unsigned int* __restrict__ remap, const unsigned int* __restrict__ wedge, const unsigned char* __restrict__ lock, const unsigned char* __restrict__ kind,
    unsigned char* __restrict__ newkind)
{
	size_t vi = gtid();
	if (vi >= n)
		return;
	unsigned int i = (unsigned int)vi;
	unsigned char k = kind[i];
	newkind[i] = k;
	if (remap[i] != i || (k != kSeam && k != kLocked))
		return;
	bool protect = false;
	unsigned int v = i;
	do
	{
		protect |= lock && (lock[v] & kVertexProtect) != 0;
		v = wedge[v];
	} while (v != i);
	do
	{
		for (unsigned int j = off[v]; j < off[v + 1] && !protect; ++j)
		{
			unsigned int nx, pv;
			cornerNeighbours(idx, csr[j], nx, pv);
			protect |= !hasEdgeWedged(nx, v, idx, off, csr, remap, wedge);
		}
		v = wedge[v];
	} while (v != i);
	newkind[i] = protect ? k : (unsigned char)kComplex;
}

__global__ void kPermissiveWedges(size_t n, const unsigned int* __restrict__ remap, const unsigned char* __restrict__ newkind, unsigned char* kind)
{
	size_t i = gtid();
	if (i >= n)
		return;
	unsigned char k = kind[i];
	kind[i] = (k == kSeam || k == kLocked) ? newkind[remap[i]] : k;
}

// ---------------------------------------------------------------- setup: sparse subset (buildSparseRemap :242-294)

__global__ void kFirstUse(const unsigned int* __restrict__ idx, size_t n, unsigned int* first)
{
	size_t p = gtid();
	if (p < n)
		atomicMin(&first[idx[p]], (unsigned int)p);
}

__global__ void kFirstFlags(const unsigned int* __restrict__ idx, size_t n, const unsigned int* __restrict__ first, unsigned int* __restrict__ flags)
{
	size_t p = gtid();
	if (p < n)
		flags[p] = first[idx[p]] == (unsigned int)p;
}

// dense id of a vertex = rank of its first use among all first uses (order of first appearance)
__global__ void kSparseIds(const unsigned int* __restrict__ idx, size_t n, const unsigned int* __restrict__ first, const unsigned int* __restrict__ rank,
    unsigned int* __restrict__ dense_idx, unsigned int* __restrict__ sparse_remap)
{
	size_t p = gtid();
	if (p >= n)
		return;
	unsigned int v = idx[p];
	unsigned int f = first[v];
	unsigned int d = rank[f];
	dense_idx[p] = d;
	if (f == (unsigned int)p)
		sparse_remap[d] = v;
}

__global__ void kSparseGather(const unsigned int* __restrict__ sparse_remap, size_t u, const float* __restrict__ pos, size_t pstride_f,
    const float* __restrict__ attr, size_t astride_f, size_t acount, const unsigned char* __restrict__ lock, float* __restrict__ pos_out,
    float* __restrict__ attr_out, unsigned char* __restrict__ lock_out)
{
	size_t d = gtid();
	if (d >= u)
		return;
	unsigned int v = sparse_remap[d];
	const float* p = pos + (size_t)v * pstride_f;
	pos_out[d * 3 + 0] = p[0];
	pos_out[d * 3 + 1] = p[1];
	pos_out[d * 3 + 2] = p[2];
	if (attr)
		for (size_t k = 0; k < acount; ++k)
			attr_out[d * acount + k] = attr[(size_t)v * astride_f + k];
	if (lock)
		lock_out[d] = lock[v];
}

// the update mode on a sparse subset: the compact copies (updated in place by the inner run)
// back into the caller's buffers; vertices the solve left alone carry their gathered bits back
__global__ void kSparseScatterBack(const unsigned int* __restrict__ sparse_remap, size_t u, const float* __restrict__ cpos, const float* __restrict__ cattr,
    size_t acount, float* pos, size_t pstride_f, float* attr, size_t astride_f)
{
	size_t d = gtid();
	if (d >= u)
		return;
	unsigned int v = sparse_remap[d];
	float* p = pos + (size_t)v * pstride_f;
	p[0] = cpos[d * 3 + 0];
	p[1] = cpos[d * 3 + 1];
	p[2] = cpos[d * 3 + 2];
	if (attr)
		for (size_t k = 0; k < acount; ++k)
			attr[(size_t)v * astride_f + k] = cattr[d * acount + k];
}

__global__ void kSparseOut(const unsigned int* __restrict__ in, size_t n, const unsigned int* __restrict__ sparse_remap, unsigned int* __restrict__ out)
{
	size_t p = gtid();
	if (p < n)
		out[p] = sparse_remap[in[p]];
}

// ---------------------------------------------------------------- setup: quadrics

// Per primary vertex r, in the order the reference accumulates into vertex_quadrics[r]:
// face quadrics of its faces in face order (fillFaceQuadrics :1057-1082), then the point
// quadric (fillVertexQuadrics :1084-1106), then border/seam edge quadrics in (face, edge,
// i0-then-i1) order (fillEdgeQuadrics :1108-1157). The corners of r's position group in
// increasing order are r's own list (`off/csr`, vertex -> corner lists with corners in
// increasing order) when r is its only wedge, else the merge of its wedges' lists.

// the border/seam edges of face f (vertices tv, kinds tk) that end at r's group, folded into Q
__device__ __forceinline__ void foldEdges(Quadric& Q, unsigned int r, const unsigned int (&tv)[3], const unsigned char (&tk)[3], const float4* __restrict__ pos,
    const unsigned int* __restrict__ remap, const unsigned int* __restrict__ loop, const unsigned int* __restrict__ loopback)
{
#pragma unroll
	for (int ed = 0; ed < 3; ++ed)
	{
		const int ne = ed == 2 ? 0 : ed + 1, pe = ed == 0 ? 2 : ed - 1;
		unsigned int i0 = tv[ed], i1 = tv[ne];
		unsigned char k0 = tk[ed], k1 = tk[ne];
		bool b0 = k0 == kBorder || k0 == kSeam, b1 = k1 == kBorder || k1 == kSeam;
		if (!b0 && !b1)
			continue;
		if (b0 && loop[i0] != i1)
			continue;
		if (b1 && loopback[i1] != i0)
			continue;
		bool to0 = remap[i0] == r, to1 = remap[i1] == r;
		if (!to0 && !to1)
			continue;
		unsigned int i2 = tv[pe];
		float weight = (k0 == kBorder || k1 == kBorder) ? 10.f : 0.5f;
		V3 p0 = ldpos(pos, i0), p1 = ldpos(pos, i1), p2 = ldpos(pos, i2);
		Quadric E = qedge(p0, p1, p2, weight);
		Quadric T = qtriangle(p0, p1, p2, weight);
		T.w = 0;
		qadd(E, T);
		if (to0)
			qadd(Q, E);
		if (to1)
			qadd(Q, E);
	}
}

// the smallest corner above `after` (or any, when first) among the lists of r's wedges; ~0u past
// the last. Each list is sorted, so a binary search per wedge finds its candidate.
__device__ unsigned int nextGroupCorner(unsigned int r, unsigned int after, bool first, const unsigned int* __restrict__ wedge,
    const unsigned int* __restrict__ off, const unsigned int* __restrict__ csr)
{
	unsigned int best = ~0u, v = r;
	do
	{
		unsigned int lo = off[v], hi = off[v + 1];
		while (lo < hi)
		{
			const unsigned int mid = (lo + hi) / 2;
			if (first || csr[mid] > after)
				hi = mid;
			else
				lo = mid + 1;
		}
		if (lo < off[v + 1])
			best = min(best, csr[lo]);
		v = wedge[v];
	} while (v != r);
	return best;
}

__global__ void kFillQuadrics(const unsigned int* __restrict__ idx, const unsigned int* __restrict__ off, const unsigned int* __restrict__ csr, size_t n,
    const float4* __restrict__ pos, const unsigned int* __restrict__ remap, const unsigned int* __restrict__ wedge, const unsigned char* __restrict__ kind,
    const unsigned int* __restrict__ loop, const unsigned int* __restrict__ loopback, const unsigned char* __restrict__ lock, float factor,
    Quadric* __restrict__ vq, float4* __restrict__ vg)
{
	size_t vi = gtid();
	if (vi >= n)
		return;
	unsigned int r = (unsigned int)vi;
	if (remap[r] != r)
	{
		stquadric(vq, r, qzero());
		if (vg)
			vg[r] = make_float4(0.f, 0.f, 0.f, 0.f);
		return;
	}
	const bool single = wedge[r] == r;
	unsigned int b = off[r], e = off[r + 1];
	Quadric Q = qzero();
	float4 G = make_float4(0.f, 0.f, 0.f, 0.f); // volume gradient (update mode with attributes), the same face order
	if (single)
	{
		// corners in groups of kFillBatch: the group's loads are issued together (past the end the
		// last corner is loaded again), then its faces fold in corner order
		for (unsigned int j = b; j < e; j += kFillBatch)
		{
			uint3 t[kFillBatch];
#pragma unroll
			for (unsigned int q = 0; q < kFillBatch; ++q)
			{
				unsigned int f = csr[min(j + q, e - 1)] / 3;
				t[q] = make_uint3(idx[f * 3 + 0], idx[f * 3 + 1], idx[f * 3 + 2]);
			}
			V3 p[kFillBatch][3];
#pragma unroll
			for (unsigned int q = 0; q < kFillBatch; ++q)
			{
				p[q][0] = ldpos(pos, t[q].x);
				p[q][1] = ldpos(pos, t[q].y);
				p[q][2] = ldpos(pos, t[q].z);
			}
#pragma unroll
			for (unsigned int q = 0; q < kFillBatch; ++q)
				if (j + q < e)
				{
					Quadric F = qtriangle(p[q][0], p[q][1], p[q][2], 1.f);
					qadd(Q, F);
					if (vg)
						gadd(G, qvolumeGrad(p[q][0], p[q][1], p[q][2]));
				}
		}
	}
	else
	{
		// a group of several wedges (rare): its corners one at a time, merged from the wedges' lists
		for (unsigned int c = nextGroupCorner(r, 0, true, wedge, off, csr); c != ~0u; c = nextGroupCorner(r, c, false, wedge, off, csr))
		{
			const unsigned int f = c / 3;
			const V3 p0 = ldpos(pos, idx[f * 3 + 0]), p1 = ldpos(pos, idx[f * 3 + 1]), p2 = ldpos(pos, idx[f * 3 + 2]);
			Quadric F = qtriangle(p0, p1, p2, 1.f);
			qadd(Q, F);
			if (vg)
				gadd(G, qvolumeGrad(p0, p1, p2));
		}
	}
	if (vg)
		vg[r] = G;
	bool priority = lock && (lock[r] & kVertexPriority) != 0;
	float w = Q.w * (priority ? 1.0f : factor);
	V3 p = ldpos(pos, r);
	Quadric P = qpoint(p.x, p.y, p.z, w);
	qadd(Q, P);
	// edge quadrics need an open edge at the vertex or a wedge of it: a manifold vertex is a
	// single wedge with no open edge (kinds only move away from manifold after classification)
	if (kind[r] == kManifold)
	{
		stquadric(vq, r, Q);
		return;
	}

	// a face shows up once per corner it has in the group: its edges fold in once
	unsigned int lastf = ~0u;
	if (single)
	{
		for (unsigned int j = b; j < e; j += kFillBatch)
		{
			unsigned int fs[kFillBatch];
			unsigned int tv[kFillBatch][3];
			unsigned char tk[kFillBatch][3];
#pragma unroll
			for (unsigned int q = 0; q < kFillBatch; ++q)
			{
				fs[q] = csr[min(j + q, e - 1)] / 3;
#pragma unroll
				for (int c = 0; c < 3; ++c)
					tv[q][c] = idx[fs[q] * 3 + c];
			}
#pragma unroll
			for (unsigned int q = 0; q < kFillBatch; ++q)
#pragma unroll
				for (int c = 0; c < 3; ++c)
					tk[q][c] = kind[tv[q][c]];
#pragma unroll
			for (unsigned int q = 0; q < kFillBatch; ++q)
			{
				if (j + q >= e || fs[q] == lastf)
					continue;
				lastf = fs[q];
				foldEdges(Q, r, tv[q], tk[q], pos, remap, loop, loopback);
			}
		}
	}
	else
	{
		for (unsigned int c = nextGroupCorner(r, 0, true, wedge, off, csr); c != ~0u; c = nextGroupCorner(r, c, false, wedge, off, csr))
		{
			const unsigned int f = c / 3;
			if (f == lastf)
				continue;
			lastf = f;
			const unsigned int tv[3] = {idx[f * 3 + 0], idx[f * 3 + 1], idx[f * 3 + 2]};
			const unsigned char tk[3] = {kind[tv[0]], kind[tv[1]], kind[tv[2]]};
			foldEdges(Q, r, tv, tk, pos, remap, loop, loopback);
		}
	}
	stquadric(vq, r, Q);
}

// rescaleAttributes :605-621 (zero-weight attributes already dropped on the host)
struct AttrMap
{
	unsigned int src[kMaxAttributes];
	float weight[kMaxAttributes];
	int count;
};

__global__ void kRescaleAttributes(const float* __restrict__ data, size_t stride_f, size_t n, AttrMap am, float* __restrict__ out)
{
	size_t i = gtid();
	if (i >= n)
		return;
	for (int k = 0; k < am.count; ++k)
		out[i * am.count + k] = data[i * stride_f + am.src[k]] * am.weight[k];
}

// fillAttributeQuadrics :1159-1179 per raw vertex v over its faces in face order
template <int MAXA>
__global__ void kFillAttributeQuadrics(const unsigned int* __restrict__ idx, const unsigned int* __restrict__ off, const unsigned int* __restrict__ csr,
    size_t n, const float4* __restrict__ pos, const float* __restrict__ attr, int count, Quadric* __restrict__ aq, float4* __restrict__ ag)
{
	size_t vi = gtid();
	if (vi >= n)
		return;
	unsigned int v = (unsigned int)vi;
	Quadric Q = qzero();
	float4 G[MAXA];
#pragma unroll
	for (int k = 0; k < MAXA; ++k)
		G[k] = make_float4(0.f, 0.f, 0.f, 0.f);
	// up to 8 attributes: two faces' loads (positions and attributes into registers) are issued
	// together, then the two fold in corner order; wider attribute sets go one face at a time
	constexpr unsigned int B = MAXA <= 8 ? 2 : 1;
	const unsigned int b = off[v], e = off[v + 1];
	for (unsigned int j = b; j < e; j += B)
	{
		uint3 t[B];
#pragma unroll
		for (unsigned int q = 0; q < B; ++q)
		{
			unsigned int f = csr[min(j + q, e - 1)] / 3;
			t[q] = make_uint3(idx[f * 3 + 0], idx[f * 3 + 1], idx[f * 3 + 2]);
		}
		if constexpr (MAXA <= 8)
		{
			V3 p[B][3];
			float at[B][3][MAXA];
#pragma unroll
			for (unsigned int q = 0; q < B; ++q)
			{
				const unsigned int tc[3] = {t[q].x, t[q].y, t[q].z};
#pragma unroll
				for (int c = 0; c < 3; ++c)
				{
					p[q][c] = ldpos(pos, tc[c]);
#pragma unroll
					for (int k = 0; k < MAXA; ++k)
						at[q][c][k] = k < count ? __ldg(attr + (size_t)tc[c] * count + k) : 0.f;
				}
			}
#pragma unroll
			for (unsigned int q = 0; q < B; ++q)
				if (j + q < e)
					addAttributeQuadric<MAXA>(Q, G, count, p[q][0], p[q][1], p[q][2], at[q][0], at[q][1], at[q][2]);
		}
		else
			addAttributeQuadric<MAXA>(Q, G, count, ldpos(pos, t[0].x), ldpos(pos, t[0].y), ldpos(pos, t[0].z), attr + (size_t)t[0].x * count,
			    attr + (size_t)t[0].y * count, attr + (size_t)t[0].z * count);
	}
	stquadric(aq, v, Q);
#pragma unroll
	for (int k = 0; k < MAXA; ++k)
		if (k < count)
			ag[(size_t)v * count + k] = G[k];
}

// boundEdgeCollapses :1292-1308 numerator: sum of degrees of manifold and seam vertices (one
// global add per block: the adds all go to one address)
__global__ void __launch_bounds__(kThreads) kDualCount(const unsigned int* __restrict__ off, const unsigned char* __restrict__ kind, size_t n,
    unsigned long long* dual)
{
	__shared__ unsigned int wsum[kThreads / 32];
	size_t i = gtid();
	unsigned int d = 0;
	if (i < n)
	{
		unsigned char k = kind[i];
		d = (k == kManifold || k == kSeam) ? (off[i + 1] - off[i]) : 0;
	}
	for (int o = 16; o > 0; o >>= 1)
		d += __shfl_down_sync(0xffffffffu, d, o);
	if ((threadIdx.x & 31) == 0)
		wsum[threadIdx.x >> 5] = d;
	__syncthreads();
	if (threadIdx.x == 0)
	{
		unsigned long long b = 0;
		for (int q = 0; q < kThreads / 32; ++q)
			b += wsum[q];
		if (b)
			atomicAdd(dual, b);
	}
}

__global__ void kCapacity(size_t index_count, Scalars* sc)
{
	if (threadIdx.x == 0 && blockIdx.x == 0)
		sc->capacity = (unsigned int)((index_count - sc->dual / 2) + 3);
}

// ---------------------------------------------------------------- pass: adjacency

// corners per vertex of the current index buffer, welded by remap; each corner keeps the count
// before it as its slot in its vertex's list, so the fill below needs no atomics. lv: the live
// pass's buffer and count, and the slots go to its next buffer (free until the compaction)
__global__ void kCountCorners(const unsigned int* __restrict__ res, size_t n, const unsigned int* __restrict__ remap, unsigned int* __restrict__ cnt,
    unsigned int* __restrict__ slot, const PassLive* lv)
{
	if (lv)
	{
		if (lv->stop)
			return;
		res = lv->res;
		n = lv->indices;
		slot = lv->res_next;
	}
	const size_t i = gtid();
	if (i - (threadIdx.x & 31) >= n)
		return; // the whole warp is past the corners
	// corners of the same vertex among the warp's 32 (neighbouring triangles share vertices) take
	// their slots with one atomic add; a list's order is arbitrary anyway
	const unsigned int lane = threadIdx.x & 31;
	const bool valid = i < n;
	const unsigned int v = valid ? remap[res[i]] : ~0u;
	// lanes past the end share a key and are masked out of every group
	const unsigned int peers = __match_any_sync(0xffffffffu, v) & __ballot_sync(0xffffffffu, valid);
	const unsigned int leader = __ffs(peers) - 1;
	unsigned int base = 0;
	if (valid && lane == leader)
		base = atomicAdd(&cnt[v], __popc(peers));
	base = __shfl_sync(0xffffffffu, base, leader);
	if (valid)
		slot[i] = base + __popc(peers & ((1u << lane) - 1u));
}

// half-edges {next, prev} of every vertex in its list (the order within a list is arbitrary: the
// flip test and the one-ring checks do not depend on it)
__global__ void kAdjFill(const unsigned int* __restrict__ res, size_t tris, const unsigned int* __restrict__ remap, const unsigned int* __restrict__ off,
    const unsigned int* __restrict__ slot, uint2* __restrict__ adj, const PassLive* lv, size_t adj_cap)
{
	if (lv)
	{
		if (lv->stop)
			return;
		res = lv->res;
		tris = lv->tris;
		slot = lv->res_next;
	}
	size_t t = gtid();
	if (t >= tris)
		return;
	const unsigned int v[3] = {remap[res[t * 3 + 0]], remap[res[t * 3 + 1]], remap[res[t * 3 + 2]]};
#pragma unroll
	for (int c = 0; c < 3; ++c)
	{
		const size_t at = size_t(off[v[c]]) + slot[t * 3 + c];
		if (at < adj_cap) // in range whenever the offsets' scan completed
			adj[at] = make_uint2(v[c == 2 ? 0 : c + 1], v[c == 0 ? 2 : c - 1]);
	}
}

// ---------------------------------------------------------------- pass: pick

// pickEdgeCollapses :1323-1368 for edge e of one triangle; returns false if not a candidate
__device__ __forceinline__ bool pickEdge(unsigned int i0, unsigned int i1, const unsigned int* __restrict__ remap, const unsigned char* __restrict__ kind,
    const unsigned int* __restrict__ loop, const unsigned int* __restrict__ loopback, unsigned int& v0, unsigned int& v1, unsigned int& bidi)
{
	unsigned int r0 = remap[i0], r1 = remap[i1];
	if (r0 == r1)
		return false;
	unsigned int k0 = kind[i0], k1 = kind[i1];
	bool c01 = canCollapse(k0, k1), c10 = canCollapse(k1, k0);
	if (!(c01 | c10))
		return false;
	if (hasOpposite(k0, k1) && r1 > r0)
		return false;
	if ((k0 == kBorder || k0 == kSeam) && k1 != kManifold && loop[i0] != i1)
		return false;
	if ((k1 == kBorder || k1 == kSeam) && k0 != kManifold && loopback[i1] != i0)
		return false;
	if (c01 & c10)
	{
		v0 = i0, v1 = i1, bidi = 1;
	}
	else
	{
		v0 = c01 ? i0 : i1;
		v1 = c01 ? i1 : i0;
		bidi = 0;
	}
	return true;
}

// a triangle's picked edges as 3 bits each (bit 0: a candidate, bit 1: bidirectional, bit 2:
// from the edge's second vertex), so the emit needs no vertex gathers
__device__ __forceinline__ unsigned int pickCode(const unsigned int a[3], const unsigned int* __restrict__ remap, const unsigned char* __restrict__ kind,
    const unsigned int* __restrict__ loop, const unsigned int* __restrict__ loopback)
{
	unsigned int code = 0;
#pragma unroll
	for (int e = 0; e < 3; ++e)
	{
		unsigned int v0, v1, bd;
		if (pickEdge(a[e], a[e == 2 ? 0 : e + 1], remap, kind, loop, loopback, v0, v1, bd))
			code |= (1u | (bd << 1) | ((v0 != a[e]) << 2)) << (3 * e);
	}
	return code;
}

// candidates per block of kThreads triangles (the scan runs over blocks, not triangles) and
// each triangle's pick code. lv: counts of the live pass; the grid covers the first pass's
// triangles and blocks past the live count write zero, so the scan over the full range is the
// scan of the live one
__global__ void __launch_bounds__(kThreads) kPickCount(const unsigned int* __restrict__ res, size_t tris, const unsigned int* __restrict__ remap,
    const unsigned char* __restrict__ kind, const unsigned int* __restrict__ loop, const unsigned int* __restrict__ loopback,
    unsigned int* __restrict__ bcnt, unsigned short* __restrict__ codes, const PassLive* lv)
{
	__shared__ unsigned int sm[kThreads / 32 + 1];
	if (lv)
	{
		if (lv->stop)
			return;
		res = lv->res;
		tris = lv->tris;
	}
	const size_t t = gtid();
	unsigned int c = 0;
	if (t < tris)
	{
		const unsigned int a[3] = {res[t * 3 + 0], res[t * 3 + 1], res[t * 3 + 2]};
		const unsigned int code = pickCode(a, remap, kind, loop, loopback);
		codes[t] = (unsigned short)code;
		c = __popc(code & 0x49u);
	}
	unsigned int total;
	blockExclusiveScan<kThreads>(c, sm, &total);
	if (threadIdx.x == 0)
		bcnt[blockIdx.x] = total;
}

// emits the candidates of every triangle whose prefix leaves room for three more
// (the capacity check at :1319-1320 stops at the first triangle that does not); a triangle's
// prefix is its block's scanned count plus the block-local prefix
__global__ void __launch_bounds__(kThreads) kPickEmit(const unsigned int* __restrict__ res, size_t tris, const unsigned short* __restrict__ codes,
    const unsigned int* __restrict__ boffs, Scalars* sc, uint4* __restrict__ crec, const PassLive* lv)
{
	__shared__ unsigned int sm[kThreads / 32 + 1];
	if (lv)
	{
		if (lv->stop)
			return;
		res = lv->res;
		tris = lv->tris;
	}
	const size_t t = gtid();
	const unsigned int code = t < tris ? codes[t] : 0u;
	unsigned int total;
	const unsigned int pre = blockExclusiveScan<kThreads>(__popc(code & 0x49u), sm, &total);
	if (t >= tris)
		return;
	unsigned int o = boffs[blockIdx.x] + pre;
	if ((size_t)o + 3 > sc->capacity)
	{
		atomicMin(&sc->pick_trunc, o);
		return;
	}
	const unsigned int a[3] = {res[t * 3 + 0], res[t * 3 + 1], res[t * 3 + 2]};
#pragma unroll
	for (int e = 0; e < 3; ++e)
	{
		const unsigned int f = (code >> (3 * e)) & 7u;
		if (f & 1u)
		{
			const unsigned int x = a[e], y = a[e == 2 ? 0 : e + 1];
			crec[o++] = (f & 4u) ? make_uint4(y, x, 0u, 0u) : make_uint4(x, y, (f >> 1) & 1u, 0u);
		}
	}
}

// ---------------------------------------------------------------- pass: rank

#ifndef MO_RANK_THREADS
#define MO_RANK_THREADS 256
#endif
constexpr unsigned int kRankThreads = MO_RANK_THREADS; // threads per block of kRank (one candidate each)

// rankEdgeCollapses :1374-1450, one candidate per thread. The candidate {v0, v1, bidi} becomes,
// in place, {i0, i1, error bits, kind of i0} with the cheaper direction first; its decision
// record {r0, r1, begin and end of r0's adjacency}, its error bits and its kind are written
// beside it. Candidates stay in pick (triangle) order from here on: the sort only gives each
// its sorted position, and the decision rounds walk pick order, where neighbouring candidates
// share vertices.
__global__ void kRank(size_t count, uint4* __restrict__ crec, uint4* __restrict__ cring, unsigned int* __restrict__ cerr, unsigned char* __restrict__ ckind,
    const float4* __restrict__ pos, const Quadric* __restrict__ vq, const unsigned int* __restrict__ remap, const unsigned int* __restrict__ wedge,
    const unsigned char* __restrict__ kind, const unsigned int* __restrict__ loop, const unsigned int* __restrict__ loopback,
    const unsigned int* __restrict__ adj_off, const float* __restrict__ attr, const Quadric* __restrict__ aq, const float4* __restrict__ ag, int ac,
    const PassLive* lv)
{
	if (lv)
	{
		if (lv->stop)
			return;
		count = lv->count;
	}
	size_t c = gtid();
	if (c >= count)
		return;
	const uint4 cand = crec[c];
	const unsigned int i0 = cand.x, i1 = cand.y;
	const bool bidi = cand.z != 0;
	const unsigned int ra = remap[i0], rb = remap[i1];
	V3 p0 = ldpos(pos, i0), p1 = ldpos(pos, i1);

	float ei = qerror(ldquadric(vq, ra), p1);
	float ej = bidi ? qerror(ldquadric(vq, rb), p0) : FLT_MAX;

	if (ac)
	{
		ei += qerrorAttr(ldquadric(aq, i0), ag + (size_t)i0 * ac, ac, p1, attr + (size_t)i1 * ac);
		ej += bidi ? qerrorAttr(ldquadric(aq, i1), ag + (size_t)i1 * ac, ac, p0, attr + (size_t)i0 * ac) : 0;

		if (kind[i0] == kSeam)
		{
			unsigned int s0 = wedge[i0];
			unsigned int s1 = loop[i0] == i1 ? loopback[s0] : loop[s0];
			s1 = (s1 != ~0u) ? s1 : wedge[i1];
			V3 ps0 = ldpos(pos, s0), ps1 = ldpos(pos, s1);
			ei += qerrorAttr(ldquadric(aq, s0), ag + (size_t)s0 * ac, ac, ps1, attr + (size_t)s1 * ac);
			ej += bidi ? qerrorAttr(ldquadric(aq, s1), ag + (size_t)s1 * ac, ac, ps0, attr + (size_t)s0 * ac) : 0;
		}
		else
		{
			if (kind[i0] == kComplex)
				for (unsigned int v = wedge[i0]; v != i0; v = wedge[v])
				{
					unsigned int t = complexTarget(v, i1, remap, loop, loopback);
					ei += qerrorAttr(ldquadric(aq, v), ag + (size_t)v * ac, ac, ldpos(pos, t), attr + (size_t)t * ac);
				}
			if (kind[i1] == kComplex && bidi)
				for (unsigned int v = wedge[i1]; v != i1; v = wedge[v])
				{
					unsigned int t = complexTarget(v, i0, remap, loop, loopback);
					ej += qerrorAttr(ldquadric(aq, v), ag + (size_t)v * ac, ac, ldpos(pos, t), attr + (size_t)t * ac);
				}
		}
	}

	const bool rev = bidi & (ej < ei);
	const unsigned int s0 = rev ? i1 : i0, s1 = rev ? i0 : i1;
	const unsigned int r0 = rev ? rb : ra, r1 = rev ? ra : rb;
	float err = ej < ei ? ej : ei;
	unsigned int bits = __float_as_uint(err);
	const unsigned char ks = kind[s0];
	crec[c] = make_uint4(s0, s1, bits, ks);
	cring[c] = make_uint4(r0, r1, adj_off[r0], adj_off[r0 + 1]);
	cerr[c] = bits;
	ckind[c] = ks;
}

// ---------------------------------------------------------------- pass: sort
//
// sortEdgeCollapses (:1452-1496) is a stable counting sort on the 12-bit key of each candidate's
// error (2560 bins). It runs as one here: a 2560-bin histogram per tile of candidates, one
// exclusive scan over the bin-major histogram matrix (which gives, for every tile and bin, the
// sorted position of the tile's first candidate with that key), and a stable scatter. The
// scatter gives each candidate its sorted position (rank, in pick order) and writes, at that
// position, the error bits and kind that the stop rules read in sorted order. The matrix has one
// column per live tile (its row stride is the live tile count), so its scan covers the live
// candidates only.
constexpr unsigned int kKeyBins = 2560;
constexpr unsigned int kKeyWarps = kThreads / 32;
constexpr size_t kKeyScatterSmem = kKeyBins * sizeof(unsigned int) + size_t(kKeyWarps) * kKeyBins * sizeof(unsigned short);

// candidates per thread of a sort tile, by the largest count the sort sees: small counts take
// small tiles (more blocks for a short sort), large ones 4096-candidate tiles (a smaller matrix)
inline unsigned int keySortItems(size_t n)
{
	return n <= (size_t(1) << 19) ? 4u : (n <= (size_t(1) << 21) ? 8u : 16u);
}

__host__ __device__ inline unsigned int keySortTiles(size_t n, unsigned int items)
{
	const size_t tile = size_t(items) * kThreads;
	return unsigned((n + tile - 1) / tile);
}

// scratch words of sortCandidates for any count up to n and any tile: the histogram matrix (at
// most one column per 1024 candidates) and its scan
size_t keySortScratchWords(size_t n)
{
	const size_t m = std::max<size_t>(keySortTiles(n, 4), 1) * kKeyBins;
	return ((m + 63) & ~size_t(63)) + scanScratchWords(m);
}

template <unsigned int ITEMS>
__global__ void __launch_bounds__(kThreads) kKeyHist(const unsigned int* __restrict__ cerr, size_t n, unsigned int* __restrict__ hist, const PassLive* lv)
{
	__shared__ unsigned int sh[kKeyBins];
	if (lv)
	{
		if (lv->stop)
			return;
		n = lv->count;
	}
	const unsigned int tiles = keySortTiles(n, ITEMS);
	if (blockIdx.x >= tiles)
		return;
	for (unsigned int b = threadIdx.x; b < kKeyBins; b += kThreads)
		sh[b] = 0;
	__syncthreads();
	const size_t t0 = (size_t)blockIdx.x * ITEMS * kThreads + threadIdx.x;
	unsigned int kb[ITEMS];
#pragma unroll
	for (unsigned int q = 0; q < ITEMS; ++q)
	{
		const size_t i = t0 + (size_t)q * kThreads;
		kb[q] = i < n ? sortKey(__ldg(cerr + i)) : kKeyBins;
	}
#pragma unroll
	for (unsigned int q = 0; q < ITEMS; ++q)
		if (kb[q] < kKeyBins)
			atomicAdd(&sh[kb[q]], 1u);
	__syncthreads();
	for (unsigned int b = threadIdx.x; b < kKeyBins; b += kThreads)
		hist[(size_t)b * tiles + blockIdx.x] = sh[b];
}

// Stable scatter of one tile. Warp w takes the tile's 32 * ITEMS consecutive candidates from
// w * 32 * ITEMS on, 32 at a time in order; equal keys among the 32 are ranked by lane
// (match_any) against per-warp key counters, and each candidate keeps its key and its rank within
// the warp in registers. The warp counters of each key are then turned into offsets in warp
// order, and every candidate is placed after the earlier ones of its key: equal keys keep pick
// order, as the reference's counting sort keeps collapse order.
template <unsigned int ITEMS>
__global__ void __launch_bounds__(kThreads) kKeyScatter(const unsigned int* __restrict__ cerr, const unsigned char* __restrict__ ckind, size_t n,
    const unsigned int* __restrict__ hist, unsigned int* __restrict__ rank, unsigned int* __restrict__ serr, unsigned char* __restrict__ skind,
    const PassLive* lv)
{
	extern __shared__ __align__(16) unsigned char key_smem[];
	unsigned int* gbase = reinterpret_cast<unsigned int*>(key_smem);               // sorted position of the tile's first candidate per key
	unsigned short* wcnt = reinterpret_cast<unsigned short*>(gbase + kKeyBins);   // per warp and key: count, then offset in the tile
	if (lv)
	{
		if (lv->stop)
			return;
		n = lv->count;
	}
	const unsigned int tiles = keySortTiles(n, ITEMS);
	if (blockIdx.x >= tiles)
		return;
	const size_t tile0 = (size_t)blockIdx.x * ITEMS * kThreads;
	const unsigned int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const size_t w0 = tile0 + (size_t)w * 32 * ITEMS + lane;
	unsigned int eb[ITEMS];
#pragma unroll
	for (unsigned int q = 0; q < ITEMS; ++q)
	{
		const size_t i = w0 + (size_t)q * 32;
		eb[q] = i < n ? __ldg(cerr + i) : 0u;
	}
	for (unsigned int b = threadIdx.x; b < kKeyBins; b += kThreads)
	{
		gbase[b] = hist[(size_t)b * tiles + blockIdx.x];
#pragma unroll
		for (unsigned int q = 0; q < kKeyWarps; ++q)
			wcnt[q * kKeyBins + b] = 0;
	}
	__syncthreads();
	unsigned short* mine = wcnt + w * kKeyBins;
	unsigned short rk[ITEMS]; // rank among the warp's candidates of the same key
#pragma unroll
	for (unsigned int q = 0; q < ITEMS; ++q)
	{
		const bool valid = w0 + (size_t)q * 32 < n;
		const unsigned int key = valid ? sortKey(eb[q]) : kKeyBins + lane;
		const unsigned int peers = __match_any_sync(0xffffffffu, key);
		const unsigned int leader = __ffs(peers) - 1;
		unsigned int before = 0;
		if (valid && lane == leader)
		{
			before = mine[key];
			mine[key] = (unsigned short)(before + __popc(peers));
		}
		before = __shfl_sync(0xffffffffu, before, leader);
		rk[q] = (unsigned short)(before + __popc(peers & ((1u << lane) - 1u)));
		__syncwarp();
	}
	__syncthreads();
	for (unsigned int b = threadIdx.x; b < kKeyBins; b += kThreads)
	{
		unsigned int run = 0;
#pragma unroll
		for (unsigned int q = 0; q < kKeyWarps; ++q)
		{
			const unsigned int c = wcnt[q * kKeyBins + b];
			wcnt[q * kKeyBins + b] = (unsigned short)run;
			run += c;
		}
	}
	__syncthreads();
#pragma unroll
	for (unsigned int q = 0; q < ITEMS; ++q)
	{
		const size_t i = w0 + (size_t)q * 32;
		if (i < n)
		{
			const unsigned int key = sortKey(eb[q]);
			const unsigned int pos = gbase[key] + mine[key] + rk[q];
			rank[i] = pos;
			if (pos < n) // in range whenever the histogram scan completed
			{
				serr[pos] = eb[q];
				skind[pos] = __ldg(ckind + i);
			}
		}
	}
}

// ---------------------------------------------------------------- pass: perform
//
// kPerform runs, in one cooperative launch per pass, everything from the ranked candidates to
// the next pass's index buffer: the decision rounds (performEdgeCollapses :1498-1636 made
// order-free), the stop rules as a prefix scan over sorted order, the collapse_remap writes and
// quadric merges of the committed prefix (:1574-1616, updateQuadrics :1638-1673), the loop remap
// (:1845-1864) and the order-preserving index compaction (:1811-1843). Phases are separated by
// grid barriers (mo_grid.cuh); data written by other blocks in an earlier phase is read through
// L2 (ld.global.cg).
//
// Candidates are identified by their sorted position k (the serial order of the reference's
// loop), but the rounds visit them in pick order c, where k = rank[c]: pick order follows the
// index buffer, so the candidates a warp takes share vertices, and their per-vertex gathers and
// mark atomics fall on a few cache sectors instead of one each.

__device__ __forceinline__ unsigned long long roundTag(unsigned int round)
{
	return (unsigned long long)(0xFFFFFFFFu - round) << 32;
}

__device__ __forceinline__ bool earlierThan(unsigned long long v, unsigned long long tag, unsigned int k)
{
	return (v >> 32) == (tag >> 32) && (unsigned int)v < k;
}

struct PerformArgs
{
	// candidates in pick order: {i0, i1, error bits, kind of i0}, {r0, r1, adjacency range of r0}
	// and the sorted position of each
	unsigned int count;
	const uint4* crec;
	const uint4* cring;
	const unsigned int* rank;
	// by sorted position
	const unsigned char* skind;
	const unsigned int* serr;
	unsigned char* status;
	// per-vertex decision state, marks alternating by round parity (a mark is the round's tag in the
	// high word and the candidate's sorted position in the low word; later rounds have smaller tags):
	//  * minT[p][v]: the earliest undecided candidate with endpoint v; 0 once a commit took v;
	//  * minS[2 v + p]: the earliest undecided candidate that moves v; once a commit moved v, the
	//    pair holds {that commit's sorted position, v's target}, both with tag 0.
	// Every pass starts by setting both to ~0 for all vertices.
	unsigned int vcount;
	unsigned long long* minT[2];
	unsigned long long* minS;
	unsigned int* cr;
	unsigned int* list[2];     // undecided candidates (pick order), one region per block
	unsigned int* commits;     // committed candidates (pick order), one region per block
	// mesh
	const unsigned int* adj_off;
	const uint2* adj;
	const float4* pos;
	const unsigned int* remap;
	const unsigned int* wedge;
	unsigned int* loop;
	unsigned int* loopback;
	Quadric* vq;
	Quadric* aq;
	float4* ag;
	int ac;
	float4* vg; // volume gradients (update mode with attributes), else nullptr
	// stop rules
	unsigned int prev_err_bits;
	float error_limit;
	unsigned long long goal;
	unsigned int first_window;
	unsigned int round_base;
	// compaction
	const unsigned int* res;
	unsigned int* res_next;
	unsigned int tris;
	uint4* blk;
	Scalars* sc;
	// device-resident pass loop (else nullptr): count, goal, first_window, round_base, tris, res,
	// res_next and the previous result error come from here instead of the fields above
	const PassLive* live;
};

// Decision rule: candidate k is decided once nothing earlier in sorted order can change its
// outcome:
//  * an earlier candidate already committed on one of its endpoints -> locked (final: any
//    commit seen on an endpoint has a smaller sorted position);
//  * otherwise it waits until it is the earliest undecided candidate on both endpoints (minT)
//    and no undecided earlier candidate moves a vertex of its one-ring (minS); then the flip
//    test runs against the one-ring as moved by earlier commits only (moving commit < k).

// the commit of a decided candidate: r0 moves to its target and both endpoints lock
__device__ __forceinline__ void commitOne(const PerformArgs& a, unsigned int c, unsigned int k, unsigned int r0, unsigned int r1)
{
	const uint4 cd = __ldg(a.crec + c);
	const unsigned int i0 = cd.x, i1 = cd.y;
	const unsigned char kd = (unsigned char)cd.w;
	unsigned int target;
	if (kd == kComplex)
		target = complexTarget(r0, i1, a.remap, a.loop, a.loopback);
	else if (kd == kSeam)
	{
		unsigned int s0 = a.wedge[i0];
		unsigned int s1 = a.loop[i0] == i1 ? a.loopback[s0] : a.loop[s0];
		s1 = (s1 != ~0u) ? s1 : a.wedge[i1];
		target = (s0 == r0) ? s1 : i1;
	}
	else
		target = i1;
	*reinterpret_cast<ulonglong2*>(a.minS + 2 * (size_t)r0) = make_ulonglong2(k, target);
	a.minT[0][r0] = 0;
	a.minT[1][r0] = 0;
	a.minT[0][r1] = 0;
	a.minT[1][r1] = 0;
	a.status[k] = kCommit;
}

// The rule runs in three stages per round, each over the candidates the stage before left (so
// lanes stay busy): the endpoint marks (in the rounds loop); one walk over the one-ring
// (ringDecide) for the waits, the flip test and the commit; and last the candidates that still
// wait: locked at once if a commit of this round took an endpoint, else marked for the next round.

#ifndef MO_RING_BATCH
#define MO_RING_BATCH 2
#endif

enum
{
	kRingWaits = 0,
	kRingFlip = 1,
	kRingCommit = 2,
};

// One walk over the one-ring of r0. If an undecided earlier candidate moves a vertex of it, the
// candidate waits. Otherwise the flip test (hasTriangleFlips :1201-1232) sees the one-ring as
// moved by earlier commits only, and the candidate is rejected or commits. The whole ring is
// checked for waits before a flip decides anything: a wait means an earlier decision is still
// open that may move a vertex the test reads.
__device__ __forceinline__ int ringDecide(const PerformArgs& a, unsigned int c, unsigned int k, const uint4& rec, unsigned int round)
{
	const unsigned int r0 = rec.x, r1 = rec.y, b = rec.z, e = rec.w;
	const unsigned long long tag = roundTag(round);
	const unsigned int p = round & 1;
	const V3 v0 = ldpos(a.pos, r0), v1 = ldpos(a.pos, r1);
	bool flip = false;
	constexpr int FB = MO_RING_BATCH;
	for (unsigned int j = b; j < e; j += FB)
	{
		uint2 ed[FB];
		ulonglong2 sx[FB], sy[FB];
		float4 px[FB], py[FB];
#pragma unroll
		for (int q = 0; q < FB; ++q)
		{
			ed[q] = j + q < e ? __ldg(a.adj + j + q) : make_uint2(r1, r1); // r1 is in the ring already
			sx[q] = __ldcg(reinterpret_cast<const ulonglong2*>(a.minS) + ed[q].x);
			sy[q] = __ldcg(reinterpret_cast<const ulonglong2*>(a.minS) + ed[q].y);
			px[q] = __ldg(a.pos + ed[q].x);
			py[q] = __ldg(a.pos + ed[q].y);
		}
		bool wait = false;
#pragma unroll
		for (int q = 0; q < FB; ++q)
			wait |= earlierThan(p ? sx[q].y : sx[q].x, tag, k) | earlierThan(p ? sy[q].y : sy[q].x, tag, k);
		if (wait)
			return kRingWaits;
		if (flip)
			continue;
#pragma unroll
		for (int q = 0; q < FB; ++q)
		{
			// moved by an earlier commit: the pair holds {commit, target} with tag 0
			const bool mvx = (sx[q].x >> 32) == 0 && (unsigned int)sx[q].x < k;
			const bool mvy = (sy[q].x >> 32) == 0 && (unsigned int)sy[q].x < k;
			const unsigned int va = mvx ? (unsigned int)sx[q].y : ed[q].x;
			const unsigned int vb = mvy ? (unsigned int)sy[q].y : ed[q].y;
			if (va == r1 || vb == r1 || va == vb)
				continue;
			const V3 pa = mvx ? ldpos(a.pos, va) : V3{px[q].x, px[q].y, px[q].z};
			const V3 pb = mvy ? ldpos(a.pos, vb) : V3{py[q].x, py[q].y, py[q].z};
			flip |= triFlip(pa, pb, v0, v1);
		}
	}
	if (flip)
	{
		a.status[k] = kSkipFlip;
		return kRingFlip;
	}
	commitOne(a, c, k, r0, r1);
	return kRingCommit;
}

__device__ __forceinline__ void markCandidate(const PerformArgs& a, unsigned int k, const uint4& rec, unsigned int round)
{
	unsigned long long key = roundTag(round) | k;
	atomicMin(&a.minT[round & 1][rec.x], key);
	atomicMin(&a.minT[round & 1][rec.y], key);
	atomicMin(&a.minS[2 * (size_t)rec.x + (round & 1)], key);
}

// per sorted candidate: triangles removed if committed, flip rejection, committed error
__device__ __forceinline__ void stopTerms(unsigned char st, unsigned char kd, unsigned int errbits, unsigned int& tri, unsigned int& flip, unsigned int& errc)
{
	bool commit = st == kCommit;
	tri = commit ? (kd == kBorder ? 1u : 2u) : 0u;
	flip = st == kSkipFlip;
	float e = __uint_as_float(errbits);
	errc = (commit && e == e) ? errbits : 0u; // NaN never raises result_error
}

// block-wide exclusive scan of (sum, sum, max) triples; returns the block totals
__device__ __forceinline__ uint3 blockScan3(unsigned int& t, unsigned int& f, unsigned int& m, unsigned int (*sm)[33])
{
	unsigned int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	unsigned int it = t, iff = f, im = m;
	for (int o = 1; o < 32; o <<= 1)
	{
		unsigned int x = __shfl_up_sync(0xffffffffu, it, o), y = __shfl_up_sync(0xffffffffu, iff, o), z = __shfl_up_sync(0xffffffffu, im, o);
		if (lane >= (unsigned)o)
			it += x, iff += y, im = max(im, z);
	}
	unsigned int pm = __shfl_up_sync(0xffffffffu, im, 1);
	if (lane == 31)
		sm[0][w] = it, sm[1][w] = iff, sm[2][w] = im;
	__syncthreads();
	if (threadIdx.x == 0)
	{
		unsigned int x = 0, y = 0, z = 0;
		for (unsigned int q = 0; q < blockDim.x / 32; ++q)
		{
			unsigned int a = sm[0][q], b = sm[1][q], c = sm[2][q];
			sm[0][q] = x, sm[1][q] = y, sm[2][q] = z;
			x += a, y += b, z = max(z, c);
		}
		sm[0][32] = x, sm[1][32] = y, sm[2][32] = z;
	}
	__syncthreads();
	unsigned int et = sm[0][w] + it - t, ef = sm[1][w] + iff - f, em = max(sm[2][w], lane ? pm : 0u);
	uint3 tot = make_uint3(sm[0][32], sm[1][32], sm[2][32]);
	__syncthreads();
	t = et, f = ef, m = em;
	return tot;
}

__device__ __forceinline__ bool keepTriangle(const unsigned int* __restrict__ res, size_t t, const unsigned int* cr, const unsigned int* __restrict__ remap,
    uint3& out)
{
	unsigned int v0 = __ldcg(cr + res[t * 3 + 0]), v1 = __ldcg(cr + res[t * 3 + 1]), v2 = __ldcg(cr + res[t * 3 + 2]);
	unsigned int r0 = remap[v0], r1 = remap[v1], r2 = remap[v2];
	out = make_uint3(v0, v1, v2);
	return r0 != r1 && r0 != r2 && r1 != r2;
}

// attribute quadric and gradient rows of vertex v added into those of vertex t (t != v)
__device__ __forceinline__ void mergeRows(const Quadric* __restrict__ vq, Quadric* __restrict__ tq, const float4* __restrict__ vg, float4* __restrict__ tg,
    int ac)
{
	Quadric A = ldquadric(tq, 0);
	qadd(A, ldquadric(vq, 0));
	stquadric(tq, 0, A);
	for (int q = 0; q < ac; ++q)
	{
		float4 g = tg[q], h = vg[q];
		g.x += h.x, g.y += h.y, g.z += h.z, g.w += h.w;
		tg[q] = g;
	}
}

__device__ __forceinline__ void mergeAttributes(const PerformArgs& a, unsigned int v, unsigned int t)
{
	Quadric A = ldquadric(a.aq, t);
	qadd(A, ldquadric(a.aq, v));
	stquadric(a.aq, t, A);
	const int ac = a.ac;
	for (int q = 0; q < ac; ++q)
	{
		float4 g = a.ag[(size_t)t * ac + q], h = a.ag[(size_t)v * ac + q];
		g.x += h.x, g.y += h.y, g.z += h.z, g.w += h.w;
		a.ag[(size_t)t * ac + q] = g;
	}
}

// the collapse_remap writes and quadric merges of one committed candidate; attribute sources
// of one commit merge in increasing vertex order, as updateQuadrics' vertex loop does.
// Commits of one pass touch disjoint vertices (no two share an endpoint, and every vertex
// written belongs to the position of r0 or r1), so a commit reads only values that no other
// commit of the pass writes.
__device__ void applyComplexCommit(const PerformArgs& a, unsigned int r0, unsigned int r1, unsigned int i0, unsigned int i1, unsigned int& derrbits)
{
	Quadric Q1 = ldquadric(a.vq, r1);
	Quadric Q0 = ldquadric(a.vq, r0);
	unsigned int v = i0;
	do
	{
		a.cr[v] = complexTarget(v, i1, a.remap, a.loop, a.loopback);
		v = a.wedge[v];
	} while (v != i0);
	qadd(Q1, Q0);
	stquadric(a.vq, r1, Q1);
	if (a.vg)
	{
		float4 g = a.vg[r1];
		gadd(g, a.vg[r0]);
		a.vg[r1] = g;
	}
	if (a.ac)
	{
		// all wedges of the source, in increasing vertex order (selection by repeated minimum)
		unsigned int last = 0;
		bool first = true;
		for (;;)
		{
			unsigned int best = ~0u;
			v = i0;
			do
			{
				if ((first || v > last) && v < best)
					best = v;
				v = a.wedge[v];
			} while (v != i0);
			if (best == ~0u)
				break;
			mergeAttributes(a, best, a.cr[best]);
			last = best;
			first = false;
		}
		float d = qerror(Q0, ldpos(a.pos, a.remap[a.cr[r0]]));
		derrbits = d == d ? __float_as_uint(d) : 0u;
	}
}

// the commit of candidate c (pick order)
__device__ void applyCommit(const PerformArgs& a, unsigned int c, unsigned int& errbits, unsigned int& derrbits)
{
	const uint4 rec = __ldg(a.cring + c);
	const uint4 cd = __ldg(a.crec + c);
	const unsigned int r0 = rec.x, r1 = rec.y, i0 = cd.x, i1 = cd.y;
	const unsigned char kd = (unsigned char)cd.w;
	const float e = __uint_as_float(cd.z);
	errbits = e == e ? cd.z : 0u;
	if (kd == kComplex)
	{
		applyComplexCommit(a, r0, r1, i0, i1, derrbits);
		return;
	}

	// collapse_remap: cr[i0] = i1, then for a seam cr[s0] = s1 (s0 may be i0 itself, which
	// then ends at s1); the targets are known here, so nothing is read back from cr
	unsigned int s0 = ~0u, s1 = ~0u;
	if (kd == kSeam)
	{
		s0 = a.wedge[i0];
		unsigned int li = a.loop[i0];
		s1 = li == i1 ? a.loopback[s0] : a.loop[s0];
		s1 = (s1 != ~0u) ? s1 : a.wedge[i1];
	}
	unsigned int mv0 = i0, mv1 = ~0u; // moved vertices, at most two, in increasing order
	if (s0 != ~0u && s0 != i0)
		mv0 = min(i0, s0), mv1 = max(i0, s0);
	const unsigned int t0 = mv0 == s0 ? s1 : i1;

	// the rows read and written below belong to distinct vertices (r0 != r1, and t0 is a wedge
	// of r1 while mv0 is one of r0), which the restrict-qualified row pointers tell the compiler,
	// so it can issue the loads ahead of the stores; cr is written last
	const Quadric* __restrict__ q0 = a.vq + r0;
	Quadric* __restrict__ q1 = a.vq + r1;
	const int ac = a.ac;
	V3 pr = {0.f, 0.f, 0.f};
	if (ac)
	{
		const unsigned int tr = r0 == s0 ? s1 : (r0 == i0 ? i1 : __ldcg(a.cr + r0));
		pr = ldpos(a.pos, __ldg(a.remap + tr));
	}
	Quadric Q1 = ldquadric(q1, 0);
	Quadric Q0 = ldquadric(q0, 0);
	qadd(Q1, Q0);
	stquadric(q1, 0, Q1);
	if (a.vg)
	{
		const float4* __restrict__ g0 = a.vg + r0;
		float4* __restrict__ g1 = a.vg + r1;
		float4 g = *g1;
		gadd(g, *g0);
		*g1 = g;
	}
	if (ac)
	{
		mergeRows(a.aq + mv0, a.aq + t0, a.ag + (size_t)mv0 * ac, a.ag + (size_t)t0 * ac, ac);
		if (mv1 != ~0u)
		{
			// after the first merge: both may share a target
			const unsigned int t1 = mv1 == s0 ? s1 : i1;
			mergeRows(a.aq + mv1, a.aq + t1, a.ag + (size_t)mv1 * ac, a.ag + (size_t)t1 * ac, ac);
		}
		float d = qerror(Q0, pr);
		derrbits = d == d ? __float_as_uint(d) : 0u;
	}
	a.cr[i0] = i1;
	if (s0 != ~0u)
		a.cr[s0] = s1;
}

// kPerform phases timed by block 0 between grid barriers (SM clock cycles)
enum
{
	kPhInit = 0,
	kPhMarks = 1,
	kPhRounds = 2,
	kPhStop = 3,
	kPhApply = 4,
	kPhLoops = 5,
	kPhScan = 6,
	kPhEmit = 7,
};

// kept in shared memory (one thread of one block uses it), so it holds no registers in the
// kernel's other threads; the round trace's count is kept beside it
struct PhaseClock
{
	long long* s; // [0, 8): cycles per phase, [8]: the last lap's clock, [9]: rounds traced
	__device__ void start(const Scalars* sc)
	{
		s[8] = clock64();
		for (int i = 0; i < 8; ++i)
			s[i] = 0;
		s[9] = sc->trace_count;
	}
	__device__ long long last() const
	{
		return s[8];
	}
	__device__ void lap(int phase)
	{
		long long t = clock64();
		s[phase] += t - s[8];
		s[8] = t;
	}
};

#ifndef MO_PERFORM_THREADS
#define MO_PERFORM_THREADS 256 // threads per block of the pass kernel
#endif
#ifndef MO_PERFORM_MIN_BLOCKS
#define MO_PERFORM_MIN_BLOCKS (1024 / MO_PERFORM_THREADS) // resident blocks per SM the pass kernel is compiled for (64 registers)
#endif
constexpr unsigned int kPerformThreads = MO_PERFORM_THREADS;

__global__ void __launch_bounds__(kPerformThreads, MO_PERFORM_MIN_BLOCKS) kPerform(PerformArgs a)
{
	__shared__ unsigned int s_app[4];
	__shared__ unsigned int s_stage[2][kStageChunk]; // candidates passed to stage B, and kept for stage C (wait)
	__shared__ unsigned int s_commits;               // this block's commits so far
	__shared__ long long s_clock[10];
	PhaseClock pc{s_clock};
	const bool timer = blockIdx.x == 0 && threadIdx.x == 0;
	if (timer)
		pc.start(a.sc);
	__shared__ unsigned int sm[3][33];
	Scalars* sc = a.sc;
	const unsigned int G = gridDim.x;
	const size_t gthreads = (size_t)G * blockDim.x;
	const unsigned int lane = threadIdx.x & 31;

	// per-pass scalars: the launch parameters, or the device-resident loop's live state
	unsigned int count = a.count, tris = a.tris, first_window = a.first_window, round_base = a.round_base, prev_err = a.prev_err_bits;
	unsigned long long goal = a.goal;
	float error_limit = a.error_limit;
	const unsigned int* res = a.res;
	unsigned int* res_next = a.res_next;
	if (a.live)
	{
		const PassLive* lv = a.live;
		if (lv->stop)
			return;
		count = lv->count;
		tris = lv->tris;
		first_window = lv->first_window;
		round_base = lv->round_base;
		goal = lv->goal;
		res = lv->res;
		res_next = lv->res_next;
		prev_err = sc->result_error_bits;
		error_limit = lv->error_limit;
	}

	// per-vertex state of the pass, streamed: collapse_remap, and both parities of both marks (the
	// marks the window's candidates set below come after the barrier)
	for (size_t i = gtid(); i < a.vcount; i += gthreads)
	{
		a.cr[i] = (unsigned int)i;
		a.minT[0][i] = ~0ull;
		a.minT[1][i] = ~0ull;
		reinterpret_cast<ulonglong2*>(a.minS)[i] = make_ulonglong2(~0ull, ~0ull);
	}
	gridBarrier(sc->bar, &sc->grid_error);

	unsigned int round = round_base;
	unsigned long long active_sum = 0;
	unsigned int K0 = 0, K1 = min(count, first_window);
	unsigned int carryT = 0, carryF = 0, carryM = prev_err;
	unsigned int windows = 0;

	// block b's candidates are the pick-order tiles b, b + G, b + 2G, ... of blockDim each; its
	// undecided and committed candidates live in its own region of the lists
	const unsigned int stride = G * blockDim.x;
	const unsigned int tiles = (count + stride - 1) / stride;
	const size_t region = (size_t)blockIdx.x * tiles * blockDim.x;
	unsigned int* const commits = a.commits + region;
	if (threadIdx.x == 0)
		s_commits = 0;

	// warp-aggregated append of the lanes whose flag is set to dst at the shared counter
	auto append = [&](bool flag, unsigned int v, unsigned int* counter, unsigned int* dst) {
		unsigned int m = __ballot_sync(0xffffffffu, flag);
		if (m)
		{
			unsigned int leader = __ffs(m) - 1, o = 0;
			if (lane == leader)
				o = atomicAdd(counter, __popc(m));
			o = __shfl_sync(0xffffffffu, o, leader);
			if (flag)
				dst[o + __popc(m & ((1u << lane) - 1u))] = v;
		}
	};

	for (;;)
	{
		// ---- decision rounds over the sorted window [K0, K1)
		++windows;
		for (size_t c = gtid(); c < count; c += gthreads)
		{
			const unsigned int k = __ldg(a.rank + c);
			if (k >= K0 && k < K1)
				markCandidate(a, k, __ldg(a.cring + c), round + 1);
		}
		if (gtid() == 0)
			sc->act_count[(round + 2) % 3] = 0; // appended to by the window's first round
		gridBarrier(sc->bar, &sc->grid_error);
		if (timer)
			pc.lap(windows == 1 ? kPhInit : kPhMarks);

		// the first round walks the block's tiles and takes the window's candidates among them;
		// the block keeps the candidates it left undecided in its region of the lists, compacted
		// with shared-memory atomics, and walks that region in the later rounds; only the
		// per-round total crosses blocks (one global add per block, read after the barrier)
		unsigned int nb = tiles * blockDim.x; // this block's undecided candidates (slots in the first round)
		unsigned int n = K1 - K0;             // all blocks'
		bool first = true;
		unsigned int guard = 0;
		unsigned int gerr = __ldcg(&sc->grid_error); // read again with each round's total, in one round trip
		while (n)
		{
			++round;
			if (++guard > count + 1 || gerr)
				break;
			active_sum += n;
			const unsigned int* cur = a.list[round & 1] + region;
			unsigned int* next = a.list[(round + 1) & 1] + region;
			unsigned int* next_total = &sc->act_count[(round + 1) % 3];
			// the total round+1 adds to; every thread read it (as round-2's result) before the
			// barrier that ended round-1
			if (gtid() == 0)
				sc->act_count[(round + 2) % 3] = 0;
			if (threadIdx.x == 0)
				s_app[0] = 0;
			for (unsigned int c0 = 0; c0 < nb; c0 += kStageChunk)
			{
				const unsigned int c1 = min(nb, c0 + kStageChunk);
				if (threadIdx.x == 0)
					s_app[1] = 0, s_app[3] = 0;
				__syncthreads();
				// stage A: endpoint marks; kStageItems candidates per thread, their loads issued together
				const unsigned long long tag = roundTag(round);
				const unsigned long long* minT = a.minT[round & 1];
				for (unsigned int base = c0; base < c1; base += blockDim.x * kStageItems)
				{
					unsigned int cc[kStageItems], kk[kStageItems];
					bool ok[kStageItems];
#pragma unroll
					for (unsigned int q = 0; q < kStageItems; ++q)
					{
						const unsigned int x = base + q * blockDim.x + threadIdx.x;
						const unsigned int g = (x - threadIdx.x) * G + blockIdx.x * blockDim.x + threadIdx.x;
						ok[q] = x < c1 && (!first || g < count);
						cc[q] = ok[q] ? (first ? g : __ldcg(cur + x)) : 0u;
					}
					uint2 ends[kStageItems];
#pragma unroll
					for (unsigned int q = 0; q < kStageItems; ++q)
					{
						kk[q] = ok[q] ? __ldg(a.rank + cc[q]) : 0u;
						const uint4 rec = ok[q] ? __ldg(a.cring + cc[q]) : make_uint4(0, 0, 0, 0);
						ends[q] = make_uint2(rec.x, rec.y);
					}
#pragma unroll
					for (unsigned int q = 0; q < kStageItems; ++q)
						ok[q] = ok[q] && (!first || (kk[q] >= K0 && kk[q] < K1));
					unsigned long long m0[kStageItems], m1[kStageItems];
#pragma unroll
					for (unsigned int q = 0; q < kStageItems; ++q)
					{
						m0[q] = ok[q] ? __ldcg(minT + ends[q].x) : 1ull;
						m1[q] = ok[q] ? __ldcg(minT + ends[q].y) : 1ull;
					}
#pragma unroll
					for (unsigned int q = 0; q < kStageItems; ++q)
					{
						const unsigned long long mine = tag | kk[q];
						const bool taken = m0[q] == 0 || m1[q] == 0; // a commit took an endpoint
						const bool locked = ok[q] && taken;
						const bool keep = ok[q] && !taken && (m0[q] != mine || m1[q] != mine);
						const bool pass = ok[q] && !taken && !keep;
						if (locked)
							a.status[kk[q]] = kSkipLocked;
						append(keep, cc[q], &s_app[3], s_stage[1]);
						append(pass, cc[q], &s_app[1], s_stage[0]);
					}
				}
				__syncthreads();
				// stage B: the one-ring's marks, the flip test and the commit, in one walk
				const unsigned int nB = s_app[1];
				for (unsigned int base = 0; base < nB; base += blockDim.x)
				{
					const unsigned int x = base + threadIdx.x;
					int r = kRingFlip;
					unsigned int c = 0;
					if (x < nB)
					{
						c = s_stage[0][x];
						r = ringDecide(a, c, __ldg(a.rank + c), __ldg(a.cring + c), round);
					}
					append(r == kRingWaits, c, &s_app[3], s_stage[1]);
					append(r == kRingCommit, c, &s_commits, commits);
				}
				__syncthreads();
				// stage C: the candidates that wait. A commit of this round (this block's, or another's
				// whose write is already seen) on an endpoint locks one now: that commit is earlier,
				// so the lock is final, and the candidates waiting on this one need not wait a round
				// more for it. The others mark their endpoints for the next round.
				const unsigned int nD = s_app[3];
				for (unsigned int base = 0; base < nD; base += blockDim.x * kStageItems)
				{
					unsigned int cc[kStageItems], kk[kStageItems];
					uint2 ends[kStageItems];
#pragma unroll
					for (unsigned int q = 0; q < kStageItems; ++q)
					{
						const unsigned int x = base + q * blockDim.x + threadIdx.x;
						cc[q] = x < nD ? s_stage[1][x] : ~0u;
						kk[q] = cc[q] != ~0u ? __ldg(a.rank + cc[q]) : 0u;
						const uint4 rec = cc[q] != ~0u ? __ldg(a.cring + cc[q]) : make_uint4(0, 0, 0, 0);
						ends[q] = make_uint2(rec.x, rec.y);
					}
					unsigned long long m0[kStageItems], m1[kStageItems];
#pragma unroll
					for (unsigned int q = 0; q < kStageItems; ++q)
					{
						m0[q] = cc[q] != ~0u ? __ldcg(minT + ends[q].x) : 1ull;
						m1[q] = cc[q] != ~0u ? __ldcg(minT + ends[q].y) : 1ull;
					}
#pragma unroll
					for (unsigned int q = 0; q < kStageItems; ++q)
					{
						const bool valid = cc[q] != ~0u;
						const bool taken = m0[q] == 0 || m1[q] == 0;
						if (valid && taken)
							a.status[kk[q]] = kSkipLocked;
						if (valid && !taken)
						{
							const unsigned long long key = roundTag(round + 1) | kk[q];
							atomicMin(&a.minT[(round + 1) & 1][ends[q].x], key);
							atomicMin(&a.minT[(round + 1) & 1][ends[q].y], key);
							atomicMin(&a.minS[2 * (size_t)ends[q].x + ((round + 1) & 1)], key);
						}
						append(valid && !taken, cc[q], &s_app[0], next);
					}
				}
				__syncthreads();
			}
			__syncthreads(); // the counter's reset is seen when the block had no candidates
			nb = s_app[0];
			if (threadIdx.x == 0 && nb)
				atomicAdd(next_total, nb);
			gridBarrier(sc->bar, &sc->grid_error);
			if (timer)
			{
				long long before = pc.last();
				pc.lap(kPhRounds);
				const unsigned int tc = (unsigned int)s_clock[9];
				if (tc < 512)
				{
					sc->trace[2 * tc] = n;
					sc->trace[2 * tc + 1] = (unsigned int)((pc.last() - before) >> 4);
					sc->trace_count = tc + 1;
					s_clock[9] = tc + 1;
				}
			}
			const unsigned int nn = __ldcg(next_total);
			gerr = __ldcg(&sc->grid_error);
			if (nn >= n)
			{
				if (gtid() == 0)
					atomicOr(&sc->grid_error, 2u);
				break;
			}
			n = nn;
			first = false;
		}
		if (__ldcg(&sc->grid_error))
			break;

		// ---- stop rules over [K0, K1): block chunks, thread sub-chunks, carried prefix
		const unsigned int len = K1 - K0;
		const unsigned int per_block = (len + G - 1) / G;
		const unsigned int c0 = min(K1, K0 + blockIdx.x * per_block), c1 = min(K1, c0 + per_block);
		const unsigned int per_thread = (c1 - c0 + blockDim.x - 1) / blockDim.x;
		const unsigned int t0 = min(c1, c0 + threadIdx.x * per_thread), t1 = min(c1, t0 + per_thread);
		unsigned int sT = 0, sF = 0, sM = 0;
		for (unsigned int k = t0; k < t1; ++k)
		{
			unsigned int tt, ff, ee;
			stopTerms(__ldcg(a.status + k), __ldg(a.skind + k), __ldg(a.serr + k), tt, ff, ee);
			sT += tt, sF += ff, sM = max(sM, ee);
		}
		unsigned int eT = sT, eF = sF, eM = sM;
		uint3 tot = blockScan3(eT, eF, eM, sm);
		if (threadIdx.x == 0)
			a.blk[blockIdx.x] = make_uint4(tot.x, tot.y, tot.z, 0);
		gridBarrier(sc->bar, &sc->grid_error);
		if (blockIdx.x == 0)
		{
			// exclusive prefix over the block totals with the carry of earlier windows
			unsigned int rT = carryT, rF = carryF, rM = carryM;
			for (unsigned int q0 = 0; q0 < G; q0 += blockDim.x)
			{
				unsigned int q = q0 + threadIdx.x;
				uint4 v = q < G ? __ldcg(a.blk + q) : make_uint4(0, 0, 0, 0);
				unsigned int x = v.x, y = v.y, z = v.z;
				uint3 ct = blockScan3(x, y, z, sm);
				if (q < G)
					a.blk[q] = make_uint4(rT + x, rF + y, max(rM, z), 0);
				rT += ct.x, rF += ct.y, rM = max(rM, ct.z);
			}
			if (threadIdx.x == 0)
				sc->carry[0] = rT, sc->carry[1] = rF, sc->carry[2] = rM;
		}
		gridBarrier(sc->bar, &sc->grid_error);
		{
			uint4 bb = __ldcg(a.blk + blockIdx.x);
			unsigned long long T = (unsigned long long)bb.x + eT;
			unsigned long long F = (unsigned long long)bb.y + eF;
			unsigned int M = max(bb.z, eM);
			const unsigned long long egoal0 = goal / 2;
			// the error goal moves with the flip count only: the last one read is kept with its
			// position, and read at all only when the rule's other two terms hold
			unsigned long long goal_at = ~0ull;
			float error_goal = FLT_MAX;
			for (unsigned int k = t0; k < t1; ++k)
			{
				float e = __uint_as_float(__ldg(a.serr + k));
				unsigned int reason = 0;
				if (e > error_limit)
					reason = 1;
				else if (T >= goal)
					reason = 2;
				else if (T > goal / 6 && e > __uint_as_float(M))
				{
					const unsigned long long eg = egoal0 + F;
					if (eg != goal_at)
					{
						goal_at = eg;
						error_goal = eg < count ? 1.5f * __uint_as_float(__ldg(a.serr + eg)) : FLT_MAX;
					}
					if (e > error_goal)
						reason = 3;
				}
				if (reason)
				{
					atomicMin(&sc->cut, ((unsigned long long)k << 2) | reason);
					break;
				}
				unsigned int tt, ff, ee;
				stopTerms(__ldcg(a.status + k), __ldg(a.skind + k), __ldg(a.serr + k), tt, ff, ee);
				T += tt, F += ff, M = max(M, ee);
			}
		}
		gridBarrier(sc->bar, &sc->grid_error);
		if (timer)
			pc.lap(kPhStop);
		if (__ldcg(&sc->cut) != ~0ull || K1 == count || __ldcg(&sc->grid_error))
			break;
		carryT = __ldcg(&sc->carry[0]);
		carryF = __ldcg(&sc->carry[1]);
		carryM = __ldcg(&sc->carry[2]);
		K0 = K1;
		K1 = (unsigned int)min((unsigned long long)count, 2ull * K1);
	}
	if (__ldcg(&sc->grid_error))
		return;

	// ---- apply the committed prefix. Commits are independent (no two share an endpoint), so
	// any order gives the same result: each block applies its own commits (pick order, so their
	// quadric rows are near one another) whose sorted position is inside the prefix. The
	// decisions of the prefix are counted over sorted order.
	const unsigned long long cutv = __ldcg(&sc->cut);
	const unsigned int cut = cutv == ~0ull ? count : (unsigned int)(cutv >> 2);
	unsigned int nd = 0, ns = 0, ni = 0, em = 0, dm = 0;
	for (size_t k = gtid(); k < cut; k += gthreads)
	{
		const unsigned char st = __ldcg(a.status + k);
		nd += st == kCommit, ns += st == kSkipLocked, ni += st == kSkipFlip;
	}
	{
		const unsigned int mc = s_commits; // every append to it was followed by a block barrier
		for (unsigned int x = threadIdx.x; x < mc; x += blockDim.x)
		{
			const unsigned int c = commits[x];
			if (__ldg(a.rank + c) < cut)
			{
				unsigned int eb = 0, db = 0;
				applyCommit(a, c, eb, db);
				em = max(em, eb), dm = max(dm, db);
			}
		}
	}
	{
		unsigned int x = nd, y = ns, z = em;
		uint3 t1 = blockScan3(x, y, z, sm);
		unsigned int p = ni, q = 0, r = dm;
		uint3 t2 = blockScan3(p, q, r, sm);
		if (threadIdx.x == 0)
		{
			if (t1.x)
				atomicAdd(&sc->done, t1.x);
			if (t1.y)
				atomicAdd(&sc->skipped, t1.y);
			if (t2.x)
				atomicAdd(&sc->invalid, t2.x);
			if (t1.z)
				atomicMax(&sc->result_error_bits, t1.z);
			if (t2.z)
				atomicMax(&sc->vertex_error_bits, t2.z);
		}
	}
	gridBarrier(sc->bar, &sc->grid_error);
	if (timer)
		pc.lap(kPhApply);
	if (__ldcg(&sc->done) == 0 || __ldcg(&sc->grid_error))
	{
		if (timer)
			for (int i = 0; i < 8; ++i)
				atomicAdd(&sc->phase_cycles[i], (unsigned long long)s_clock[i]);
		if (gtid() == 0)
		{
			sc->rounds = round - round_base;
			sc->active_sum = active_sum;
			sc->windows = windows;
		}
		return;
	}

	// ---- loop remap (in place: targets are fixed points of collapse_remap) and kept-triangle counts
	for (size_t i = gtid(); i < a.vcount; i += gthreads)
	{
		unsigned int* arrs[2] = {a.loop, a.loopback};
		for (int q = 0; q < 2; ++q)
		{
			unsigned int* L = arrs[q];
			unsigned int l = L[i];
			if (l == ~0u)
				continue;
			unsigned int r = __ldcg(a.cr + l);
			if (i == r)
			{
				unsigned int ll = __ldcg(L + l);
				L[i] = ll != ~0u ? __ldcg(a.cr + ll) : ~0u;
			}
			else
				L[i] = r;
		}
	}
	const unsigned int tper_block = (tris + G - 1) / G;
	const unsigned int tb0 = min(tris, blockIdx.x * tper_block), tb1 = min(tris, tb0 + tper_block);
	const unsigned int tper_thread = (tb1 - tb0 + blockDim.x - 1) / blockDim.x;
	const unsigned int tt0 = min(tb1, tb0 + threadIdx.x * tper_thread), tt1 = min(tb1, tt0 + tper_thread);
	unsigned int kept = 0;
	for (unsigned int t = tt0; t < tt1; ++t)
	{
		uint3 o;
		kept += keepTriangle(res, t, a.cr, a.remap, o);
	}
	unsigned int ek = kept, d1 = 0, d2 = 0;
	uint3 ktot = blockScan3(ek, d1, d2, sm);
	if (threadIdx.x == 0)
		a.blk[blockIdx.x] = make_uint4(ktot.x, 0, 0, 0);
	gridBarrier(sc->bar, &sc->grid_error);
	if (timer)
		pc.lap(kPhLoops);
	if (blockIdx.x == 0)
	{
		unsigned int run = 0;
		for (unsigned int q0 = 0; q0 < G; q0 += blockDim.x)
		{
			unsigned int q = q0 + threadIdx.x;
			unsigned int x = q < G ? __ldcg(&a.blk[q].x) : 0u, y = 0, z = 0;
			uint3 ct = blockScan3(x, y, z, sm);
			if (q < G)
				a.blk[q].y = run + x;
			run += ct.x;
		}
		if (threadIdx.x == 0)
		{
			sc->tri_total = run;
			sc->rounds = round - round_base;
			sc->active_sum = active_sum;
			sc->windows = windows;
		}
	}
	gridBarrier(sc->bar, &sc->grid_error);
	if (timer)
		pc.lap(kPhScan);
	{
		unsigned int w = __ldcg(&a.blk[blockIdx.x].y) + ek;
		for (unsigned int t = tt0; t < tt1; ++t)
		{
			uint3 o;
			if (keepTriangle(res, t, a.cr, a.remap, o))
			{
				res_next[(size_t)w * 3 + 0] = o.x;
				res_next[(size_t)w * 3 + 1] = o.y;
				res_next[(size_t)w * 3 + 2] = o.z;
				w++;
			}
		}
	}
	if (timer)
	{
		pc.lap(kPhEmit);
		for (int i = 0; i < 8; ++i)
			atomicAdd(&sc->phase_cycles[i], (unsigned long long)s_clock[i]);
	}
}

// ---------------------------------------------------------------- prune (buildComponents / measureComponents / pruneComponents, :1866-2024)

__device__ __forceinline__ unsigned int ufFind(unsigned int* parent, unsigned int x)
{
	unsigned int p = __ldcg(parent + x);
	while (p != x)
	{
		unsigned int gp = __ldcg(parent + p);
		if (gp != p)
			atomicCAS(parent + x, p, gp); // path halving
		x = p;
		p = __ldcg(parent + x);
	}
	return x;
}

// lock-free union-find over the welded edges: the larger root is linked under the smaller, so

// ---------------------------------------------------------------- the update mode (meshopt_simplifyWithUpdate)
//
// After the passes the vertices the result still uses get the optimal position of their
// quadric (solvePositions :1675-1763) and attributes (solveAttributes :1765-1809), written back
// to the caller's buffers (finalizeVertices :623-665). The reference solves positions in
// vertex order, in place: a vertex's checks see the new positions of lower-index neighbours
// and the old ones of higher-index neighbours. Here a vertex is solved once every lower-index
// neighbour that is solved at all is final, reading final positions below its index and the
// original ones above it: the same values, in rounds (the lowest pending vertex is always
// ready, so every round makes progress).

// vertices the result uses, and their positions' primaries (:2580-2587)
__global__ void kMarkUpdate(const unsigned int* __restrict__ res, size_t n, const unsigned int* __restrict__ remap, unsigned char* update)
{
	size_t i = gtid();
	if (i >= n)
		return;
	unsigned int v = res[i];
	update[remap[v]] = 1;
	update[v] = 1;
}

__device__ __forceinline__ bool positionSolved(unsigned char k)
{
	return !(k == kLocked || k == kSeam || k == kBorder);
}

// solved primaries go to the first list; every other vertex keeps its position and is final
__global__ void kSolveList(size_t n, const unsigned char* __restrict__ update, const unsigned int* __restrict__ remap, const unsigned char* __restrict__ kind,
    unsigned int* __restrict__ done, unsigned int* __restrict__ list, unsigned int* count)
{
	size_t vi = gtid();
	if (vi >= n)
		return;
	unsigned int i = (unsigned int)vi;
	bool cand = update[i] && remap[i] == i && positionSolved(kind[i]);
	done[i] = cand ? 0u : 1u;
	if (cand)
		list[atomicAdd(count, 1u)] = i;
}

struct SolveArgs
{
	unsigned int* list[2];
	unsigned int* done;
	const unsigned int* adj_off;
	const uint2* adj;
	const float4* pos;   // positions before the solve
	float4* pos_new;     // solved positions (starts as a copy of pos)
	const Quadric* vq;
	const Quadric* aq;
	const float4* ag;
	const float4* vg;
	int ac;
	const unsigned int* wedge;
	unsigned int max_rounds;
	Scalars* sc;
};

// the reference's checks for one vertex (:1698-1759); true with the accepted position in p
__device__ bool solveVertex(const SolveArgs& a, unsigned int i, V3& p)
{
	const V3 vp = ldpos(a.pos, i);
	Quadric Q = ldquadric(a.vq, i);
	Quadric R = qpoint(vp.x, vp.y, vp.z, Q.w * 1e-4f);
	qadd(Q, R);
	float4 GV = make_float4(0.f, 0.f, 0.f, 0.f);
	if (a.ac)
	{
		unsigned int v = i;
		do
		{
			qreduceAttr(Q, ldquadric(a.aq, v), a.ag + (size_t)v * a.ac, a.ac);
			v = a.wedge[v];
		} while (v != i);
		if (a.vg)
			GV = a.vg[i];
	}
	if (!qsolve(p, Q, GV))
		return false;

	// neighbours as the reference's loop sees them at i's turn
	auto npos = [&](unsigned int x) {
		if (x < i)
		{
			float4 q = __ldcg(a.pos_new + x);
			return V3{q.x, q.y, q.z};
		}
		return ldpos(a.pos, x);
	};
	const unsigned int b = a.adj_off[i], e = a.adj_off[i + 1];
	float radius = 0.f;
	for (unsigned int j = b; j < e; ++j)
	{
		uint2 ed = a.adj[j];
		V3 va = npos(ed.x), vb = npos(ed.y);
		float da = (va.x - vp.x) * (va.x - vp.x) + (va.y - vp.y) * (va.y - vp.y) + (va.z - vp.z) * (va.z - vp.z);
		float db = (vb.x - vp.x) * (vb.x - vp.x) + (vb.y - vp.y) * (vb.y - vp.y) + (vb.z - vp.z) * (vb.z - vp.z);
		radius = radius < da ? da : radius;
		radius = radius < db ? db : radius;
	}
	float nr = sqrtf(radius);
	float dp = (p.x - vp.x) * (p.x - vp.x) + (p.y - vp.y) * (p.y - vp.y) + (p.z - vp.z) * (p.z - vp.z);
	if (dp > nr * nr)
		return false;
	for (unsigned int j = b; j < e; ++j)
	{
		uint2 ed = a.adj[j];
		if (triFlip(npos(ed.x), npos(ed.y), vp, p))
			return false;
	}
	const Quadric Q0 = ldquadric(a.vq, i);
	if (qerror(Q0, p) > qerror(Q0, vp) * 1.5f + 1e-6f)
		return false;
	return true;
}

__global__ void __launch_bounds__(kThreads) kSolvePositions(SolveArgs a)
{
	Scalars* sc = a.sc;
	const size_t gthreads = (size_t)gridDim.x * blockDim.x;
	const unsigned int lane = threadIdx.x & 31;
	unsigned int n = __ldcg(&sc->solve_pending[1]);
	unsigned int round = 0;
	while (n)
	{
		++round;
		if (round > a.max_rounds || __ldcg(&sc->grid_error))
		{
			if (gtid() == 0)
				atomicOr(&sc->grid_error, 2u);
			break;
		}
		const unsigned int* cur = a.list[round & 1];
		unsigned int* next = a.list[(round + 1) & 1];
		unsigned int* next_count = &sc->solve_pending[(round + 1) % 3];
		if (gtid() == 0)
			sc->solve_pending[(round + 2) % 3] = 0;
		for (size_t base = (size_t)blockIdx.x * blockDim.x; base < n; base += gthreads)
		{
			size_t x = base + threadIdx.x;
			bool keep = false;
			unsigned int i = 0;
			if (x < n)
			{
				i = __ldcg(cur + x);
				bool ready = true;
				for (unsigned int j = a.adj_off[i], e = a.adj_off[i + 1]; j < e && ready; ++j)
				{
					uint2 ed = a.adj[j];
					ready = !((ed.x < i && __ldcg(a.done + ed.x) == 0) || (ed.y < i && __ldcg(a.done + ed.y) == 0));
				}
				if (ready)
				{
					__threadfence(); // the final positions behind the flags read above
					V3 p;
					if (solveVertex(a, i, p))
						a.pos_new[i] = make_float4(p.x, p.y, p.z, 0.f);
					__threadfence();
					atomicExch(a.done + i, 1u);
				}
				else
					keep = true;
			}
			unsigned int m = __ballot_sync(0xffffffffu, keep);
			if (m)
			{
				unsigned int leader = __ffs(m) - 1, o = 0;
				if (lane == leader)
					o = atomicAdd(next_count, __popc(m));
				o = __shfl_sync(0xffffffffu, o, leader);
				if (keep)
					next[o + __popc(m & ((1u << lane) - 1u))] = i;
			}
		}
		gridBarrier(sc->bar, &sc->grid_error);
		unsigned int nn = __ldcg(next_count);
		if (nn >= n)
		{
			if (gtid() == 0)
				atomicOr(&sc->grid_error, 2u);
			break;
		}
		n = nn;
	}
	if (gtid() == 0)
		sc->solve_rounds = round;
}

// wedges take their primary's solved position (:1691-1695)
__global__ void kSolveWedges(size_t n, const unsigned char* __restrict__ update, const unsigned int* __restrict__ remap, const unsigned char* __restrict__ kind,
    float4* pos_new)
{
	size_t vi = gtid();
	if (vi >= n)
		return;
	unsigned int i = (unsigned int)vi;
	if (update[i] && remap[i] != i && positionSolved(kind[i]))
		pos_new[i] = pos_new[remap[i]];
}

// solveAttributes :1765-1809, one thread per solved primary over its wedges
__global__ void kSolveAttributes(size_t n, const unsigned char* __restrict__ update, const unsigned int* __restrict__ remap, const unsigned int* __restrict__ wedge,
    const unsigned char* __restrict__ kind, const float4* __restrict__ pos_new, const Quadric* __restrict__ aq, const float4* __restrict__ ag, int ac,
    float* attr)
{
	size_t vi = gtid();
	if (vi >= n)
		return;
	unsigned int i = (unsigned int)vi;
	if (!update[i] || remap[i] != i)
		return;
	const float4 pn = pos_new[i];
	for (int k = 0; k < ac; ++k)
	{
		unsigned int shared = ~0u;
		if (kind[i] == kComplex)
		{
			shared = i;
			for (unsigned int v = wedge[i]; v != i; v = wedge[v])
				if (attr[(size_t)v * ac + k] != attr[(size_t)i * ac + k])
					shared = ~0u;
				else if (shared != ~0u && ldquadric(aq, v).w > ldquadric(aq, shared).w)
					shared = v;
		}
		unsigned int v = i;
		do
		{
			unsigned int r = shared == ~0u ? v : shared;
			float aw = ldquadric(aq, r).w;
			float4 g = ag[(size_t)r * ac + k];
			float iw = aw == 0 ? 0.f : 1.f / aw;
			attr[(size_t)v * ac + k] = (g.x * pn.x + g.y * pn.y + g.z * pn.z + g.w) * iw;
			v = wedge[v];
		} while (v != i);
	}
}

// finalizeVertices :623-665: undo the rescale and the attribute weights into the caller's buffers
__global__ void kFinalizeVertices(size_t n, const unsigned char* __restrict__ update, const unsigned char* __restrict__ lock, const unsigned char* __restrict__ kind,
    const float4* __restrict__ pos_new, const Scalars* __restrict__ sc, float* positions, size_t pstride_f, const float* __restrict__ attr, AttrMap am,
    float* attributes, size_t astride_f)
{
	size_t vi = gtid();
	if (vi >= n)
		return;
	if (!update[vi] || (lock && (lock[vi] & kVertexLock)))
		return;
	if (kind[vi] != kLocked)
	{
		const float4 p = pos_new[vi];
		const float scale = sc->extent;
		float* v = positions + vi * pstride_f;
		v[0] = p.x * scale + sc->minv[0];
		v[1] = p.y * scale + sc->minv[1];
		v[2] = p.z * scale + sc->minv[2];
	}
	for (int k = 0; k < am.count; ++k)
		attributes[vi * astride_f + am.src[k]] = attr[vi * am.count + k] / am.weight[k];
}

// ---------------------------------------------------------------- device-resident pass loop
//
// The pass loop (src/simplifier.cpp:2493-2541) recorded once into a CUDA graph as the body of
// a WHILE conditional node: every kernel of a pass reads the pass's counts from PassLive, the
// grids cover the first (largest) pass, and kPassEnd decides on the device whether another
// pass runs, so the loop needs no host round trip.

// After the pick: the pass's candidate count, triangle goal and first window (the host loop's
// arithmetic), and the per-pass resets of kPerform's scalars. No candidate ends the loop (the
// host loop's break at C == 0).
// the pass loop's squared error limit (:2489-2491) from the extent kMinMaxFinal left, with the
// host's operations: target_error^2 / scale^2, scale = the extent for ErrorAbsolute, else 1
__global__ void kErrorLimit(Scalars* sc, float target_error, int absolute)
{
	const float s = absolute ? sc->extent : 1.f;
	sc->live.error_limit = (target_error * target_error) / (s * s);
}

__global__ void kPassPrep(Scalars* sc)
{
	PassLive& lv = sc->live;
	if (lv.stop)
		return;
	unsigned int C = min(sc->pick_total, sc->pick_trunc);
	lv.count = C;
	if (C == 0)
	{
		lv.stop = 1;
		return;
	}
	lv.sort_cells = keySortTiles(C, lv.sort_items) * kKeyBins;
	unsigned long long goal = (unsigned long long)(lv.indices - lv.target) / 3;
	lv.goal = goal;
	double wf = lv.window_factor * double(goal / 2) + 4096.0;
	lv.first_window = unsigned(double(C) < wf ? double(C) : wf);
	sc->bar[0] = 0;
	sc->bar[1] = 0;
	sc->grid_error = 0;
	sc->cut = ~0ull;
	sc->done = 0;
	sc->skipped = 0;
	sc->invalid = 0;
}

// After kPerform: the pass's counters (as the host loop records them), the next pass's index
// buffer and counts, and the loop condition.
__global__ void kPassEnd(Scalars* sc, cudaGraphConditionalHandle handle, unsigned int max_passes)
{
	PassLive& lv = sc->live;
	lv.iterations++;
	if (!lv.stop)
	{
		if (sc->grid_error || sc->scan_error)
			lv.stop = 1; // reported by the host after the loop
		else
		{
			const unsigned long long cutv = sc->cut;
			const unsigned int C = lv.count;
			const unsigned int cut = cutv == ~0ull ? C : (unsigned int)(cutv >> 2);
			if (lv.passes < kMaxPassStats)
			{
				PassStats& ps = sc->pstats[lv.passes];
				ps.triangles = lv.tris;
				ps.candidates = C;
				ps.evaluated = cut < C ? cut + 1 : C;
				ps.done = sc->done;
				ps.skipped = sc->skipped;
				ps.invalid = sc->invalid;
				ps.stop = cutv == ~0ull ? 0u : (unsigned int)(cutv & 3);
				ps.rounds = sc->rounds;
				ps.active = (unsigned int)sc->active_sum;
				ps.windows = sc->windows;
			}
			lv.window_factor = nextWindowFactor(lv.window_base, lv.goal, cut < C ? cut + 1 : C);
			lv.round_base += sc->rounds;
			lv.passes++;
			if (sc->done == 0)
				lv.stop = 1;
			else
			{
				lv.tris = sc->tri_total;
				lv.indices = sc->tri_total * 3;
				const unsigned int* r = lv.res;
				lv.res = lv.res_next;
				lv.res_next = const_cast<unsigned int*>(r);
				if (lv.indices <= lv.target)
					lv.stop = 1;
				else if (lv.passes >= max_passes)
				{
					lv.stop = 1;
					sc->grid_error |= 4u;
				}
			}
		}
	}
	cudaGraphSetConditional(handle, lv.stop ? 0u : 1u);
}


// a component's root is its smallest primary vertex, as the reference's union-find leaves it
__global__ void kUnionEdges(const unsigned int* __restrict__ idx, size_t tris, const unsigned int* __restrict__ remap, unsigned int* parent)
{
	size_t t = gtid();
	if (t >= tris)
		return;
	for (int e = 0; e < 3; ++e)
	{
		unsigned int a = remap[idx[t * 3 + e]], b = remap[idx[t * 3 + (e == 2 ? 0 : e + 1)]];
		for (int guard = 0; guard < 1 << 20; ++guard)
		{
			unsigned int ra = ufFind(parent, a), rb = ufFind(parent, b);
			if (ra == rb)
				break;
			unsigned int hi = max(ra, rb), lo = min(ra, rb);
			if (atomicCAS(parent + hi, hi, lo) == hi)
				break;
		}
	}
}

__global__ void kComponentRoots(size_t n, const unsigned int* __restrict__ remap, unsigned int* parent, unsigned int* __restrict__ rootflag)
{
	size_t i = gtid();
	if (i >= n)
		return;
	unsigned int r = remap[i] == i ? ufFind(parent, (unsigned int)i) : ~0u;
	rootflag[i] = r == (unsigned int)i;
}

// component ids in order of their roots (next_component++ over primaries in vertex order)
__global__ void kComponentIds(size_t n, const unsigned int* __restrict__ remap, unsigned int* parent, const unsigned int* __restrict__ rootrank,
    unsigned int* __restrict__ comp)
{
	size_t i = gtid();
	if (i >= n)
		return;
	unsigned int r = ufFind(parent, remap[(unsigned int)i]);
	comp[i] = rootrank[r];
}

// center = average position (sums in vertex order, as measureComponents), radius^2 = max
// squared distance; one thread per component over its vertices sorted by (component, index)
__global__ void kMeasureComponents(size_t ncomp, const unsigned int* __restrict__ off, const unsigned int* __restrict__ verts,
    const float4* __restrict__ pos, float* __restrict__ err)
{
	size_t c = gtid();
	if (c >= ncomp)
		return;
	unsigned int b = off[c], e = off[c + 1];
	float sx = 0.f, sy = 0.f, sz = 0.f, sw = 0.f;
	for (unsigned int j = b; j < e; ++j)
	{
		float4 p = pos[verts[j]];
		sx += p.x;
		sy += p.y;
		sz += p.z;
		sw += 1;
	}
	float iw = sw == 0.f ? 0.f : 1.f / sw;
	sx *= iw;
	sy *= iw;
	sz *= iw;
	float r2 = 0.f;
	for (unsigned int j = b; j < e; ++j)
	{
		float4 p = pos[verts[j]];
		float dx = p.x - sx, dy = p.y - sy, dz = p.z - sz;
		float r = dx * dx + dy * dy + dz * dz;
		r2 = r2 < r ? r : r2;
	}
	err[c] = r2;
}

__global__ void kMinFloat(const float* __restrict__ v, size_t n, unsigned int* out)
{
	size_t i = gtid();
	if (i < n)
		atomicMin(out, __float_as_uint(v[i])); // non-negative errors: bits order as floats
}

// largest component error not above the cutoff (cleanup loop, :2557-2560)
__global__ void kMaxBelow(const float* __restrict__ v, size_t n, float cutoff, unsigned int* out)
{
	size_t i = gtid();
	if (i < n && v[i] <= cutoff && v[i] > 0.f)
		atomicMax(out, __float_as_uint(v[i]));
}

__device__ __forceinline__ bool pruneKeep(const unsigned int* __restrict__ res, size_t t, const unsigned int* __restrict__ comp,
    const float* __restrict__ err, float cutoff, uint3& tri, float& e)
{
	tri = make_uint3(res[t * 3], res[t * 3 + 1], res[t * 3 + 2]);
	e = err[comp[tri.x]];
	return e > cutoff;
}

__global__ void __launch_bounds__(kThreads) kPruneCount(const unsigned int* __restrict__ res, size_t tris, const unsigned int* __restrict__ comp,
    const float* __restrict__ err, float cutoff, unsigned int* __restrict__ blkcnt, unsigned int* minerr)
{
	size_t t = gtid();
	uint3 tri;
	float e = 0.f;
	bool keep = t < tris && pruneKeep(res, t, comp, err, cutoff, tri, e);
	if (keep)
		atomicMin(minerr, __float_as_uint(e));
	unsigned int c = __syncthreads_count(keep);
	if (threadIdx.x == 0)
		blkcnt[blockIdx.x] = c;
}

__global__ void __launch_bounds__(kThreads) kPruneEmit(const unsigned int* __restrict__ res, size_t tris, const unsigned int* __restrict__ comp,
    const float* __restrict__ err, float cutoff, const unsigned int* __restrict__ blkoff, unsigned int* __restrict__ out)
{
	__shared__ unsigned int smem[kThreads / 32 + 1];
	size_t t = gtid();
	uint3 tri = make_uint3(0, 0, 0);
	float e = 0.f;
	bool keep = t < tris && pruneKeep(res, t, comp, err, cutoff, tri, e);
	unsigned int total;
	unsigned int pre = blockExclusiveScan<kThreads>(keep ? 1u : 0u, smem, &total);
	if (keep)
	{
		size_t w = (size_t)(blkoff[blockIdx.x] + pre) * 3;
		out[w] = tri.x, out[w + 1] = tri.y, out[w + 2] = tri.z;
	}
}

// meshopt_SimplifyInternalDebug (:2601-2614): vertex kind in bits 28-30, loop bit 31
__global__ void kDebugBits(unsigned int* res, size_t tris, const unsigned char* __restrict__ kind, const unsigned int* __restrict__ loop,
    const unsigned int* __restrict__ loopback)
{
	size_t t = gtid();
	if (t >= tris)
		return;
	unsigned int a = res[t * 3], b = res[t * 3 + 1], c = res[t * 3 + 2];
	res[t * 3 + 0] = a | ((unsigned int)kind[a] << 28) | ((unsigned int)(loop[a] == b || loopback[b] == a) << 31);
	res[t * 3 + 1] = b | ((unsigned int)kind[b] << 28) | ((unsigned int)(loop[b] == c || loopback[c] == b) << 31);
	res[t * 3 + 2] = c | ((unsigned int)kind[c] << 28) | ((unsigned int)(loop[c] == a || loopback[a] == c) << 31);
}

// ---------------------------------------------------------------- workspace

struct Carver
{
	char* base;
	size_t off = 0;
	template <class T>
	T* take(size_t count)
	{
		size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
		T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
		off += bytes ? bytes : 256;
		return p;
	}
};

struct Work
{
	Scalars* sc;
	float* partial;
	float4* pos_raw;
	float4* pos;
	unsigned int *remap, *wedge, *table, *slot, *flags;
	unsigned char* kind;
	unsigned int *loop, *loopback;
	float* attr;
	Quadric *vq, *aq;
	float4* ag;
	unsigned int *off_raw, *csr_raw, *comp_off, *cnt, *tcnt;
	unsigned int *keys_a, *vals_a, *keys_b, *vals_b;
	unsigned int *res0, *res1;
	unsigned int *adj_off, *fill;
	uint2* adj;
	uint4 *crec, *cring; // candidates in pick order (pick, then rank in place) and their decision records
	unsigned int* cerr;   // their error bits (setup: scratch of the duplicate and corner sorts)
	unsigned char* ckind; // their kinds
	unsigned int* rank;   // their sorted positions
	unsigned int* serr;   // error bits by sorted position (setup: each corner's slot in its remapped list)
	unsigned char *skind, *status; // kinds and decisions by sorted position
	unsigned int *act0, *act1, *commits;
	unsigned long long *minT, *minS;
	unsigned char* touched; // setup scratch (the permissive kinds)
	unsigned int* cr;
	unsigned int *comp, *parent;
	float* comp_err;
	uint4* blk;
	unsigned int* blkcnt;
	unsigned int* scratch;
	unsigned int* scratch2; // the pick's block-count scan, beside the adjacency scan in the pass loop
	unsigned int hash_mask;
	// the update mode only
	float4* vg;              // volume gradients (with attributes)
	float4* pos_new;         // solved positions
	unsigned char* vupdate;  // vertices the result uses (and their positions' primaries)
	unsigned int* sdone;     // position solve: 0 while the vertex is a pending candidate
	unsigned int *slist0, *slist1;
};

inline float __uint_as_float_host(unsigned int u)
{
	float f;
	memcpy(&f, &u, 4);
	return f;
}

size_t hashBuckets(size_t count)
{
	size_t b = 1;
	while (b < count + count / 4)
		b *= 2;
	return b;
}

// the undecided-candidate lists hold one region of whole blockDim tiles per kPerform block:
// at most the window plus one tile per block
constexpr size_t kListSlack = size_t(1) << 19;

size_t layout(Work& w, char* base, size_t I, size_t V, size_t ac, bool solve = false)
{
	Carver c{base};
	size_t Vp = V + 1;
	size_t cap = I + 4;              // collapse capacity bound (boundEdgeCollapses <= I + 3)
	size_t big = std::max(cap, Vp + 4); // sort buffers also hold the duplicate-vertex list (<= V)
	size_t T = I / 3 + 1;
	size_t hb = hashBuckets(V ? V : 1);
	w.hash_mask = (unsigned int)(hb - 1);
	w.sc = c.take<Scalars>(1);
	w.partial = c.take<float>(6 * 4096);
	w.pos_raw = c.take<float4>(Vp);
	w.pos = c.take<float4>(Vp);
	w.remap = c.take<unsigned int>(Vp);
	w.wedge = c.take<unsigned int>(Vp);
	w.table = c.take<unsigned int>(hb);
	w.slot = c.take<unsigned int>(Vp);
	w.flags = c.take<unsigned int>(Vp + 1);
	w.kind = c.take<unsigned char>(Vp);
	w.loop = c.take<unsigned int>(Vp);
	w.loopback = c.take<unsigned int>(Vp);
	w.attr = c.take<float>(Vp * (ac ? ac : 1));
	w.vq = c.take<Quadric>(Vp);
	w.aq = c.take<Quadric>(ac ? Vp : 1);
	w.ag = c.take<float4>(ac ? Vp * ac : 1);
	w.off_raw = c.take<unsigned int>(Vp + 1);
	w.csr_raw = c.take<unsigned int>(I + 1);
	w.comp_off = c.take<unsigned int>(Vp + 1);
	w.cnt = c.take<unsigned int>(Vp + 1);
	w.tcnt = c.take<unsigned int>(T + 2);
	w.keys_a = c.take<unsigned int>(big);
	w.vals_a = c.take<unsigned int>(big);
	w.keys_b = c.take<unsigned int>(big);
	w.vals_b = c.take<unsigned int>(big);
	w.res0 = c.take<unsigned int>(I + 1);
	w.res1 = c.take<unsigned int>(I + 1);
	w.adj_off = c.take<unsigned int>(Vp + 1);
	w.fill = c.take<unsigned int>(Vp);
	w.adj = c.take<uint2>(I + 1);
	w.crec = c.take<uint4>(big);
	w.cring = c.take<uint4>(cap);
	w.cerr = c.take<unsigned int>(big);
	w.ckind = c.take<unsigned char>(cap);
	w.rank = c.take<unsigned int>(cap);
	w.serr = c.take<unsigned int>(cap);
	w.skind = c.take<unsigned char>(cap);
	w.status = c.take<unsigned char>(cap);
	w.act0 = c.take<unsigned int>(cap + kListSlack); // per-block regions of whole tiles
	w.act1 = c.take<unsigned int>(cap + kListSlack);
	w.commits = c.take<unsigned int>(cap + kListSlack);
	w.minT = c.take<unsigned long long>(2 * Vp);
	w.minS = c.take<unsigned long long>(2 * Vp);
	w.touched = c.take<unsigned char>(Vp);
	w.comp = c.take<unsigned int>(Vp);
	w.parent = c.take<unsigned int>(Vp + 1);
	w.comp_err = c.take<float>(Vp + 1);
	w.cr = c.take<unsigned int>(Vp);
	w.blk = c.take<uint4>(std::max<size_t>(cap / kStopTile + 2, 8192)); // >= blocks of any cooperative launch
	w.blkcnt = c.take<unsigned int>(T / kThreads + 2);
	size_t sw = std::max(std::max(scanScratchWords(I + Vp + 2), radixScratchWords(big)), std::max(scanScratchWords(T + 2), keySortScratchWords(cap)));
	w.scratch = c.take<unsigned int>(sw);
	w.scratch2 = c.take<unsigned int>(scanScratchWords(T / kThreads + 2));
	const size_t Vs = solve ? Vp : 0;
	w.vg = (solve && ac) ? c.take<float4>(Vp) : nullptr;
	w.pos_new = c.take<float4>(Vs);
	w.vupdate = c.take<unsigned char>(Vs);
	w.sdone = c.take<unsigned int>(Vs);
	w.slist0 = c.take<unsigned int>(Vs + kListSlack * (solve ? 1 : 0));
	w.slist1 = c.take<unsigned int>(Vs + kListSlack * (solve ? 1 : 0));
	return c.off;
}

int bitsFor(size_t maxval)
{
	int b = 1;
	while (b < 32 && (size_t(1) << b) <= maxval)
		++b;
	return b;
}

// The pass's counting sort (kKeyHist, scan, kKeyScatter) of up to n candidates, in tiles of
// items * 256 (items: 4, 8 or 16): their sorted positions into w.rank, the error bits and kinds by
// sorted position into w.serr and w.skind. lv: the device-resident loop's live state (the grids
// cover n; the kernels and the scan take the live count from it, whose sort_items must equal
// items), else nullptr.
void sortCandidates(const Work& w, size_t n, cudaStream_t stream, const PassLive* lv, ScanSync ss, unsigned int items)
{
	if (n == 0)
		return;
	const unsigned int tiles = keySortTiles(n, items);
	const size_t m = size_t(tiles) * kKeyBins;
	unsigned int* hist = w.scratch;
	unsigned int* sscratch = w.scratch + ((m + 63) & ~size_t(63));
	if (lv)
		ss.n_dev = &lv->sort_cells;
	if (items == 4)
		MO_LAUNCH(kKeyHist<4>, tiles, kThreads, 0, stream, w.cerr, n, hist, lv);
	else if (items == 8)
		MO_LAUNCH(kKeyHist<8>, tiles, kThreads, 0, stream, w.cerr, n, hist, lv);
	else
		MO_LAUNCH(kKeyHist<16>, tiles, kThreads, 0, stream, w.cerr, n, hist, lv);
	scanExclusive(hist, hist, m, nullptr, sscratch, stream, ss);
	if (items == 4)
		MO_LAUNCH(kKeyScatter<4>, tiles, kThreads, kKeyScatterSmem, stream, w.cerr, w.ckind, n, hist, w.rank, w.serr, w.skind, lv);
	else if (items == 8)
		MO_LAUNCH(kKeyScatter<8>, tiles, kThreads, kKeyScatterSmem, stream, w.cerr, w.ckind, n, hist, w.rank, w.serr, w.skind, lv);
	else
		MO_LAUNCH(kKeyScatter<16>, tiles, kThreads, kKeyScatterSmem, stream, w.cerr, w.ckind, n, hist, w.rank, w.serr, w.skind, lv);
}

} // namespace

// ---------------------------------------------------------------- tuning

Tuning Tuning::fromEnvironment()
{
	Tuning t;
	if (const char* v = getenv("MESHOPTGPU_PERFORM_BLOCKS_PER_SM"))
		t.perform_blocks_per_sm = std::max(1, atoi(v));
	if (const char* v = getenv("MESHOPTGPU_WINDOW_FACTOR"))
		t.window_factor = std::max(0.0, atof(v));
	if (const char* v = getenv("MESHOPTGPU_DEVICE_LOOP"))
		t.device_loop = atoi(v) != 0;
	return t;
}

// ---------------------------------------------------------------- arena

DeviceArena::~DeviceArena()
{
	release();
}

void DeviceArena::release()
{
	if (base_)
		cudaFree(base_);
	base_ = nullptr;
	cap_ = 0;
}

void DeviceArena::reserve(size_t bytes)
{
	if (bytes <= cap_)
		return;
	release();
	size_t want = std::max(bytes, cap_ + cap_ / 4);
	MO_CUDA_CHECK(cudaMalloc(&base_, want));
	cap_ = want;
}

// ---------------------------------------------------------------- driver

Simplifier::Simplifier(int device) : device_(device)
{
	MO_CUDA_CHECK(cudaSetDevice(device));
	MO_CUDA_CHECK(cudaMallocHost(&pinned_, kPinnedBytes));
	MO_CUDA_CHECK(cudaStreamCreateWithFlags(&capture_, cudaStreamNonBlocking));
	MO_CUDA_CHECK(cudaStreamCreateWithFlags(&capture2_, cudaStreamNonBlocking));
	MO_CUDA_CHECK(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
	MO_CUDA_CHECK(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming));
	int sms = 0, per_sm = 0;
	MO_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
	MO_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kPerform, kPerformThreads, 0));
	MO_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&solve_per_sm_, kSolvePositions, kThreads, 0));
	MO_CUDA_CHECK(cudaFuncSetAttribute(kKeyScatter<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kKeyScatterSmem)));
	MO_CUDA_CHECK(cudaFuncSetAttribute(kKeyScatter<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kKeyScatterSmem)));
	MO_CUDA_CHECK(cudaFuncSetAttribute(kKeyScatter<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kKeyScatterSmem)));
	cudaDeviceGetAttribute(&clock_khz_, cudaDevAttrClockRate, device);
	sms_ = sms;
	coop_blocks_ = unsigned(std::max(1, sms * std::max(per_sm, 1)));
	tuning_ = Tuning::fromEnvironment();
	perform_blocks_ = std::min(coop_blocks_, unsigned(std::max(1, sms * tuning_.perform_blocks_per_sm)));
	coopScanCapacity(); // cached now: the pass loop's scans may first run while it is recorded
}

void Simplifier::dropLoopGraph()
{
	if (loop_.exec)
		cudaGraphExecDestroy(loop_.exec);
	if (loop_.graph)
		cudaGraphDestroy(loop_.graph);
	loop_ = LoopGraph{};
}

Simplifier::~Simplifier()
{
	dropLoopGraph();
	if (capture_)
		cudaStreamDestroy(capture_);
	if (capture2_)
		cudaStreamDestroy(capture2_);
	if (fork_)
		cudaEventDestroy(fork_);
	if (join_)
		cudaEventDestroy(join_);
	if (pinned_)
		cudaFreeHost(pinned_);
}

size_t Simplifier::workspaceBytes(size_t index_count, size_t vertex_count, size_t attribute_count)
{
	Work w;
	return layout(w, nullptr, index_count, vertex_count, attribute_count);
}

// Sparse subset (meshopt_SimplifySparse): the indices are rewritten to dense ids in order of
// first appearance, the used vertices are gathered into a compact mesh, the compact mesh is
// simplified, and the result is mapped back to the original vertex ids (:2367-2369, :2616-2619).
RunResult Simplifier::runSparse(const MeshDesc& m, unsigned int* d_out, cudaStream_t stream, PhaseTimes* times, SetupDump* dump)
{
	const size_t I = m.index_count, V = m.vertex_count;
	const size_t ac = m.attribute_count; // every attribute column is gathered; zero weights are dropped later
	// layout of the compact mesh in its own arena (the inner run uses the main one)
	auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
	size_t b_first = al((V + 1) * 4), b_flags = al((I + 1) * 4), b_rank = al((I + 1) * 4), b_dense = al((I + 1) * 4), b_map = al((I + 1) * 4);
	size_t b_pos = al((I + 1) * 12), b_attr = al((I + 1) * 4 * (ac ? ac : 1)), b_lock = al(I + 1), b_res = al((I + 1) * 4), b_scan = al(scanScratchWords(I + 2) * 4);
	size_t b_sc = 256;
	sparse_arena_.reserve(b_first + b_flags + b_rank + b_dense + b_map + b_pos + b_attr + b_lock + b_res + b_scan + b_sc);
	char* base = sparse_arena_.base();
	unsigned int* first = reinterpret_cast<unsigned int*>(base);
	unsigned int* flags = reinterpret_cast<unsigned int*>(base += b_first);
	unsigned int* rank = reinterpret_cast<unsigned int*>(base += b_flags);
	unsigned int* dense = reinterpret_cast<unsigned int*>(base += b_rank);
	unsigned int* smap = reinterpret_cast<unsigned int*>(base += b_dense);
	float* cpos = reinterpret_cast<float*>(base += b_map);
	float* cattr = reinterpret_cast<float*>(base += b_pos);
	unsigned char* clock = reinterpret_cast<unsigned char*>(base += b_attr);
	unsigned int* cres = reinterpret_cast<unsigned int*>(base += b_lock);
	unsigned int* scratch = reinterpret_cast<unsigned int*>(base += b_res);
	unsigned int* total = reinterpret_cast<unsigned int*>(base += b_scan);

	MO_CUDA_CHECK(cudaMemsetAsync(total, 0, 8, stream));
	if (m.indices_ready)
		MO_CUDA_CHECK(cudaStreamWaitEvent(stream, m.indices_ready, 0));
	if (I)
		MO_LAUNCH(kValidateIndices, gridFor(I, kThreads), kThreads, 0, stream, m.indices, I, V, total + 1);
	unsigned int hv[2] = {0, 0};
	MO_CUDA_CHECK(cudaMemcpyAsync(pinned_, total, 8, cudaMemcpyDeviceToHost, stream));
	MO_CUDA_CHECK(cudaStreamSynchronize(stream));
	memcpy(hv, pinned_, 8);
	if (hv[1])
		throw std::invalid_argument("index out of range of vertex_count");

	MO_CUDA_CHECK(cudaMemsetAsync(first, 0xFF, (V + 1) * 4, stream));
	if (I)
	{
		const unsigned int gI = gridFor(I, kThreads);
		MO_LAUNCH(kFirstUse, gI, kThreads, 0, stream, m.indices, I, first);
		MO_LAUNCH(kFirstFlags, gI, kThreads, 0, stream, m.indices, I, first, flags);
		scanExclusive(flags, rank, I, total, scratch, stream);
		MO_LAUNCH(kSparseIds, gI, kThreads, 0, stream, m.indices, I, first, rank, dense, smap);
	}
	else
		MO_CUDA_CHECK(cudaMemsetAsync(total, 0, 4, stream));
	MO_CUDA_CHECK(cudaMemcpyAsync(pinned_, total, 4, cudaMemcpyDeviceToHost, stream));
	MO_CUDA_CHECK(cudaStreamSynchronize(stream));
	const size_t U = pinned_[0];
	if (ac && m.attributes_ready)
		MO_CUDA_CHECK(cudaStreamWaitEvent(stream, m.attributes_ready, 0));
	if (U)
		MO_LAUNCH(kSparseGather, gridFor(U, kThreads), kThreads, 0, stream, smap, U, m.positions, m.positions_stride / 4, ac ? m.attributes : nullptr,
		    m.attributes_stride / 4, ac, m.lock, cpos, cattr, m.lock ? clock : nullptr);

	MeshDesc cm = m;
	cm.indices = dense;
	cm.vertex_count = U;
	cm.positions = cpos;
	cm.positions_stride = 12;
	cm.attributes = ac ? cattr : nullptr;
	cm.attributes_ready = nullptr;
	cm.indices_ready = nullptr;
	cm.attributes_stride = ac * 4;
	cm.lock = m.lock ? clock : nullptr;
	cm.options = m.options & ~(kOptSparse | kOptInternalDebug); // debug bits are not produced for sparse subsets (:2602)
	const bool solve = (m.options & kOptInternalSolve) != 0;
	if (solve)
	{
		cm.update_positions = cpos;
		cm.update_attributes = ac ? cattr : nullptr;
	}
	RunResult rr = run(cm, cres, stream, times, dump);
	if (solve && U)
		MO_LAUNCH(kSparseScatterBack, gridFor(U, kThreads), kThreads, 0, stream, smap, U, cpos, cattr, ac, m.update_positions, m.positions_stride / 4,
		    ac ? m.update_attributes : nullptr, m.attributes_stride / 4);
	if (rr.index_count)
		MO_LAUNCH(kSparseOut, gridFor(rr.index_count, kThreads), kThreads, 0, stream, cres, rr.index_count, smap, d_out);
	MO_CUDA_CHECK(cudaStreamSynchronize(stream));
	return rr;
}

float Simplifier::scale(const float* d_positions, size_t vertex_count, size_t stride, cudaStream_t stream)
{
	MO_CUDA_CHECK(cudaSetDevice(device_));
	Work w;
	size_t bytes = layout(w, nullptr, 0, vertex_count, 0);
	arena_.reserve(bytes);
	layout(w, arena_.base(), 0, vertex_count, 0);
	size_t V = vertex_count;
	if (V)
		MO_LAUNCH(kGatherPositions, gridFor(V, kThreads), kThreads, 0, stream, d_positions, stride / 4, V, w.pos_raw);
	size_t per = (V + kMinMaxMaxThreads - 1) / kMinMaxMaxThreads;
	per = per ? per : 1;
	unsigned int mmb = gridFor((V + per - 1) / per, kMinMaxThreads);
	MO_LAUNCH(kMinMaxPartial, mmb, kMinMaxThreads, 0, stream, w.pos_raw, V, per, w.partial);
	MO_LAUNCH(kMinMaxFinal, 1, kMinMaxThreads, 0, stream, w.partial, mmb, w.sc);
	Scalars* h = reinterpret_cast<Scalars*>(pinned_);
	MO_CUDA_CHECK(cudaMemcpyAsync(h, w.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
	MO_CUDA_CHECK(cudaStreamSynchronize(stream));
	probe().collect();
	return h->extent;
}

RunResult Simplifier::run(const MeshDesc& m, unsigned int* d_out, cudaStream_t stream, PhaseTimes* times, SetupDump* dump)
{
	MO_CUDA_CHECK(cudaSetDevice(device_));
	if (m.options & kOptSparse)
		return runSparse(m, d_out, stream, times, dump);
	RunResult rr;
	const size_t I = m.index_count, V = m.vertex_count;

	// attributes with weight > 0 only (:2410-2421)
	AttrMap am{};
	am.count = 0;
	for (size_t k = 0; k < m.attribute_count; ++k)
		if (m.weights[k] > 0)
		{
			am.src[am.count] = (unsigned int)k;
			am.weight[am.count] = m.weights[k];
			am.count++;
		}
	const int ac = am.count;
	const bool solve = (m.options & kOptInternalSolve) != 0;
	if (solve && (!m.update_positions || (ac && !m.update_attributes)))
		throw std::invalid_argument("the update mode needs writable position (and attribute) buffers");

	Work w;
	size_t bytes = layout(w, nullptr, I, V, ac, solve);
	arena_.reserve(bytes);
	layout(w, arena_.base(), I, V, ac, solve);

	Scalars* hs = reinterpret_cast<Scalars*>(pinned_);
	auto readScalars = [&]() {
		MO_CUDA_CHECK(cudaMemcpyAsync(hs, w.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
		MO_CUDA_CHECK(cudaStreamSynchronize(stream));
		if (hs->scan_error)
			throw std::runtime_error("grid barrier wait limit reached in a scan");
	};
	// scans and sorts of this run: one cooperative launch per scan (the run's stream is the only
	// one that uses these words)
	ScanSync ss;
	ss.bar = w.sc->scan_bar;
	ss.err = &w.sc->scan_error;
	ss.max_blocks = tuning_.perform_grid_cap > 0 ? unsigned(tuning_.perform_grid_cap) : 0u; // the pass kernel's share of the GPU
	// per-triangle pick codes live in the decision-record array, which rank fills only after the pick
	unsigned short* const pick_codes = reinterpret_cast<unsigned short*>(w.cring);

	cudaEvent_t ev[16];
	bool timed = times != nullptr;
	if (timed)
		for (auto& e : ev)
			MO_CUDA_CHECK(cudaEventCreate(&e));
	float acc_adj = 0, acc_pick = 0, acc_rank = 0, acc_sort = 0, acc_perf = 0, acc_apply = 0;
	auto elapsed = [&](int a, int b) {
		float ms = 0;
		MO_CUDA_CHECK(cudaEventElapsedTime(&ms, ev[a], ev[b]));
		return ms;
	};

	if (timed)
		MO_CUDA_CHECK(cudaEventRecord(ev[0], stream));

	MO_CUDA_CHECK(cudaMemsetAsync(w.sc, 0, sizeof(Scalars), stream));

	// ---- setup
	const unsigned int gV = gridFor(V, kThreads), gI = gridFor(I, kThreads);
	if (V)
		MO_LAUNCH(kGatherPositions, gV, kThreads, 0, stream, m.positions, m.positions_stride / 4, V, w.pos_raw);

	// position remap + wedges
	MO_CUDA_CHECK(cudaMemsetAsync(w.table, 0xFF, size_t(w.hash_mask + 1) * 4, stream));
	if (V)
	{
		MO_LAUNCH(kHashInsert, gV, kThreads, 0, stream, w.pos_raw, V, w.table, w.hash_mask, w.slot, &w.sc->probe_fail);
		MO_LAUNCH(kHashRemap, gV, kThreads, 0, stream, w.table, w.slot, V, w.remap, w.wedge, w.flags);
		scanExclusive(w.flags, w.flags, V, &w.sc->dup_count, w.scratch, stream, ss);
	}
	// vertex -> corner lists in corner order: raw (classification, attribute quadrics) and
	// remapped (position quadrics). Their offsets and largest degrees come before the host read
	// below, which decides how the lists are filled.
	// each corner's slot in its vertex's list, in res1 (free until the passes)
	unsigned int* const slot_raw = w.res1;
	// the counts in one pass over the indices, in the offset array itself (scanned in place); the
	// count also validates the indices (the first kernel that reads them), and the host read
	// below reports a bad index before anything else uses the lists. A position group's corners
	// are the merge of its wedges' lists (the quadric fill walks them), so no welded list is built.
	MO_CUDA_CHECK(cudaMemsetAsync(w.off_raw, 0, (V + 1) * 4, stream));
	if (m.indices_ready)
		MO_CUDA_CHECK(cudaStreamWaitEvent(stream, m.indices_ready, 0));
	if (I)
		MO_LAUNCH(kCountCornerLists, gI, kThreads, 0, stream, m.indices, I, V, w.off_raw, slot_raw, &w.sc->bad_index, w.res0);
	scanExclusive(w.off_raw, w.off_raw, V + 1, nullptr, w.scratch, stream, ss);
	if (V)
		MO_LAUNCH(kMaxDegree, gV, kThreads, 0, stream, w.off_raw, V, &w.sc->max_degree);
	// flags now hold offsets; recompute flags from remap in the compaction kernel
	readScalars();
	if (hs->bad_index)
		throw std::invalid_argument("index out of range of vertex_count");
	if (hs->probe_fail)
		throw std::runtime_error("position hash table overflow");
	const size_t D = hs->dup_count;
	if (D)
	{
		// rebuild the dup flags (the scan consumed them) into cnt, then compact
		MO_LAUNCH(kHashRemap, gV, kThreads, 0, stream, w.table, w.slot, V, w.remap, w.wedge, w.cnt);
		MO_LAUNCH(kCompactFlagged, gV, kThreads, 0, stream, w.cnt, w.flags, w.remap, V, w.keys_b, w.vals_b);
		radixSortPairs(w.keys_b, w.vals_b, w.keys_a, w.vals_a, w.cerr, reinterpret_cast<unsigned int*>(w.crec), D, bitsFor(V), w.scratch, stream, nullptr, ss);
		MO_LAUNCH(kWedgeLink, gridFor(D, kThreads), kThreads, 0, stream, w.keys_a, w.vals_a, D, w.wedge);
	}

	const int vbits = bitsFor(V ? V - 1 : 0);
	if (hs->max_degree <= kCornerSortMax)
	{
		// few corners per vertex: fill and sort each list in place
		if (I && V)
		{
			MO_LAUNCH(kCornerFill, gI, kThreads, 0, stream, w.res0, nullptr, I, w.off_raw, slot_raw, w.csr_raw);
			MO_LAUNCH(kCornerSort, gV, kThreads, 0, stream, w.off_raw, V, w.csr_raw);
		}
	}
	else
	{
		// a vertex with many corners: a stable radix sort by vertex
		radixSortPairs(w.res0, nullptr, w.keys_a, w.csr_raw, w.keys_b, w.vals_b, I, vbits, w.scratch, stream, nullptr, ss);
	}

	// classification
	if (V)
	{
		MO_LAUNCH(kOpenEdges, gV, kThreads, 0, stream, w.res0, w.off_raw, w.csr_raw, V, w.loop, w.loopback);
		MO_LAUNCH(kClassify, gV, kThreads, 0, stream, V, w.remap, w.wedge, w.loop, w.loopback, w.kind);
		if (m.options & kOptPermissive)
		{
			MO_LAUNCH(kPermissivePrimary, gV, kThreads, 0, stream, V, w.res0, w.off_raw, w.csr_raw, w.remap, w.wedge, m.lock, w.kind, w.touched);
			MO_LAUNCH(kPermissiveWedges, gV, kThreads, 0, stream, V, w.remap, w.touched, w.kind);
		}
		if (m.lock)
		{
			MO_LAUNCH(kLockMark, gV, kThreads, 0, stream, V, m.lock, w.remap, w.kind);
			MO_LAUNCH(kLockSpread, gV, kThreads, 0, stream, V, w.remap, w.kind);
		}
		if (m.options & kOptLockBorder)
			MO_LAUNCH(kLockBorder, gV, kThreads, 0, stream, V, w.kind);
	}

	// rescale
	size_t per = (V + kMinMaxMaxThreads - 1) / kMinMaxMaxThreads;
	per = per ? per : 1;
	unsigned int mmb = gridFor((V + per - 1) / per, kMinMaxThreads);
	MO_LAUNCH(kMinMaxPartial, mmb, kMinMaxThreads, 0, stream, w.pos_raw, V, per, w.partial);
	MO_LAUNCH(kMinMaxFinal, 1, kMinMaxThreads, 0, stream, w.partial, mmb, w.sc);
	if (V)
		MO_LAUNCH(kRescale, gV, kThreads, 0, stream, w.pos_raw, V, w.sc, w.pos);
	if (ac && V)
	{
		if (m.attributes_ready)
			MO_CUDA_CHECK(cudaStreamWaitEvent(stream, m.attributes_ready, 0));
		MO_LAUNCH(kRescaleAttributes, gV, kThreads, 0, stream, m.attributes, m.attributes_stride / 4, V, am, w.attr);
	}

	// quadrics
	float factor = (m.options & kOptRegularizeLight) ? 1e-2f : ((m.options & kOptRegularize) ? 1e-1f : 1e-7f);
	if (V)
		MO_LAUNCH(kFillQuadrics, gV, kThreads, 0, stream, w.res0, w.off_raw, w.csr_raw, V, w.pos, w.remap, w.wedge, w.kind, w.loop, w.loopback, m.lock, factor, w.vq,
		    (solve && ac) ? w.vg : nullptr);
	if (ac && V)
	{
		if (ac <= 4)
			MO_LAUNCH(kFillAttributeQuadrics<4>, gridFor(V, 128), 128, 0, stream, w.res0, w.off_raw, w.csr_raw, V, w.pos, w.attr, ac, w.aq, w.ag);
		else if (ac <= 8)
			MO_LAUNCH(kFillAttributeQuadrics<8>, gridFor(V, 128), 128, 0, stream, w.res0, w.off_raw, w.csr_raw, V, w.pos, w.attr, ac, w.aq, w.ag);
		else if (ac <= 16)
			MO_LAUNCH(kFillAttributeQuadrics<16>, gridFor(V, 128), 128, 0, stream, w.res0, w.off_raw, w.csr_raw, V, w.pos, w.attr, ac, w.aq, w.ag);
		else
			MO_LAUNCH(kFillAttributeQuadrics<32>, gridFor(V, 64), 64, 0, stream, w.res0, w.off_raw, w.csr_raw, V, w.pos, w.attr, ac, w.aq, w.ag);
	}
	size_t comp_count = 0;
	if ((m.options & kOptPrune) && V)
	{
		// components of the welded mesh, numbered in root order, then their radii
		MO_LAUNCH(kIota, gV, kThreads, 0, stream, w.parent, V);
		if (I)
			MO_LAUNCH(kUnionEdges, gridFor(I / 3, kThreads), kThreads, 0, stream, w.res0, I / 3, w.remap, w.parent);
		MO_LAUNCH(kComponentRoots, gV, kThreads, 0, stream, V, w.remap, w.parent, w.flags);
		scanExclusive(w.flags, w.fill, V, &w.sc->dup_count, w.scratch, stream, ss);
		MO_LAUNCH(kComponentIds, gV, kThreads, 0, stream, V, w.remap, w.parent, w.fill, w.comp);
		readScalars();
		comp_count = hs->dup_count;
		MO_CUDA_CHECK(cudaMemsetAsync(w.cnt, 0, (comp_count + 1) * 4, stream));
		MO_LAUNCH(kCountKeys, gV, kThreads, 0, stream, w.comp, nullptr, V, w.cnt);
		scanExclusive(w.cnt, w.comp_off, comp_count + 1, nullptr, w.scratch, stream, ss);
		radixSortPairs(w.comp, nullptr, w.keys_a, w.vals_a, w.keys_b, w.vals_b, V, bitsFor(comp_count ? comp_count - 1 : 0), w.scratch, stream, nullptr, ss);
		MO_LAUNCH(kMeasureComponents, gridFor(comp_count, kThreads), kThreads, 0, stream, comp_count, w.comp_off, w.vals_a, w.pos, w.comp_err);
	}
	if (V)
		MO_LAUNCH(kDualCount, gV, kThreads, 0, stream, w.off_raw, w.kind, V, &w.sc->dual);
	MO_LAUNCH(kCapacity, 1, 32, 0, stream, I, w.sc);
	MO_CUDA_CHECK(cudaGetLastError());

	// The device-resident pass loop (below) takes no host values from setup: its graph is
	// recorded and instantiated while the setup kernels run, and the extent is read after it.
	// Pruning, the debug bit and per-phase event timing need the host between passes.
	const bool device_loop =
	    tuning_.device_loop && !timed && !dump && !(m.options & (kOptPrune | kOptInternalDebug)) && I > m.target_index_count;
	float vertex_scale = 0.f, error_scale = 1.f, error_limit = 0.f;
	auto takeScale = [&]() {
		vertex_scale = hs->extent;
		rr.scale = vertex_scale;
		error_scale = (m.options & kOptErrorAbsolute) ? vertex_scale : 1.f;
		error_limit = (m.target_error * m.target_error) / (error_scale * error_scale);
	};
	if (!device_loop)
	{
		readScalars();
		takeScale();
	}

	if (dump)
	{
		MO_CUDA_CHECK(cudaStreamSynchronize(stream));
		dump->remap.resize(V);
		dump->wedge.resize(V);
		dump->loop.resize(V);
		dump->loopback.resize(V);
		dump->kind.resize(V);
		dump->positions.resize(V * 3);
		dump->quadrics.resize(V * 11);
		MO_CUDA_CHECK(cudaMemcpy(dump->remap.data(), w.remap, V * 4, cudaMemcpyDeviceToHost));
		MO_CUDA_CHECK(cudaMemcpy(dump->wedge.data(), w.wedge, V * 4, cudaMemcpyDeviceToHost));
		MO_CUDA_CHECK(cudaMemcpy(dump->loop.data(), w.loop, V * 4, cudaMemcpyDeviceToHost));
		MO_CUDA_CHECK(cudaMemcpy(dump->loopback.data(), w.loopback, V * 4, cudaMemcpyDeviceToHost));
		MO_CUDA_CHECK(cudaMemcpy(dump->kind.data(), w.kind, V, cudaMemcpyDeviceToHost));
		std::vector<float4> p4(V);
		std::vector<Quadric> q(V);
		MO_CUDA_CHECK(cudaMemcpy(p4.data(), w.pos, V * 16, cudaMemcpyDeviceToHost));
		MO_CUDA_CHECK(cudaMemcpy(q.data(), w.vq, V * sizeof(Quadric), cudaMemcpyDeviceToHost));
		for (size_t i = 0; i < V; ++i)
		{
			dump->positions[i * 3 + 0] = p4[i].x;
			dump->positions[i * 3 + 1] = p4[i].y;
			dump->positions[i * 3 + 2] = p4[i].z;
			memcpy(&dump->quadrics[i * 11], &q[i], 11 * 4);
		}
		if (ac)
		{
			dump->attr_quadrics.resize(V * 11);
			dump->attr_gradients.resize(V * 4 * ac);
			MO_CUDA_CHECK(cudaMemcpy(q.data(), w.aq, V * sizeof(Quadric), cudaMemcpyDeviceToHost));
			for (size_t i = 0; i < V; ++i)
				memcpy(&dump->attr_quadrics[i * 11], &q[i], 11 * 4);
			MO_CUDA_CHECK(cudaMemcpy(dump->attr_gradients.data(), w.ag, V * 16 * ac, cudaMemcpyDeviceToHost));
		}
		dump->capacity = hs->capacity;
		dump->scale = vertex_scale;
	}

	if (timed)
		MO_CUDA_CHECK(cudaEventRecord(ev[1], stream));

	// ---- pass loop (src/simplifier.cpp:2493-2541)
	size_t result_count = I;
	unsigned int* res = w.res0;
	unsigned int* res_next = w.res1;
	unsigned int result_error_bits = 0;
	float vertex_error = 0.f;
	float comp_next = 0.f;
	// pruneComponents (:1996-2024): keep triangles of components above the cutoff, in order;
	// comp_next becomes the smallest error among the components left
	auto prune = [&](float cutoff) {
		const size_t T = result_count / 3;
		const unsigned int gT = gridFor(T, kThreads);
		MO_CUDA_CHECK(cudaMemsetAsync(&w.sc->done, 0xFF, 4, stream)); // min error of kept components
		if (T)
		{
			MO_LAUNCH(kPruneCount, gT, kThreads, 0, stream, res, T, w.comp, w.comp_err, cutoff, w.blkcnt, &w.sc->done);
			scanExclusive(w.blkcnt, w.blkcnt, gT, &w.sc->tri_total, w.scratch, stream, ss);
			MO_LAUNCH(kPruneEmit, gT, kThreads, 0, stream, res, T, w.comp, w.comp_err, cutoff, w.blkcnt, res_next);
		}
		else
			MO_CUDA_CHECK(cudaMemsetAsync(&w.sc->tri_total, 0, 4, stream));
		readScalars();
		unsigned int mb = hs->done;
		comp_next = mb == ~0u ? FLT_MAX : __uint_as_float_host(mb);
		result_count = size_t(hs->tri_total) * 3;
		std::swap(res, res_next);
	};
	if (comp_count)
	{
		MO_CUDA_CHECK(cudaMemsetAsync(&w.sc->done, 0xFF, 4, stream));
		MO_LAUNCH(kMinFloat, gridFor(comp_count, kThreads), kThreads, 0, stream, w.comp_err, comp_count, &w.sc->done);
		readScalars();
		comp_next = __uint_as_float_host(hs->done);
	}
	else if (m.options & kOptPrune)
		comp_next = FLT_MAX;
	int passes = 0;
	double window_factor = tuning_.window_factor; // the host loop's first-window factor, as kPassEnd adapts it
	unsigned int round_base = 0; // decision rounds are numbered across the run (mark tags never repeat)

	// ---- the pass loop on the device: one pass recorded into the body of a WHILE conditional
	// node, replayed until kPassEnd ends it
	if (device_loop)
	{
		// grids cover the capacity bound (boundEdgeCollapses <= I + 3); the kernels stop at the
		// live counts
		const size_t T0 = I / 3, capn = I + 3;
		PassLive init{};
		init.res = w.res0;
		init.res_next = w.res1;
		init.indices = unsigned(I);
		init.tris = unsigned(T0);
		init.target = unsigned(m.target_index_count);
		const unsigned int sort_items = sort_items_ ? sort_items_ : keySortItems(capn);
		init.sort_items = sort_items;
		init.window_factor = tuning_.window_factor;
		init.window_base = tuning_.window_factor;
		MO_CUDA_CHECK(cudaMemcpyAsync(&w.sc->live, &init, sizeof(init), cudaMemcpyHostToDevice, stream));
		MO_CUDA_CHECK(cudaMemsetAsync(&w.sc->result_error_bits, 0, 4, stream));
		MO_LAUNCH(kErrorLimit, 1, 1, 0, stream, w.sc, m.target_error, (m.options & kOptErrorAbsolute) ? 1 : 0);
		const PassLive* lv = &w.sc->live;

		// grid of the pass kernel
		unsigned int blocks = std::max(1u, std::min(perform_blocks_, gridFor(std::max(std::max(capn, V), T0), kPerformThreads)));
		if (tuning_.perform_grid_cap > 0)
			blocks = std::min(blocks, unsigned(tuning_.perform_grid_cap));
		if (size_t(blocks) * kPerformThreads > kListSlack)
			throw std::runtime_error("kPerform grid exceeds the candidate list slack");

		LaunchProbe& lp = probe();
		const bool reuse = loop_.exec && loop_.base == arena_.base() && loop_.I == I && loop_.V == V && loop_.ac == ac && loop_.solve == solve &&
		                   loop_.blocks == blocks && loop_.sort_items == sort_items && loop_.scan_blocks == ss.max_blocks;
		if (!reuse)
		{
			dropLoopGraph();
			// the new graph and its executable are released if recording or instantiation fails
			struct GraphGuard
			{
				cudaGraph_t graph = nullptr;
				cudaGraphExec_t exec = nullptr;
				~GraphGuard()
				{
					if (exec)
						cudaGraphExecDestroy(exec);
					if (graph)
						cudaGraphDestroy(graph);
				}
			} guard;
			MO_CUDA_CHECK(cudaGraphCreate(&guard.graph, 0));
			cudaGraph_t graph = guard.graph;
			cudaGraphConditionalHandle handle;
			MO_CUDA_CHECK(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
			cudaGraphNodeParams cp = {};
			cp.type = cudaGraphNodeTypeConditional;
			cp.conditional.handle = handle;
			cp.conditional.type = cudaGraphCondTypeWhile;
			cp.conditional.size = 1;
			cudaGraphNode_t loop_node;
			MO_CUDA_CHECK(cudaGraphAddNode(&loop_node, graph, nullptr, nullptr, 0, &cp));
			cudaGraph_t body = cp.conditional.phGraph_out[0];

			const unsigned long long launches0 = lp.launches;
			cudaStream_t cs = capture_; // recording only: nothing runs on it
			MO_CUDA_CHECK(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
			lp.capturing = true;
			try
			{
				const unsigned int gI = gridFor(I, kThreads), gT0 = gridFor(T0, kThreads);
				// the pick (its own scan scratch and barrier words) and the adjacency are independent:
				// two branches of the body, joined before the rank
				cudaStream_t cs2 = capture2_;
				ScanSync ss2 = ss;
				ss2.bar = w.sc->scan_bar2;
				MO_CUDA_CHECK(cudaEventRecord(fork_, cs));
				MO_CUDA_CHECK(cudaStreamWaitEvent(cs2, fork_, 0));
				MO_LAUNCH(kPickCount, gT0, kThreads, 0, cs2, nullptr, T0, w.remap, w.kind, w.loop, w.loopback, w.tcnt, pick_codes, lv);
				scanExclusive(w.tcnt, w.tcnt, gT0, &w.sc->pick_total, w.scratch2, cs2, ss2);
				MO_CUDA_CHECK(cudaMemsetAsync(&w.sc->pick_trunc, 0xFF, 4, cs2));
				MO_LAUNCH(kPickEmit, gT0, kThreads, 0, cs2, nullptr, T0, pick_codes, w.tcnt, w.sc, w.crec, lv);
				MO_CUDA_CHECK(cudaEventRecord(join_, cs2));
				MO_CUDA_CHECK(cudaMemsetAsync(w.cnt, 0, (V + 1) * 4, cs));
				MO_LAUNCH(kCountCorners, gI, kThreads, 0, cs, nullptr, I, w.remap, w.cnt, nullptr, lv);
				scanExclusive(w.cnt, w.adj_off, V + 1, nullptr, w.scratch, cs, ss);
				MO_LAUNCH(kAdjFill, gT0, kThreads, 0, cs, nullptr, T0, w.remap, w.adj_off, nullptr, w.adj, lv, I);
				MO_CUDA_CHECK(cudaStreamWaitEvent(cs, join_, 0));
				MO_LAUNCH(kPassPrep, 1, 1, 0, cs, w.sc);
				MO_LAUNCH(kRank, gridFor(capn, kRankThreads), kRankThreads, 0, cs, capn, w.crec, w.cring, w.cerr, w.ckind, w.pos, w.vq, w.remap, w.wedge, w.kind, w.loop, w.loopback,
				    w.adj_off, w.attr, w.aq, w.ag, ac, lv);
				sortCandidates(w, capn, cs, lv, ss, sort_items);
				PerformArgs pa;
				pa.count = 0;
				pa.crec = w.crec;
				pa.cring = w.cring;
				pa.rank = w.rank;
				pa.skind = w.skind;
				pa.serr = w.serr;
				pa.status = w.status;
				pa.vcount = unsigned(V);
				pa.minT[0] = w.minT;
				pa.minT[1] = w.minT + (V + 1);
				pa.minS = w.minS;
				pa.cr = w.cr;
				pa.list[0] = w.act0;
				pa.list[1] = w.act1;
				pa.commits = w.commits;
				pa.adj_off = w.adj_off;
				pa.adj = w.adj;
				pa.pos = w.pos;
				pa.remap = w.remap;
				pa.wedge = w.wedge;
				pa.loop = w.loop;
				pa.loopback = w.loopback;
				pa.vq = w.vq;
				pa.aq = w.aq;
				pa.ag = w.ag;
				pa.ac = ac;
				pa.vg = (solve && ac) ? w.vg : nullptr;
				pa.prev_err_bits = 0;
				pa.error_limit = 0.f; // the live state's
				pa.goal = 0;
				pa.first_window = 0;
				pa.round_base = 0;
				pa.res = nullptr;
				pa.res_next = nullptr;
				pa.tris = 0;
				pa.blk = w.blk;
				pa.sc = w.sc;
				pa.live = lv;
				void* params[] = {&pa};
				lp.launches++;
				MO_CUDA_CHECK(cudaLaunchCooperativeKernel((const void*)kPerform, dim3(blocks), dim3(kPerformThreads), params, 0, cs));
				MO_LAUNCH(kPassEnd, 1, 1, 0, cs, w.sc, handle, unsigned(T0 + 1));
			}
			catch (...)
			{
				lp.capturing = false;
				cudaGraph_t dead = nullptr;
				cudaStreamEndCapture(cs, &dead);
				throw;
			}
			lp.capturing = false;
			cudaGraph_t captured = nullptr;
			MO_CUDA_CHECK(cudaStreamEndCapture(cs, &captured));
			MO_CUDA_CHECK(cudaGraphInstantiate(&guard.exec, graph, 0));
			loop_.body_launches = lp.launches - launches0;
			lp.launches = launches0; // counted below, once per replay
			loop_.graph = guard.graph;
			loop_.exec = guard.exec;
			guard.graph = nullptr;
			guard.exec = nullptr;
			loop_.base = arena_.base();
			loop_.I = I;
			loop_.V = V;
			loop_.ac = ac;
			loop_.solve = solve;
			loop_.blocks = blocks;
			loop_.sort_items = sort_items;
			loop_.scan_blocks = ss.max_blocks;
		}
		MO_CUDA_CHECK(cudaGraphLaunch(loop_.exec, stream));
		readScalars();
		takeScale();
		lp.launches += loop_.body_launches * hs->live.iterations;
		if (hs->grid_error)
			throw std::runtime_error(hs->grid_error & 4 ? "pass loop did not converge"
			                                            : (hs->grid_error & 2 ? "collapse decision round made no progress" : "grid barrier wait limit reached"));
		passes = int(hs->live.passes);
		for (int p = 0; p < passes && p < kMaxPassStats; ++p)
			rr.pass[p] = hs->pstats[p];
		result_error_bits = hs->result_error_bits;
		result_count = hs->live.indices;
		res = const_cast<unsigned int*>(hs->live.res);
	}
	else
	while (result_count > m.target_index_count)
	{
		const size_t T = result_count / 3;
		const unsigned int gT = gridFor(T, kThreads);
		if (timed)
			MO_CUDA_CHECK(cudaEventRecord(ev[2], stream));

		// adjacency of the current result, welded by remap
		MO_CUDA_CHECK(cudaMemsetAsync(w.cnt, 0, (V + 1) * 4, stream));
		MO_LAUNCH(kCountCorners, gridFor(result_count, kThreads), kThreads, 0, stream, res, result_count, w.remap, w.cnt, res_next, nullptr);
		scanExclusive(w.cnt, w.adj_off, V + 1, nullptr, w.scratch, stream, ss);
		MO_LAUNCH(kAdjFill, gT, kThreads, 0, stream, res, T, w.remap, w.adj_off, res_next, w.adj, nullptr, I);
		if (timed)
			MO_CUDA_CHECK(cudaEventRecord(ev[3], stream));

		// pick
		MO_LAUNCH(kPickCount, gT, kThreads, 0, stream, res, T, w.remap, w.kind, w.loop, w.loopback, w.tcnt, pick_codes, nullptr);
		scanExclusive(w.tcnt, w.tcnt, gT, &w.sc->pick_total, w.scratch, stream, ss);
		MO_CUDA_CHECK(cudaMemsetAsync(&w.sc->pick_trunc, 0xFF, 4, stream));
		MO_LAUNCH(kPickEmit, gT, kThreads, 0, stream, res, T, pick_codes, w.tcnt, w.sc, w.crec, nullptr);
		readScalars();
		const size_t C = std::min<size_t>(hs->pick_total, hs->pick_trunc);
		if (timed)
			MO_CUDA_CHECK(cudaEventRecord(ev[4], stream));
		if (C == 0)
			break;

		// rank + sort
		MO_LAUNCH(kRank, gridFor(C, kRankThreads), kRankThreads, 0, stream, C, w.crec, w.cring, w.cerr, w.ckind, w.pos, w.vq, w.remap, w.wedge, w.kind, w.loop, w.loopback,
		    w.adj_off, w.attr, w.aq, w.ag, ac, nullptr);
		if (timed)
			MO_CUDA_CHECK(cudaEventRecord(ev[5], stream));
		sortCandidates(w, C, stream, nullptr, ss, sort_items_ ? sort_items_ : keySortItems(C));
		if (timed)
			MO_CUDA_CHECK(cudaEventRecord(ev[6], stream));

		// perform: decisions, stop rules, apply, loop remap and compaction in one cooperative launch
		const size_t goal = (result_count - m.target_index_count) / 3;
		{
			PerformArgs pa;
			pa.count = unsigned(C);
			pa.crec = w.crec;
			pa.cring = w.cring;
			pa.rank = w.rank;
			pa.skind = w.skind;
			pa.serr = w.serr;
			pa.status = w.status;
			pa.vcount = unsigned(V);
			pa.minT[0] = w.minT;
			pa.minT[1] = w.minT + (V + 1);
			pa.minS = w.minS;
			pa.cr = w.cr;
			pa.list[0] = w.act0;
			pa.list[1] = w.act1;
			pa.commits = w.commits;
			pa.adj_off = w.adj_off;
			pa.adj = w.adj;
			pa.pos = w.pos;
			pa.remap = w.remap;
			pa.wedge = w.wedge;
			pa.loop = w.loop;
			pa.loopback = w.loopback;
			pa.vq = w.vq;
			pa.aq = w.aq;
			pa.ag = w.ag;
			pa.ac = ac;
			pa.vg = (solve && ac) ? w.vg : nullptr;
			pa.prev_err_bits = result_error_bits;
			pa.error_limit = error_limit;
			pa.goal = goal;
			double wf = window_factor * double(goal / 2) + 4096.0;
			pa.first_window = unsigned(std::min<double>(double(C), wf));
			pa.round_base = round_base;
			pa.res = res;
			pa.res_next = res_next;
			pa.tris = unsigned(T);
			pa.blk = w.blk;
			pa.live = nullptr;
			pa.sc = w.sc;
			MO_CUDA_CHECK(cudaMemsetAsync(w.sc->bar, 0, sizeof(unsigned int) * 3, stream));
			MO_CUDA_CHECK(cudaMemsetAsync(&w.sc->cut, 0xFF, 8, stream));
			MO_CUDA_CHECK(cudaMemsetAsync(&w.sc->done, 0, 12, stream));
			MO_CUDA_CHECK(cudaMemcpyAsync(&w.sc->result_error_bits, &result_error_bits, 4, cudaMemcpyHostToDevice, stream));
			unsigned int want = gridFor(std::max(std::max(C, V), T), kPerformThreads);
			unsigned int blocks = std::max(1u, std::min(perform_blocks_, want));
			if (tuning_.perform_grid_cap > 0)
				blocks = std::min(blocks, unsigned(tuning_.perform_grid_cap));
			if (size_t(blocks) * kPerformThreads > kListSlack)
				throw std::runtime_error("kPerform grid exceeds the candidate list slack");
			void* params[] = {&pa};
			cudaEvent_t e0 = probeBegin("kPerform", stream);
			MO_CUDA_CHECK(cudaLaunchCooperativeKernel((const void*)kPerform, dim3(blocks), dim3(kPerformThreads), params, 0, stream));
			probeEnd(e0, stream);
		}
		if (timed)
			MO_CUDA_CHECK(cudaEventRecord(ev[7], stream));
		readScalars();
		if (hs->grid_error)
			throw std::runtime_error(hs->grid_error & 2 ? "collapse decision round made no progress" : "grid barrier wait limit reached");
		const unsigned long long cutv = hs->cut;
		const size_t cut = cutv == ~0ull ? C : size_t(cutv >> 2);
		const unsigned int reason = cutv == ~0ull ? 0 : unsigned(cutv & 3);
		round_base += hs->rounds;
		if (passes < kMaxPassStats)
		{
			PassStats& ps = rr.pass[passes];
			ps.triangles = unsigned(T);
			ps.candidates = unsigned(C);
			ps.evaluated = unsigned(cut < C ? cut + 1 : C);
			ps.done = hs->done;
			ps.skipped = hs->skipped;
			ps.invalid = hs->invalid;
			ps.stop = reason;
			ps.rounds = hs->rounds;
			ps.active = unsigned(hs->active_sum);
			ps.windows = hs->windows;
		}
		window_factor = nextWindowFactor(tuning_.window_factor, goal, cut < C ? cut + 1 : C);
		passes++;
		result_error_bits = hs->result_error_bits;
		if (hs->done == 0)
			break;
		const float derr_pass = __uint_as_float_host(hs->vertex_error_bits);
		result_count = size_t(hs->tri_total) * 3;
		std::swap(res, res_next);
		vertex_error = ac == 0 ? __uint_as_float_host(result_error_bits) : derr_pass;
		if ((m.options & kOptPrune) && result_count > m.target_index_count && comp_next <= vertex_error)
			prune(vertex_error);
		if (timed)
		{
			const std::array<float, 5> ph = {elapsed(2, 3), elapsed(3, 4), elapsed(4, 5), elapsed(5, 6), elapsed(6, 7)};
			acc_adj += ph[0];
			acc_pick += ph[1];
			acc_rank += ph[2];
			acc_sort += ph[3];
			acc_perf += ph[4];
			rr.pass_phase_ms.push_back(ph);
		}
	}

	// prune cleanup (:2543-2569): remove small components towards the error limit
	bool comp_stale = true;
	while ((m.options & kOptPrune) && result_count > m.target_index_count && comp_next <= error_limit)
	{
		float cutoff = comp_next * 1.5f < error_limit ? comp_next * 1.5f : error_limit;
		MO_CUDA_CHECK(cudaMemsetAsync(&w.sc->skipped, 0, 4, stream));
		if (comp_count)
			MO_LAUNCH(kMaxBelow, gridFor(comp_count, kThreads), kThreads, 0, stream, w.comp_err, comp_count, cutoff, &w.sc->skipped);
		readScalars();
		const float maxerr = __uint_as_float_host(hs->skipped);
		const size_t before = result_count;
		prune(cutoff);
		if (result_count == before && !comp_stale)
			break;
		comp_stale = false;
		float re = __uint_as_float_host(result_error_bits);
		re = re < maxerr ? maxerr : re;
		memcpy(&result_error_bits, &re, 4);
		vertex_error = vertex_error < maxerr ? maxerr : vertex_error;
	}

	// the update mode (:2575-2599): solve the vertices the result uses and write them back
	if (solve && V)
	{
		const size_t T = result_count / 3;
		MO_CUDA_CHECK(cudaMemsetAsync(w.vupdate, 0, V, stream));
		MO_CUDA_CHECK(cudaMemsetAsync(w.cnt, 0, (V + 1) * 4, stream));
		MO_CUDA_CHECK(cudaMemsetAsync(w.sc->solve_pending, 0, sizeof(w.sc->solve_pending), stream));
		unsigned int* slot = res == w.res0 ? w.res1 : w.res0; // the index buffer the result is not in
		if (result_count)
		{
			MO_LAUNCH(kMarkUpdate, gridFor(result_count, kThreads), kThreads, 0, stream, res, result_count, w.remap, w.vupdate);
			MO_LAUNCH(kCountCorners, gridFor(result_count, kThreads), kThreads, 0, stream, res, result_count, w.remap, w.cnt, slot, nullptr);
		}
		scanExclusive(w.cnt, w.adj_off, V + 1, nullptr, w.scratch, stream, ss);
		if (T)
			MO_LAUNCH(kAdjFill, gridFor(T, kThreads), kThreads, 0, stream, res, T, w.remap, w.adj_off, slot, w.adj, nullptr, I);
		MO_CUDA_CHECK(cudaMemcpyAsync(w.pos_new, w.pos, V * sizeof(float4), cudaMemcpyDeviceToDevice, stream));
		const unsigned int gV = gridFor(V, kThreads);
		MO_LAUNCH(kSolveList, gV, kThreads, 0, stream, V, w.vupdate, w.remap, w.kind, w.sdone, w.slist1, &w.sc->solve_pending[1]);
		{
			SolveArgs sa;
			sa.list[0] = w.slist0;
			sa.list[1] = w.slist1;
			sa.done = w.sdone;
			sa.adj_off = w.adj_off;
			sa.adj = w.adj;
			sa.pos = w.pos;
			sa.pos_new = w.pos_new;
			sa.vq = w.vq;
			sa.aq = w.aq;
			sa.ag = w.ag;
			sa.vg = ac ? w.vg : nullptr;
			sa.ac = ac;
			sa.wedge = w.wedge;
			sa.max_rounds = unsigned(V + 2);
			sa.sc = w.sc;
			// co-resident blocks of this kernel (its own register count), as many as the pass kernel's at most
			unsigned int resident = unsigned(std::max(1, solve_per_sm_ * sms_));
			unsigned int blocks = std::max(1u, std::min(std::min(perform_blocks_, resident), gV));
			MO_CUDA_CHECK(cudaMemsetAsync(w.sc->bar, 0, sizeof(unsigned int) * 3, stream));
			void* params[] = {&sa};
			cudaEvent_t e0 = probeBegin("kSolvePositions", stream);
			MO_CUDA_CHECK(cudaLaunchCooperativeKernel((const void*)kSolvePositions, dim3(blocks), dim3(kThreads), params, 0, stream));
			probeEnd(e0, stream);
		}
		MO_LAUNCH(kSolveWedges, gV, kThreads, 0, stream, V, w.vupdate, w.remap, w.kind, w.pos_new);
		if (ac)
			MO_LAUNCH(kSolveAttributes, gV, kThreads, 0, stream, V, w.vupdate, w.remap, w.wedge, w.kind, w.pos_new, w.aq, w.ag, ac, w.attr);
		MO_LAUNCH(kFinalizeVertices, gV, kThreads, 0, stream, V, w.vupdate, m.lock, w.kind, w.pos_new, w.sc, m.update_positions, m.positions_stride / 4,
		    w.attr, am, ac ? m.update_attributes : nullptr, m.attributes_stride / 4);
	}

	if ((m.options & kOptInternalDebug) && result_count)
		MO_LAUNCH(kDebugBits, gridFor(result_count / 3, kThreads), kThreads, 0, stream, res, result_count / 3, w.kind, w.loop, w.loopback);

	if (result_count)
		MO_CUDA_CHECK(cudaMemcpyAsync(d_out, res, result_count * 4, cudaMemcpyDeviceToDevice, stream));
	if (timed)
		MO_CUDA_CHECK(cudaEventRecord(ev[9], stream));
	MO_CUDA_CHECK(cudaStreamSynchronize(stream));
	MO_CUDA_CHECK(cudaGetLastError());
	probe().collect();

	float rerr;
	memcpy(&rerr, &result_error_bits, 4);
	{
		const int khz = clock_khz_;
		readScalars();
		for (int i = 0; i < 8; ++i)
			rr.perform_phase_ms[i] = khz ? float(double(hs->phase_cycles[i]) / khz) : 0.f;
		rr.round_trace.clear();
		for (unsigned int i = 0; i < hs->trace_count && i < 512; ++i)
			rr.round_trace.push_back({hs->trace[2 * i], khz ? float(double(hs->trace[2 * i + 1]) * 16.0 / khz * 1e3) : 0.f});
		if (solve && hs->grid_error)
			throw std::runtime_error(hs->grid_error & 2 ? "position solve made no progress" : "grid barrier wait limit reached in the position solve");
	}
	rr.index_count = result_count;
	rr.result_error_sq = rerr;
	rr.result_error = sqrtf(rerr) * error_scale;
	rr.passes = passes;
	if (timed)
	{
		times->setup = elapsed(0, 1);
		times->adjacency = acc_adj;
		times->pick = acc_pick;
		times->rank = acc_rank;
		times->sort = acc_sort;
		times->perform = acc_perf;
		times->apply = acc_apply;
		times->total = elapsed(0, 9);
		for (auto& e : ev)
			cudaEventDestroy(e);
	}
	return rr;
}

} // namespace mogpu
