// mo_batch.cu - many small meshes simplified in one persistent launch.
//
// Each CTA takes meshes from a device work queue (an atomic ticket) and runs the whole
// edge-collapse simplification of one mesh (meshopt_simplifyEdge, src/simplifier.cpp:2344-2626,
// positions only) with block-level phases. The scratch of a mesh lives in shared memory when
// it fits the launch's dynamic shared memory, otherwise in a per-CTA slab of global memory;
// every phase addresses it through generic pointers, so one code path serves both.
//
// Inside a CTA the greedy collapse loop (performEdgeCollapses :1498-1636) runs in one of two
// exact forms. For a mesh in shared memory it runs as the reference writes it, on one warp:
// lane 0 walks the sorted candidates and evaluates the stop rules, locks and commits, and the
// 32 lanes split the one-ring of the flip test (hasTriangleFlips :1201-1232). For a mesh in a
// global slab it runs as block-level decision rounds (the rule of the multi-CTA kPerform),
// which hide the global-memory latency a serial walk would pay per candidate. All other phases
// use the whole block.
#include "mo_common.cuh"
#include "mo_prims.cuh"
#include "mo_probe.cuh"
#include "mo_batch.cuh"
#include <tuple>
#include <map>

#include <algorithm>
#include <cstring>
#include <mutex>

namespace mogpu
{

namespace
{

constexpr unsigned int kSortBinsC = 2560;

struct CtaWork
{
	unsigned int* idx;      // I: current result indices (compacted in place)
	float4* pos;            // V: rescaled positions
	unsigned int* remap;    // V
	unsigned int* wedge;    // V
	unsigned int* loop;     // V
	unsigned int* loopback; // V
	unsigned char* kind;    // V
	unsigned char* locked;  // V
	Quadric* vq;            // V
	unsigned int* adj_off;  // V + 1
	uint2* adj;             // I
	unsigned int* fill;     // V
	unsigned int* cr;       // V
	unsigned int* table;    // H
	unsigned int* cv0;      // cap
	unsigned int* cv1;      // cap
	unsigned int* cerr;     // cap
	unsigned int* order;    // cap
	unsigned int* hist;     // 2560
	unsigned int* red;      // 64 words of block-reduction scratch
	unsigned long long* minT;  // V: round-tagged earliest undecided candidate touching the vertex
	unsigned long long* minS;  // V: ... whose source is the vertex
	unsigned long long* moved; // V: (sorted index of the moving commit << 32) | target, ~0: not moved
	unsigned char* status;     // cap: decision per sorted position
	unsigned int* list0;       // cap: undecided candidates of the round
	unsigned int* list1;       // cap
	unsigned int* sort_tmp;    // cap: the sort's first digit pass
	unsigned int* back;        // V: sparse meshes, local vertex -> vertex of the shared buffer
	float* attr;               // V * ac: rescaled attributes
	Quadric* aq;               // V: attribute quadrics (per wedge)
	float4* ag;                // V * ac: attribute gradients
};

__host__ __device__ inline size_t alignUp(size_t v, size_t a)
{
	return (v + a - 1) & ~(a - 1);
}

__host__ __device__ inline size_t hashBucketsFor(size_t count)
{
	size_t b = 1;
	while (b < count + count / 4)
		b *= 2;
	return b;
}

// vertices a mesh's workspace is carved for: its own, or for a sparse mesh at most one per index
__host__ __device__ inline size_t localVertexBound(size_t I, size_t vertex_count, bool sparse)
{
	return sparse ? (I < vertex_count ? I : vertex_count) : vertex_count;
}

// Carves the workspace of a mesh with I indices, V (local) vertices and ac attributes from
// `base` (nullptr: size only). The decision-round state (rounds = true) is only carved for
// meshes in a global slab: meshes in shared memory run the serial warp loop without it.
__host__ __device__ inline size_t carve(CtaWork& w, char* base, size_t I, size_t V, size_t ac, bool sparse, bool rounds)
{
	size_t off = 0;
	size_t H = hashBucketsFor(V ? V : 1);
	size_t cap = I + 4;
	auto take = [&](size_t bytes) {
		char* p = base ? base + off : nullptr;
		off = alignUp(off + bytes, 16);
		return p;
	};
	w.idx = reinterpret_cast<unsigned int*>(take(I * 4));
	w.pos = reinterpret_cast<float4*>(take(V * 16));
	w.remap = reinterpret_cast<unsigned int*>(take(V * 4));
	w.wedge = reinterpret_cast<unsigned int*>(take(V * 4));
	w.loop = reinterpret_cast<unsigned int*>(take(V * 4));
	w.loopback = reinterpret_cast<unsigned int*>(take(V * 4));
	w.kind = reinterpret_cast<unsigned char*>(take(V));
	w.locked = reinterpret_cast<unsigned char*>(take(V));
	w.vq = reinterpret_cast<Quadric*>(take(V * sizeof(Quadric)));
	w.adj_off = reinterpret_cast<unsigned int*>(take((V + 1) * 4));
	w.adj = reinterpret_cast<uint2*>(take(I * 8));
	w.fill = reinterpret_cast<unsigned int*>(take(V * 4));
	w.cr = reinterpret_cast<unsigned int*>(take(V * 4));
	w.back = sparse ? reinterpret_cast<unsigned int*>(take(V * 4)) : nullptr;
	w.attr = ac ? reinterpret_cast<float*>(take(V * ac * 4)) : nullptr;
	w.aq = ac ? reinterpret_cast<Quadric*>(take(V * sizeof(Quadric))) : nullptr;
	w.ag = ac ? reinterpret_cast<float4*>(take(V * ac * 16)) : nullptr;
	// the hash table (64-bit entries for a sparse mesh's first-use table) is only live during
	// setup; the candidate arrays only during passes
	size_t shared_at = off;
	w.table = reinterpret_cast<unsigned int*>(take(H * (sparse ? 8 : 4)));
	size_t after_table = off;
	off = shared_at;
	w.cv0 = reinterpret_cast<unsigned int*>(take(cap * 4));
	w.cv1 = reinterpret_cast<unsigned int*>(take(cap * 4));
	w.cerr = reinterpret_cast<unsigned int*>(take(cap * 4));
	w.order = reinterpret_cast<unsigned int*>(take(cap * 4));
	w.hist = reinterpret_cast<unsigned int*>(take(kSortBinsC * 4)); // >= 8 warps x 256 digit counters
	w.red = reinterpret_cast<unsigned int*>(take(64 * 4));
	w.sort_tmp = reinterpret_cast<unsigned int*>(take(cap * 4));
	w.minT = rounds ? reinterpret_cast<unsigned long long*>(take(V * 8)) : nullptr;
	w.minS = rounds ? reinterpret_cast<unsigned long long*>(take(V * 8)) : nullptr;
	w.moved = rounds ? reinterpret_cast<unsigned long long*>(take(V * 8)) : nullptr;
	w.status = rounds ? reinterpret_cast<unsigned char*>(take(cap)) : nullptr;
	w.list0 = rounds ? reinterpret_cast<unsigned int*>(take(cap * 4)) : nullptr;
	w.list1 = rounds ? reinterpret_cast<unsigned int*>(take(cap * 4)) : nullptr;
	return off > after_table ? off : after_table;
}

// ---------------------------------------------------------------- block helpers

// exclusive scan of data[0..n) in place over the block; returns the total
template <int NT>
__device__ unsigned int blockScanArray(unsigned int* data, unsigned int n, unsigned int* red)
{
	// each thread scans a contiguous run; one block scan of the run totals
	const unsigned int per = (n + NT - 1) / NT;
	const unsigned int b = min(n, threadIdx.x * per), e = min(n, b + per);
	unsigned int sum = 0;
	for (unsigned int i = b; i < e; ++i)
		sum += data[i];
	unsigned int tot;
	unsigned int run = blockExclusiveScan<NT>(sum, red, &tot);
	for (unsigned int i = b; i < e; ++i)
	{
		unsigned int v = data[i];
		data[i] = run;
		run += v;
	}
	__syncthreads();
	return tot;
}

// One pass of a stable LSD radix sort of candidate indices on 8 bits of their sort key: up to 8
// warps each own a contiguous segment, count its digits (counters digit-major, then warp, so
// one scan gives every (digit, warp) its start), and scatter the segment in order. Equal digits
// keep segment order and index order inside a segment. src == nullptr: the identity.
template <int NT>
__device__ void blockDigitPass(const unsigned int* cerr, const unsigned int* src, unsigned int* dst, unsigned int C, int shift, unsigned int* cnt,
    unsigned int* red)
{
	constexpr unsigned int NW = NT / 32 < 8 ? NT / 32 : 8; // counters: NW * 256 words
	const unsigned int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const unsigned int seg = (C + NW - 1) / NW;
	const unsigned int s0 = min(C, warp * seg), s1 = warp < NW ? min(C, s0 + seg) : s0;
	for (unsigned int i = threadIdx.x; i < NW * 256; i += NT)
		cnt[i] = 0;
	__syncthreads();
	for (unsigned int b = s0; b < s1; b += 32)
	{
		unsigned int x = b + lane;
		bool valid = x < s1;
		unsigned int v = valid ? (src ? src[x] : x) : 0u;
		unsigned int d = valid ? ((sortKey(cerr[v]) >> shift) & 255u) : 256u + lane;
		unsigned int peers = __match_any_sync(0xffffffffu, d);
		if (valid && lane == (unsigned int)(__ffs(peers) - 1))
			cnt[d * NW + warp] += __popc(peers);
		__syncwarp();
	}
	__syncthreads();
	blockScanArray<NT>(cnt, NW * 256, red);
	for (unsigned int b = s0; b < s1; b += 32)
	{
		unsigned int x = b + lane;
		bool valid = x < s1;
		unsigned int v = valid ? (src ? src[x] : x) : 0u;
		unsigned int d = valid ? ((sortKey(cerr[v]) >> shift) & 255u) : 256u + lane;
		unsigned int peers = __match_any_sync(0xffffffffu, d);
		unsigned int leader = __ffs(peers) - 1;
		unsigned int base = 0;
		if (valid && lane == leader)
		{
			base = cnt[d * NW + warp];
			cnt[d * NW + warp] = base + __popc(peers);
		}
		base = __shfl_sync(0xffffffffu, base, leader);
		if (valid)
			dst[base + __popc(peers & ((1u << lane) - 1u))] = v;
		__syncwarp();
	}
	__syncthreads();
}

template <int NT>
__device__ unsigned int blockSum(unsigned int v, unsigned int* red)
{
	unsigned int tot;
	blockExclusiveScan<NT>(v, red, &tot);
	__syncthreads();
	return tot;
}

__device__ __forceinline__ unsigned int mix32b(unsigned int h)
{
	h ^= h >> 16;
	h *= 0x7feb352du;
	h ^= h >> 15;
	h *= 0x846ca68bu;
	h ^= h >> 16;
	return h;
}

__device__ __forceinline__ unsigned int posBitsB(float f)
{
	unsigned int u = __float_as_uint(f);
	return u == 0x80000000u ? 0u : u;
}

// ordered min/max folds, see rescalePositions :551-567 (leftmost of equal values, NaN skipped)
__device__ __forceinline__ float fmin_l(float l, float r)
{
	return l > r ? r : l;
}

__device__ __forceinline__ float fmax_l(float l, float r)
{
	return l < r ? r : l;
}

// ---------------------------------------------------------------- one mesh

// FULL = false compiles out the sparse subset, attributes, vertex_lock and Permissive, so that
// positions-only batches run the lean instantiation
template <int NT, bool FULL>
__device__ void simplifyMesh(const BatchDesc& d, CtaWork& w, BatchResult* out, bool serial)
{
	const unsigned int tid = threadIdx.x;
	const unsigned int I = d.index_count;
	const float* P = d.positions;
	const unsigned int sf = d.stride_f;
	const unsigned int ac = FULL ? d.ac : 0;
	const unsigned char* const vlock = FULL ? d.lock : nullptr;
	unsigned int* const back = FULL ? w.back : nullptr; // sparse: local vertex -> vertex of the shared buffer
	__shared__ unsigned int s_flag, s_unique;
	__shared__ float s_mm[NT / 32][6];
	__shared__ float s_minv[3], s_scale, s_extent;
	__shared__ unsigned int s_cap, s_count, s_trunc, s_done, s_errbits, s_next, s_stall;
	__shared__ unsigned long long s_cut;
	__shared__ unsigned int s_carry[3];
	__shared__ unsigned int s_maxes[NT];

	if (tid == 0)
		s_flag = 0, s_stall = 0;
	__syncthreads();
	for (unsigned int i = tid; i < I; i += NT)
	{
		unsigned int v = d.indices[i];
		w.idx[i] = v;
		if (v >= d.vertex_count)
			s_flag = 1;
	}
	__syncthreads();
	if (s_flag)
	{
		if (tid == 0)
			*out = BatchResult{I, 0.f, 0, 2};
		for (unsigned int i = tid; i < I; i += NT)
			d.out[i] = d.indices[i];
		return;
	}

	// ---- sparse subset (buildSparseRemap :242-294): local ids in order of first use. A
	// 64-bit table keyed by the shared-buffer vertex keeps its first index position (atomicMin);
	// the positions that are first uses, ranked by a block scan, give the local ids.
	unsigned int V = d.vertex_count;
	if (back)
	{
		unsigned long long* t64 = reinterpret_cast<unsigned long long*>(w.table);
		const unsigned int HS = (unsigned int)hashBucketsFor(localVertexBound(I, d.vertex_count, true) ? localVertexBound(I, d.vertex_count, true) : 1);
		const unsigned int smask = HS - 1;
		for (unsigned int i = tid; i < HS; i += NT)
			t64[i] = ~0ull;
		__syncthreads();
		for (unsigned int p = tid; p < I; p += NT)
		{
			unsigned int v = w.idx[p];
			unsigned long long key = ((unsigned long long)v << 32) | p;
			unsigned int b = mix32b(v) & smask, slot = 0;
			for (unsigned int probe = 0; probe <= smask; ++probe)
			{
				unsigned long long cur = t64[b];
				if (cur == ~0ull)
				{
					unsigned long long prev = atomicCAS(&t64[b], ~0ull, key);
					if (prev == ~0ull)
					{
						slot = b;
						break;
					}
					cur = prev;
				}
				if ((unsigned int)(cur >> 32) == v)
				{
					atomicMin(&t64[b], key);
					slot = b;
					break;
				}
				b = (b + probe + 1) & smask;
			}
			w.adj[p].x = slot;
		}
		__syncthreads();
		for (unsigned int p = tid; p < I; p += NT)
			w.adj[p].y = (unsigned int)t64[w.adj[p].x]; // first position of this vertex
		__syncthreads();
		// the table is dead from here: its region holds the candidate arrays later
		for (unsigned int p = tid; p < I; p += NT)
			w.cv0[p] = w.adj[p].y == p;
		__syncthreads();
		unsigned int unique = blockScanArray<NT>(w.cv0, I, w.red);
		for (unsigned int p = tid; p < I; p += NT)
			if (w.adj[p].y == p)
				back[w.cv0[p]] = w.idx[p];
		__syncthreads();
		for (unsigned int p = tid; p < I; p += NT)
			w.idx[p] = w.cv0[w.adj[p].y];
		if (tid == 0)
			s_unique = unique;
		__syncthreads();
		V = s_unique;
	}
	auto src = [&](unsigned int i) { return back ? back[i] : i; };

	// ---- position remap (buildPositionRemap :195-214) in a block-local hash table
	const unsigned int H = (unsigned int)hashBucketsFor(V ? V : 1), mask = H - 1;
	for (unsigned int i = tid; i < H; i += NT)
		w.table[i] = ~0u;
	__syncthreads();
	for (unsigned int i = tid; i < V; i += NT)
	{
		const float* p = P + (size_t)src(i) * sf;
		float x = p[0], y = p[1], z = p[2];
		unsigned int h = mix32b(posBitsB(x) * 0x9e3779b1u ^ mix32b(posBitsB(y) + 0x85ebca6bu) ^ mix32b(posBitsB(z) * 0xc2b2ae35u + 1u));
		unsigned int b = h & mask, slot = ~0u;
		for (unsigned int probe = 0; probe <= mask; ++probe)
		{
			unsigned int cur = w.table[b];
			if (cur == ~0u)
			{
				unsigned int prev = atomicCAS(&w.table[b], ~0u, i);
				if (prev == ~0u)
				{
					slot = b;
					break;
				}
				cur = prev;
			}
			const float* q = P + (size_t)src(cur) * sf;
			if (q[0] == x && q[1] == y && q[2] == z)
			{
				atomicMin(&w.table[b], i);
				slot = b;
				break;
			}
			b = (b + probe + 1) & mask;
		}
		w.remap[i] = slot; // slot for now
	}
	__syncthreads();
	for (unsigned int i = tid; i < V; i += NT)
	{
		unsigned int s = w.remap[i];
		w.remap[i] = s == ~0u ? i : w.table[s];
	}
	__syncthreads();
	// wedge cycle (:229-239): dup i -> previous member of its class (or the primary); the
	// primary -> largest duplicate
	for (unsigned int i = tid; i < V; i += NT)
	{
		w.wedge[i] = i;
		w.fill[i] = 0;
	}
	__syncthreads();
	for (unsigned int i = tid; i < V; i += NT)
	{
		unsigned int r = w.remap[i];
		if (r == i)
			continue;
		unsigned int pred = r;
		for (unsigned int j = r + 1; j < i; ++j)
			if (w.remap[j] == r)
				pred = j;
		w.wedge[i] = pred;
		atomicMax(&w.fill[r], i);
	}
	__syncthreads();
	for (unsigned int i = tid; i < V; i += NT)
		if (w.remap[i] == i && w.fill[i])
			w.wedge[i] = w.fill[i];
	__syncthreads();

	// ---- rescale (rescalePositions :544-603): ordered folds over contiguous thread chunks
	{
		float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		unsigned int per = (V + NT - 1) / NT, b0 = min(V, tid * per), b1 = min(V, b0 + per);
		for (unsigned int i = b0; i < b1; ++i)
		{
			const float* p = P + (size_t)src(i) * sf;
			for (int j = 0; j < 3; ++j)
			{
				mn[j] = mn[j] > p[j] ? p[j] : mn[j];
				mx[j] = mx[j] < p[j] ? p[j] : mx[j];
			}
		}
		for (int o = 1; o < 32; o <<= 1)
			for (int j = 0; j < 3; ++j)
			{
				float a = __shfl_down_sync(0xffffffffu, mn[j], o), c = __shfl_down_sync(0xffffffffu, mx[j], o);
				if ((tid & 31) + o < 32 && ((tid & (2 * o - 1)) == 0))
					mn[j] = fmin_l(mn[j], a), mx[j] = fmax_l(mx[j], c);
			}
		if ((tid & 31) == 0)
			for (int j = 0; j < 3; ++j)
				s_mm[tid >> 5][j] = mn[j], s_mm[tid >> 5][3 + j] = mx[j];
		__syncthreads();
		if (tid == 0)
		{
			for (int q = 1; q < NT / 32; ++q)
				for (int j = 0; j < 3; ++j)
					s_mm[0][j] = fmin_l(s_mm[0][j], s_mm[q][j]), s_mm[0][3 + j] = fmax_l(s_mm[0][3 + j], s_mm[q][3 + j]);
			float extent = 0.f;
			extent = (s_mm[0][3] - s_mm[0][0]) < extent ? extent : (s_mm[0][3] - s_mm[0][0]);
			extent = (s_mm[0][4] - s_mm[0][1]) < extent ? extent : (s_mm[0][4] - s_mm[0][1]);
			extent = (s_mm[0][5] - s_mm[0][2]) < extent ? extent : (s_mm[0][5] - s_mm[0][2]);
			s_extent = extent;
			s_scale = extent == 0 ? 0.f : 1.f / extent;
			for (int j = 0; j < 3; ++j)
				s_minv[j] = s_mm[0][j];
		}
		__syncthreads();
		for (unsigned int i = tid; i < V; i += NT)
		{
			const float* p = P + (size_t)src(i) * sf;
			w.pos[i] = make_float4((p[0] - s_minv[0]) * s_scale, (p[1] - s_minv[1]) * s_scale, (p[2] - s_minv[2]) * s_scale, 0.f);
		}
		// rescaleAttributes (:605-621): weighted copies of the used attributes
		if constexpr (FULL)
			if (ac)
				for (unsigned int x = tid; x < V * ac; x += NT)
				{
					unsigned int i = x / ac, k = x - i * ac;
					w.attr[x] = d.attributes[(size_t)src(i) * d.attr_stride_f + d.amap->src[k]] * d.amap->weight[k];
				}
	}

	// ---- raw adjacency (updateEdgeAdjacency :52-109, no remap): corner lists, unordered
	for (unsigned int i = tid; i <= V; i += NT)
		w.adj_off[i] = 0;
	__syncthreads();
	for (unsigned int p = tid; p < I; p += NT)
		atomicAdd(&w.adj_off[w.idx[p]], 1u);
	__syncthreads();
	blockScanArray<NT>(w.adj_off, V + 1, w.red);
	for (unsigned int i = tid; i < V; i += NT)
		w.fill[i] = 0;
	__syncthreads();
	for (unsigned int p = tid; p < I; p += NT)
	{
		unsigned int v = w.idx[p];
		unsigned int s = w.adj_off[v] + atomicAdd(&w.fill[v], 1u);
		unsigned int f = p / 3, c = p - f * 3;
		w.adj[s] = make_uint2(w.idx[f * 3 + (c == 2 ? 0 : c + 1)], w.idx[f * 3 + (c == 0 ? 2 : c - 1)]);
	}
	__syncthreads();

	// ---- classification (classifyVertices :364-542, open edges from each vertex's own list)
	for (unsigned int v = tid; v < V; v += NT)
	{
		unsigned int b = w.adj_off[v], e = w.adj_off[v + 1];
		bool degen = false;
		for (unsigned int j = b; j < e; ++j)
			degen |= w.adj[j].x == v;
		unsigned int outc = 0, outt = ~0u, inc = 0, ins = ~0u;
		if (!degen)
			for (unsigned int j = b; j < e; ++j)
			{
				uint2 ej = w.adj[j];
				bool bk = false, fwd = false;
				for (unsigned int q = b; q < e; ++q)
				{
					uint2 eq = w.adj[q];
					bk |= eq.y == ej.x;
					fwd |= eq.x == ej.y;
				}
				if (!bk)
					outc++, outt = ej.x;
				if (!fwd)
					inc++, ins = ej.y;
			}
		w.loop[v] = degen ? v : (outc == 0 ? ~0u : (outc == 1 ? outt : v));
		w.loopback[v] = degen ? v : (inc == 0 ? ~0u : (inc == 1 ? ins : v));
	}
	__syncthreads();
	for (unsigned int i = tid; i < V; i += NT)
	{
		unsigned int r = w.remap[i], wi = w.wedge[r];
		unsigned char k;
		if (wi == r)
		{
			unsigned int openi = w.loopback[r], openo = w.loop[r];
			if (openi == ~0u && openo == ~0u)
				k = kManifold;
			else if (openi != ~0u && openo != ~0u && w.remap[openi] == w.remap[openo] && openi != r)
				k = kSeam;
			else if (openi != r && openo != r)
				k = kBorder;
			else
				k = kLocked;
		}
		else if (w.wedge[wi] == r)
		{
			unsigned int openiv = w.loopback[r], openov = w.loop[r], openiw = w.loopback[wi], openow = w.loop[wi];
			if (openiv != ~0u && openiv != r && openov != ~0u && openov != r && openiw != ~0u && openiw != wi && openow != ~0u && openow != wi)
				k = (w.remap[openiv] == w.remap[openow] && w.remap[openov] == w.remap[openiw] && w.remap[openiv] != w.remap[openov]) ? kSeam : kLocked;
			else
				k = kLocked;
		}
		else
			k = kLocked;
		w.kind[i] = k;
	}
	__syncthreads();
	if (FULL && (d.options & kOptPermissive))
	{
		// Permissive (:481-515): a seam or locked primary becomes Complex unless a wedge is
		// protected or has a half-edge with no opposite in position space (hasEdge :345-362);
		// the new kinds are staged in `locked` (unused until the passes), then copied to wedges
		for (unsigned int i = tid; i < V; i += NT)
		{
			unsigned char k = w.kind[i];
			unsigned char nk = k;
			if (w.remap[i] == i && (k == kSeam || k == kLocked))
			{
				bool protect = false;
				unsigned int v = i;
				do
				{
					protect |= vlock && (vlock[src(v)] & kVertexProtect) != 0;
					v = w.wedge[v];
				} while (v != i);
				do
				{
					for (unsigned int j = w.adj_off[v]; j < w.adj_off[v + 1] && !protect; ++j)
					{
						// hasEdge(nx -> v) over the wedges of nx
						unsigned int a = w.adj[j].x, rb = w.remap[v], u = a;
						bool found = false;
						do
						{
							for (unsigned int q = w.adj_off[u]; q < w.adj_off[u + 1] && !found; ++q)
								found = w.remap[w.adj[q].x] == rb;
							u = w.wedge[u];
						} while (u != a && !found);
						protect |= !found;
					}
					v = w.wedge[v];
				} while (v != i);
				nk = protect ? k : (unsigned char)kComplex;
			}
			w.locked[i] = nk;
		}
		__syncthreads();
		for (unsigned int i = tid; i < V; i += NT)
		{
			unsigned char k = w.kind[i];
			if (k == kSeam || k == kLocked)
				w.kind[i] = w.locked[w.remap[i]];
		}
		__syncthreads();
	}
	if (vlock)
	{
		// vertex_lock (:517-531): a locked wedge locks its whole position
		for (unsigned int i = tid; i < V; i += NT)
			if (vlock[src(i)] & kVertexLock)
				w.kind[w.remap[i]] = kLocked;
		__syncthreads();
		for (unsigned int i = tid; i < V; i += NT)
			if (w.kind[w.remap[i]] == kLocked)
				w.kind[i] = kLocked;
		__syncthreads();
	}
	if (d.options & kOptLockBorder)
	{
		for (unsigned int i = tid; i < V; i += NT)
			if (w.kind[i] == kBorder)
				w.kind[i] = kLocked;
		__syncthreads();
	}

	// ---- capacity (boundEdgeCollapses :1292-1308) from the raw degrees
	{
		unsigned int dual = 0;
		for (unsigned int i = tid; i < V; i += NT)
		{
			unsigned char k = w.kind[i];
			dual += (k == kManifold || k == kSeam) ? (w.adj_off[i + 1] - w.adj_off[i]) : 0;
		}
		unsigned int tot = blockSum<NT>(dual, w.red);
		if (tid == 0)
			s_cap = I - tot / 2 + 3;
	}

	// ---- corner lists in corner order (remapped for the position quadrics, raw for the
	// attribute quadrics), then the quadric folds (:1057-1179)
	auto cornerLists = [&](bool remapped) {
		for (unsigned int i = tid; i <= V; i += NT)
			w.adj_off[i] = 0;
		__syncthreads();
		for (unsigned int p = tid; p < I; p += NT)
			atomicAdd(&w.adj_off[remapped ? w.remap[w.idx[p]] : w.idx[p]], 1u);
		__syncthreads();
		blockScanArray<NT>(w.adj_off, V + 1, w.red);
		for (unsigned int i = tid; i < V; i += NT)
			w.fill[i] = 0;
		__syncthreads();
		for (unsigned int p = tid; p < I; p += NT)
		{
			unsigned int v = remapped ? w.remap[w.idx[p]] : w.idx[p];
			w.adj[w.adj_off[v] + atomicAdd(&w.fill[v], 1u)].x = p;
		}
		__syncthreads();
		for (unsigned int v = tid; v < V; v += NT)
		{
			// insertion sort of the vertex's corners (few per vertex)
			unsigned int b = w.adj_off[v], e = w.adj_off[v + 1];
			for (unsigned int j = b + 1; j < e; ++j)
			{
				unsigned int x = w.adj[j].x;
				unsigned int q = j;
				while (q > b && w.adj[q - 1].x > x)
				{
					w.adj[q].x = w.adj[q - 1].x;
					--q;
				}
				w.adj[q].x = x;
			}
		}
		__syncthreads();
	};
	cornerLists(true);
	{
		const float factor = (d.options & kOptRegularizeLight) ? 1e-2f : ((d.options & kOptRegularize) ? 1e-1f : 1e-7f);
		for (unsigned int r = tid; r < V; r += NT)
		{
			if (w.remap[r] != r)
			{
				stquadric(w.vq, r, qzero());
				continue;
			}
			unsigned int b = w.adj_off[r], e = w.adj_off[r + 1];
			Quadric Q = qzero();
			for (unsigned int j = b; j < e; ++j)
			{
				unsigned int f = w.adj[j].x / 3;
				unsigned int i0 = w.idx[f * 3 + 0], i1 = w.idx[f * 3 + 1], i2 = w.idx[f * 3 + 2];
				float4 a0 = w.pos[i0], a1 = w.pos[i1], a2 = w.pos[i2];
				Quadric F = qtriangle(V3{a0.x, a0.y, a0.z}, V3{a1.x, a1.y, a1.z}, V3{a2.x, a2.y, a2.z}, 1.f);
				qadd(Q, F);
			}
			bool priority = vlock && (vlock[src(r)] & kVertexPriority) != 0;
			float wt = Q.w * (priority ? 1.0f : factor);
			float4 pr = w.pos[r];
			Quadric Pq = qpoint(pr.x, pr.y, pr.z, wt);
			qadd(Q, Pq);
			unsigned int lastf = ~0u;
			for (unsigned int j = b; j < e; ++j)
			{
				unsigned int f = w.adj[j].x / 3;
				if (f == lastf)
					continue;
				lastf = f;
				for (int ed = 0; ed < 3; ++ed)
				{
					unsigned int i0 = w.idx[f * 3 + ed], i1 = w.idx[f * 3 + (ed == 2 ? 0 : ed + 1)];
					unsigned char k0 = w.kind[i0], k1 = w.kind[i1];
					bool b0 = k0 == kBorder || k0 == kSeam, b1 = k1 == kBorder || k1 == kSeam;
					if (!b0 && !b1)
						continue;
					if (b0 && w.loop[i0] != i1)
						continue;
					if (b1 && w.loopback[i1] != i0)
						continue;
					bool to0 = w.remap[i0] == r, to1 = w.remap[i1] == r;
					if (!to0 && !to1)
						continue;
					unsigned int i2 = w.idx[f * 3 + (ed == 0 ? 2 : ed - 1)];
					float weight = (k0 == kBorder || k1 == kBorder) ? 10.f : 0.5f;
					float4 a0 = w.pos[i0], a1 = w.pos[i1], a2 = w.pos[i2];
					V3 p0{a0.x, a0.y, a0.z}, p1{a1.x, a1.y, a1.z}, p2{a2.x, a2.y, a2.z};
					Quadric E = qedge(p0, p1, p2, weight);
					Quadric Tq = qtriangle(p0, p1, p2, weight);
					Tq.w = 0;
					qadd(E, Tq);
					if (to0)
						qadd(Q, E);
					if (to1)
						qadd(Q, E);
				}
			}
			stquadric(w.vq, r, Q);
		}
	}
	__syncthreads();
	if constexpr (FULL)
	{
		if (ac)
		{
			// fillAttributeQuadrics (:1159-1179): per wedge over its faces in face order; the
			// gradients accumulate in place (each vertex is owned by one thread)
			cornerLists(false);
			for (unsigned int v = tid; v < V; v += NT)
			{
				float4* G = w.ag + (size_t)v * ac;
				for (unsigned int k = 0; k < ac; ++k)
					G[k] = make_float4(0.f, 0.f, 0.f, 0.f);
				Quadric Q = qzero();
				for (unsigned int j = w.adj_off[v]; j < w.adj_off[v + 1]; ++j)
				{
					unsigned int f = w.adj[j].x / 3;
					unsigned int i0 = w.idx[f * 3 + 0], i1 = w.idx[f * 3 + 1], i2 = w.idx[f * 3 + 2];
					float4 a0 = w.pos[i0], a1 = w.pos[i1], a2 = w.pos[i2];
					addAttributeQuadric<32>(Q, G, (int)ac, V3{a0.x, a0.y, a0.z}, V3{a1.x, a1.y, a1.z}, V3{a2.x, a2.y, a2.z}, w.attr + (size_t)i0 * ac,
					    w.attr + (size_t)i1 * ac, w.attr + (size_t)i2 * ac);
				}
				stquadric(w.aq, v, Q);
			}
			__syncthreads();
		}
	}

	// ---- pass loop (:2493-2541)
	const float error_scale = (d.options & kOptErrorAbsolute) ? s_extent : 1.f;
	const float error_limit = (d.target_error * d.target_error) / (error_scale * error_scale);
	unsigned int result_count = I;
	float result_error = 0.f;
	unsigned int passes = 0;
	unsigned int round = 0; // decision rounds are numbered across passes, so mark tags never repeat

	while (result_count > d.target_index_count)
	{
		const unsigned int T = result_count / 3;

		// adjacency of the current result, welded by remap (unordered lists)
		for (unsigned int i = tid; i <= V; i += NT)
			w.adj_off[i] = 0;
		__syncthreads();
		for (unsigned int p = tid; p < result_count; p += NT)
			atomicAdd(&w.adj_off[w.remap[w.idx[p]]], 1u);
		__syncthreads();
		blockScanArray<NT>(w.adj_off, V + 1, w.red);
		for (unsigned int i = tid; i < V; i += NT)
			w.fill[i] = 0;
		__syncthreads();
		for (unsigned int t = tid; t < T; t += NT)
		{
			unsigned int a = w.remap[w.idx[t * 3 + 0]], b = w.remap[w.idx[t * 3 + 1]], c = w.remap[w.idx[t * 3 + 2]];
			w.adj[w.adj_off[a] + atomicAdd(&w.fill[a], 1u)] = make_uint2(b, c);
			w.adj[w.adj_off[b] + atomicAdd(&w.fill[b], 1u)] = make_uint2(c, a);
			w.adj[w.adj_off[c] + atomicAdd(&w.fill[c], 1u)] = make_uint2(a, b);
		}
		__syncthreads();

		// pick (pickEdgeCollapses :1310-1372): each thread takes a contiguous run of triangles,
		// counts its candidates, and after one block scan emits them in triangle order; the
		// capacity check stops at the first triangle that has no room for three more
		if (tid == 0)
			s_trunc = ~0u;
		{
			auto pickEdgeB = [&](unsigned int i0, unsigned int i1, unsigned int& v0, unsigned int& v1, unsigned int& bd) {
				unsigned int r0 = w.remap[i0], r1 = w.remap[i1];
				if (r0 == r1)
					return false;
				unsigned int k0 = w.kind[i0], k1 = w.kind[i1];
				bool c01 = canCollapse(k0, k1), c10 = canCollapse(k1, k0);
				if (!(c01 | c10))
					return false;
				if (hasOpposite(k0, k1) && r1 > r0)
					return false;
				if ((k0 == kBorder || k0 == kSeam) && k1 != kManifold && w.loop[i0] != i1)
					return false;
				if ((k1 == kBorder || k1 == kSeam) && k0 != kManifold && w.loopback[i1] != i0)
					return false;
				if (c01 & c10)
					v0 = i0, v1 = i1, bd = 1;
				else
					v0 = c01 ? i0 : i1, v1 = c01 ? i1 : i0, bd = 0;
				return true;
			};
			const unsigned int per = (T + NT - 1) / NT;
			const unsigned int t0 = min(T, tid * per), t1 = min(T, t0 + per);
			unsigned int n = 0;
			for (unsigned int t = t0; t < t1; ++t)
				for (int e = 0; e < 3; ++e)
				{
					unsigned int v0, v1, bd;
					n += pickEdgeB(w.idx[t * 3 + e], w.idx[t * 3 + (e == 2 ? 0 : e + 1)], v0, v1, bd);
				}
			unsigned int tot;
			unsigned int o = blockExclusiveScan<NT>(n, w.red, &tot);
			if (tid == 0)
				s_count = tot;
			for (unsigned int t = t0; t < t1; ++t)
			{
				if (o + 3 > s_cap)
				{
					atomicMin(&s_trunc, o);
					break;
				}
				for (int e = 0; e < 3; ++e)
				{
					unsigned int v0, v1, bd;
					if (pickEdgeB(w.idx[t * 3 + e], w.idx[t * 3 + (e == 2 ? 0 : e + 1)], v0, v1, bd))
					{
						w.cv0[o] = v0, w.cv1[o] = v1, w.cerr[o] = bd;
						o++;
					}
				}
			}
			__syncthreads();
		}
		const unsigned int C = min(s_count, s_trunc);
		if (C == 0)
			break;

		// rank (rankEdgeCollapses :1374-1450)
		for (unsigned int c = tid; c < C; c += NT)
		{
			unsigned int i0 = w.cv0[c], i1 = w.cv1[c];
			bool bidi = w.cerr[c] != 0;
			float4 a0 = w.pos[i0], a1 = w.pos[i1];
			V3 p0{a0.x, a0.y, a0.z}, p1{a1.x, a1.y, a1.z};
			float ei = qerror(ldquadric(w.vq, w.remap[i0]), p1);
			float ej = bidi ? qerror(ldquadric(w.vq, w.remap[i1]), p0) : FLT_MAX;
			if (ac)
			{
				auto term = [&](unsigned int v, unsigned int t) {
					float4 pt = w.pos[t];
					return qerrorAttr(ldquadric(w.aq, v), w.ag + (size_t)v * ac, (int)ac, V3{pt.x, pt.y, pt.z}, w.attr + (size_t)t * ac);
				};
				ei += term(i0, i1);
				ej += bidi ? term(i1, i0) : 0;
				if (w.kind[i0] == kSeam)
				{
					unsigned int s0 = w.wedge[i0];
					unsigned int s1 = w.loop[i0] == i1 ? w.loopback[s0] : w.loop[s0];
					s1 = (s1 != ~0u) ? s1 : w.wedge[i1];
					ei += term(s0, s1);
					ej += bidi ? term(s1, s0) : 0;
				}
				else
				{
					if (FULL && w.kind[i0] == kComplex)
						for (unsigned int v = w.wedge[i0]; v != i0; v = w.wedge[v])
							ei += term(v, complexTarget(v, i1, w.remap, w.loop, w.loopback));
					if (FULL && w.kind[i1] == kComplex && bidi)
						for (unsigned int v = w.wedge[i1]; v != i1; v = w.wedge[v])
							ej += term(v, complexTarget(v, i0, w.remap, w.loop, w.loopback));
				}
			}
			bool rev = bidi & (ej < ei);
			w.cv0[c] = rev ? i1 : i0;
			w.cv1[c] = rev ? i0 : i1;
			w.cerr[c] = __float_as_uint(ej < ei ? ej : ei);
		}
		// sort (sortEdgeCollapses :1452-1496): the same stable order on the 12-bit key as two
		// stable 8-bit digit passes (low byte, then the high four bits)
		blockDigitPass<NT>(w.cerr, nullptr, w.sort_tmp, C, 0, w.hist, w.red);
		blockDigitPass<NT>(w.cerr, w.sort_tmp, w.order, C, 8, w.hist, w.red);
		for (unsigned int i = tid; i < V; i += NT)
			w.cr[i] = i, w.locked[i] = 0;
		__syncthreads();

		const unsigned int goal = (result_count - d.target_index_count) / 3;
		if (serial)
		{
			// meshes in shared memory: the reference's serial loop on one warp is cheaper than rounds
			for (unsigned int i = tid; i < V; i += NT)
				w.cr[i] = i, w.locked[i] = 0;
			__syncthreads();

			// perform (performEdgeCollapses :1498-1636) on warp 0, serial order, lanes split the flip test
			if (tid < 32)
			{
				const unsigned int lane = tid;
				unsigned int edge_collapses = 0, triangle_collapses = 0, edge_goal = goal / 2;
				for (unsigned int i = 0; i < C; ++i)
				{
					unsigned int c = w.order[i];
					float err = __uint_as_float(w.cerr[c]);
					if (err > error_limit)
						break;
					if (triangle_collapses >= goal)
						break;
					float error_goal = edge_goal < C ? 1.5f * __uint_as_float(w.cerr[w.order[edge_goal]]) : FLT_MAX;
					if (err > error_goal && err > result_error && triangle_collapses > goal / 6)
						break;
					unsigned int i0 = w.cv0[c], i1 = w.cv1[c];
					unsigned int r0 = w.remap[i0], r1 = w.remap[i1];
					unsigned char kd = w.kind[i0];
					if (w.locked[r0] | w.locked[r1])
						continue;
					// flip test, lanes over r0's one-ring
					unsigned int b = w.adj_off[r0], e = w.adj_off[r0 + 1];
					float4 a0 = w.pos[r0], a1 = w.pos[r1];
					V3 v0{a0.x, a0.y, a0.z}, v1{a1.x, a1.y, a1.z};
					bool flip = false;
					for (unsigned int j = b + lane; j < e; j += 32)
					{
						uint2 ed = w.adj[j];
						unsigned int va = w.cr[ed.x], vb = w.cr[ed.y];
						if (va == r1 || vb == r1 || va == vb)
							continue;
						float4 pa = w.pos[va], pb = w.pos[vb];
						flip |= triFlip(V3{pa.x, pa.y, pa.z}, V3{pb.x, pb.y, pb.z}, v0, v1);
					}
					if (__any_sync(0xffffffffu, flip))
					{
						edge_goal++;
						continue;
					}
					if (lane == 0)
					{
						if (FULL && kd == kComplex)
						{
							unsigned int v = i0;
							do
							{
								w.cr[v] = complexTarget(v, i1, w.remap, w.loop, w.loopback);
								v = w.wedge[v];
							} while (v != i0);
						}
						else if (kd == kSeam)
						{
							unsigned int s0 = w.wedge[i0];
							unsigned int s1 = w.loop[i0] == i1 ? w.loopback[s0] : w.loop[s0];
							s1 = (s1 != ~0u) ? s1 : w.wedge[i1];
							w.cr[i0] = i1;
							w.cr[s0] = s1;
						}
						else
							w.cr[i0] = i1;
						w.locked[r0] = 1;
						w.locked[r1] = 1;
					}
					__syncwarp();
					triangle_collapses += (kd == kBorder) ? 1 : 2;
					edge_collapses++;
					result_error = result_error < err ? err : result_error;
				}
				if (lane == 0)
				{
					s_done = edge_collapses;
					s_errbits = __float_as_uint(result_error);
				}
			}
		}
		else
		{
			// perform (performEdgeCollapses :1498-1636) in block-level decision rounds: a candidate is
			// decided once nothing earlier in sorted order can change its outcome (the rule of the
			// multi-CTA path's kPerform), over a window of sorted order that grows until the stop
			// rules fire; the stop rules are a prefix scan of the decisions
			for (unsigned int i = tid; i < V; i += NT)
				w.locked[i] = 0, w.moved[i] = ~0ull, w.minT[i] = ~0ull, w.minS[i] = ~0ull;
			for (unsigned int k = tid; k < C; k += NT)
				w.status[k] = kUndecided;
			if (tid == 0)
				s_cut = ~0ull, s_carry[0] = 0, s_carry[1] = 0, s_carry[2] = __float_as_uint(result_error);
			__syncthreads();
			{
				unsigned int K0 = 0, K1 = (unsigned int)min((unsigned long long)C, 2ull * (goal / 2) + 64ull);
				for (;;)
				{
					// rounds over [K0, K1)
					unsigned int n = K1 - K0;
					bool first = true;
					unsigned int* cur = w.list0;
					unsigned int* nxt = w.list1;
					while (n)
					{
						++round;
						const unsigned long long tag = (unsigned long long)(0xFFFFFFFFu - round) << 32;
						for (unsigned int x = tid; x < n; x += NT)
						{
							unsigned int k = first ? K0 + x : cur[x];
							unsigned int c = w.order[k];
							unsigned int r0 = w.remap[w.cv0[c]], r1 = w.remap[w.cv1[c]];
							atomicMin(&w.minT[r0], tag | k);
							atomicMin(&w.minT[r1], tag | k);
							atomicMin(&w.minS[r0], tag | k);
						}
						if (tid == 0)
							s_next = 0;
						__syncthreads();
						for (unsigned int base = 0; base < n; base += NT)
						{
							unsigned int x = base + tid;
							bool keep = false;
							unsigned int k = 0;
							if (x < n)
							{
								k = first ? K0 + x : cur[x];
								unsigned int c = w.order[k];
								unsigned int i0 = w.cv0[c], i1 = w.cv1[c];
								unsigned int r0 = w.remap[i0], r1 = w.remap[i1];
								const unsigned long long mine = tag | k;
								if (w.locked[r0] | w.locked[r1])
									w.status[k] = kSkipLocked;
								else if (w.minT[r0] != mine || w.minT[r1] != mine)
									keep = true;
								else
								{
									unsigned int b = w.adj_off[r0], e = w.adj_off[r0 + 1];
									for (unsigned int j = b; j < e && !keep; ++j)
									{
										uint2 ed = w.adj[j];
										unsigned long long sx = w.minS[ed.x], sy = w.minS[ed.y];
										keep = ((sx >> 32) == (tag >> 32) && (unsigned int)sx < k) || ((sy >> 32) == (tag >> 32) && (unsigned int)sy < k);
									}
									if (!keep)
									{
										float4 a0 = w.pos[r0], a1 = w.pos[r1];
										V3 v0{a0.x, a0.y, a0.z}, v1{a1.x, a1.y, a1.z};
										bool flip = false;
										for (unsigned int j = b; j < e && !flip; ++j)
										{
											uint2 ed = w.adj[j];
											unsigned long long mx = w.moved[ed.x], my = w.moved[ed.y];
											unsigned int va = (unsigned int)(mx >> 32) < k ? (unsigned int)mx : ed.x;
											unsigned int vb = (unsigned int)(my >> 32) < k ? (unsigned int)my : ed.y;
											if (va == r1 || vb == r1 || va == vb)
												continue;
											float4 pa = w.pos[va], pb = w.pos[vb];
											flip = triFlip(V3{pa.x, pa.y, pa.z}, V3{pb.x, pb.y, pb.z}, v0, v1);
										}
										if (flip)
											w.status[k] = kSkipFlip;
										else
										{
											unsigned int target = i1;
											if (FULL && w.kind[i0] == kComplex)
												target = complexTarget(r0, i1, w.remap, w.loop, w.loopback);
											else if (w.kind[i0] == kSeam)
											{
												unsigned int s0 = w.wedge[i0];
												unsigned int s1 = w.loop[i0] == i1 ? w.loopback[s0] : w.loop[s0];
												s1 = (s1 != ~0u) ? s1 : w.wedge[i1];
												target = (s0 == r0) ? s1 : i1;
											}
											w.moved[r0] = ((unsigned long long)k << 32) | target;
											w.locked[r0] = 1;
											w.locked[r1] = 1;
											w.status[k] = kCommit;
										}
									}
								}
							}
							unsigned int m = __ballot_sync(0xffffffffu, keep);
							if (keep)
							{
								unsigned int lane = tid & 31;
								unsigned int leader = __ffs(m) - 1;
								unsigned int o = 0;
								if (lane == leader)
									o = atomicAdd(&s_next, __popc(m));
								o = __shfl_sync(m, o, leader);
								nxt[o + __popc(m & ((1u << lane) - 1u))] = k;
							}
						}
						__syncthreads();
						unsigned int nn = s_next;
						__syncthreads();
						if (nn >= n)
						{
							if (tid == 0)
								s_stall = 1;
							break;
						}
						n = nn;
						first = false;
						unsigned int* t = cur;
						cur = nxt;
						nxt = t;
					}
					// stop rules over [K0, K1): contiguous thread chunks, block scan, carried prefix
					const unsigned int len = K1 - K0, per = (len + NT - 1) / NT;
					const unsigned int t0 = min(K1, K0 + tid * per), t1 = min(K1, t0 + per);
					unsigned int sT = 0, sF = 0, sM = 0;
					for (unsigned int k = t0; k < t1; ++k)
					{
						unsigned char st = w.status[k];
						unsigned int c = w.order[k];
						float e = __uint_as_float(w.cerr[c]);
						if (st == kCommit)
						{
							sT += w.kind[w.cv0[c]] == kBorder ? 1u : 2u;
							if (e == e)
								sM = max(sM, w.cerr[c]);
						}
						sF += st == kSkipFlip;
					}
					unsigned int eT, eF;
					{
						unsigned int tot;
						eT = blockExclusiveScan<NT>(sT, w.red, &tot);
						__syncthreads();
						eF = blockExclusiveScan<NT>(sF, w.red, &tot);
						__syncthreads();
					}
					// exclusive max over the threads before this one (in thread order)
					s_maxes[tid] = sM;
					__syncthreads();
					unsigned int eM = 0;
					for (unsigned int q = 0; q < tid; ++q)
						eM = max(eM, s_maxes[q]);
					unsigned long long T = (unsigned long long)s_carry[0] + eT, F = (unsigned long long)s_carry[1] + eF;
					unsigned int M = max(s_carry[2], eM);
					for (unsigned int k = t0; k < t1; ++k)
					{
						unsigned int c = w.order[k];
						float e = __uint_as_float(w.cerr[c]);
						unsigned int reason = 0;
						if (e > error_limit)
							reason = 1;
						else if (T >= goal)
							reason = 2;
						else
						{
							unsigned long long eg = goal / 2 + F;
							float error_goal = eg < C ? 1.5f * __uint_as_float(w.cerr[w.order[eg]]) : FLT_MAX;
							if (e > error_goal && e > __uint_as_float(M) && T > goal / 6)
								reason = 3;
						}
						if (reason)
						{
							atomicMin(&s_cut, ((unsigned long long)k << 2) | reason);
							break;
						}
						unsigned char st = w.status[k];
						if (st == kCommit)
						{
							T += w.kind[w.cv0[c]] == kBorder ? 1u : 2u;
							if (e == e)
								M = max(M, w.cerr[c]);
						}
						F += st == kSkipFlip;
					}
					__syncthreads();
					if (s_cut != ~0ull || K1 == C || s_stall)
						break;
					// carry the prefix over the window into the next one
					if (tid == NT - 1)
					{
						s_carry[0] = (unsigned int)T;
						s_carry[1] = (unsigned int)F;
						s_carry[2] = M;
					}
					__syncthreads();
					K0 = K1;
					K1 = (unsigned int)min((unsigned long long)C, 2ull * K1);
				}
			}
			// apply the committed prefix: collapse_remap writes, done count, result error
			{
				const unsigned int cut = s_cut == ~0ull ? C : (unsigned int)(s_cut >> 2);
				for (unsigned int i = tid; i < V; i += NT)
					w.cr[i] = i;
				__syncthreads();
				unsigned int done = 0, em = 0;
				for (unsigned int k = tid; k < cut; k += NT)
				{
					if (w.status[k] != kCommit)
						continue;
					unsigned int c = w.order[k];
					unsigned int i0 = w.cv0[c], i1 = w.cv1[c];
					if (FULL && w.kind[i0] == kComplex)
					{
						unsigned int v = i0;
						do
						{
							w.cr[v] = complexTarget(v, i1, w.remap, w.loop, w.loopback);
							v = w.wedge[v];
						} while (v != i0);
					}
					else if (w.kind[i0] == kSeam)
					{
						unsigned int s0 = w.wedge[i0];
						unsigned int s1 = w.loop[i0] == i1 ? w.loopback[s0] : w.loop[s0];
						s1 = (s1 != ~0u) ? s1 : w.wedge[i1];
						w.cr[i0] = i1;
						w.cr[s0] = s1;
					}
					else
						w.cr[i0] = i1;
					done++;
					float e = __uint_as_float(w.cerr[c]);
					if (e == e)
						em = max(em, w.cerr[c]);
				}
				unsigned int tot;
				blockExclusiveScan<NT>(done, w.red, &tot);
				__syncthreads();
				s_maxes[tid] = em;
				__syncthreads();
				if (tid == 0)
				{
					unsigned int mm = __float_as_uint(result_error);
					for (unsigned int q = 0; q < NT; ++q)
						mm = max(mm, s_maxes[q]);
					s_done = tot;
					s_errbits = mm;
				}
			}
		}
		__syncthreads();
		result_error = __uint_as_float(s_errbits);
		passes++;
		if (s_done == 0 || s_stall)
			break;

		// updateQuadrics (:1638-1673): every target receives at most one source per pass. The
		// moved wedges of one commit all belong to its source position (whose primary always
		// moves), and no other commit targets their targets, so each moved primary merges the
		// attribute quadrics of its wedges in increasing vertex order, as the reference's vertex
		// loop does
		for (unsigned int i = tid; i < V; i += NT)
		{
			unsigned int t = w.cr[i];
			if (t == i || w.remap[i] != i)
				continue;
			unsigned int r1 = w.remap[t];
			Quadric Q = ldquadric(w.vq, r1);
			qadd(Q, ldquadric(w.vq, i));
			stquadric(w.vq, r1, Q);
			if constexpr (FULL)
			{
				if (ac)
				{
					unsigned int last = 0;
					bool firstw = true;
					for (;;)
					{
						unsigned int best = ~0u, v = i;
						do
						{
							if ((firstw || v > last) && v < best)
								best = v;
							v = w.wedge[v];
						} while (v != i);
						if (best == ~0u)
							break;
						unsigned int tb = w.cr[best];
						if (tb != best)
						{
							Quadric A = ldquadric(w.aq, tb);
							qadd(A, ldquadric(w.aq, best));
							stquadric(w.aq, tb, A);
							for (unsigned int q = 0; q < ac; ++q)
							{
								float4 g = w.ag[(size_t)tb * ac + q], h = w.ag[(size_t)best * ac + q];
								g.x += h.x, g.y += h.y, g.z += h.z, g.w += h.w;
								w.ag[(size_t)tb * ac + q] = g;
							}
						}
						last = best;
						firstw = false;
					}
				}
			}
		}
		// remapEdgeLoops (:1845-1864), in place
		for (unsigned int i = tid; i < V; i += NT)
		{
			unsigned int* arrs[2] = {w.loop, w.loopback};
			for (int q = 0; q < 2; ++q)
			{
				unsigned int* L = arrs[q];
				unsigned int l = L[i];
				if (l == ~0u)
					continue;
				unsigned int r = w.cr[l];
				if (i == r)
				{
					unsigned int ll = L[l];
					L[i] = ll != ~0u ? w.cr[ll] : ~0u;
				}
				else
					L[i] = r;
			}
		}
		__syncthreads();
		// remapIndexBuffer (:1811-1843): in-place order-preserving compaction by chunks
		unsigned int written = 0;
		for (unsigned int base = 0; base < T; base += NT)
		{
			unsigned int t = base + tid;
			unsigned int v0 = 0, v1 = 0, v2 = 0;
			bool keep = false;
			if (t < T)
			{
				v0 = w.cr[w.idx[t * 3]], v1 = w.cr[w.idx[t * 3 + 1]], v2 = w.cr[w.idx[t * 3 + 2]];
				unsigned int r0 = w.remap[v0], r1 = w.remap[v1], r2 = w.remap[v2];
				keep = r0 != r1 && r0 != r2 && r1 != r2;
			}
			unsigned int tot;
			unsigned int ex = blockExclusiveScan<NT>(keep ? 1u : 0u, w.red, &tot);
			if (keep)
			{
				unsigned int o = (written + ex) * 3;
				w.idx[o] = v0, w.idx[o + 1] = v1, w.idx[o + 2] = v2;
			}
			written += tot;
			__syncthreads();
		}
		result_count = written * 3;
	}

	for (unsigned int i = tid; i < result_count; i += NT)
		d.out[i] = src(w.idx[i]);
	if (tid == 0)
		*out = BatchResult{result_count, sqrtf(result_error) * error_scale, passes, s_stall ? 3u : 0u};
}

template <int NT, bool FULL>
__global__ void __launch_bounds__(NT) kBatch(const BatchDesc* __restrict__ descs, unsigned int count, unsigned int* ticket, BatchResult* results,
    char* slabs, size_t slab_bytes, unsigned int smem_bytes)
{
	extern __shared__ __align__(16) char smem[];
	__shared__ unsigned int s_job;
	for (;;)
	{
		if (threadIdx.x == 0)
			s_job = atomicAdd(ticket, 1u);
		__syncthreads();
		unsigned int job = s_job;
		if (job >= count)
			break;
		BatchDesc d = descs[job];
		CtaWork w;
		const bool sparse = FULL && (d.options & kOptSparse) != 0;
		const size_t vb = localVertexBound(d.index_count, d.vertex_count, sparse);
		const unsigned int ac = FULL ? d.ac : 0;
		const bool in_smem = carve(w, nullptr, d.index_count, vb, ac, sparse, false) <= smem_bytes;
		char* base = in_smem ? smem : slabs + (size_t)blockIdx.x * slab_bytes;
		carve(w, base, d.index_count, vb, ac, sparse, !in_smem);
		simplifyMesh<NT, FULL>(d, w, &results[job], in_smem);
		__syncthreads();
	}
}

} // namespace

size_t batchWorkspaceBytes(size_t index_count, size_t vertex_count, size_t ac, bool sparse, bool rounds)
{
	CtaWork w;
	return carve(w, nullptr, index_count, localVertexBound(index_count, vertex_count, sparse), ac, sparse, rounds);
}

// the dynamic shared-memory limit of every batch kernel instance is raised once, to the
// device's opt-in maximum: setting it per launch would race between threads launching batches
// with different sizes
void raiseSmemLimits()
{
	static std::once_flag once;
	std::call_once(once, [] {
		int dev = 0, optin = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
		int limit = optin - 4096; // room for the kernel's static shared memory
		cudaFuncSetAttribute(kBatch<128, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
		cudaFuncSetAttribute(kBatch<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
		cudaFuncSetAttribute(kBatch<512, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
		cudaFuncSetAttribute(kBatch<128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
		cudaFuncSetAttribute(kBatch<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
		cudaFuncSetAttribute(kBatch<512, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
	});
}

template <bool FULL>
void launchBatchT(const BatchDesc* d_descs, unsigned int count, unsigned int* d_ticket, BatchResult* d_results, char* d_slabs, size_t slab_bytes,
    unsigned int smem_bytes, unsigned int blocks, int threads, cudaStream_t stream)
{
	switch (threads)
	{
	case 128:
		MO_LAUNCH((kBatch<128, FULL>), blocks, 128, smem_bytes, stream, d_descs, count, d_ticket, d_results, d_slabs, slab_bytes, smem_bytes);
		break;
	case 512:
		MO_LAUNCH((kBatch<512, FULL>), blocks, 512, smem_bytes, stream, d_descs, count, d_ticket, d_results, d_slabs, slab_bytes, smem_bytes);
		break;
	default:
		MO_LAUNCH((kBatch<256, FULL>), blocks, 256, smem_bytes, stream, d_descs, count, d_ticket, d_results, d_slabs, slab_bytes, smem_bytes);
		break;
	}
}

void launchBatch(const BatchDesc* d_descs, unsigned int count, unsigned int* d_ticket, BatchResult* d_results, char* d_slabs, size_t slab_bytes,
    unsigned int smem_bytes, unsigned int blocks, int threads, bool full, cudaStream_t stream)
{
	raiseSmemLimits();
	MO_CUDA_CHECK(cudaMemsetAsync(d_ticket, 0, sizeof(unsigned int), stream));
	if (full)
		launchBatchT<true>(d_descs, count, d_ticket, d_results, d_slabs, slab_bytes, smem_bytes, blocks, threads, stream);
	else
		launchBatchT<false>(d_descs, count, d_ticket, d_results, d_slabs, slab_bytes, smem_bytes, blocks, threads, stream);
	MO_CUDA_CHECK(cudaGetLastError());
}

template <bool FULL>
int blocksPerSMT(int threads, unsigned int smem_bytes)
{
	int n = 0;
	if (threads == 128)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kBatch<128, FULL>, 128, smem_bytes);
	else if (threads == 512)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kBatch<512, FULL>, 512, smem_bytes);
	else
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kBatch<256, FULL>, 256, smem_bytes);
	return n;
}

// occupancy per (device, threads, shared memory, variant), queried once each: driver queries
// are not free, and a batch call makes one
int batchBlocksPerSM(int threads, unsigned int smem_bytes, bool full)
{
	raiseSmemLimits();
	static std::mutex lock;
	static std::map<std::tuple<int, int, unsigned int, bool>, int> known;
	int dev = 0;
	cudaGetDevice(&dev);
	const auto key = std::make_tuple(dev, threads, smem_bytes, full);
	{
		std::lock_guard<std::mutex> g(lock);
		auto it = known.find(key);
		if (it != known.end())
			return it->second;
	}
	const int n = full ? blocksPerSMT<true>(threads, smem_bytes) : blocksPerSMT<false>(threads, smem_bytes);
	std::lock_guard<std::mutex> g(lock);
	known[key] = n;
	return n;
}

} // namespace mogpu
