// mo_meshlets.cu - meshopt_buildMeshletsFlex (src/clusterizer.cpp:1035-1224) for many index
// subsets of one vertex buffer: the re-clusterization a cluster-LOD builder runs on every
// simplified group (demo/clusterlod.h:266-296).
//
// The algorithm is a serial greedy: every step appends the best triangle next to the current
// meshlet, and the choice depends on all earlier ones. Here one warp builds one group's meshlets,
// and groups run side by side. Inside a group, lane 0 runs the order-dependent bookkeeping (the
// area sum, the kd-tree, seeds, appends, list removal) exactly as the reference orders it, and
// the warp shares the wide steps:
//  - group-local vertex ids in first-use order (a hash table keyed by vertex, a warp scan);
//  - every vertex's triangle list in face order (ranks among equal vertices from match_any, so
//    corners enter their lists in corner order, as the reference's fill loop does);
//  - the triangle cones;
//  - the neighbour search of every step: lanes scan the lists of different meshlet vertices and
//    a warp reduction picks the smallest (priority, score, scan position), which is the
//    reference's first best triangle in its scan order. A NaN score breaks that ordering, so a
//    step that meets one is scanned again by lane 0 alone, in the reference's order;
//  - each meshlet vertex's best seed neighbour when a meshlet ends.
// The reference keys its per-vertex arrays by the caller's vertex index; nothing in its result
// depends on that numbering, only on vertex identity and on the order vertices enter a meshlet,
// so group-local ids give the same meshlets.
#include "mo_meshlets.cuh"
#include "mo_common.cuh"
#include "mo_prims.cuh"
#include "mo_probe.cuh"

#include <float.h>
#include <type_traits>

namespace mogpu
{

namespace
{

constexpr unsigned int kMaxSeeds = 256; // kMeshletMaxSeeds, :27
constexpr unsigned int kAddSeeds = 4;   // kMeshletAddSeeds, :28
constexpr int kMaxDepth = 50;           // kMeshletMaxTreeDepth, :31
constexpr unsigned int kLeafSize = 8;   // :1090
constexpr int kMaxWarpsPerBlock = 4;

struct Cone
{
	float px, py, pz, nx, ny, nz;
};

// kd-tree node (:473-485): axis 3 = leaf of `children` points (this node and the ones after);
// a branch's right subtree starts children + 1 nodes after it
struct KDNode
{
	unsigned int word; // split (float bits) or point index
	unsigned int axis;
	unsigned int children;
};

size_t align256(size_t n)
{
	return (n + 255) & ~size_t(255);
}

__host__ __device__ inline unsigned int tableSize(unsigned int I)
{
	unsigned int h = 64;
	while (h < 2 * I)
		h *= 2;
	return h;
}

// one group's scratch, carved from its base in a fixed order (host and device agree)
struct Scratch
{
	unsigned int *hkey, *hpos, *hid, *slot, *lidx, *gid, *cnt, *off, *fill, *adj, *mvl, *kdidx, *vbest, *seeds;
	short* used;
	unsigned char* emitted;
	Cone* cones;
	float* area;
	KDNode* nodes;
};

__host__ __device__ inline size_t carve(Scratch& s, char* base, unsigned int I)
{
	const unsigned int F = I / 3, H = tableSize(I);
	size_t o = 0;
	auto take = [&](size_t bytes) {
		char* p = base ? base + o : nullptr;
		o += (bytes + 15) & ~size_t(15);
		return p;
	};
	s.hkey = reinterpret_cast<unsigned int*>(take(size_t(H) * 4));
	s.hpos = reinterpret_cast<unsigned int*>(take(size_t(H) * 4));
	s.hid = reinterpret_cast<unsigned int*>(take(size_t(H) * 4));
	s.slot = reinterpret_cast<unsigned int*>(take(size_t(I) * 4));
	s.lidx = reinterpret_cast<unsigned int*>(take(size_t(I) * 4));
	s.gid = reinterpret_cast<unsigned int*>(take(size_t(I) * 4));
	s.cnt = reinterpret_cast<unsigned int*>(take(size_t(I) * 4));
	s.off = reinterpret_cast<unsigned int*>(take(size_t(I) * 4));
	s.fill = reinterpret_cast<unsigned int*>(take(size_t(I) * 4));
	s.adj = reinterpret_cast<unsigned int*>(take(size_t(I) * 4));
	s.mvl = reinterpret_cast<unsigned int*>(take(size_t(I) * 4));
	s.kdidx = reinterpret_cast<unsigned int*>(take(size_t(F) * 4));
	s.vbest = reinterpret_cast<unsigned int*>(take(256 * 3 * 4));
	s.seeds = reinterpret_cast<unsigned int*>(take(kMaxSeeds * 4));
	s.used = reinterpret_cast<short*>(take(size_t(I) * 2));
	s.emitted = reinterpret_cast<unsigned char*>(take(F));
	s.cones = reinterpret_cast<Cone*>(take(size_t(F) * sizeof(Cone)));
	s.area = reinterpret_cast<float*>(take(size_t(F) * 4));
	s.nodes = reinterpret_cast<KDNode*>(take(size_t(F) * 2 * sizeof(KDNode)));
	return o;
}

__device__ __forceinline__ unsigned int hashVertex(unsigned int v)
{
	v ^= v >> 16;
	v *= 0x7feb352du;
	v ^= v >> 15;
	v *= 0x846ca68bu;
	v ^= v >> 16;
	return v;
}

__device__ __forceinline__ float dist3(float ax, float ay, float az, float bx, float by, float bz)
{
	float dx = ax - bx, dy = ay - by, dz = az - bz;
	return sqrtf(dx * dx + dy * dy + dz * dz);
}

// getMeshletScore, :173-179
__device__ __forceinline__ float meshletScore(float distance, float spread, float cone_weight, float expected_radius)
{
	float cone = 1.f - spread * cone_weight;
	float clamped = cone < 1e-3f ? 1e-3f : cone;
	return (1 + distance / expected_radius * (1 - cone_weight)) * clamped;
}

// topology priority of a candidate triangle (:318-335)
__device__ __forceinline__ int neighborPriority(const Scratch& s, unsigned int t)
{
	unsigned int a = s.lidx[t * 3 + 0], b = s.lidx[t * 3 + 1], c = s.lidx[t * 3 + 2];
	int extra = (s.used[a] < 0) + (s.used[b] < 0) + (s.used[c] < 0);
	unsigned int la = s.cnt[a], lb = s.cnt[b], lc = s.cnt[c];
	if (extra == 0)
		return 0;
	if (la == 1 || lb == 1 || lc == 1)
		return 1;
	if ((la == 2) + (lb == 2) + (lc == 2) >= 2)
		return 1 + extra;
	return 2 + extra;
}

__device__ __forceinline__ float neighborScore(const Scratch& s, unsigned int t, const Cone& mc, float cone_weight, float radius)
{
	const Cone& tc = s.cones[t];
	float distance = dist3(tc.px, tc.py, tc.pz, mc.px, mc.py, mc.pz);
	float spread = tc.nx * mc.nx + tc.ny * mc.ny + tc.nz * mc.nz;
	return meshletScore(distance, spread, cone_weight, radius);
}

// getNeighborTriangle, :302-362, in the reference's scan order (lane 0 only)
__device__ unsigned int neighborSerial(const Scratch& s, unsigned int voff, unsigned int vcount, const Cone& mc, float cone_weight, float radius)
{
	unsigned int best = ~0u;
	int best_priority = 5;
	float best_score = FLT_MAX;
	for (unsigned int i = 0; i < vcount; ++i)
	{
		unsigned int v = s.mvl[voff + i];
		const unsigned int* list = s.adj + s.off[v];
		const unsigned int n = s.cnt[v];
		for (unsigned int j = 0; j < n; ++j)
		{
			unsigned int t = list[j];
			int priority = neighborPriority(s, t);
			if (priority > best_priority)
				continue;
			float score = neighborScore(s, t, mc, cone_weight, radius);
			if (priority < best_priority || score < best_score)
			{
				best = t;
				best_priority = priority;
				best_score = score;
			}
		}
	}
	return best;
}

// the same choice by the whole warp: lane l scans the lists of meshlet vertices l, l + 32, ...,
// then the warp takes the smallest (priority, score, scan position); *nan is set when a score
// was NaN (the warp's answer is then not the reference's)
__device__ unsigned int neighborWarp(const Scratch& s, unsigned int voff, unsigned int vcount, const Cone& mc, float cone_weight, float radius, bool* nan)
{
	const unsigned int lane = threadIdx.x & 31;
	unsigned int best = ~0u;
	unsigned long long key = ~0ull; // scan position: (meshlet vertex, list entry)
	int bp = 5;
	float bs = FLT_MAX;
	bool sawnan = false;
	for (unsigned int i = lane; i < vcount; i += 32)
	{
		unsigned int v = s.mvl[voff + i];
		const unsigned int* list = s.adj + s.off[v];
		const unsigned int n = s.cnt[v];
		for (unsigned int j = 0; j < n; ++j)
		{
			unsigned int t = list[j];
			int priority = neighborPriority(s, t);
			if (priority > bp)
				continue;
			float score = neighborScore(s, t, mc, cone_weight, radius);
			sawnan |= score != score;
			if (priority < bp || score < bs)
			{
				best = t;
				bp = priority;
				bs = score;
				key = ((unsigned long long)i << 32) | j;
			}
		}
	}
	for (int o = 16; o > 0; o >>= 1)
	{
		unsigned int ob = __shfl_xor_sync(0xffffffffu, best, o);
		unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
		int op = __shfl_xor_sync(0xffffffffu, bp, o);
		float os = __shfl_xor_sync(0xffffffffu, bs, o);
		bool take = op < bp || (op == bp && (os < bs || (os == bs && ok < key)));
		if (take)
		{
			best = ob;
			bp = op;
			bs = os;
			key = ok;
		}
	}
	*nan = __any_sync(0xffffffffu, sawnan);
	return __shfl_sync(0xffffffffu, best, 0);
}

// kdtreeBuild, :532-581, depth first on an explicit stack (lane 0): a subtree's nodes start
// where the previous one in that order ended, and a right subtree records its distance from its
// parent when it starts, which is after the whole left subtree
__device__ void kdBuild(const Scratch& s, unsigned int F, unsigned int* err)
{
	struct Task
	{
		unsigned int start, count, parent;
		int depth;
	} stack[kMaxDepth + 8];
	int top = 0;
	stack[top++] = Task{0, F, ~0u, 0};
	unsigned int next = 0;
	while (top > 0)
	{
		Task t = stack[--top];
		const unsigned int offset = next;
		if (t.parent != ~0u)
			s.nodes[t.parent].children = offset - t.parent - 1;
		unsigned int* idx = s.kdidx + t.start;
		bool leaf = t.count <= kLeafSize;
		float split = 0.f;
		int axis = 0;
		unsigned int middle = 0;
		if (!leaf)
		{
			float mean[3] = {0.f, 0.f, 0.f}, vars[3] = {0.f, 0.f, 0.f};
			float runc = 1, runs = 1;
			for (unsigned int i = 0; i < t.count; ++i, runc += 1.f, runs = 1.f / runc)
			{
				const Cone& c = s.cones[idx[i]];
				const float p[3] = {c.px, c.py, c.pz};
				for (int k = 0; k < 3; ++k)
				{
					float delta = p[k] - mean[k];
					mean[k] += delta * runs;
					vars[k] += delta * (p[k] - mean[k]);
				}
			}
			axis = (vars[0] >= vars[1] && vars[0] >= vars[2]) ? 0 : (vars[1] >= vars[2] ? 1 : 2);
			split = mean[axis];
			// kdtreePartition, :487-506
			unsigned int m = 0;
			for (unsigned int i = 0; i < t.count; ++i)
			{
				const Cone& c = s.cones[idx[i]];
				float v = axis == 0 ? c.px : (axis == 1 ? c.py : c.pz);
				unsigned int tmp = idx[m];
				idx[m] = idx[i];
				idx[i] = tmp;
				m += v < split;
			}
			middle = m;
			leaf = middle <= kLeafSize / 2 || middle >= t.count - kLeafSize / 2 || t.depth >= kMaxDepth;
		}
		if (leaf)
		{
			// kdtreeBuildLeaf, :508-530
			s.nodes[offset] = KDNode{idx[0], 3u, t.count};
			for (unsigned int i = 1; i < t.count; ++i)
				s.nodes[offset + i] = KDNode{idx[i], 3u, ~0u >> 2};
			next = offset + t.count;
			continue;
		}
		s.nodes[offset] = KDNode{__float_as_uint(split), unsigned(axis), 0u};
		next = offset + 1;
		if (top + 2 > kMaxDepth + 8)
		{
			atomicOr(err, 2u);
			return;
		}
		stack[top++] = Task{t.start + middle, t.count - middle, offset, t.depth + 1};
		stack[top++] = Task{t.start, middle, ~0u, t.depth + 1};
	}
}

// kdtreeNearest, :583-639, on an explicit stack in the recursion's order (lane 0): a branch
// leaves "its second child, if the split is within the best distance then" under its first
// child; emptied leaves and branches are switched off on the way
__device__ void kdNearest(const Scratch& s, const float* pos, unsigned int* result, float* limit)
{
	struct Frame
	{
		unsigned int node;
		float dist; // >= 0: a deferred second child, visited if dist <= limit; < 0: visit
	} stack[2 * kMaxDepth + 8];
	int top = 0;
	stack[top++] = Frame{0, -1.f};
	while (top > 0)
	{
		Frame f = stack[--top];
		if (f.dist >= 0.f && !(f.dist <= *limit))
			continue;
		const unsigned int root = f.node;
		KDNode& node = s.nodes[root];
		if (node.children == 0)
			continue;
		if (node.axis == 3)
		{
			bool inactive = true;
			for (unsigned int i = 0; i < node.children; ++i)
			{
				unsigned int index = s.nodes[root + i].word;
				if (s.emitted[index])
					continue;
				inactive = false;
				const Cone& c = s.cones[index];
				float d = dist3(c.px, c.py, c.pz, pos[0], pos[1], pos[2]);
				if (d < *limit)
				{
					*result = index;
					*limit = d;
				}
			}
			if (inactive)
				node.children = 0;
		}
		else
		{
			float delta = pos[node.axis] - __uint_as_float(node.word);
			unsigned int first = (delta <= 0) ? 0 : node.children;
			unsigned int second = first ^ node.children;
			if ((s.nodes[root + 1 + first].children | s.nodes[root + 1 + second].children) == 0)
				node.children = 0;
			if (top + 2 > 2 * kMaxDepth + 8)
				return;
			// a NaN delta is never <= limit, so that child is skipped as the recursion skips it
			stack[top++] = Frame{root + 1 + second, delta != delta ? FLT_MAX : fabsf(delta)};
			stack[top++] = Frame{root + 1 + first, -1.f};
		}
	}
}

// meshopt_optimizeMeshletLevel (src/meshletutils.cpp:366-554) on one meshlet, by one warp: at
// every position the scan over the remaining triangles runs 32 at a time (the stop after the
// level-th edge match found with a ballot, then the first best score up to it), the shift and
// the bookkeeping on lane 0; 8-bit timestamps and valences wrap as the reference's do
struct MeshletOpt
{
	unsigned char idx[512 * 3];
	unsigned char cache[256];
	unsigned int valence[256];
	short remap[256];
	unsigned int order[256];
};

__device__ void optimizeMeshletWarp(unsigned int* verts, unsigned char* tris, unsigned int vc, unsigned int tc, int level, MeshletOpt& o)
{
	const unsigned int lane = threadIdx.x & 31;
	const unsigned char cutoff = 3;
	for (unsigned int k = lane; k < tc * 3; k += 32)
		o.idx[k] = tris[k];
	for (unsigned int v = lane; v < vc; v += 32)
	{
		o.cache[v] = 0;
		o.valence[v] = 0;
	}
	__syncwarp();
	for (unsigned int k = lane; k < tc * 3; k += 32)
		atomicAdd(&o.valence[o.idx[k]], 1u);
	__syncwarp();
	unsigned char cache_last = 128;
	for (unsigned int i = 0; i < tc; ++i)
	{
		int next = -1, next_score = -1, edges = 0;
		bool done = false;
		for (unsigned int j0 = i; j0 < tc && !done; j0 += 32)
		{
			const unsigned int j = j0 + lane;
			const bool valid = j < tc;
			int score = -2, match = 0;
			if (valid)
			{
				unsigned char a = o.idx[j * 3 + 0], b = o.idx[j * 3 + 1], c = o.idx[j * 3 + 2];
				unsigned char ad = (unsigned char)(cache_last - o.cache[a]);
				unsigned char bd = (unsigned char)(cache_last - o.cache[b]);
				unsigned char cd = (unsigned char)(cache_last - o.cache[c]);
				match = (ad < cutoff) + (bd < cutoff) + (cd < cutoff);
				if (level)
				{
					int va = o.valence[a] & 0xFF, vb = o.valence[b] & 0xFF, vcc = o.valence[c] & 0xFF;
					int vmin = va < vb ? va : vb;
					vmin = vcc < vmin ? vcc : vmin;
					score = (match * 1024 + (1023 - ad - bd - cd)) * 256 + (255 - vmin);
				}
				else
					score = match;
			}
			// the scan stops at the edge match that makes `level` of them (the first one at level 0)
			const unsigned int em = __ballot_sync(0xffffffffu, valid && match >= 2);
			const int need = level ? level - edges : 1;
			unsigned int last = 31;
			if (__popc(em) >= need)
			{
				unsigned int m = em;
				for (int q = 1; q < need; ++q)
					m &= m - 1;
				last = __ffs(m) - 1;
				done = true;
			}
			edges += __popc(em & (last == 31 ? 0xffffffffu : ((2u << last) - 1u)));
			// the first best score among the scanned ones
			int bs = (valid && lane <= last) ? score : -2;
			unsigned int bj = (valid && lane <= last) ? j : ~0u;
			for (int off = 16; off > 0; off >>= 1)
			{
				int os = __shfl_xor_sync(0xffffffffu, bs, off);
				unsigned int oj = __shfl_xor_sync(0xffffffffu, bj, off);
				if (os > bs || (os == bs && oj < bj))
					bs = os, bj = oj;
			}
			if (bs > next_score)
			{
				next = int(bj);
				next_score = bs;
			}
		}
		if (lane == 0)
		{
			const unsigned int n = unsigned(next);
			unsigned char a = o.idx[n * 3 + 0], b = o.idx[n * 3 + 1], c = o.idx[n * 3 + 2];
			for (unsigned int k = n * 3; k > i * 3; --k) // the triangles before it shift forward
				o.idx[k + 2] = o.idx[k - 1];
			o.idx[i * 3 + 0] = a;
			o.idx[i * 3 + 1] = b;
			o.idx[i * 3 + 2] = c;
			unsigned char stamp = (unsigned char)(cache_last + 1);
			o.cache[a] = o.cache[b] = o.cache[c] = stamp;
			o.valence[a] = (o.valence[a] - 1) & 0xFF;
			o.valence[b] = (o.valence[b] - 1) & 0xFF;
			o.valence[c] = (o.valence[c] - 1) & 0xFF;
		}
		cache_last++;
		__syncwarp();
	}
	if (lane == 0)
	{
		if (level >= 1)
		{
			for (unsigned int v = 0; v < vc; ++v)
				o.cache[v] = 0;
			for (unsigned int i = 0; i < tc; ++i)
			{
				unsigned char a = o.idx[i * 3 + 0], b = o.idx[i * 3 + 1], c = o.idx[i * 3 + 2];
				if (!o.cache[a] && o.cache[b] && !o.cache[c])
				{
					unsigned char t = a;
					a = b, b = c, c = t;
				}
				else if (!o.cache[a] && !o.cache[b] && !o.cache[c])
				{
					bool ab = false, bc = false, ca = false;
					for (unsigned int j = i + 1; j < tc && j <= i + cutoff; ++j)
					{
						unsigned char oa = o.idx[j * 3 + 0], ob = o.idx[j * 3 + 1], oc = o.idx[j * 3 + 2];
						ab |= (oa == b && ob == a) || (ob == b && oc == a) || (oc == b && oa == a);
						bc |= (oa == c && ob == b) || (ob == c && oc == b) || (oc == c && oa == b);
						ca |= (oa == a && ob == c) || (ob == a && oc == c) || (oc == a && oa == c);
					}
					if (ab && !bc)
					{
						unsigned char t = a;
						a = b, b = c, c = t;
					}
					else if ((ab && !ca) || (!ab && bc && !ca))
					{
						unsigned char t = c;
						c = b, b = a, a = t;
					}
				}
				o.idx[i * 3 + 0] = a, o.idx[i * 3 + 1] = b, o.idx[i * 3 + 2] = c;
				o.cache[a] = o.cache[b] = o.cache[c] = 1;
			}
		}
		// vertices renumbered in first-use order
		for (unsigned int v = 0; v < vc; ++v)
			o.remap[v] = -1;
		unsigned int n = 0;
		for (unsigned int k = 0; k < tc * 3; ++k)
		{
			short r = o.remap[o.idx[k]];
			if (r < 0)
			{
				r = short(n);
				o.remap[o.idx[k]] = r;
				o.order[n++] = verts[o.idx[k]];
			}
			o.idx[k] = (unsigned char)r;
		}
		for (unsigned int v = 0; v < n; ++v)
			verts[v] = o.order[v];
	}
	__syncwarp();
	for (unsigned int k = lane; k < tc * 3; k += 32)
		tris[k] = o.idx[k];
	__syncwarp();
}

__global__ void __launch_bounds__(kMaxWarpsPerBlock * 32) kMeshletsFlex(MeshletBatch b)
{
	const unsigned int lane = threadIdx.x & 31;
	const unsigned int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
	if (g >= b.groups)
		return;
	const unsigned long long i0 = b.offsets[g], i1 = b.offsets[g + 1];
	const unsigned int I = unsigned(i1 - i0) / 3 * 3, F = I / 3;
	const unsigned int* indices = b.indices + i0;
	if (F == 0)
	{
		if (lane == 0)
			b.counts[g] = 0;
		return;
	}
	Scratch s;
	carve(s, b.scratch + b.scratch_off[g], I);
	const unsigned int H = tableSize(I);
	unsigned int* out = b.meshlets + b.meshlet_base[g] * 4;
	const unsigned long long out_rows = b.meshlet_base[g + 1] - b.meshlet_base[g];
	unsigned int* mverts = b.mverts + i0;
	unsigned char* mtris = b.mtris + i0;

	// ---- group-local vertex ids in first-use order
	for (unsigned int h = lane; h < H; h += 32)
	{
		s.hkey[h] = ~0u;
		s.hpos[h] = ~0u;
	}
	__syncwarp();
	for (unsigned int p = lane; p < I; p += 32)
	{
		unsigned int v = indices[p];
		if (v >= b.vertex_count)
		{
			atomicOr(b.error, 1u);
			v = 0;
		}
		unsigned int h = hashVertex(v) & (H - 1);
		for (unsigned int probe = 0; probe < H; ++probe)
		{
			unsigned int k = atomicCAS(&s.hkey[h], ~0u, v);
			if (k == ~0u || k == v)
			{
				atomicMin(&s.hpos[h], p);
				s.slot[p] = h;
				break;
			}
			h = (h + 1) & (H - 1);
		}
	}
	__syncwarp();
	unsigned int U = 0;
	for (unsigned int base = 0; base < I; base += 32)
	{
		const unsigned int p = base + lane;
		const bool first = p < I && s.hpos[s.slot[p]] == p;
		const unsigned int m = __ballot_sync(0xffffffffu, first);
		if (first)
		{
			unsigned int id = U + __popc(m & ((1u << lane) - 1u));
			s.hid[s.slot[p]] = id;
			unsigned int v = indices[p];
			s.gid[id] = v < b.vertex_count ? v : 0u;
		}
		U += __popc(m);
	}
	// the arrays the greedy loop reads at every step move to this warp's shared memory, in the
	// order of their use per step, while they fit (U is known now)
	{
		extern __shared__ __align__(16) char pool[];
		char* base = pool + (threadIdx.x >> 5) * b.pool_bytes;
		size_t used_bytes = 0;
		auto promote = [&](auto*& ptr, size_t bytes) {
			bytes = (bytes + 15) & ~size_t(15);
			if (used_bytes + bytes <= b.pool_bytes)
			{
				ptr = reinterpret_cast<std::remove_reference_t<decltype(ptr)>>(base + used_bytes);
				used_bytes += bytes;
			}
		};
		promote(s.cnt, size_t(U) * 4);
		promote(s.off, size_t(U) * 4);
		promote(s.used, size_t(U) * 2);
		promote(s.lidx, size_t(I) * 4);
		promote(s.adj, size_t(I) * 4);
		promote(s.mvl, size_t(I) * 4);
		promote(s.emitted, F);
		promote(s.cones, size_t(F) * sizeof(Cone));
	}
	__syncwarp();
	for (unsigned int p = lane; p < I; p += 32)
		s.lidx[p] = s.hid[s.slot[p]];
	for (unsigned int v = lane; v < U; v += 32)
	{
		s.cnt[v] = 0;
		s.fill[v] = 0;
		s.used[v] = -1;
	}
	for (unsigned int t = lane; t < F; t += 32)
		s.emitted[t] = 0;
	__syncwarp();

	// ---- triangle lists per vertex, in face order (corner order)
	for (unsigned int p = lane; p < I; p += 32)
		atomicAdd(&s.cnt[s.lidx[p]], 1u);
	__syncwarp();
	{
		unsigned int run = 0;
		for (unsigned int base = 0; base < U; base += 32)
		{
			const unsigned int v = base + lane;
			unsigned int c = v < U ? s.cnt[v] : 0u, x = c;
			for (int o = 1; o < 32; o <<= 1)
			{
				unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
				if (lane >= (unsigned)o)
					x += y;
			}
			if (v < U)
				s.off[v] = run + x - c;
			run += __shfl_sync(0xffffffffu, x, 31);
		}
	}
	__syncwarp();
	for (unsigned int base = 0; base < I; base += 32)
	{
		const unsigned int p = base + lane;
		const bool valid = p < I;
		const unsigned int v = valid ? s.lidx[p] : (0x80000000u | lane);
		const unsigned int peers = __match_any_sync(0xffffffffu, v);
		const unsigned int leader = __ffs(peers) - 1;
		unsigned int o = 0;
		if (valid && lane == leader)
			o = atomicAdd(&s.fill[v], __popc(peers));
		o = __shfl_sync(0xffffffffu, o, leader);
		if (valid)
			s.adj[s.off[v] + o + __popc(peers & ((1u << lane) - 1u))] = p / 3;
	}

	// ---- triangle cones (computeTriangleCones, :201-241)
	for (unsigned int t = lane; t < F; t += 32)
	{
		const float* p0 = b.positions + size_t(b.stride_f) * s.gid[s.lidx[t * 3 + 0]];
		const float* p1 = b.positions + size_t(b.stride_f) * s.gid[s.lidx[t * 3 + 1]];
		const float* p2 = b.positions + size_t(b.stride_f) * s.gid[s.lidx[t * 3 + 2]];
		float p10[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
		float p20[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
		float nx = p10[1] * p20[2] - p10[2] * p20[1];
		float ny = p10[2] * p20[0] - p10[0] * p20[2];
		float nz = p10[0] * p20[1] - p10[1] * p20[0];
		float area = sqrtf(nx * nx + ny * ny + nz * nz);
		float inv = (area == 0.f) ? 0.f : 1.f / area;
		Cone c;
		c.px = (p0[0] + p1[0] + p2[0]) / 3.f;
		c.py = (p0[1] + p1[1] + p2[1]) / 3.f;
		c.pz = (p0[2] + p1[2] + p2[2]) / 3.f;
		c.nx = nx * inv;
		c.ny = ny * inv;
		c.nz = nz * inv;
		s.cones[t] = c;
		s.area[t] = area;
		s.kdidx[t] = t;
	}
	__syncwarp();

	// ---- serial setup (lane 0): mesh area in face order, the kd-tree, the corner, the first seed
	float radius = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
	unsigned int initial = ~0u;
	if (lane == 0)
	{
		float mesh_area = 0.f;
		for (unsigned int t = 0; t < F; ++t)
			mesh_area += s.area[t];
		float tri_area_avg = mesh_area / float(F) * 0.5f;
		radius = sqrtf(tri_area_avg * float(b.max_triangles)) * 0.5f;
		kdBuild(s, F, b.error);
		cx = FLT_MAX, cy = FLT_MAX, cz = FLT_MAX;
		for (unsigned int t = 0; t < F; ++t)
		{
			const Cone& c = s.cones[t];
			cx = cx > c.px ? c.px : cx;
			cy = cy > c.py ? c.py : cy;
			cz = cz > c.pz ? c.pz : cz;
		}
		float initial_score = FLT_MAX;
		for (unsigned int t = 0; t < F; ++t)
		{
			const Cone& c = s.cones[t];
			float d = dist3(c.px, c.py, c.pz, cx, cy, cz);
			if (initial == ~0u || d < initial_score)
			{
				initial = t;
				initial_score = d;
			}
		}
	}
	radius = __shfl_sync(0xffffffffu, radius, 0);
	cx = __shfl_sync(0xffffffffu, cx, 0);
	cy = __shfl_sync(0xffffffffu, cy, 0);
	cz = __shfl_sync(0xffffffffu, cz, 0);
	initial = __shfl_sync(0xffffffffu, initial, 0);
	__syncwarp();

	// ---- the greedy loop (:1125-1216); every lane holds the same meshlet state
	unsigned int m_voff = 0, m_toff = 0, m_vc = 0, m_tc = 0; // the current meshlet
	unsigned int offset = 0, seed_count = 0;
	Cone acc = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
	for (unsigned int step = 0; step <= F; ++step)
	{
		// getMeshletCone, :181-199
		Cone mc = acc;
		{
			float center_scale = m_tc == 0 ? 0.f : 1.f / float(m_tc);
			mc.px *= center_scale;
			mc.py *= center_scale;
			mc.pz *= center_scale;
			float len = mc.nx * mc.nx + mc.ny * mc.ny + mc.nz * mc.nz;
			float axis_scale = len == 0.f ? 0.f : 1.f / sqrtf(len);
			mc.nx *= axis_scale;
			mc.ny *= axis_scale;
			mc.nz *= axis_scale;
		}
		unsigned int best;
		if (offset == 0 && m_tc == 0)
			best = initial;
		else
		{
			bool nan = false;
			best = neighborWarp(s, m_voff, m_vc, mc, b.cone_weight, radius, &nan);
			if (nan)
			{
				if (lane == 0)
					best = neighborSerial(s, m_voff, m_vc, mc, b.cone_weight, radius);
				best = __shfl_sync(0xffffffffu, best, 0);
			}
		}
		bool split = false;
		if (best == ~0u)
		{
			// no adjacent triangle: the nearest unemitted one (kdtreeNearest)
			float distance = FLT_MAX;
			if (lane == 0)
			{
				const float pos[3] = {mc.px, mc.py, mc.pz};
				kdNearest(s, pos, &best, &distance);
			}
			best = __shfl_sync(0xffffffffu, best, 0);
			distance = __shfl_sync(0xffffffffu, distance, 0);
			split = m_tc >= b.min_triangles && b.split_factor > 0 && distance > radius * b.split_factor;
		}
		if (best == ~0u)
			break;
		__syncwarp();
		const int best_extra = (s.used[s.lidx[best * 3 + 0]] < 0) + (s.used[s.lidx[best * 3 + 1]] < 0) + (s.used[s.lidx[best * 3 + 2]] < 0);
		if (split || m_vc + best_extra > b.max_vertices || m_tc >= b.max_triangles)
		{
			// each meshlet vertex's neighbour with the smallest live count (appendSeedTriangles,
			// :364-430, inner loop), then the seed bookkeeping in vertex order on lane 0
			for (unsigned int i = lane; i < m_vc; i += 32)
			{
				unsigned int v = s.mvl[m_voff + i];
				const unsigned int* list = s.adj + s.off[v];
				const unsigned int n = s.cnt[v];
				unsigned int bn = ~0u, bn_live = ~0u;
				for (unsigned int j = 0; j < n; ++j)
				{
					unsigned int t = list[j];
					unsigned int l = s.cnt[s.lidx[t * 3 + 0]] + s.cnt[s.lidx[t * 3 + 1]] + s.cnt[s.lidx[t * 3 + 2]];
					if (l < bn_live)
					{
						bn = t;
						bn_live = l;
					}
				}
				float score = 0.f;
				if (bn != ~0u)
				{
					const Cone& c = s.cones[bn];
					score = dist3(c.px, c.py, c.pz, cx, cy, cz);
				}
				s.vbest[i * 3 + 0] = bn;
				s.vbest[i * 3 + 1] = bn_live;
				s.vbest[i * 3 + 2] = __float_as_uint(score);
			}
			__syncwarp();
			if (lane == 0)
			{
				// pruneSeedTriangles, :432-445
				unsigned int r = 0;
				for (unsigned int i = 0; i < seed_count; ++i)
				{
					unsigned int sd = s.seeds[i];
					s.seeds[r] = sd;
					r += s.emitted[sd] == 0;
				}
				seed_count = (r + kAddSeeds <= kMaxSeeds) ? r : kMaxSeeds - kAddSeeds;
				unsigned int bs[kAddSeeds], bl[kAddSeeds];
				float bsc[kAddSeeds];
				for (unsigned int i = 0; i < kAddSeeds; ++i)
				{
					bs[i] = ~0u;
					bl[i] = ~0u;
					bsc[i] = FLT_MAX;
				}
				for (unsigned int i = 0; i < m_vc; ++i)
				{
					unsigned int bn = s.vbest[i * 3 + 0];
					if (bn == ~0u)
						continue;
					unsigned int live = s.vbest[i * 3 + 1];
					float score = __uint_as_float(s.vbest[i * 3 + 2]);
					for (unsigned int j = 0; j < kAddSeeds; ++j)
						if (live < bl[j] || (live == bl[j] && score <= bsc[j]))
						{
							bs[j] = bn;
							bl[j] = live;
							bsc[j] = score;
							break;
						}
				}
				for (unsigned int i = 0; i < kAddSeeds; ++i)
					if (bs[i] != ~0u)
						s.seeds[seed_count++] = bs[i];
				// selectSeedTriangle, :447-471
				unsigned int bseed = ~0u, blive = ~0u;
				float bscore = FLT_MAX;
				for (unsigned int i = 0; i < seed_count; ++i)
				{
					unsigned int sd = s.seeds[i];
					unsigned int live = s.cnt[s.lidx[sd * 3 + 0]] + s.cnt[s.lidx[sd * 3 + 1]] + s.cnt[s.lidx[sd * 3 + 2]];
					const Cone& c = s.cones[sd];
					float score = dist3(c.px, c.py, c.pz, cx, cy, cz);
					if (live < blive || (live == blive && score < bscore))
					{
						bseed = sd;
						blive = live;
						bscore = score;
					}
				}
				best = bseed != ~0u ? bseed : best;
			}
			best = __shfl_sync(0xffffffffu, best, 0);
			seed_count = __shfl_sync(0xffffffffu, seed_count, 0);
		}

		// appendMeshlet (:243-300), the list removal (:1177-1199) and the emitted flag on lane 0
		unsigned int reset = 0;
		if (lane == 0)
		{
			const unsigned int v3[3] = {s.lidx[best * 3 + 0], s.lidx[best * 3 + 1], s.lidx[best * 3 + 2]};
			const int extra = (s.used[v3[0]] < 0) + (s.used[v3[1]] < 0) + (s.used[v3[2]] < 0);
			if (m_vc + extra > b.max_vertices || m_tc >= b.max_triangles || split)
			{
				if (offset < out_rows)
				{
					out[offset * 4 + 0] = m_voff;
					out[offset * 4 + 1] = m_toff;
					out[offset * 4 + 2] = m_vc;
					out[offset * 4 + 3] = m_tc;
				}
				else
					atomicOr(b.error, 4u);
				for (unsigned int j = 0; j < m_vc; ++j)
					s.used[s.mvl[m_voff + j]] = -1;
				m_voff += m_vc;
				m_toff += m_tc * 3;
				m_vc = 0;
				m_tc = 0;
				reset = 1;
			}
			for (int k = 0; k < 3; ++k)
				if (s.used[v3[k]] < 0)
				{
					s.used[v3[k]] = short(m_vc);
					if (m_voff + m_vc < I)
					{
						s.mvl[m_voff + m_vc] = v3[k];
						mverts[m_voff + m_vc] = s.gid[v3[k]];
					}
					else
						atomicOr(b.error, 4u);
					m_vc++;
				}
			if (m_toff + m_tc * 3 + 2 < I)
				for (int k = 0; k < 3; ++k)
					mtris[m_toff + m_tc * 3 + k] = (unsigned char)s.used[v3[k]];
			else
				atomicOr(b.error, 4u);
			m_tc++;
			// the emitted triangle leaves its vertices' lists (swap with the last)
			for (int k = 0; k < 3; ++k)
			{
				const unsigned int v = v3[k];
				unsigned int* list = s.adj + s.off[v];
				const unsigned int n = s.cnt[v];
				for (unsigned int i = 0; i < n; ++i)
					if (list[i] == best)
					{
						list[i] = list[n - 1];
						s.cnt[v] = n - 1;
						break;
					}
			}
			s.emitted[best] = 1;
			offset += reset;
		}
		m_voff = __shfl_sync(0xffffffffu, m_voff, 0);
		m_toff = __shfl_sync(0xffffffffu, m_toff, 0);
		m_vc = __shfl_sync(0xffffffffu, m_vc, 0);
		m_tc = __shfl_sync(0xffffffffu, m_tc, 0);
		offset = __shfl_sync(0xffffffffu, offset, 0);
		reset = __shfl_sync(0xffffffffu, reset, 0);
		if (reset)
			acc = Cone{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
		const Cone& c = s.cones[best];
		acc.px += c.px;
		acc.py += c.py;
		acc.pz += c.pz;
		acc.nx += c.nx;
		acc.ny += c.ny;
		acc.nz += c.nz;
		__syncwarp();
	}
	if (lane == 0)
	{
		if (m_tc)
		{
			if (offset < out_rows)
			{
				out[offset * 4 + 0] = m_voff;
				out[offset * 4 + 1] = m_toff;
				out[offset * 4 + 2] = m_vc;
				out[offset * 4 + 3] = m_tc;
			}
			else
				atomicOr(b.error, 4u);
			offset++;
		}
		b.counts[g] = offset;
	}
}

// meshopt_optimizeMeshletLevel on every meshlet, as clusterize runs it (demo/clusterlod.h:292-300):
// one warp per meshlet row of the batch; a row past its group's meshlet count has nothing to do
__global__ void __launch_bounds__(kMaxWarpsPerBlock * 32) kOptimizeMeshlets(MeshletBatch b, unsigned long long rows)
{
	__shared__ MeshletOpt opt[kMaxWarpsPerBlock];
	const unsigned long long r = (unsigned long long)blockIdx.x * kMaxWarpsPerBlock + (threadIdx.x >> 5);
	if (r >= rows)
		return;
	// the group whose rows hold r: the last g with meshlet_base[g] <= r
	unsigned int lo = 0, hi = b.groups;
	while (hi - lo > 1)
	{
		unsigned int mid = (lo + hi) / 2;
		if (b.meshlet_base[mid] <= r)
			lo = mid;
		else
			hi = mid;
	}
	const unsigned int g = lo;
	const unsigned long long k = r - b.meshlet_base[g];
	if (k >= b.counts[g])
		return;
	const unsigned long long i0 = b.offsets[g];
	const unsigned int I = unsigned(b.offsets[g + 1] - i0) / 3 * 3;
	const unsigned int* row = b.meshlets + r * 4;
	const unsigned int vo = row[0], to = row[1], vc = row[2], tc = row[3];
	if (vc <= 256 && tc <= 512 && vo + vc <= I && to + tc * 3 <= I)
		optimizeMeshletWarp(b.mverts + i0 + vo, b.mtris + i0 + to, vc, tc, b.optimize_level, opt[threadIdx.x >> 5]);
}

} // namespace

size_t meshletBound(size_t index_count, size_t max_vertices, size_t max_triangles)
{
	size_t conservative = max_vertices - 2;
	size_t by_vertices = (index_count + conservative - 1) / conservative;
	size_t by_triangles = (index_count / 3 + max_triangles - 1) / max_triangles;
	return by_vertices > by_triangles ? by_vertices : by_triangles;
}

size_t meshletScratchBytes(size_t index_count)
{
	Scratch s;
	return align256(carve(s, nullptr, unsigned(index_count / 3 * 3)));
}

void buildMeshletsBatch(const MeshletBatch& b, cudaStream_t stream)
{
	if (!b.groups)
		return;
	// with a shared pool, one warp per block (the pool sets how many fit on an SM); without, four
	const unsigned int warps = b.pool_bytes ? 1 : kMaxWarpsPerBlock;
	const unsigned int blocks = (b.groups + warps - 1) / warps;
	MO_LAUNCH(kMeshletsFlex, blocks, warps * 32, warps * b.pool_bytes, stream, b);
	if (b.optimize_level >= 0 && b.rows)
		MO_LAUNCH(kOptimizeMeshlets, unsigned((b.rows + kMaxWarpsPerBlock - 1) / kMaxWarpsPerBlock), kMaxWarpsPerBlock * 32, 0, stream, b, b.rows);
	MO_CUDA_CHECK(cudaGetLastError());
}

} // namespace mogpu
