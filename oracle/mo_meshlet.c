/* mo_meshlet.c - CPU restatement of meshopt_buildMeshletsFlex (src/clusterizer.cpp:1035-1224),
 * the re-clusterization step of a cluster-LOD level (demo/clusterlod.h:266-296).
 *
 * Test infrastructure only: the parity tests and the benchmark's CPU-baseline leg call it; the
 * library never does. Compiled with -ffp-contract=off, like the reference build it is checked
 * against (oracle/_ref/libclod_ref.so, which holds the reference's own clusterizer.cpp).
 *
 * It is written the way the GPU kernel works, so that the golden vectors pin that design too:
 *  - vertices are numbered densely in first-use order (group-local ids); the reference keys its
 *    per-vertex arrays by the caller's vertex index, and nothing in its result depends on the
 *    numbering, only on identity and on the order vertices enter a meshlet;
 *  - each vertex's triangle list holds its triangles in face order, as both reference adjacency
 *    builders leave them (:40-86, :88-152), and emitted triangles leave it by swap-with-last;
 *  - the kd-tree nearest search runs on an explicit stack in the reference's recursion order.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mo_oracle.h"

#define MO_MAX_SEEDS 256  /* kMeshletMaxSeeds, :27 */
#define MO_ADD_SEEDS 4    /* kMeshletAddSeeds, :28 */
#define MO_MAX_DEPTH 50   /* kMeshletMaxTreeDepth, :31 */
#define MO_LEAF_SIZE 8    /* :1090 */

typedef struct
{
	float px, py, pz, nx, ny, nz;
} MoCone;

/* kd-tree node (:473-485): split or point index; axis 3 marks a leaf, whose `children` counts
 * its points (stored in it and the nodes after it); a branch's right subtree starts children + 1
 * nodes after it */
typedef struct
{
	union
	{
		float split;
		unsigned int index;
	} u;
	unsigned int axis;
	unsigned int children;
} MoNode;

typedef struct
{
	unsigned int vertex_offset, triangle_offset, vertex_count, triangle_count;
} MoMeshlet;

size_t mo_buildMeshletsBound(size_t index_count, size_t max_vertices, size_t max_triangles)
{
	/* :1017-1033 */
	size_t conservative = max_vertices - 2;
	size_t by_vertices = (index_count + conservative - 1) / conservative;
	size_t by_triangles = (index_count / 3 + max_triangles - 1) / max_triangles;
	return by_vertices > by_triangles ? by_vertices : by_triangles;
}

/* getMeshletScore, :173-179 */
static float meshletScore(float distance, float spread, float cone_weight, float expected_radius)
{
	float cone = 1.f - spread * cone_weight;
	float clamped = cone < 1e-3f ? 1e-3f : cone;
	return (1 + distance / expected_radius * (1 - cone_weight)) * clamped;
}

/* getMeshletCone, :181-199 */
static MoCone meshletCone(const MoCone* acc, unsigned int triangle_count)
{
	MoCone r = *acc;
	float center_scale = triangle_count == 0 ? 0.f : 1.f / (float)triangle_count;
	r.px *= center_scale;
	r.py *= center_scale;
	r.pz *= center_scale;
	float len = r.nx * r.nx + r.ny * r.ny + r.nz * r.nz;
	float axis_scale = len == 0.f ? 0.f : 1.f / sqrtf(len);
	r.nx *= axis_scale;
	r.ny *= axis_scale;
	r.nz *= axis_scale;
	return r;
}

/* kdtreePartition, :487-506: swap every element to the boundary, advance it for those below */
static size_t kdPartition(unsigned int* idx, size_t count, const MoCone* pts, int axis, float pivot)
{
	size_t m = 0;
	for (size_t i = 0; i < count; ++i)
	{
		const float* p = &pts[idx[i]].px;
		float v = p[axis];
		unsigned int t = idx[m];
		idx[m] = idx[i];
		idx[i] = t;
		m += v < pivot;
	}
	return m;
}

/* kdtreeBuildLeaf, :508-530 */
static size_t kdLeaf(size_t offset, MoNode* nodes, const unsigned int* idx, size_t count)
{
	nodes[offset].u.index = idx[0];
	nodes[offset].axis = 3;
	nodes[offset].children = (unsigned int)count;
	for (size_t i = 1; i < count; ++i)
	{
		nodes[offset + i].u.index = idx[i];
		nodes[offset + i].axis = 3;
		nodes[offset + i].children = ~0u >> 2;
	}
	return offset + count;
}

/* kdtreeBuild, :532-581 (recursion depth <= MO_MAX_DEPTH + 1) */
static size_t kdBuild(size_t offset, MoNode* nodes, const MoCone* pts, unsigned int* idx, size_t count, int depth)
{
	if (count <= MO_LEAF_SIZE)
		return kdLeaf(offset, nodes, idx, count);
	float mean[3] = {0, 0, 0}, vars[3] = {0, 0, 0};
	float runc = 1, runs = 1;
	/* Welford, in point order */
	for (size_t i = 0; i < count; ++i, runc += 1.f, runs = 1.f / runc)
	{
		const float* p = &pts[idx[i]].px;
		for (int k = 0; k < 3; ++k)
		{
			float delta = p[k] - mean[k];
			mean[k] += delta * runs;
			vars[k] += delta * (p[k] - mean[k]);
		}
	}
	int axis = (vars[0] >= vars[1] && vars[0] >= vars[2]) ? 0 : (vars[1] >= vars[2] ? 1 : 2);
	float split = mean[axis];
	size_t middle = kdPartition(idx, count, pts, axis, split);
	if (middle <= MO_LEAF_SIZE / 2 || middle >= count - MO_LEAF_SIZE / 2 || depth >= MO_MAX_DEPTH)
		return kdLeaf(offset, nodes, idx, count);
	nodes[offset].u.split = split;
	nodes[offset].axis = (unsigned int)axis;
	size_t next = kdBuild(offset + 1, nodes, pts, idx, middle, depth + 1);
	nodes[offset].children = (unsigned int)(next - offset - 1);
	return kdBuild(next, nodes, pts, idx + middle, count - middle, depth + 1);
}

/* kdtreeNearest, :583-639, on an explicit stack: a branch pushes "the second child, if the
 * distance to the split is within the limit then" below its first child, which is the order the
 * recursion visits them in; emptied leaves and branches are switched off on the way */
typedef struct
{
	unsigned int node;
	unsigned int second; /* 1: a deferred second child, visited if dist <= limit */
	float dist;
} MoFrame;

static void kdNearest(MoNode* nodes, const MoCone* pts, const unsigned char* emitted, const float* pos, unsigned int* result, float* limit)
{
	MoFrame stack[2 * MO_MAX_DEPTH + 8];
	int top = 0;
	stack[top].node = 0;
	stack[top].second = 0;
	stack[top].dist = 0.f;
	top++;
	while (top > 0)
	{
		MoFrame f = stack[--top];
		if (f.second && !(f.dist <= *limit))
			continue;
		unsigned int root = f.node;
		MoNode* node = &nodes[root];
		if (node->children == 0)
			continue;
		if (node->axis == 3)
		{
			int inactive = 1;
			for (unsigned int i = 0; i < node->children; ++i)
			{
				unsigned int index = nodes[root + i].u.index;
				if (emitted[index])
					continue;
				inactive = 0;
				const float* p = &pts[index].px;
				float dx = p[0] - pos[0], dy = p[1] - pos[1], dz = p[2] - pos[2];
				float d = sqrtf(dx * dx + dy * dy + dz * dz);
				if (d < *limit)
				{
					*result = index;
					*limit = d;
				}
			}
			if (inactive)
				node->children = 0;
		}
		else
		{
			float delta = pos[node->axis] - node->u.split;
			unsigned int first = (delta <= 0) ? 0 : node->children;
			unsigned int second = first ^ node->children;
			if ((nodes[root + 1 + first].children | nodes[root + 1 + second].children) == 0)
				node->children = 0;
			stack[top].node = root + 1 + second;
			stack[top].second = 1;
			stack[top].dist = fabsf(delta);
			top++;
			stack[top].node = root + 1 + first;
			stack[top].second = 0;
			stack[top].dist = 0.f;
			top++;
		}
	}
}

static int cmpU64(const void* a, const void* b)
{
	unsigned long long x = *(const unsigned long long*)a, y = *(const unsigned long long*)b;
	return x < y ? -1 : (x > y ? 1 : 0);
}

typedef struct
{
	unsigned int* counts;  /* live triangles per local vertex (the list length) */
	unsigned int* offsets;
	unsigned int* data;
} MoAdj;

/* appendMeshlet, :243-300 (without the index-span limit, which the reference builds without) */
static int appendMeshlet(MoMeshlet* m, unsigned int a, unsigned int b, unsigned int c, short* used, MoMeshlet* out,
    unsigned int* mverts, unsigned char* mtris, size_t offset, size_t max_vertices, size_t max_triangles, int split)
{
	int extra = (used[a] < 0) + (used[b] < 0) + (used[c] < 0);
	int result = 0;
	if (m->vertex_count + extra > max_vertices || m->triangle_count >= max_triangles || split)
	{
		out[offset] = *m;
		for (unsigned int j = 0; j < m->vertex_count; ++j)
			used[mverts[m->vertex_offset + j]] = -1;
		m->vertex_offset += m->vertex_count;
		m->triangle_offset += m->triangle_count * 3;
		m->vertex_count = 0;
		m->triangle_count = 0;
		result = 1;
	}
	unsigned int v[3] = {a, b, c};
	for (int k = 0; k < 3; ++k)
		if (used[v[k]] < 0)
		{
			used[v[k]] = (short)m->vertex_count;
			mverts[m->vertex_offset + m->vertex_count++] = v[k];
		}
	for (int k = 0; k < 3; ++k)
		mtris[m->triangle_offset + m->triangle_count * 3 + k] = (unsigned char)used[v[k]];
	m->triangle_count++;
	return result;
}

/* getNeighborTriangle, :302-362: the first triangle, in the order of the meshlet's vertices and
 * their lists, with the smallest (topology priority, score) */
static unsigned int neighborTriangle(const MoMeshlet* m, const MoCone* mc, const unsigned int* mverts, const unsigned int* lidx, const MoAdj* adj,
    const MoCone* cones, const short* used, float radius, float cone_weight)
{
	unsigned int best = ~0u;
	int best_priority = 5;
	float best_score = FLT_MAX;
	const unsigned int* live = adj->counts;
	for (unsigned int i = 0; i < m->vertex_count; ++i)
	{
		unsigned int v = mverts[m->vertex_offset + i];
		const unsigned int* list = adj->data + adj->offsets[v];
		for (unsigned int j = 0; j < adj->counts[v]; ++j)
		{
			unsigned int t = list[j];
			unsigned int a = lidx[t * 3 + 0], b = lidx[t * 3 + 1], c = lidx[t * 3 + 2];
			int extra = (used[a] < 0) + (used[b] < 0) + (used[c] < 0);
			int priority;
			if (extra == 0)
				priority = 0;
			else if (live[a] == 1 || live[b] == 1 || live[c] == 1)
				priority = 1;
			else if ((live[a] == 2) + (live[b] == 2) + (live[c] == 2) >= 2)
				priority = 1 + extra;
			else
				priority = 2 + extra;
			if (priority > best_priority)
				continue;
			const MoCone* tc = &cones[t];
			float dx = tc->px - mc->px, dy = tc->py - mc->py, dz = tc->pz - mc->pz;
			float distance = sqrtf(dx * dx + dy * dy + dz * dz);
			float spread = tc->nx * mc->nx + tc->ny * mc->ny + tc->nz * mc->nz;
			float score = meshletScore(distance, spread, cone_weight, radius);
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

/* appendSeedTriangles, :364-430 */
static size_t appendSeeds(unsigned int* seeds, const MoMeshlet* m, const unsigned int* mverts, const unsigned int* lidx, const MoAdj* adj,
    const MoCone* cones, float cx, float cy, float cz)
{
	unsigned int best_seeds[MO_ADD_SEEDS], best_live[MO_ADD_SEEDS];
	float best_score[MO_ADD_SEEDS];
	const unsigned int* live = adj->counts;
	for (int i = 0; i < MO_ADD_SEEDS; ++i)
	{
		best_seeds[i] = ~0u;
		best_live[i] = ~0u;
		best_score[i] = FLT_MAX;
	}
	for (unsigned int i = 0; i < m->vertex_count; ++i)
	{
		unsigned int v = mverts[m->vertex_offset + i];
		unsigned int bn = ~0u, bn_live = ~0u;
		const unsigned int* list = adj->data + adj->offsets[v];
		for (unsigned int j = 0; j < adj->counts[v]; ++j)
		{
			unsigned int t = list[j];
			unsigned int l = live[lidx[t * 3 + 0]] + live[lidx[t * 3 + 1]] + live[lidx[t * 3 + 2]];
			if (l < bn_live)
			{
				bn = t;
				bn_live = l;
			}
		}
		if (bn == ~0u)
			continue;
		float dx = cones[bn].px - cx, dy = cones[bn].py - cy, dz = cones[bn].pz - cz;
		float score = sqrtf(dx * dx + dy * dy + dz * dz);
		for (int j = 0; j < MO_ADD_SEEDS; ++j)
			if (bn_live < best_live[j] || (bn_live == best_live[j] && score <= best_score[j]))
			{
				best_seeds[j] = bn;
				best_live[j] = bn_live;
				best_score[j] = score;
				break;
			}
	}
	size_t n = 0;
	for (int i = 0; i < MO_ADD_SEEDS; ++i)
		if (best_seeds[i] != ~0u)
			seeds[n++] = best_seeds[i];
	return n;
}

/* pruneSeedTriangles, :432-445 */
static size_t pruneSeeds(unsigned int* seeds, size_t count, const unsigned char* emitted)
{
	size_t r = 0;
	for (size_t i = 0; i < count; ++i)
	{
		unsigned int s = seeds[i];
		seeds[r] = s;
		r += emitted[s] == 0;
	}
	return r;
}

/* selectSeedTriangle, :447-471 */
static unsigned int selectSeed(const unsigned int* seeds, size_t count, const unsigned int* lidx, const unsigned int* live, const MoCone* cones, float cx,
    float cy, float cz)
{
	unsigned int best = ~0u, best_live = ~0u;
	float best_score = FLT_MAX;
	for (size_t i = 0; i < count; ++i)
	{
		unsigned int s = seeds[i];
		unsigned int l = live[lidx[s * 3 + 0]] + live[lidx[s * 3 + 1]] + live[lidx[s * 3 + 2]];
		float dx = cones[s].px - cx, dy = cones[s].py - cy, dz = cones[s].pz - cz;
		float score = sqrtf(dx * dx + dy * dy + dz * dz);
		if (l < best_live || (l == best_live && score < best_score))
		{
			best = s;
			best_live = l;
			best_score = score;
		}
	}
	return best;
}

size_t mo_buildMeshletsFlex(unsigned int* meshlets, unsigned int* meshlet_vertices, unsigned char* meshlet_triangles, const unsigned int* indices,
    size_t index_count, const float* vertex_positions, size_t vertex_count, size_t vertex_positions_stride, size_t max_vertices, size_t min_triangles,
    size_t max_triangles, float cone_weight, float split_factor)
{
	(void)vertex_count;
	if (index_count == 0)
		return 0;
	const size_t F = index_count / 3, stride = vertex_positions_stride / sizeof(float);
	MoMeshlet* out = (MoMeshlet*)meshlets;

	/* group-local vertex ids in first-use order, through a sorted copy of (vertex, position) */
	unsigned int* lidx = (unsigned int*)malloc(index_count * sizeof(unsigned int));
	unsigned int* global = (unsigned int*)malloc(index_count * sizeof(unsigned int)); /* local id -> caller's index */
	unsigned int U = 0;
	{
		unsigned long long* key = (unsigned long long*)malloc(index_count * sizeof(unsigned long long));
		for (size_t i = 0; i < index_count; ++i)
			key[i] = ((unsigned long long)indices[i] << 32) | (unsigned long long)i;
		/* sorted by (vertex, position): each run's first entry is the vertex's first use */
		unsigned int* first = (unsigned int*)malloc(index_count * sizeof(unsigned int));
		qsort(key, index_count, sizeof(unsigned long long), cmpU64);
		for (size_t i = 0; i < index_count; ++i)
		{
			size_t j = i;
			unsigned int v = (unsigned int)(key[i] >> 32);
			unsigned int pos0 = (unsigned int)key[i];
			while (j < index_count && (unsigned int)(key[j] >> 32) == v)
				++j;
			for (size_t q = i; q < j; ++q)
				first[(unsigned int)key[q]] = pos0;
			i = j - 1;
		}
		/* number first uses in index order */
		unsigned int* id_at_first = (unsigned int*)malloc(index_count * sizeof(unsigned int));
		for (size_t i = 0; i < index_count; ++i)
			if (first[i] == (unsigned int)i)
			{
				id_at_first[i] = U;
				global[U] = indices[i];
				U++;
			}
		for (size_t i = 0; i < index_count; ++i)
			lidx[i] = id_at_first[first[i]];
		free(id_at_first);
		free(first);
		free(key);
	}

	/* triangle lists per local vertex, in face order */
	MoAdj adj;
	adj.counts = (unsigned int*)calloc(U, sizeof(unsigned int));
	adj.offsets = (unsigned int*)malloc(U * sizeof(unsigned int));
	adj.data = (unsigned int*)malloc(index_count * sizeof(unsigned int));
	for (size_t i = 0; i < index_count; ++i)
		adj.counts[lidx[i]]++;
	{
		unsigned int off = 0;
		for (unsigned int v = 0; v < U; ++v)
		{
			adj.offsets[v] = off;
			off += adj.counts[v];
		}
		unsigned int* fill = (unsigned int*)calloc(U, sizeof(unsigned int));
		for (size_t t = 0; t < F; ++t)
			for (int k = 0; k < 3; ++k)
			{
				unsigned int v = lidx[t * 3 + k];
				adj.data[adj.offsets[v] + fill[v]++] = (unsigned int)t;
			}
		free(fill);
	}

	unsigned char* emitted = (unsigned char*)calloc(F, 1);

	/* computeTriangleCones, :201-241; the mesh area sums in face order */
	MoCone* cones = (MoCone*)malloc(F * sizeof(MoCone));
	float mesh_area = 0;
	for (size_t t = 0; t < F; ++t)
	{
		const float* p0 = vertex_positions + stride * indices[t * 3 + 0];
		const float* p1 = vertex_positions + stride * indices[t * 3 + 1];
		const float* p2 = vertex_positions + stride * indices[t * 3 + 2];
		float p10[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
		float p20[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
		float nx = p10[1] * p20[2] - p10[2] * p20[1];
		float ny = p10[2] * p20[0] - p10[0] * p20[2];
		float nz = p10[0] * p20[1] - p10[1] * p20[0];
		float area = sqrtf(nx * nx + ny * ny + nz * nz);
		float inv = (area == 0.f) ? 0.f : 1.f / area;
		cones[t].px = (p0[0] + p1[0] + p2[0]) / 3.f;
		cones[t].py = (p0[1] + p1[1] + p2[1]) / 3.f;
		cones[t].pz = (p0[2] + p1[2] + p2[2]) / 3.f;
		cones[t].nx = nx * inv;
		cones[t].ny = ny * inv;
		cones[t].nz = nz * inv;
		mesh_area += area;
	}
	float tri_area_avg = mesh_area / (float)F * 0.5f;
	float radius = sqrtf(tri_area_avg * (float)max_triangles) * 0.5f;

	unsigned int* kdidx = (unsigned int*)malloc(F * sizeof(unsigned int));
	for (size_t t = 0; t < F; ++t)
		kdidx[t] = (unsigned int)t;
	MoNode* nodes = (MoNode*)malloc(F * 2 * sizeof(MoNode));
	kdBuild(0, nodes, cones, kdidx, F, 0);

	float cx = FLT_MAX, cy = FLT_MAX, cz = FLT_MAX;
	for (size_t t = 0; t < F; ++t)
	{
		cx = cx > cones[t].px ? cones[t].px : cx;
		cy = cy > cones[t].py ? cones[t].py : cy;
		cz = cz > cones[t].pz ? cones[t].pz : cz;
	}

	short* used = (short*)malloc(U * sizeof(short));
	for (unsigned int v = 0; v < U; ++v)
		used[v] = -1;

	unsigned int initial = ~0u;
	float initial_score = FLT_MAX;
	for (size_t t = 0; t < F; ++t)
	{
		float dx = cones[t].px - cx, dy = cones[t].py - cy, dz = cones[t].pz - cz;
		float s = sqrtf(dx * dx + dy * dy + dz * dz);
		if (initial == ~0u || s < initial_score)
		{
			initial = (unsigned int)t;
			initial_score = s;
		}
	}

	unsigned int seeds[MO_MAX_SEEDS];
	size_t seed_count = 0;
	MoMeshlet m = {0, 0, 0, 0};
	size_t offset = 0;
	MoCone acc = {0, 0, 0, 0, 0, 0};
	/* meshlet_vertices hold local ids while building, caller's indices at the end */
	for (;;)
	{
		MoCone mc = meshletCone(&acc, m.triangle_count);
		unsigned int best;
		if (offset == 0 && m.triangle_count == 0)
			best = initial;
		else
			best = neighborTriangle(&m, &mc, meshlet_vertices, lidx, &adj, cones, used, radius, cone_weight);
		int split = 0;
		if (best == ~0u)
		{
			float pos[3] = {mc.px, mc.py, mc.pz};
			unsigned int index = ~0u;
			float distance = FLT_MAX;
			kdNearest(nodes, cones, emitted, pos, &index, &distance);
			best = index;
			split = m.triangle_count >= min_triangles && split_factor > 0 && distance > radius * split_factor;
		}
		if (best == ~0u)
			break;
		int best_extra = (used[lidx[best * 3 + 0]] < 0) + (used[lidx[best * 3 + 1]] < 0) + (used[lidx[best * 3 + 2]] < 0);
		if (split || (m.vertex_count + best_extra > max_vertices || m.triangle_count >= max_triangles))
		{
			seed_count = pruneSeeds(seeds, seed_count, emitted);
			seed_count = (seed_count + MO_ADD_SEEDS <= MO_MAX_SEEDS) ? seed_count : MO_MAX_SEEDS - MO_ADD_SEEDS;
			seed_count += appendSeeds(seeds + seed_count, &m, meshlet_vertices, lidx, &adj, cones, cx, cy, cz);
			unsigned int s = selectSeed(seeds, seed_count, lidx, adj.counts, cones, cx, cy, cz);
			best = s != ~0u ? s : best;
		}
		unsigned int a = lidx[best * 3 + 0], b = lidx[best * 3 + 1], c = lidx[best * 3 + 2];
		if (appendMeshlet(&m, a, b, c, used, out, meshlet_vertices, meshlet_triangles, offset, max_vertices, max_triangles, split))
		{
			offset++;
			memset(&acc, 0, sizeof(acc));
		}
		/* the emitted triangle leaves its vertices' lists (swap with the last) */
		for (int k = 0; k < 3; ++k)
		{
			unsigned int v = lidx[best * 3 + k];
			unsigned int* list = adj.data + adj.offsets[v];
			unsigned int n = adj.counts[v];
			for (unsigned int i = 0; i < n; ++i)
				if (list[i] == best)
				{
					list[i] = list[n - 1];
					adj.counts[v]--;
					break;
				}
		}
		acc.px += cones[best].px;
		acc.py += cones[best].py;
		acc.pz += cones[best].pz;
		acc.nx += cones[best].nx;
		acc.ny += cones[best].ny;
		acc.nz += cones[best].nz;
		emitted[best] = 1;
	}
	if (m.triangle_count)
		out[offset++] = m;

	/* local ids -> the caller's vertex indices */
	if (offset)
	{
		const MoMeshlet* last = &out[offset - 1];
		for (unsigned int i = 0; i < last->vertex_offset + last->vertex_count; ++i)
			meshlet_vertices[i] = global[meshlet_vertices[i]];
	}

	free(nodes);
	free(kdidx);
	free(used);
	free(cones);
	free(emitted);
	free(adj.data);
	free(adj.offsets);
	free(adj.counts);
	free(global);
	free(lidx);
	return offset;
}

/* meshopt_optimizeMeshletLevel (src/meshletutils.cpp:366-554): triangles reordered for vertex
 * reuse (a greedy pick over the remaining triangles with 8-bit cache timestamps and valences,
 * which wrap as the reference's unsigned char counters do), rotated for compressibility at
 * level >= 1, then vertices renumbered in first-use order. */
void mo_optimizeMeshletLevel(unsigned int* meshlet_vertices, size_t vertex_count, unsigned char* meshlet_triangles, size_t triangle_count, int level)
{
	unsigned char* idx = meshlet_triangles;
	unsigned char cache[256], valence[256];
	memset(cache, 0, vertex_count);
	memset(valence, 0, vertex_count);
	unsigned char cache_last = 128;
	const unsigned char cutoff = 3;
	for (size_t i = 0; i < triangle_count * 3; ++i)
		valence[idx[i]]++;
	for (size_t i = 0; i < triangle_count; ++i)
	{
		int next = -1, next_score = -1, edges = 0;
		for (size_t j = i; j < triangle_count; ++j)
		{
			unsigned char a = idx[j * 3 + 0], b = idx[j * 3 + 1], c = idx[j * 3 + 2];
			unsigned char ad = (unsigned char)(cache_last - cache[a]);
			unsigned char bd = (unsigned char)(cache_last - cache[b]);
			unsigned char cd = (unsigned char)(cache_last - cache[c]);
			int match = (ad < cutoff) + (bd < cutoff) + (cd < cutoff);
			int score;
			if (level)
			{
				int vmin = valence[a] < valence[b] ? valence[a] : valence[b];
				vmin = valence[c] < vmin ? valence[c] : vmin;
				score = (match * 1024 + (1023 - ad - bd - cd)) * 256 + (255 - vmin);
			}
			else
				score = match;
			if (score > next_score)
			{
				next = (int)j;
				next_score = score;
			}
			if (level ? (match >= 2 && ++edges >= level) : (match >= 2))
				break;
		}
		unsigned char a = idx[next * 3 + 0], b = idx[next * 3 + 1], c = idx[next * 3 + 2];
		memmove(idx + (i + 1) * 3, idx + i * 3, (size_t)(next - (int)i) * 3);
		idx[i * 3 + 0] = a;
		idx[i * 3 + 1] = b;
		idx[i * 3 + 2] = c;
		cache_last++;
		cache[a] = cache[b] = cache[c] = cache_last;
		valence[a]--;
		valence[b]--;
		valence[c]--;
	}
	if (level >= 1)
	{
		memset(cache, 0, vertex_count);
		for (size_t i = 0; i < triangle_count; ++i)
		{
			unsigned char a = idx[i * 3 + 0], b = idx[i * 3 + 1], c = idx[i * 3 + 2];
			if (!cache[a] && cache[b] && !cache[c])
			{
				unsigned char t = a;
				a = b, b = c, c = t;
			}
			else if (!cache[a] && !cache[b] && !cache[c])
			{
				int ab = 0, bc = 0, ca = 0;
				for (size_t j = i + 1; j < triangle_count && j <= i + cutoff; ++j)
				{
					unsigned char oa = idx[j * 3 + 0], ob = idx[j * 3 + 1], oc = idx[j * 3 + 2];
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
			idx[i * 3 + 0] = a, idx[i * 3 + 1] = b, idx[i * 3 + 2] = c;
			cache[a] = cache[b] = cache[c] = 1;
		}
	}
	unsigned int order[256];
	short remap[256];
	for (size_t v = 0; v < vertex_count; ++v)
		remap[v] = -1;
	size_t n = 0;
	for (size_t i = 0; i < triangle_count * 3; ++i)
	{
		short* r = &remap[idx[i]];
		if (*r < 0)
		{
			*r = (short)n;
			order[n++] = meshlet_vertices[idx[i]];
		}
		idx[i] = (unsigned char)*r;
	}
	memcpy(meshlet_vertices, order, n * sizeof(unsigned int));
}

/* the clusterize step's per-meshlet pass (demo/clusterlod.h:292-300) over a build's output */
void mo_optimizeMeshlets(const unsigned int* meshlets, size_t meshlet_count, unsigned int* meshlet_vertices, unsigned char* meshlet_triangles, int level)
{
	for (size_t i = 0; i < meshlet_count; ++i)
	{
		const unsigned int* m = meshlets + i * 4;
		mo_optimizeMeshletLevel(meshlet_vertices + m[0], m[2], meshlet_triangles + m[1], m[3], level);
	}
}
