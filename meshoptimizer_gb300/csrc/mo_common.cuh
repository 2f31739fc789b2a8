// mo_common.cuh - shared device types and FP32 quadric arithmetic for the GB300 simplifier.
//
// Every floating-point expression here keeps the operation order of meshoptimizer's
// src/simplifier.cpp so that results are bit-identical to the reference CPU code. The
// library is compiled with --fmad=false (no a*b+c contraction) and IEEE division and
// square root (nvcc's defaults without fast-math); both are required for that.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>

namespace mogpu
{

// vertex kinds, src/simplifier.cpp:296-305
enum : unsigned char
{
	kManifold = 0,
	kBorder = 1,
	kSeam = 2,
	kComplex = 3,
	kLocked = 4,
};

// option bits, meshoptimizer.h:466-482
enum : unsigned int
{
	kOptLockBorder = 1u << 0,
	kOptSparse = 1u << 1,
	kOptErrorAbsolute = 1u << 2,
	kOptPrune = 1u << 3,
	kOptRegularize = 1u << 4,
	kOptPermissive = 1u << 5,
	kOptRegularizeLight = 1u << 6,
	kOptInternalSolve = 1u << 29, // meshopt_simplifyWithUpdate's mode (src/simplifier.cpp:2340)
	kOptInternalDebug = 1u << 30,
};

// vertex_lock flags, meshoptimizer.h:488-495
enum : unsigned char
{
	kVertexLock = 1,
	kVertexProtect = 2,
	kVertexPriority = 4,
};

// collapse decision states
enum : unsigned char
{
	kUndecided = 0,
	kCommit = 1,
	kSkipLocked = 2,
	kSkipFlip = 3,
};

// Collapse rule tables (src/simplifier.cpp:311-331), packed as 5-bit row masks:
// bit j of row i is table[i][j].
__host__ __device__ __forceinline__ bool canCollapse(unsigned k0, unsigned k1)
{
	// rows: {11111, 10010, 10100, 11000, 00000} with bit j = column j
	const unsigned rows = (0x1Fu) | (0x12u << 5) | (0x14u << 10) | (0x18u << 15) | (0x00u << 20);
	return (rows >> (k0 * 5 + k1)) & 1;
}

__host__ __device__ __forceinline__ bool hasOpposite(unsigned k0, unsigned k1)
{
	// rows: {1,1,1,1,1}, {1,0,1,0,0}, {1,1,1,0,1}, {1,0,0,0,0}, {1,0,1,0,0}
	const unsigned rows = (0x1Fu) | (0x05u << 5) | (0x17u << 10) | (0x01u << 15) | (0x05u << 20);
	return (rows >> (k0 * 5 + k1)) & 1;
}

struct Quadric
{
	float a00, a11, a22;
	float a10, a20, a21;
	float b0, b1, b2, c;
	float w;
	float pad;
};

static_assert(sizeof(Quadric) == 48, "Quadric is padded to three float4");

struct V3
{
	float x, y, z;
};

__device__ __forceinline__ V3 ldpos(const float4* pos, unsigned int i)
{
	float4 p = __ldg(pos + i);
	return V3{p.x, p.y, p.z};
}

__device__ __forceinline__ Quadric ldquadric(const Quadric* q, unsigned int i)
{
	const float4* p = reinterpret_cast<const float4*>(q + i);
	float4 a = p[0], b = p[1], c = p[2];
	return Quadric{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, 0.f};
}

__device__ __forceinline__ void stquadric(Quadric* q, unsigned int i, const Quadric& Q)
{
	float4* p = reinterpret_cast<float4*>(q + i);
	p[0] = make_float4(Q.a00, Q.a11, Q.a22, Q.a10);
	p[1] = make_float4(Q.a20, Q.a21, Q.b0, Q.b1);
	p[2] = make_float4(Q.b2, Q.c, Q.w, 0.f);
}

__device__ __forceinline__ Quadric qzero()
{
	return Quadric{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
}

// quadricAdd, :716-729
__device__ __forceinline__ void qadd(Quadric& Q, const Quadric& R)
{
	Q.a00 += R.a00;
	Q.a11 += R.a11;
	Q.a22 += R.a22;
	Q.a10 += R.a10;
	Q.a20 += R.a20;
	Q.a21 += R.a21;
	Q.b0 += R.b0;
	Q.b1 += R.b1;
	Q.b2 += R.b2;
	Q.c += R.c;
	Q.w += R.w;
}

// normalize, :702-714
__device__ __forceinline__ float vnormalize(V3& v)
{
	float length = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
	if (length > 0)
	{
		v.x /= length;
		v.y /= length;
		v.z /= length;
	}
	return length;
}

// quadricEval, :751-773
__device__ __forceinline__ float qeval(const Quadric& Q, const V3& v)
{
	float rx = Q.b0, ry = Q.b1, rz = Q.b2;
	rx += Q.a10 * v.y;
	ry += Q.a21 * v.z;
	rz += Q.a20 * v.x;
	rx *= 2;
	ry *= 2;
	rz *= 2;
	rx += Q.a00 * v.x;
	ry += Q.a11 * v.y;
	rz += Q.a22 * v.z;
	float r = Q.c;
	r += rx * v.x;
	r += ry * v.y;
	r += rz * v.z;
	return r;
}

// quadricError (position), :775-781
__device__ __forceinline__ float qerror(const Quadric& Q, const V3& v)
{
	float r = qeval(Q, v);
	float s = Q.w == 0.f ? 0.f : 1.f / Q.w;
	return fabsf(r) * s;
}

// quadricFromPlane, :800-818
__device__ __forceinline__ Quadric qplane(float a, float b, float c, float d, float w)
{
	float aw = a * w, bw = b * w, cw = c * w, dw = d * w;
	Quadric Q;
	Q.a00 = a * aw;
	Q.a11 = b * bw;
	Q.a22 = c * cw;
	Q.a10 = a * bw;
	Q.a20 = a * cw;
	Q.a21 = b * cw;
	Q.b0 = a * dw;
	Q.b1 = b * dw;
	Q.b2 = c * dw;
	Q.c = d * dw;
	Q.w = w;
	Q.pad = 0.f;
	return Q;
}

// quadricFromPoint, :820-829
__device__ __forceinline__ Quadric qpoint(float x, float y, float z, float w)
{
	Quadric Q;
	Q.a00 = Q.a11 = Q.a22 = w;
	Q.a10 = Q.a20 = Q.a21 = 0;
	Q.b0 = -x * w;
	Q.b1 = -y * w;
	Q.b2 = -z * w;
	Q.c = (x * x + y * y + z * z) * w;
	Q.w = w;
	Q.pad = 0.f;
	return Q;
}

// quadricFromTriangle, :831-845
__device__ __forceinline__ Quadric qtriangle(const V3& p0, const V3& p1, const V3& p2, float weight)
{
	V3 p10 = {p1.x - p0.x, p1.y - p0.y, p1.z - p0.z};
	V3 p20 = {p2.x - p0.x, p2.y - p0.y, p2.z - p0.z};
	V3 n = {p10.y * p20.z - p10.z * p20.y, p10.z * p20.x - p10.x * p20.z, p10.x * p20.y - p10.y * p20.x};
	float area = vnormalize(n);
	float distance = n.x * p0.x + n.y * p0.y + n.z * p0.z;
	return qplane(n.x, n.y, n.z, -distance, sqrtf(area) * weight);
}

// quadricFromTriangleEdge, :847-868
__device__ __forceinline__ Quadric qedge(const V3& p0, const V3& p1, const V3& p2, float weight)
{
	V3 p10 = {p1.x - p0.x, p1.y - p0.y, p1.z - p0.z};
	float lengthsq = p10.x * p10.x + p10.y * p10.y + p10.z * p10.z;
	float length = sqrtf(lengthsq);
	V3 p20 = {p2.x - p0.x, p2.y - p0.y, p2.z - p0.z};
	float p20p = p20.x * p10.x + p20.y * p10.y + p20.z * p10.z;
	V3 perp = {p20.x * lengthsq - p10.x * p20p, p20.y * lengthsq - p10.y * p20p, p20.z * lengthsq - p10.z * p20p};
	vnormalize(perp);
	float distance = perp.x * p0.x + perp.y * p0.y + perp.z * p0.z;
	return qplane(perp.x, perp.y, perp.z, -distance, length * weight);
}

// hasTriangleFlip, :1182-1199: does triangle ABC flip when C is replaced with D?
__device__ __forceinline__ bool triFlip(const V3& a, const V3& b, const V3& c, const V3& d)
{
	V3 eb = {b.x - a.x, b.y - a.y, b.z - a.z};
	V3 ec = {c.x - a.x, c.y - a.y, c.z - a.z};
	V3 ed = {d.x - a.x, d.y - a.y, d.z - a.z};
	V3 nbc = {eb.y * ec.z - eb.z * ec.y, eb.z * ec.x - eb.x * ec.z, eb.x * ec.y - eb.y * ec.x};
	V3 nbd = {eb.y * ed.z - eb.z * ed.y, eb.z * ed.x - eb.x * ed.z, eb.x * ed.y - eb.y * ed.x};
	float ndp = nbc.x * nbd.x + nbc.y * nbd.y + nbc.z * nbd.z;
	float abc = nbc.x * nbc.x + nbc.y * nbc.y + nbc.z * nbc.z;
	float abd = nbd.x * nbd.x + nbd.y * nbd.y + nbd.z * nbd.z;
	return ndp <= 0.25f * sqrtf(abc * abd);
}

// sortEdgeCollapses key, :1458-1471: 12 bits of exponent+mantissa, clamped to 2559
__device__ __forceinline__ unsigned int sortKey(unsigned int errorbits)
{
	unsigned int key = (errorbits << 1) >> 20;
	return key < 2560u ? key : 2559u;
}

// quadricFromAttributes :870-950 for one face, accumulated into Q/G of one vertex
template <int MAXA>
__device__ __forceinline__ void addAttributeQuadric(Quadric& Qacc, float4* Gacc, int count, const V3& p0, const V3& p1, const V3& p2,
    const float* __restrict__ va0, const float* __restrict__ va1, const float* __restrict__ va2)
{
	V3 p10 = {p1.x - p0.x, p1.y - p0.y, p1.z - p0.z};
	V3 p20 = {p2.x - p0.x, p2.y - p0.y, p2.z - p0.z};
	V3 nn = {p10.y * p20.z - p10.z * p20.y, p10.z * p20.x - p10.x * p20.z, p10.x * p20.y - p10.y * p20.x};
	float area = sqrtf(nn.x * nn.x + nn.y * nn.y + nn.z * nn.z) * 0.5f;
	float w = area;
	const V3& v0 = p10;
	const V3& v1 = p20;
	float d00 = v0.x * v0.x + v0.y * v0.y + v0.z * v0.z;
	float d01 = v0.x * v1.x + v0.y * v1.y + v0.z * v1.z;
	float d11 = v1.x * v1.x + v1.y * v1.y + v1.z * v1.z;
	float denom = d00 * d11 - d01 * d01;
	float denomr = denom == 0 ? 0.f : 1.f / denom;
	float gx1 = (d11 * v0.x - d01 * v1.x) * denomr;
	float gx2 = (d00 * v1.x - d01 * v0.x) * denomr;
	float gy1 = (d11 * v0.y - d01 * v1.y) * denomr;
	float gy2 = (d00 * v1.y - d01 * v0.y) * denomr;
	float gz1 = (d11 * v0.z - d01 * v1.z) * denomr;
	float gz2 = (d00 * v1.z - d01 * v0.z) * denomr;

	Quadric Q = qzero();
	Q.w = w;
#pragma unroll
	for (int k = 0; k < MAXA; ++k)
	{
		if (k >= count)
			break;
		float a0 = va0[k], a1 = va1[k], a2 = va2[k];
		float gx = gx1 * (a1 - a0) + gx2 * (a2 - a0);
		float gy = gy1 * (a1 - a0) + gy2 * (a2 - a0);
		float gz = gz1 * (a1 - a0) + gz2 * (a2 - a0);
		float gw = a0 - p0.x * gx - p0.y * gy - p0.z * gz;
		Q.a00 += w * (gx * gx);
		Q.a11 += w * (gy * gy);
		Q.a22 += w * (gz * gz);
		Q.a10 += w * (gy * gx);
		Q.a20 += w * (gz * gx);
		Q.a21 += w * (gz * gy);
		Q.b0 += w * (gx * gw);
		Q.b1 += w * (gy * gw);
		Q.b2 += w * (gz * gw);
		Q.c += w * (gw * gw);
		Gacc[k].x += w * gx;
		Gacc[k].y += w * gy;
		Gacc[k].z += w * gz;
		Gacc[k].w += w * gw;
	}
	qadd(Qacc, Q);
}

// one attribute's term of quadricError's attribute sum (src/simplifier.cpp:784-798), added to r in
// attribute order
__device__ __forceinline__ void qattrStep(float& r, float a, const float4& g4, const V3& v, float w)
{
	float g = v.x * g4.x + v.y * g4.y + v.z * g4.z + g4.w;
	r += a * (a * w - 2 * g);
}

// quadricError with attributes (src/simplifier.cpp:784-798): position error plus the attribute terms
__device__ __forceinline__ float qerrorAttr(const Quadric& Q, const float4* __restrict__ G, int count, const V3& v, const float* __restrict__ va)
{
	float r = qeval(Q, v);
	for (int k = 0; k < count; ++k)
		qattrStep(r, va[k], G[k], v, Q.w);
	return fabsf(r);
}

// ---- the update mode (meshopt_simplifyWithUpdate)

// quadricVolumeGradient, :952-965: gradient of the signed volume under a face
__device__ __forceinline__ float4 qvolumeGrad(const V3& p0, const V3& p1, const V3& p2)
{
	V3 p10 = {p1.x - p0.x, p1.y - p0.y, p1.z - p0.z};
	V3 p20 = {p2.x - p0.x, p2.y - p0.y, p2.z - p0.z};
	V3 n = {p10.y * p20.z - p10.z * p20.y, p10.z * p20.x - p10.x * p20.z, p10.x * p20.y - p10.y * p20.x};
	float area = vnormalize(n) * 0.5f;
	return make_float4(n.x * area, n.y * area, n.z * area, (-p0.x * n.x - p0.y * n.y - p0.z * n.z) * area);
}

__device__ __forceinline__ void gadd(float4& g, const float4& h)
{
	g.x += h.x;
	g.y += h.y;
	g.z += h.z;
	g.w += h.w;
}

// quadricSolve, :967-1022: LDL^T solve of the quadric's 3x3 system, augmented with the volume
// constraint GV as a Lagrange row; false when a pivot is too small
__device__ __forceinline__ bool qsolve(V3& p, const Quadric& Q, const float4& GV)
{
	float a00 = Q.a00, a11 = Q.a11, a22 = Q.a22;
	float a10 = Q.a10, a20 = Q.a20, a21 = Q.a21;
	float x0 = -Q.b0, x1 = -Q.b1, x2 = -Q.b2;
	float eps = 1e-6f * Q.w;

	float d0 = a00;
	float l10 = a10 / d0;
	float l20 = a20 / d0;
	float d1 = a11 - a10 * l10;
	float dl21 = a21 - a20 * l10;
	float l21 = dl21 / d1;
	float d2 = a22 - a20 * l20 - dl21 * l21;

	float y0 = x0;
	float y1 = x1 - l10 * y0;
	float y2 = x2 - l20 * y0 - l21 * y1;
	float z0 = y0 / d0;
	float z1 = y1 / d1;
	float z2 = y2 / d2;

	float a30 = GV.x, a31 = GV.y, a32 = GV.z;
	float x3 = -GV.w;
	float l30 = a30 / d0;
	float dl31 = a31 - a30 * l10;
	float l31 = dl31 / d1;
	float dl32 = a32 - a30 * l20 - dl31 * l21;
	float l32 = dl32 / d2;
	float d3 = 0.f - a30 * l30 - dl31 * l31 - dl32 * l32;
	float y3 = x3 - l30 * y0 - l31 * y1 - l32 * y2;
	float z3 = fabsf(d3) > eps ? y3 / d3 : 0.f;

	float lambda = z3;
	float pz = z2 - l32 * lambda;
	float py = z1 - l21 * pz - l31 * lambda;
	float px = z0 - l10 * py - l20 * pz - l30 * lambda;
	p = V3{px, py, pz};
	return fabsf(d0) > eps && fabsf(d1) > eps && fabsf(d2) > eps;
}

// quadricReduceAttributes, :1024-1050: one wedge's attribute quadric folded into the position
// system (its gradients enter as B B^T / a)
__device__ __forceinline__ void qreduceAttr(Quadric& Q, const Quadric& A, const float4* G, int count)
{
	Q.a00 += A.a00 * Q.w;
	Q.a11 += A.a11 * Q.w;
	Q.a22 += A.a22 * Q.w;
	Q.a10 += A.a10 * Q.w;
	Q.a20 += A.a20 * Q.w;
	Q.a21 += A.a21 * Q.w;
	Q.b0 += A.b0 * Q.w;
	Q.b1 += A.b1 * Q.w;
	Q.b2 += A.b2 * Q.w;
	float iaw = A.w == 0 ? 0.f : Q.w / A.w;
	for (int k = 0; k < count; ++k)
	{
		float4 g = G[k];
		Q.a00 -= (g.x * g.x) * iaw;
		Q.a11 -= (g.y * g.y) * iaw;
		Q.a22 -= (g.z * g.z) * iaw;
		Q.a10 -= (g.x * g.y) * iaw;
		Q.a20 -= (g.x * g.z) * iaw;
		Q.a21 -= (g.y * g.z) * iaw;
		Q.b0 -= (g.x * g.w) * iaw;
		Q.b1 -= (g.y * g.w) * iaw;
		Q.b2 -= (g.z * g.w) * iaw;
	}
}

// getComplexTarget, :1278-1290
__device__ __forceinline__ unsigned int complexTarget(unsigned int v, unsigned int target, const unsigned int* remap,
    const unsigned int* loop, const unsigned int* loopback)
{
	unsigned int r = remap[target];
	unsigned int lv = loop[v];
	if (lv != ~0u && remap[lv] == r)
		return lv;
	unsigned int lb = loopback[v];
	if (lb != ~0u && remap[lb] == r)
		return lb;
	return target;
}

// atomic max on non-negative float bit patterns; NaN values are ignored as the reference's
// "a < b ? b : a" update ignores them
__device__ __forceinline__ void atomicMaxNonNegFloat(unsigned int* addr, float v)
{
	if (!(v == v))
		return;
	atomicMax(addr, __float_as_uint(v));
}

} // namespace mogpu

#define MO_CUDA_CHECK(expr)                                                                             \
	do                                                                                                  \
	{                                                                                                   \
		cudaError_t e_ = (expr);                                                                        \
		if (e_ != cudaSuccess)                                                                          \
			throw mogpu::CudaError(e_, #expr, __FILE__, __LINE__);                                      \
	} while (0)
