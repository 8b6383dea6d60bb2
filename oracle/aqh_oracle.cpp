/*
 * aqh_oracle.cpp -- CPU restatement of the aqsis REYES hider (the checker).
 *
 * TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline leg.  It is never part of the product path.
 *
 * The reference cannot be compiled in this environment (its hot-path headers
 * hard-include Boost; libtiff, flex and bison are also missing), so this file
 * restates its algorithm in plain C++17, following the reference's files op
 * for op.  It must be compiled with -ffp-contract=off and without fast-math so
 * that every float operation is rounded the way the reference's SSE build
 * rounds it.  Each function cites the reference code it follows.
 *
 * Frame-wide form.  The reference samples bucket by bucket, handing apron
 * pixels to unprocessed neighbours through cache segments
 * (libs/core/bucketprocessor.cpp:241-358, 1645-1694), so every pixel of the
 * sample region [crop - shift, crop + shift) is sampled exactly once, against
 * every micropolygon whose bound touches it, in the order the micropolygons
 * were inserted (libs/core/bucket.cpp:396-399).  This oracle keeps exactly
 * that per-sample sequence with the sample region set to the whole frame:
 * micropolygons are visited in insertion order (grid order, then iv, then iu;
 * micropolygon.cpp:770-880) and each one walks the pixels of its bound as
 * RenderMPG_Static / RenderMPG_MBOrDof do.  The per-bucket m_hasValidSamples
 * shortcut (bucketprocessor.cpp:420, 667-684) only zeroes buckets whose every
 * pixel already filters to zero, so it is not modelled.
 */
#include "aqh_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// Value types with the reference's operator semantics.
// CqVector2D (include/aqsis/math/vector2d.h), CqVector3D (vector3d.h).
struct V2 {
	float x, y;
	V2() : x(0), y(0) {}
	V2(float a, float b) : x(a), y(b) {}
};
static inline V2 operator+(V2 a, V2 b) { return V2(a.x + b.x, a.y + b.y); }
static inline V2 operator-(V2 a, V2 b) { return V2(a.x - b.x, a.y - b.y); }
static inline V2 operator-(V2 a) { return V2(-a.x, -a.y); }
static inline V2 operator*(V2 a, float f) { return V2(a.x * f, a.y * f); }
static inline V2 operator*(float f, V2 a) { return V2(f * a.x, f * a.y); }
static inline V2 operator+(float f, V2 v) { return V2(f + v.x, f + v.y); }
// vector2d.h:377-385
static inline float cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
template <class T> static inline T amin(T a, T b) { return a < b ? a : b; }  // math.h:112
template <class T> static inline T amax(T a, T b) { return a < b ? b : a; }  // math.h:123
static inline float maxNorm(V2 v) { return amax(std::fabs(v.x), std::fabs(v.y)); }
static inline V2 compMul(V2 a, V2 b) { return V2(a.x * b.x, a.y * b.y); }
// vector2d.h:132-147
static inline float mag2(V2 v) {
	if (v.y == 0.0) return v.x * v.x;
	if (v.x == 0.0) return v.y * v.y;
	return (v.x * v.x) + (v.y * v.y);
}
static inline float mag(V2 v) {
	if (v.y == 0.0) return std::fabs(v.x);
	if (v.x == 0.0) return std::fabs(v.y);
	return std::sqrt((v.x * v.x) + (v.y * v.y));
}

struct V3 {
	float x, y, z;
	V3() : x(0), y(0), z(0) {}
	V3(float a, float b, float c) : x(a), y(b), z(c) {}
};
static inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator*(float f, V3 a) { return V3(f * a.x, f * a.y, f * a.z); }
static inline float mag2(V3 v) { return v.x * v.x + v.y * v.y + v.z * v.z; }  // vector3d.h:345-348
static inline V3 vmin(V3 a, V3 b) { return V3(amin(a.x, b.x), amin(a.y, b.y), amin(a.z, b.z)); }
static inline V3 vmax(V3 a, V3 b) { return V3(amax(a.x, b.x), amax(a.y, b.y), amax(a.z, b.z)); }

// math.h:47-70
static inline long lfloor(float x) { return static_cast<long>(x) - (x < 0 && x != static_cast<long>(x)); }
static inline long lceil(float x) { return static_cast<long>(x) + (x > 0 && x != static_cast<long>(x)); }
static inline long lfloord(double x) { return static_cast<long>(x) - (x < 0 && x != static_cast<long>(x)); }
static inline long lroundd(double x) { return lfloord(x - 0.5) + 1; }

struct Bound {  // libs/core/bound.h
	V3 mn, mx;
	bool contains2D(V2 v) const {  // bound.h:144-151
		if ((v.x < mn.x || v.x > mx.x) || (v.y < mn.y || v.y > mx.y)) return false;
		return true;
	}
	bool intersects(V2 a, V2 b) const {  // bound.h:153-160
		if (a.x > mx.x || a.y > mx.y || b.x < mn.x || b.y < mn.y) return false;
		return true;
	}
	void encapsulate(const Bound& b) { mn = vmin(mn, b.mn); mx = vmax(mx, b.mx); }
	void encapsulate2(V2 v) {
		mn.x = amin(mn.x, v.x); mn.y = amin(mn.y, v.y);
		mx.x = amax(mx.x, v.x); mx.y = amax(mx.y, v.y);
	}
};

// ---------------------------------------------------------------------------
// CqInvBilinear (libs/core/bilinear.h:99-140, 250-310).
struct InvBilinear {
	V2 A, E, F, G;
	bool linear;
	void setVertices(V2 a, V2 b, V2 c, V2 d) {  // bilinear.h:260-275
		A = a;
		E = b - a;
		F = c - a;
		G = -E - c + d;
		linear = false;
		float patchSize = amax(maxNorm(F), maxNorm(E));
		float irregularity = maxNorm(G);
		if (irregularity < 1e-2 * patchSize)  // double comparison, as written
			linear = true;
	}
	template <bool unsafeInvert>
	static V2 solve(V2 M1, V2 M2, V2 b) {  // bilinear.h:298-305
		float det = cross(M1, M2);
		if (unsafeInvert || det != 0) det = 1 / det;
		return det * V2(cross(b, M2), -cross(b, M1));
	}
	V2 bilinEval(V2 uv) const {  // bilinear.h:307-310
		return A + E * uv.x + F * uv.y + G * uv.x * uv.y;
	}
	V2 operator()(V2 P) const {  // bilinear.h:277-290
		V2 uv(0.5f, 0.5f);
		uv = uv - solve<true>(E + G * uv.y, F + G * uv.x, bilinEval(uv) - P);
		if (!linear)
			uv = uv - solve<false>(E + G * uv.y, F + G * uv.x, bilinEval(uv) - P);
		return uv;
	}
};

// bilinear.h:228-236
static inline float bilerpf(float A, float B, float C, float D, V2 uv) {
	float w0 = (1 - uv.y) * (1 - uv.x);
	float w1 = (1 - uv.y) * uv.x;
	float w2 = uv.y * (1 - uv.x);
	float w3 = uv.y * uv.x;
	return w0 * A + w1 * B + w2 * C + w3 * D;
}
static inline V2 bilerp2(V2 A, V2 B, V2 C, V2 D, V2 uv) {
	float w0 = (1 - uv.y) * (1 - uv.x);
	float w1 = (1 - uv.y) * uv.x;
	float w2 = uv.y * (1 - uv.x);
	float w3 = uv.y * uv.x;
	return w0 * A + w1 * B + w2 * C + w3 * D;
}

// ---------------------------------------------------------------------------
// CqHitTestCache (micropolygon.h:520-551)
struct HitTestCache {
	V3 P[4];
	float z[4];
	float YMul[4], XMul[4], X[4], Y[4];
	int lastFailedEdge;
	V2 cocMult[4];
	V2 cocMultMin, cocMultMax;
	InvBilinear xyToUV;
};

static const int Degeneracy_Mask = 0x8000000;  // micropolygon.h:791

// Frame-level context (the parts of CqRenderer / SqOptionCache the hider reads).
struct Ctx {
	const OrcFrame* f;
	const OrcGrids* g;
	int xs, ys, spp;
	int shiftX, shiftY;
	// renderer.h:401-406
	V2 coc(float depth) const {
		float c = f->dof_mult * std::fabs(1.0f / depth - f->dof_inv_fd);
		return V2(f->dof_scale_x * c, f->dof_scale_y * c);
	}
	// renderer.cpp:1602-1617
	float minCoCForBound(const Bound& b) const {
		float z1 = b.mn.z, z2 = b.mx.z;
		float focalDist = 1 / f->dof_inv_fd;
		if ((z1 - focalDist) * (z2 - focalDist) < 0) return 0;
		float minBlur = amin(std::fabs(1 / z1 - f->dof_inv_fd), std::fabs(1 / z2 - f->dof_inv_fd));
		return f->dof_mult * amin(f->dof_scale_x, f->dof_scale_y) * minBlur;
	}
};

// One micropolygon (CqMicroPolygon / CqMicroPolygonMotion).
struct MP {
	int id;             // global insertion index
	int grid;
	int index;          // vertex index of corner A within the grid (m_Index)
	int cu;
	int indexCode;
	Bound bound;        // m_Bound (union over keys for moving micropolygons)
	int nkeys;
	const float* keyTimes;
	V3 keys[8][4];      // key vertices: A, B, C(index+cu+1), D(index+cu+2) as AppendKey
	Bound keyBound[8];
	// motion bound list (BuildBoundList)
	std::vector<Bound> subBounds;
	std::vector<float> subTimes;
	// triangle split line per key (CqMicroPolyGridBase::m_TriangleSplitLine)
	bool triangular;
	V2 splitA[8], splitB[8];
	// output cache (SqMpgSampleInfo)
	float col[4][3], opa[4][3];
	bool smooth, isOpaque, isCullable;
	int matteFlag;
	// SqGridInfo::lodBounds (micropolygon.cpp:64-66; attribute default 0 1,
	// attributes.cpp:127); the test runs when the minimum is >= 0
	float lodMin, lodMax;
	bool lodTest() const { return lodMin >= 0.0f; }
	int csgNode;  // the grid's CSG primitive node, -1 if none
	int trimSet;  // the grid's trim set when the micropolygon is marked trimmed (MarkTrimmed), else -1
	bool trimOutside;
	V2 trimUV[4];  // u v at index, index+1, index+cu+1, index+cu+2
	bool lodRejects(float level) const { return lodMin > level || level >= lodMax; }
};

static inline V3 loadP(const float* P, long long vtx) {
	return V3(P[4 * vtx], P[4 * vtx + 1], P[4 * vtx + 2]);
}

// micropolygon.cpp:1207-1284.  pP = key-0 raster points of the grid.
static int computeVertexOrder(const float* P, long long base, int index, int cu) {
	int IndexA = index, IndexB = index + 1, IndexC = index + cu + 2, IndexD = index + cu + 1;
	short CodeA = 0, CodeB = 1, CodeC = 3, CodeD = 2;
	auto p = [&](int i) { return loadP(P, base + i); };
	if (mag2(p(IndexA) - p(IndexB)) < 1e-8) {
		IndexB = IndexC; CodeB = CodeC; IndexC = IndexD; CodeC = CodeD; IndexD = -1; CodeD = -1;
	} else if (mag2(p(IndexB) - p(IndexC)) < 1e-8) {
		IndexB = IndexC; CodeB = CodeC; IndexC = IndexD; CodeC = CodeD; IndexD = -1; CodeD = -1;
	} else if (mag2(p(IndexC) - p(IndexD)) < 1e-8) {
		IndexC = IndexD; CodeC = CodeD; IndexD = -1; CodeD = -1;
	} else if (mag2(p(IndexD) - p(IndexA)) < 1e-8) {
		IndexD = IndexC; CodeD = CodeC; IndexD = -1; CodeD = -1;
	}
	V3 vA2 = p(IndexA), vB2 = p(IndexB), vC2 = p(IndexC);
	bool fFlip = ((vA2.x - vB2.x) * (vB2.y - vC2.y)) >= ((vA2.y - vB2.y) * (vB2.x - vC2.x));
	int code;
	if (!fFlip) {
		code = (CodeD == -1)
			? ((CodeA & 0x3) | ((CodeC & 0x3) << 2) | ((CodeB & 0x3) << 4) | Degeneracy_Mask)
			: ((CodeA & 0x3) | ((CodeD & 0x3) << 2) | ((CodeC & 0x3) << 4) | ((CodeB & 0x3) << 6));
	} else {
		code = (CodeD == -1)
			? ((CodeA & 0x3) | ((CodeB & 0x3) << 2) | ((CodeC & 0x3) << 4) | Degeneracy_Mask)
			: ((CodeA & 0x3) | ((CodeB & 0x3) << 2) | ((CodeC & 0x3) << 4) | ((CodeD & 0x3) << 6));
	}
	return code;
}

// micropolygon.cpp:1346-1392.  pointsIn in the natural order (A, B, index+cu+1, index+cu+2).
static void cachePointInPolyTest(const MP& mp, HitTestCache& cache, const V3* pointsIn) {
	cache.z[0] = pointsIn[0].z;
	cache.z[1] = pointsIn[1].z;
	cache.z[2] = pointsIn[2].z;
	cache.z[3] = pointsIn[3].z;
	cache.xyToUV.setVertices(V2(pointsIn[0].x, pointsIn[0].y), V2(pointsIn[1].x, pointsIn[1].y),
	                         V2(pointsIn[2].x, pointsIn[2].y), V2(pointsIn[3].x, pointsIn[3].y));
	const int c = mp.indexCode;
	const V3 points[4] = {pointsIn[(c >> 2) & 0x3], pointsIn[(c >> 4) & 0x3], pointsIn[(c >> 6) & 0x3],
	                      pointsIn[c & 0x3]};
	int j = 3;
	for (int i = 0; i < 4; ++i) {
		cache.YMul[i] = points[i].x - points[j].x;
		cache.XMul[i] = points[i].y - points[j].y;
		cache.X[i] = points[j].x;
		cache.Y[i] = points[j].y;
		j = i;
	}
	if (c & Degeneracy_Mask) {
		for (int i = 2; i < 4; ++i) {
			cache.YMul[i] = points[3].x - points[1].x;
			cache.XMul[i] = points[3].y - points[1].y;
			cache.X[i] = points[1].x;
			cache.Y[i] = points[1].y;
		}
	}
	cache.lastFailedEdge = 0;
}

// micropolygon.cpp:1295-1342
static bool fContains(HitTestCache& cache, V2 vecP, float& Depth, V2& uv) {
	float x = vecP.x, y = vecP.y;
	int e = cache.lastFailedEdge;
	for (int i = 0; i < 4; ++i) {
		float v = ((y - cache.Y[e]) * cache.YMul[e]) - ((x - cache.X[e]) * cache.XMul[e]);
		if (e & 2) {
			if (v < 0) { cache.lastFailedEdge = e; return false; }
		} else {
			if (v <= 0) { cache.lastFailedEdge = e; return false; }
		}
		e = (e + 1) & 3;
	}
	uv = cache.xyToUV(vecP);
	Depth = bilerpf(cache.z[0], cache.z[1], cache.z[2], cache.z[3], uv);
	return true;
}

// Per-pixel sample storage (SqSampleData, imagepixel.h:122-151).
struct Frag {
	int mp;
	float data[7];
	int flags;
	int csg;  // SqImageSample::csgNode: the CSG node the entry belongs to (-1: none)
};
struct Sample {
	V2 position, dofOffset;
	float time, lod;
	float occlZ;
	bool occlValid;
	int occlFlags;
	int occlMp;
	float occl[7];
	std::vector<Frag> data;
};

struct Frame {
	Ctx ctx;
	const OrcSamples* s;
	int x0, y0, w, h;  // sample region
	std::vector<Sample> samples;
	std::vector<int> dofIndex;  // per pixel per i: m_DofOffsetIndices
	int64_t splCount = 0, splBoundHits = 0, splHits = 0;
	Sample& at(int px, int py, int i) { return samples[((size_t)(py - y0) * w + (px - x0)) * ctx.spp + i]; }
	int dofIdx(int px, int py, int i) { return dofIndex[((size_t)(py - y0) * w + (px - x0)) * ctx.spp + i]; }
};

// StoreExtraData (bucketprocessor.cpp:1573-1643): the output variables of
// micropolygon `id`'s vertex A (GetIndex), found from the grids' micropolygon
// counts.
static const float* vertexAValues(const OrcGrids* g, const std::vector<int64_t>& mpStart, int id, int naov) {
	const int gi = (int)(std::upper_bound(mpStart.begin(), mpStart.end(), (int64_t)id) - mpStart.begin()) - 1;
	const int cu = g->cu[gi];
	const int m = id - (int)mpStart[gi];
	const int iv = m / cu, iu = m - iv * cu;
	return g->aov + (g->cbase[gi] + (int64_t)iv * (cu + 1) + iu) * naov;
}

// micropolygon.cpp:1443-1462
static void interpolateOutputs(const MP& mp, V2 uv, float col[3], float opa[3]) {
	if (mp.smooth) {
		float w0 = (1 - uv.x) * (1 - uv.y);
		float w1 = uv.x * (1 - uv.y);
		float w2 = (1 - uv.x) * uv.y;
		float w3 = uv.x * uv.y;
		for (int k = 0; k < 3; ++k) {
			col[k] = w0 * mp.col[0][k] + w1 * mp.col[1][k] + w2 * mp.col[2][k] + w3 * mp.col[3][k];
			opa[k] = w0 * mp.opa[0][k] + w1 * mp.opa[1][k] + w2 * mp.opa[2][k] + w3 * mp.opa[3][k];
		}
	} else {
		for (int k = 0; k < 3; ++k) { col[k] = mp.col[0][k]; opa[k] = mp.opa[0][k]; }
	}
}

// bucketprocessor.cpp:1471-1569 (AOVs and CSG not modelled).
static void storeSample(Frame& fr, const MP& mp, Sample& sd, float D, V2 uv) {
	const OrcFrame* f = fr.ctx.f;
	if (mp.isCullable && sd.occlZ <= D) return;
	fr.splHits++;
	float* hitData;
	int* hitFlags;
	if ((mp.isOpaque || (mp.matteFlag & ORC_GRID_MATTEALPHA)) && mp.isCullable) {
		if (f->display_z && f->depth_filter == ORC_DEPTH_MIDPOINT) {
			float hitPrevZ = FLT_MAX;
			if (sd.occlValid) hitPrevZ = sd.occl[6];
			if (hitPrevZ < D) {
				sd.occlZ = D;
				return;
			} else {
				sd.occlZ = hitPrevZ;
			}
		} else {
			sd.occlZ = D;
		}
		sd.occlValid = true;
		sd.occlFlags = 0;
		sd.occlMp = mp.id;
		hitData = sd.occl;
		hitFlags = &sd.occlFlags;
	} else {
		sd.data.push_back(Frag());
		sd.data.back().mp = mp.id;
		sd.data.back().csg = mp.csgNode;
		sd.data.back().flags = 0;
		hitData = sd.data.back().data;
		hitFlags = &sd.data.back().flags;
	}
	float col[3], opa[3];
	interpolateOutputs(mp, uv, col, opa);
	hitData[0] = col[0]; hitData[1] = col[1]; hitData[2] = col[2];
	hitData[3] = opa[0]; hitData[4] = opa[1]; hitData[5] = opa[2];
	hitData[6] = D;
	// Flag_Matte = 1, Flag_MatteAlpha = 2 (imagepixel.h:97-101)
	int mf = 0;
	if (mp.matteFlag & ORC_GRID_MATTE) mf |= 1;
	if (mp.matteFlag & ORC_GRID_MATTEALPHA) mf |= 2;
	*hitFlags |= mf;
}

// micropolygon.cpp:1531-1550
static bool dofSampleInBound(const Bound& bound, const HitTestCache& cache, const Sample& sample) {
	V2 dofOffset = sample.dofOffset;
	V2 samplePos = sample.position;
	V2 cocMin = samplePos + compMul(cache.cocMultMin, dofOffset);
	V2 cocMax = samplePos + compMul(cache.cocMultMax, dofOffset);
	if (dofOffset.x < 0) std::swap(cocMin.x, cocMax.x);
	if (dofOffset.y < 0) std::swap(cocMin.y, cocMax.y);
	return bound.intersects(cocMin, cocMax);
}

// TriangleSplitPoints (micropolygon.cpp:895-900): CqMotionSpec::GetMotionObjectInterpolated
// (motion.h:176-228) over the per-key split lines, lerped as
// CqTriangleSplitLine::LinearInterpolateMotionObjects (micropolygon.h:182-188).
static void triangleSplitPoints(const MP& mp, float time, V2& A, V2& B) {
	const int n = mp.nkeys;
	int i = 0;
	float Fraction = 0.0f;
	bool exact = true;
	if (n > 1) {
		const float* T = mp.keyTimes;
		if (time >= T[n - 1]) {
			i = n - 1;
		} else if (time <= T[0]) {
			i = 0;
		} else {
			i = 0;
			while (time >= T[i + 1]) i += 1;
			Fraction = (time - T[i]) / (T[i + 1] - T[i]);
			exact = (T[i] == time);
		}
	}
	if (exact) {
		A = mp.splitA[i];
		B = mp.splitB[i];
	} else {
		A = ((1.0f - Fraction) * mp.splitA[i]) + (Fraction * mp.splitA[i + 1]);
		B = ((1.0f - Fraction) * mp.splitB[i]) + (Fraction * mp.splitB[i + 1]);
	}
}

// The triangle split line test of both Sample forms (micropolygon.cpp:1630-1654,
// 1885-1907): a hit on or behind the line through the grid's far corners misses.
static bool triangleSplitKeeps(const Ctx& ctx, const MP& mp, const Sample& sample, float D, float time,
                               bool usingDof) {
	V2 vA, vB;
	triangleSplitPoints(mp, time, vA, vB);
	const float Ax = vA.x, Ay = vA.y, Bx = vB.x, By = vB.y;
	V2 hitPos = sample.position;
	if (usingDof) hitPos = hitPos + compMul(ctx.coc(D), sample.dofOffset);
	const float v = (Ay - By) * hitPos.x + (Bx - Ax) * hitPos.y + (Ax * By - Bx * Ay);
	return !(v <= 0);
}

// CqTrimLoop::TrimPoint (trimcurve.cpp:145-169): crossings of the loop's
// edges on the left of the point, by the even-odd rule.
static bool trimLoopPoint(const float* pts, int first, int size, V2 v) {
	const float x = v.x, y = v.y;
	bool odd = false;
	for (int i = 0, j = size - 1; i < size; j = i++) {
		const float ax = pts[2 * (first + i)], ay = pts[2 * (first + i) + 1];
		const float bx = pts[2 * (first + j)], by = pts[2 * (first + j) + 1];
		if (((ay < y) && (by >= y)) || ((by < y) && (ay >= y))) {
			if (ax + (y - ay) / (by - ay) * (bx - ax) < x) odd = !odd;
		}
	}
	return odd;
}

// CqTrimLoopArray::TrimPoint (trimcurve.cpp:223-237): no loops trims nothing;
// else a point inside an even number of loops is trimmed.
static bool trimPoint(const OrcGrids* g, int set, V2 v) {
	const int l0 = g->trim_set_first[set], l1 = g->trim_set_first[set + 1];
	if (l1 == l0) return false;
	int crosses = 0;
	for (int l = l0; l < l1; ++l) {
		const int p0 = g->trim_loop_first[l];
		crosses += trimLoopPoint(g->trim_points, p0, g->trim_loop_first[l + 1] - p0, v) ? 1 : 0;
	}
	return !(crosses & 1);
}

// CqTrimLoop::LineIntersects / CqTrimLoopArray::LineIntersects
// (trimcurve.cpp:172-198, 240-253).
static bool trimLine(const OrcGrids* g, int set, V2 v1, V2 v2) {
	const float x1 = v1.x, y1 = v1.y, x2 = v2.x, y2 = v2.y;
	for (int l = g->trim_set_first[set]; l < g->trim_set_first[set + 1]; ++l) {
		const int p0 = g->trim_loop_first[l], size = g->trim_loop_first[l + 1] - p0;
		const float* P = g->trim_points;
		for (int i = 0, j = size - 1; i < size; j = i++) {
			const float x3 = P[2 * (p0 + i)], y3 = P[2 * (p0 + i) + 1];
			const float x4 = P[2 * (p0 + j)], y4 = P[2 * (p0 + j) + 1];
			const float d = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
			if (d == 0.0f) continue;
			const float r = ((y1 - y3) * (x4 - x3) - (x1 - x3) * (y4 - y3)) / d;
			const float s = ((y1 - y3) * (x2 - x1) - (x1 - x3) * (y2 - y1)) / d;
			if ((r >= 0.0f) && (s >= 0.0f) && (r <= 1.0f) && (s <= 1.0f)) return true;
		}
	}
	return false;
}

// CqBasicVec3 dot product (vector3d.h:602-606)
static float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// The back-face test of one vertex (micropolygon.cpp:451-459, 1013-1017):
// Ng flipped to N's side when N is given, facing away from the eye (P . Ng >= 0).
static bool backFacing(const float* P4, const float* Ng3, const float* N3) {
	float s = 1.0f;
	if (N3) s = (dot3(N3, Ng3) < 0.0f) ? -1.0f : 1.0f;
	const float sn[3] = {s * Ng3[0], s * Ng3[1], s * Ng3[2]};
	return dot3(sn, P4) >= 0;
}

// BilinearEvaluate (bilinear.h:189-224) of CqVector2D corners.
static V2 bilinearEvaluate(V2 A, V2 B, V2 C, V2 D, float s, float t) {
	V2 AB, CD;
	if (s <= 0.0) {
		AB = A;
		CD = C;
	} else if (s >= 1.0) {
		AB = B;
		CD = D;
	} else {
		AB = V2((B.x - A.x) * s + A.x, (B.y - A.y) * s + A.y);
		CD = V2((D.x - C.x) * s + C.x, (D.y - C.y) * s + C.y);
	}
	if (t <= 0.0) return AB;
	if (t >= 1.0) return CD;
	return V2((CD.x - AB.x) * t + AB.x, (CD.y - AB.y) * t + AB.y);
}

// micropolygon.cpp:1561-1660 (static micropolygon).
static bool sampleStatic(const Ctx& ctx, const MP& mp, HitTestCache& cache, const Sample& sample, float& D, V2& uv,
                         bool usingDof, const OrcGrids* g) {
	V2 vecSample = sample.position;
	if (usingDof) {
		if (!dofSampleInBound(mp.bound, cache, sample)) return false;
		V2* coc = cache.cocMult;
		V2 dofOffset = sample.dofOffset;
		V3* P = cache.P;
		V3 points[4];
		for (int i = 0; i < 4; ++i) {
			V2 d = compMul(coc[i], dofOffset);
			points[i] = P[i] - V3(d.x, d.y, 0.0f);
		}
		cachePointInPolyTest(mp, cache, points);
	}
	if (!fContains(cache, vecSample, D, uv)) return false;
	// trimmed micropolygons (micropolygon.cpp:1592-1627): only the "inside"
	// sense rejects here
	if (mp.trimSet >= 0) {
		const V2 vR = bilinearEvaluate(mp.trimUV[0], mp.trimUV[1], mp.trimUV[2], mp.trimUV[3], uv.x, uv.y);
		if (trimPoint(g, mp.trimSet, vR) && !mp.trimOutside) return false;
	}
	return !mp.triangular || triangleSplitKeeps(ctx, mp, sample, D, sample.time, usingDof);
}

// micropolygon.cpp:1768-1914
static bool sampleMotion(const Ctx& ctx, const MP& mp, HitTestCache& cache, const Sample& sample, float& D, V2& uv,
                         float time, bool usingDof) {
	const V2 vecSample = sample.position;
	V3 points[4];
	int iIndex = 0;
	float Fraction = 0.0f;
	bool Exact = true;
	const float* T = mp.keyTimes;
	int ntimes = mp.nkeys;
	if (time > T[0]) {
		if (time >= T[ntimes - 1])
			iIndex = ntimes - 1;
		else {
			iIndex = 0;
			while (time >= T[iIndex + 1]) iIndex += 1;
			Fraction = (time - T[iIndex]) / (T[iIndex + 1] - T[iIndex]);
			Exact = (T[iIndex] == time);
		}
	}
	Bound tight;
	if (Exact) {
		tight = mp.keyBound[iIndex];
	} else {
		const Bound& b1 = mp.keyBound[iIndex];
		const Bound& b2 = mp.keyBound[iIndex + 1];
		tight.mn = (1 - Fraction) * b1.mn + Fraction * b2.mn;
		tight.mx = (1 - Fraction) * b1.mx + Fraction * b2.mx;
	}
	if (usingDof) {
		if (!dofSampleInBound(tight, cache, sample)) return false;
	} else {
		if (!tight.contains2D(vecSample)) return false;
	}
	if (Exact) {
		for (int i = 0; i < 4; ++i) points[i] = mp.keys[iIndex][i];
	} else {
		float F1 = 1.0f - Fraction;
		for (int i = 0; i < 4; ++i) points[i] = (F1 * mp.keys[iIndex][i]) + (Fraction * mp.keys[iIndex + 1][i]);
	}
	if (usingDof) {
		V2 dofOffset = sample.dofOffset;
		for (int i = 0; i < 4; ++i) {
			V2 d = compMul(ctx.coc(points[i].z), dofOffset);
			points[i] = points[i] - V3(d.x, d.y, 0.0f);
		}
	}
	cachePointInPolyTest(mp, cache, points);
	if (!fContains(cache, vecSample, D, uv)) return false;
	return !mp.triangular || triangleSplitKeeps(ctx, mp, sample, D, time, usingDof);
}

// Time-sub-bound list (micropolygon.cpp:1689-1756).
static void buildBoundList(MP& mp, unsigned timeRanges, float opentime, float closetime) {
	mp.subBounds.clear();
	mp.subTimes.clear();
	V3 cr = mp.keyBound[0].mx - mp.keyBound[0].mn;
	float polyLen2 = mag2(V2(cr.x, cr.y));
	V2 p0(mp.keys[0][0].x, mp.keys[0][0].y);
	V2 pl(mp.keys[mp.nkeys - 1][0].x, mp.keys[mp.nkeys - 1][0].y);
	float moveDist2 = mag2(p0 - pl);
	int polyLengthsMoved = amax<int>(1, (int)lfloor(std::sqrt(moveDist2 / polyLen2)));
	unsigned divisions = (unsigned)amin<int>(polyLengthsMoved, (int)timeRanges);
	float dt = (closetime - opentime) / divisions;
	float time = opentime + dt;
	int startKey = 0;
	unsigned endKey = 1;
	Bound bound = mp.keyBound[startKey];
	for (unsigned i = 0; i < divisions; i++) {
		while (time > mp.keyTimes[endKey] && endKey < (unsigned)mp.nkeys - 1) ++endKey;
		int endKey_1 = endKey - 1;
		const Bound& end0 = mp.keyBound[endKey_1];
		float end0Time = mp.keyTimes[endKey_1];
		const Bound& end1 = mp.keyBound[endKey];
		float end1Time = mp.keyTimes[endKey];
		float mix = (time - end0Time) / (end1Time - end0Time);
		Bound mid = end0;
		mid.mn = mid.mn + mix * (end1.mn - end0.mn);
		mid.mx = mid.mx + mix * (end1.mx - end0.mx);
		bound.encapsulate(mid);
		while (startKey < endKey_1) {
			startKey++;
			bound.encapsulate(mp.keyBound[startKey]);
		}
		mp.subBounds.push_back(bound);
		mp.subTimes.push_back(time - dt);
		bound = mid;
		time += dt;
	}
}

// bucketprocessor.cpp:1097-1218
static void renderStatic(Frame& fr, MP& mp) {
	const Ctx& ctx = fr.ctx;
	HitTestCache cache;
	// CacheHitTestValues(cache, false): natural-order points
	V3* P = cache.P;
	for (int i = 0; i < 4; ++i) P[i] = mp.keys[0][i];
	cachePointInPolyTest(mp, cache, P);
	const Bound& Bound = mp.bound;
	float bminx = Bound.mn.x, bmaxx = Bound.mx.x, bminy = Bound.mn.y, bmaxy = Bound.mx.y;
	int eX = (int)lceil(bmaxx), eY = (int)lceil(bmaxy);
	if (eX > fr.x0 + fr.w) eX = fr.x0 + fr.w;
	if (eY > fr.y0 + fr.h) eY = fr.y0 + fr.h;
	int sX = static_cast<int>(std::floor(bminx));
	int sY = static_cast<int>(std::floor(bminy));
	if (sY < fr.y0) sY = fr.y0;
	if (sX < fr.x0) sX = fr.x0;
	int iXSamples = ctx.xs, iYSamples = ctx.ys;
	int im = (bminx < sX) ? 0 : static_cast<int>(std::floor((bminx - sX) * iXSamples));
	int in = (bminy < sY) ? 0 : static_cast<int>(std::floor((bminy - sY) * iYSamples));
	int em = (bmaxx > eX) ? iXSamples : (int)lceil((bmaxx - (eX - 1)) * iXSamples);
	int en = (bmaxy > eY) ? iYSamples : (int)lceil((bmaxy - (eY - 1)) * iYSamples);
	if (sX >= eX || sY >= eY) return;
	for (int iY = sY; iY < eY; ++iY) {
		for (int iX = sX; iX < eX; ++iX) {
			int n = (iY == sY) ? in : 0;
			int end_n = (iY == (eY - 1)) ? en : iYSamples;
			int start_m = (iX == sX) ? im : 0;
			int end_m = (iX == (eX - 1)) ? em : iXSamples;
			int index_start = n * iXSamples + start_m;
			for (; n < end_n; n++) {
				int index = index_start;
				for (int m = start_m; m < end_m; m++, index++) {
					Sample& sd = fr.at(iX, iY, index);
					fr.splCount++;
					if (!Bound.contains2D(sd.position)) continue;
					if (mp.isCullable && Bound.mn.z > sd.occlZ) continue;
					// level of detail (bucketprocessor.cpp:1182-1190)
					if (mp.lodTest() && mp.lodRejects(sd.lod)) continue;
					fr.splBoundHits++;
					float D;
					V2 uv;
					if (sampleStatic(ctx, mp, cache, sd, D, uv, false, ctx.g)) storeSample(fr, mp, sd, D, uv);
				}
				index_start += iXSamples;
			}
		}
	}
}

// bucketprocessor.cpp:858-913 and imagepixel.h:429-436
static V2 projectToCircle(V2 pos) {
	float r = mag(pos);
	if (r == 0.0) return V2(0, 0);
	float adj = amax(std::fabs(pos.x), std::fabs(pos.y)) / r;
	return adj * pos;
}
static std::vector<Bound> calculateDofBounds(int xs, int ys) {
	std::vector<Bound> b(xs * ys);
	float dx = 2.0 / xs;
	float dy = 2.0 / ys;
	float minX = -1.0, minY = -1.0;
	int which = 0;
	for (int j = 0; j < ys; ++j) {
		for (int i = 0; i < xs; ++i) {
			V2 topLeft = projectToCircle(V2(minX, minY));
			V2 topRight = projectToCircle(V2(minX + dx, minY));
			V2 bottomLeft = projectToCircle(V2(minX, minY + dy));
			V2 bottomRight = projectToCircle(V2(minX + dx, minY + dy));
			if ((topLeft.y > 0.0 && bottomLeft.y < 0.0) || (topLeft.y < 0.0 && bottomLeft.y > 0.0)) {
				topLeft.x = minX; bottomLeft.x = minX; topRight.x = minX + dx; bottomRight.x = minX + dx;
			}
			if ((topLeft.x > 0.0 && topRight.x < 0.0) || (topLeft.x < 0.0 && topRight.x > 0.0)) {
				topLeft.y = minY; bottomLeft.y = minY + dy; topRight.y = minY; bottomRight.y = minY + dy;
			}
			b[which].mn = V3(topLeft.x, topLeft.y, 0.0f);
			b[which].mx = V3(topLeft.x, topLeft.y, 0.0f);
			b[which].encapsulate2(topRight);
			b[which].encapsulate2(bottomLeft);
			b[which].encapsulate2(bottomRight);
			which++;
			minX += dx;
		}
		minX = -1.0;
		minY += dy;
	}
	return b;
}

// bucketprocessor.cpp:1221-1469
static void renderMBOrDof(Frame& fr, MP& mp, bool isMoving, bool usingDof, const std::vector<Bound>& dofBounds) {
	const Ctx& ctx = fr.ctx;
	const OrcFrame* f = ctx.f;
	HitTestCache cache;
	// CacheHitTestValues (micropolygon.cpp:1394-1432 static, 1916-1940 motion)
	if (!isMoving) {
		for (int i = 0; i < 4; ++i) cache.P[i] = mp.keys[0][i];
		if (usingDof) {
			for (int i = 0; i < 4; ++i) cache.cocMult[i] = ctx.coc(cache.P[i].z);
			cache.cocMultMin = V2(amin(amin(cache.cocMult[0].x, cache.cocMult[1].x), amin(cache.cocMult[2].x, cache.cocMult[3].x)),
			                      amin(amin(cache.cocMult[0].y, cache.cocMult[1].y), amin(cache.cocMult[2].y, cache.cocMult[3].y)));
			cache.cocMultMax = V2(amax(amax(cache.cocMult[0].x, cache.cocMult[1].x), amax(cache.cocMult[2].x, cache.cocMult[3].x)),
			                      amax(amax(cache.cocMult[0].y, cache.cocMult[1].y), amax(cache.cocMult[2].y, cache.cocMult[3].y)));
		} else {
			cachePointInPolyTest(mp, cache, cache.P);
		}
	} else if (usingDof) {
		V2 coc1 = ctx.coc(mp.bound.mn.z);
		V2 coc2 = ctx.coc(mp.bound.mx.z);
		if (ctx.minCoCForBound(mp.bound) == 0)
			cache.cocMultMin = V2(0, 0);
		else
			cache.cocMultMin = V2(amin(coc1.x, coc2.x), amin(coc1.y, coc2.y));
		cache.cocMultMax = V2(amax(coc1.x, coc2.x), amax(coc1.y, coc2.y));
	}
	int iXSamples = ctx.xs, iYSamples = ctx.ys;
	float opentime = f->shutter_open, closetime = f->shutter_close;
	float timePerSample = 0;
	bool fastShutter = false;
	int numSamples = iXSamples * iYSamples;
	if (isMoving) {
		// isClose (math.h:174-182)
		float d = std::fabs(closetime - opentime);
		float tol = 10 * FLT_EPSILON;
		fastShutter = d <= tol * std::fabs(closetime) || d <= tol * std::fabs(opentime);
		if (!fastShutter) timePerSample = numSamples / (closetime - opentime);
	}
	const int timeRanges = std::max(4, iXSamples * iYSamples);
	int bound_maxMB = 1;
	if (isMoving) {
		buildBoundList(mp, timeRanges, opentime, closetime);
		bound_maxMB = (int)mp.subBounds.size();
	}
	int bound_maxMB_1 = bound_maxMB - 1;
	for (int bound_numMB = 0; bound_numMB < bound_maxMB; bound_numMB++) {
		float time0, time1 = 0;
		Bound B;
		if (isMoving) { B = mp.subBounds[bound_numMB]; time0 = mp.subTimes[bound_numMB]; }
		else { B = mp.bound; time0 = 0.0f; }
		int indexT0 = 0, indexT1 = 0;
		if (isMoving) {
			if (bound_numMB != bound_maxMB_1) time1 = mp.subTimes[bound_numMB + 1];
			else time1 = closetime;
			if (time1 < opentime || time0 > closetime) continue;
			if (fastShutter) { indexT0 = 0; indexT1 = numSamples; }
			else {
				indexT0 = amax<int>(0, (int)lfloor((time0 - opentime) * timePerSample));
				indexT1 = (int)lceil((time1 - opentime) * timePerSample);
			}
			// The reference reads past the sample array if rounding pushes
			// indexT1 above numSamples; clamp to stay in bounds.
			if (indexT1 > numSamples) indexT1 = numSamples;
		}
		float maxCocX = 0, maxCocY = 0;
		float bminx = B.mn.x, bmaxx = B.mx.x, bminy = B.mn.y, bmaxy = B.mx.y;
		float bminz = B.mn.z, bmaxz = B.mx.z;
		// clipping planes: the stream is already clipped; Clipping defaults (FLT_EPSILON, FLT_MAX)
		if (bminz > FLT_MAX || bmaxz < FLT_EPSILON) continue;
		float mpgbminx = bminx, mpgbmaxx = bmaxx, mpgbminy = bminy, mpgbmaxy = bmaxy;
		int bound_maxDof = 1;
		if (usingDof) {
			V2 minZCoc = ctx.coc(B.mn.z);
			V2 maxZCoc = ctx.coc(B.mx.z);
			maxCocX = amax(minZCoc.x, maxZCoc.x);
			maxCocY = amax(minZCoc.y, maxZCoc.y);
			bound_maxDof = numSamples;
		}
		for (int bound_numDof = 0; bound_numDof < bound_maxDof; bound_numDof++) {
			if (usingDof) {
				const Bound& DofBound = dofBounds[bound_numDof];
				float leftOffset = DofBound.mx.x * maxCocX;
				float rightOffset = DofBound.mn.x * maxCocX;
				float topOffset = DofBound.mx.y * maxCocY;
				float bottomOffset = DofBound.mn.y * maxCocY;
				bminx = mpgbminx - leftOffset;
				bmaxx = mpgbmaxx - rightOffset;
				bminy = mpgbminy - topOffset;
				bmaxy = mpgbmaxy - bottomOffset;
			}
			int eX = (int)lceil(bmaxx), eY = (int)lceil(bmaxy);
			if (eX > fr.x0 + fr.w) eX = fr.x0 + fr.w;
			if (eY > fr.y0 + fr.h) eY = fr.y0 + fr.h;
			int sX = static_cast<int>(std::floor(bminx));
			int sY = static_cast<int>(std::floor(bminy));
			if (sY < fr.y0) sY = fr.y0;
			if (sX < fr.x0) sX = fr.x0;
			if (sX >= eX || sY >= eY) continue;
			for (int iY = sY; iY < eY; ++iY) {
				for (int iX = sX; iX < eX; ++iX) {
					int index = usingDof ? fr.dofIdx(iX, iY, bound_numDof) : indexT0;
					do {
						Sample& sd = fr.at(iX, iY, index);
						V2 vecP = sd.position;
						float time = sd.time;
						index++;
						fr.splCount++;
						if (isMoving && (time < time0 || time > time1)) continue;
						if (usingDof) {
							Bound DofBound;
							DofBound.mn = V3(bminx, bminy, bminz);
							DofBound.mx = V3(bmaxx, bmaxy, bmaxz);
							if (!DofBound.contains2D(vecP)) continue;
						} else {
							if (!B.contains2D(vecP)) continue;
						}
						if (mp.isCullable && B.mn.z > sd.occlZ) continue;
						// level of detail (bucketprocessor.cpp:1404-1412, 1439-1447)
						if (mp.lodTest() && mp.lodRejects(sd.lod)) continue;
						fr.splBoundHits++;
						float D;
						V2 uv;
						bool hit = isMoving ? sampleMotion(ctx, mp, cache, sd, D, uv, time, usingDof)
						                    : sampleStatic(ctx, mp, cache, sd, D, uv, usingDof, ctx.g);
						if (hit) storeSample(fr, mp, sd, D, uv);
					} while (!usingDof && index < indexT1);
				}
			}
		}
	}
}

// CSG resolve of one sample's depth-sorted entries (csgtree.cpp:144-351):
// CqCSGTreeNode::ProcessSampleList, depth first over non-primitive children,
// then this node: child in/out states start false (the reference's "camera
// inside" test can never fire), every entry of a child toggles that child's
// state; entries that do not change this node's state are removed, the
// others are promoted to this node (to no node at the top of the tree).
struct CsgTree {
	const OrcGrids* g;
	bool evaluate(int node, const std::vector<char>& st) const {
		const int t = g->csg_type[node];
		if (t == ORC_CSG_UNION) {
			for (char c : st) if (c) return true;
			return false;
		}
		if (t == ORC_CSG_INTERSECTION) {
			for (char c : st) if (!c) return false;
			return true;
		}
		if (t == ORC_CSG_DIFFERENCE) {
			if (st.empty() || !st[0]) return false;
			for (size_t i = 1; i < st.size(); ++i) if (st[i]) return false;
			return true;
		}
		return false;
	}
	std::vector<int> children(int node) const {
		std::vector<int> c;
		for (int i = 0; i < g->csg_nnodes; ++i) if (g->csg_parent[i] == node) c.push_back(i);
		return c;
	}
	void process(int node, std::vector<Frag>& data) const {
		const std::vector<int> ch = children(node);
		if (g->csg_type[node] == ORC_CSG_PRIMITIVE) {
			// CqCSGNodePrimitive::ProcessSampleList (a primitive at the top)
			for (Frag& e : data) if (e.csg == node) e.csg = -1;
			return;
		}
		for (int c : ch) if (g->csg_type[c] != ORC_CSG_PRIMITIVE) process(c, data);
		std::vector<char> st(ch.size(), 0);
		bool cur = evaluate(node, st);
		for (size_t i = 0; i < data.size();) {
			int ci = -1;
			for (size_t k = 0; k < ch.size(); ++k) if (data[i].csg == ch[k]) ci = (int)k;
			if (ci < 0) { ++i; continue; }
			st[ci] = !st[ci];
			const bool nw = evaluate(node, st);
			if (nw == cur) {
				data.erase(data.begin() + i);
			} else {
				cur = nw;
				data[i].csg = g->csg_parent[node] >= 0 ? node : -1;
				++i;
			}
		}
	}
	void resolve(std::vector<Frag>& data) const {
		for (;;) {
			int start = -1;
			for (const Frag& e : data) if (e.csg >= 0) { start = e.csg; break; }
			if (start < 0) return;
			int top = start;
			while (g->csg_parent[top] >= 0) top = g->csg_parent[top];
			process(top, data);
		}
	}
};

// CqImagePixel::Combine (imagepixel.cpp:144-332)
static void combine(const OrcFrame* f, Sample& sd, const OrcGrids* g) {
	const float zt[3] = {f->zthreshold[0], f->zthreshold[1], f->zthreshold[2]};
	if (!sd.data.empty()) {
		if (sd.occlValid) {
			Frag o;
			o.mp = sd.occlMp;
			o.csg = -1;  // occluding hits never come from CSG grids (not cullable)
			o.flags = sd.occlFlags;
			std::memcpy(o.data, sd.occl, sizeof(o.data));
			sd.data.push_back(o);
		}
		// std::sort is not stable; exact depth ties are resolved in insertion
		// order here (libstdc++ insertion-sorts lists of up to 16 entries,
		// which is stable, so this matches the reference for such lists).
		std::stable_sort(sd.data.begin(), sd.data.end(),
		                 [](const Frag& a, const Frag& b) { return a.data[6] < b.data[6]; });
		// CSG (imagepixel.cpp:170-190); a list it empties leaves the sample as
		// it was (imagepixel.cpp:249: nothing is written back)
		if (g->csg_node && g->csg_nnodes > 0) {
			CsgTree{g}.resolve(sd.data);
			if (sd.data.empty()) return;
		}
		float sc[3] = {0, 0, 0}, so[3] = {0, 0, 0};
		float opaqueDepths[2] = {sd.occlZ, FLT_MAX};
		float maxOpaqueDepth = FLT_MAX;
		for (auto it = sd.data.rbegin(); it != sd.data.rend(); ++it) {
			const float* d = it->data;
			if (it->flags & 1) {  // Flag_Matte: lerp(t, x0, x1) = (1-t)*x0 + t*x1 (math.h:88-91)
				float nc[3], no[3];
				for (int k = 0; k < 3; ++k) nc[k] = (1 - d[3 + k]) * sc[k] + d[3 + k] * 0.0f;
				for (int k = 0; k < 3; ++k) no[k] = (1 - d[k]) * so[k] + d[k] * 0.0f;
				for (int k = 0; k < 3; ++k) { sc[k] = nc[k]; so[k] = no[k]; }
			} else {
				for (int k = 0; k < 3; ++k) {
					float o = d[3 + k];
					float cl = o < 0.0f ? 0.0f : (o > 1.0f ? 1.0f : o);
					sc[k] = (sc[k] * (1.0f - cl)) + d[k];
				}
				for (int k = 0; k < 3; ++k) so[k] = ((1.0f - so[k]) * d[3 + k]) + so[k];
			}
			if (d[3] >= zt[0] && d[4] >= zt[1] && d[5] >= zt[2]) {
				opaqueDepths[1] = opaqueDepths[0];
				opaqueDepths[0] = d[6];
				if (!(maxOpaqueDepth < FLT_MAX)) maxOpaqueDepth = d[6];
			}
		}
		const Frag& top = sd.data.front();
		sd.occlMp = top.mp;
		sd.occlFlags = top.flags;
		std::memcpy(sd.occl, top.data, sizeof(sd.occl));
		for (int k = 0; k < 3; ++k) { sd.occl[k] = sc[k]; sd.occl[3 + k] = so[k]; }
		sd.occlValid = true;
		float& occlDepth = sd.occl[6];
		if (f->depth_filter != ORC_DEPTH_MIN) {
			if (f->depth_filter == ORC_DEPTH_MIDPOINT) {
				if (sd.data.size() > 1) occlDepth = ((opaqueDepths[0] + opaqueDepths[1]) * 0.5f);
				else occlDepth = FLT_MAX;
			} else if (f->depth_filter == ORC_DEPTH_MAX) {
				occlDepth = maxOpaqueDepth;
			} else if (f->depth_filter == ORC_DEPTH_AVERAGE) {
				float totDepth = 0.0f;
				int totCount = 0;
				for (auto& fr : sd.data) {
					const float* d = fr.data;
					if (d[3] >= zt[0] || d[4] >= zt[1] || d[5] >= zt[2]) { totDepth += d[6]; totCount++; }
				}
				totDepth /= totCount;
				occlDepth = totDepth;
			}
		} else {
			occlDepth = opaqueDepths[0];
		}
	} else {
		if (sd.occlValid) {
			if (sd.occlFlags & 1) {
				for (int k = 0; k < 6; ++k) sd.occl[k] = 0;
			}
			if (f->depth_filter == ORC_DEPTH_MIDPOINT) sd.occl[6] = 0.5 * (sd.occl[6] + sd.occlZ);
		}
	}
}


// Float64 twin of combine() (CqImagePixel::Combine, imagepixel.cpp:144-332):
// the same entries, the same stable (depth, insertion) order and CSG resolve,
// composited back to front in double.  Called before combine(), which sorts
// and overwrites the sample in place.  Never feeds the float path.
struct Occl64 {
	bool valid;
	double d[7];
};
static void combine64(const OrcFrame* f, const Sample& sd, const OrcGrids* g, Occl64& o) {
	const double zt[3] = {f->zthreshold[0], f->zthreshold[1], f->zthreshold[2]};
	o.valid = sd.occlValid;
	for (int k = 0; k < 7; ++k) o.d[k] = sd.occl[k];
	if (!sd.data.empty()) {
		std::vector<Frag> data = sd.data;
		if (sd.occlValid) {
			Frag e;
			e.mp = sd.occlMp;
			e.csg = -1;
			e.flags = sd.occlFlags;
			std::memcpy(e.data, sd.occl, sizeof(e.data));
			data.push_back(e);
		}
		std::stable_sort(data.begin(), data.end(), [](const Frag& a, const Frag& b) { return a.data[6] < b.data[6]; });
		if (g->csg_node && g->csg_nnodes > 0) {
			CsgTree{g}.resolve(data);
			if (data.empty()) return;
		}
		double sc[3] = {0, 0, 0}, so[3] = {0, 0, 0};
		double opaqueDepths[2] = {sd.occlZ, FLT_MAX};
		double maxOpaqueDepth = FLT_MAX;
		for (auto it = data.rbegin(); it != data.rend(); ++it) {
			double d[7];
			for (int k = 0; k < 7; ++k) d[k] = it->data[k];
			if (it->flags & 1) {
				double nc[3], no[3];
				for (int k = 0; k < 3; ++k) nc[k] = (1 - d[3 + k]) * sc[k];
				for (int k = 0; k < 3; ++k) no[k] = (1 - d[k]) * so[k];
				for (int k = 0; k < 3; ++k) { sc[k] = nc[k]; so[k] = no[k]; }
			} else {
				for (int k = 0; k < 3; ++k) {
					const double op = d[3 + k];
					const double cl = op < 0.0 ? 0.0 : (op > 1.0 ? 1.0 : op);
					sc[k] = sc[k] * (1.0 - cl) + d[k];
				}
				for (int k = 0; k < 3; ++k) so[k] = (1.0 - so[k]) * d[3 + k] + so[k];
			}
			if (d[3] >= zt[0] && d[4] >= zt[1] && d[5] >= zt[2]) {
				opaqueDepths[1] = opaqueDepths[0];
				opaqueDepths[0] = d[6];
				if (!(maxOpaqueDepth < FLT_MAX)) maxOpaqueDepth = d[6];
			}
		}
		for (int k = 0; k < 7; ++k) o.d[k] = data.front().data[k];
		for (int k = 0; k < 3; ++k) { o.d[k] = sc[k]; o.d[3 + k] = so[k]; }
		o.valid = true;
		if (f->depth_filter == ORC_DEPTH_MIDPOINT) {
			o.d[6] = data.size() > 1 ? (opaqueDepths[0] + opaqueDepths[1]) * 0.5 : FLT_MAX;
		} else if (f->depth_filter == ORC_DEPTH_MAX) {
			o.d[6] = maxOpaqueDepth;
		} else if (f->depth_filter == ORC_DEPTH_AVERAGE) {
			double tot = 0.0;
			int cnt = 0;
			for (auto& e : data)
				if (e.data[3] >= zt[0] || e.data[4] >= zt[1] || e.data[5] >= zt[2]) { tot += e.data[6]; cnt++; }
			o.d[6] = tot / cnt;
		} else {
			o.d[6] = opaqueDepths[0];
		}
	} else if (sd.occlValid) {
		if (sd.occlFlags & 1)
			for (int k = 0; k < 6; ++k) o.d[k] = 0;
		if (f->depth_filter == ORC_DEPTH_MIDPOINT) o.d[6] = 0.5 * ((double)sd.occl[6] + (double)sd.occlZ);
	}
}

}  // namespace orc

using namespace orc;

// ---------------------------------------------------------------------------
// Filters (libs/core/filters.cpp), restated from the RI specification forms
// the reference uses.
extern "C" float orc_filter_eval(int filter, float x, float y, float xwidth, float ywidth) {
	switch (filter) {
	case ORC_FILTER_GAUSSIAN:  // filters.cpp:71-109
		x /= xwidth;
		y /= ywidth;
		return std::exp(-8.0 * (x * x + y * y));
	case ORC_FILTER_BOX:  // filters.cpp:129-141
		return amin((std::fabs(x) <= xwidth / 2.0 ? 1.0 : 0.0), (std::fabs(y) <= ywidth / 2.0 ? 1.0 : 0.0));
	case ORC_FILTER_TRIANGLE: {  // filters.cpp:149-161
		float hxw = xwidth / 2.0, hyw = ywidth / 2.0;
		float absx = std::fabs(x), absy = std::fabs(y);
		return amin((absx <= hxw ? (hxw - absx) / hxw : 0.0), (absy <= hyw ? (hyw - absy) / hyw : 0.0));
	}
	case ORC_FILTER_CATMULLROM: {  // filters.cpp:169-225 (RI 3.2 radial form)
		float r2 = (x * x + y * y);
		float r = std::sqrt(r2);
		return (r >= 2.0) ? 0.0 : (r < 1.0) ? (3.0 * r * r2 - 5.0 * r2 + 2.0) : (-r * r2 + 5.0 * r2 - 8.0 * r + 4.0);
	}
	case ORC_FILTER_SINC: {  // filters.cpp:233-278
		const double PI = 3.14159265358979323846;
		if (x != 0.0) { x *= PI; x = std::cos(0.5 * x / xwidth) * std::sin(x) / x; }
		else x = 1.0;
		if (y != 0.0) { y *= PI; y = std::cos(0.5 * y / ywidth) * std::sin(y) / y; }
		else y = 1.0;
		return x * y;
	}
	case ORC_FILTER_DISK: {  // filters.cpp:286-304
		double d, xx, yy;
		xx = x * x; yy = y * y;
		xwidth *= 0.5; ywidth *= 0.5;
		d = (xx) / (xwidth * xwidth) + (yy) / (ywidth * ywidth);
		return d < 1.0 ? 1.0 : 0.0;
	}
	case ORC_FILTER_BESSEL: {  // filters.cpp:312-342
		const double PI = 3.14159265358979323846;
		double d, w, xx, yy;
		xx = x * x; yy = y * y;
		xwidth *= 0.5; ywidth *= 0.5;
		w = (xx) / (xwidth * xwidth) + (yy) / (ywidth * ywidth);
		if (w < 1.0) {
			d = std::sqrt(xx + yy);
			if (d != 0.0) {
				w = std::cos(0.5 * PI * std::sqrt(w));
				return w * 2 * j1(PI * d) / d;
			}
			return PI;
		}
		return 0.0;
	}
	case ORC_FILTER_MITCHELL: {  // filters.cpp:37-63, 117-122 (B = C = 1/3)
		const float B = 1 / 3.0f, C = 1 / 3.0f;
		float ixw = 1.0f / xwidth, iyw = 1.0f / ywidth;
		auto ev = [&](float t) {
			t = std::fabs(2.f * t);
			if (t > 1.f)
				return ((-B - 6 * C) * t * t * t + (6 * B + 30 * C) * t * t + (-12 * B - 48 * C) * t + (8 * B + 24 * C)) * (1.f / 6.f);
			return ((12 - 9 * B - 6 * C) * t * t * t + (-18 + 12 * B + 6 * C) * t * t + (6 - 2 * B)) * (1.f / 6.f);
		};
		return ev(x * ixw) * ev(y * iyw);
	}
	}
	return 0.0f;
}

// bucketprocessor.cpp:811-856
extern "C" int orc_filter_table(int filter, float xw, float yw, int xs, int ys, float* out, int max_out) {
	int numSubPixels = xs * ys;
	int xmax = (int)lfloor(xw / 2.0f), ymax = (int)lfloor(yw / 2.0f);
	int n = (2 * xmax + 1) * (2 * ymax + 1) * numSubPixels;
	if (n > max_out) return -n;
	float xfwo2 = std::ceil(xw) * 0.5f;
	float yfwo2 = std::ceil(yw) * 0.5f;
	for (int py = -ymax; py <= ymax; py++) {
		for (int px = -xmax; px <= xmax; px++) {
			int subPixelIndex = ((py + ymax) * (2 * xmax + 1) + px + xmax) * numSubPixels;
			for (int sy = 0; sy < ys; sy++) {
				for (int sx = 0; sx < xs; sx++, ++subPixelIndex) {
					float fx = (sx + 0.5f) / xs + px - 0.5f;
					float fy = (sy + 0.5f) / ys + py - 0.5f;
					float w = 0;
					if (fx >= -xfwo2 && fy >= -yfwo2 && fx <= xfwo2 && fy <= yfwo2)
						w = orc_filter_eval(filter, fx, fy, std::ceil(xw), std::ceil(yw));
					out[subPixelIndex] = w;
				}
			}
		}
	}
	return n;
}

extern "C" void orc_invbilinear(const float* q, const float* P, int n, float* uv) {
	InvBilinear ib;
	ib.setVertices(V2(q[0], q[1]), V2(q[2], q[3]), V2(q[4], q[5]), V2(q[6], q[7]));
	for (int i = 0; i < n; ++i) {
		V2 r = ib(V2(P[2 * i], P[2 * i + 1]));
		uv[2 * i] = r.x;
		uv[2 * i + 1] = r.y;
	}
}

extern "C" void orc_bilerp2(const float* q, const float* uv, int n, float* P) {
	for (int i = 0; i < n; ++i) {
		V2 r = bilerp2(V2(q[0], q[1]), V2(q[2], q[3]), V2(q[4], q[5]), V2(q[6], q[7]), V2(uv[2 * i], uv[2 * i + 1]));
		P[2 * i] = r.x;
		P[2 * i + 1] = r.y;
	}
}

// ExposeBucket (bucketprocessor.cpp:766-806) over n display pixels' channels.
static void exposeChannels(const OrcFrame* f, float* chan, size_t n) {
	if (f->gain == 1.0 && f->gamma == 1.0) return;
	float oneovergamma = 1.0f / f->gamma;
	for (size_t p = 0; p < n; ++p) {
		float* c = &chan[p * 9];
		if (f->gain != 1.0) { c[0] *= f->gain; c[1] *= f->gain; c[2] *= f->gain; }
		if (f->gamma != 1.0) {
			c[0] = std::pow(c[0], oneovergamma);
			c[1] = std::pow(c[1], oneovergamma);
			c[2] = std::pow(c[2], oneovergamma);
		}
	}
}

// FormatBucketForDisplay quantize (ddmanager.cpp:1022-1119) of the channels
// `qch` of n display pixels, one dither value per pixel (or none).
static void quantizeChannels(const OrcFrame* f, const float* chan, size_t n, const float* dither, const int32_t* qch,
                             int nq, double* out) {
	for (size_t p = 0; p < n; ++p) {
		double sdither = dither ? (double)dither[p] : 0.0;
		for (int ci = 0; ci < nq; ++ci) {
			double value = chan[p * 9 + qch[ci]];
			if (f->q_one != 0) {
				value = lroundd(f->q_zero + value * (f->q_one - f->q_zero) + (f->q_dither * sdither));
				value = value < f->q_min ? f->q_min : (value > f->q_max ? f->q_max : value);
			}
			out[p * nq + ci] = value;
		}
	}
}

// The imager shader's write-back (bucketprocessor.cpp:712-743) on channels
// FilterBucket left (before exposure): Ci and Oi from the shader's colour and
// opacity (ci_oi [pixel][6]), alpha = their mean; then ExposeBucket.
extern "C" void orc_imager(const OrcFrame* f, float* chan, const float* ci_oi, int64_t n) {
	for (int64_t p = 0; p < n; ++p) {
		float* c = &chan[p * 9];
		const float* im = &ci_oi[p * 6];
		c[0] = im[0]; c[1] = im[1]; c[2] = im[2];
		c[3] = im[3]; c[4] = im[4]; c[5] = im[5];
		const float a = (im[3] + im[4] + im[5]) / 3.0f;
		c[6] = a;
	}
	exposeChannels(f, chan, (size_t)n);
}

extern "C" void orc_quantize(const OrcFrame* f, const float* chan, int64_t n, const float* dither,
                             const int32_t* qch, int nq, double* out) {
	quantizeChannels(f, chan, (size_t)n, dither, qch, nq, out);
}

extern "C" int orc_render(const OrcFrame* f, const OrcGrids* g, const OrcSamples* s, const float* ftab, OrcOut* out) {
	Frame fr;
	fr.ctx.f = f;
	fr.ctx.g = g;
	fr.ctx.xs = f->xsamples;
	fr.ctx.ys = f->ysamples;
	fr.ctx.spp = f->xsamples * f->ysamples;
	fr.ctx.shiftX = (int)lfloor(f->xfilter / 2.0f);  // bucketprocessor.cpp:36-37
	fr.ctx.shiftY = (int)lfloor(f->yfilter / 2.0f);
	fr.s = s;
	fr.x0 = s->x0; fr.y0 = s->y0; fr.w = s->w; fr.h = s->h;
	const int spp = fr.ctx.spp;
	const size_t nsamp = (size_t)fr.w * fr.h * spp;
	fr.samples.resize(nsamp);
	fr.dofIndex.resize(nsamp);
	// CqImagePixel::clear + setSamples (imagepixel.cpp:105-122, 334-359).
	const float opentime = f->shutter_open, closetime = f->shutter_close;
	for (int py = 0; py < fr.h; ++py) {
		for (int px = 0; px < fr.w; ++px) {
			const size_t pix = (size_t)py * fr.w + px;
			const size_t pbase = pix * spp;
			auto sel = [&](const uint32_t* idx) { return (size_t)(idx ? idx[pix] : pix) * spp; };
			const size_t ps = sel(s->pos_index), ds = sel(s->dof_index), ts = sel(s->time_index);
			const size_t ss = sel(s->shuffle_index), ls = sel(s->lod_index);
			V2 offset((float)(px + fr.x0), (float)(py + fr.y0));
			for (int i = 0; i < spp; ++i) {
				Sample& sd = fr.samples[pbase + i];
				sd.occlZ = FLT_MAX;
				sd.occlValid = false;
				sd.occlFlags = 0;
				sd.occlMp = -1;
				for (int k = 0; k < 7; ++k) sd.occl[k] = 0;
			}
			for (int i = 0; i < spp; ++i)
				fr.dofIndex[pbase + i] = s->shuffle ? s->shuffle[ss + i] : i;
			for (int i = 0; i < spp; ++i) {
				Sample& sd = fr.samples[pbase + i];
				sd.position = offset + V2(s->pos[2 * (ps + i)], s->pos[2 * (ps + i) + 1]);
				float t = s->time ? s->time[ts + i] : 0.0f;
				sd.time = (closetime - opentime) * t + opentime;
				sd.lod = s->lod ? s->lod[ls + i] : 0.0f;
				V2 d = s->dof ? V2(s->dof[2 * (ds + i)], s->dof[2 * (ds + i) + 1]) : V2(0.5f, 0.5f);
				fr.samples[pbase + fr.dofIndex[pbase + i]].dofOffset = projectToCircle(-1 + 2 * d);
			}
		}
	}
	const bool usingDof = f->use_dof != 0;
	std::vector<Bound> dofBounds;
	if (usingDof) dofBounds = calculateDofBounds(f->xsamples, f->ysamples);
	const bool cullable = !(f->display_z && (f->depth_filter == ORC_DEPTH_MAX || f->depth_filter == ORC_DEPTH_AVERAGE));

	int mpid = 0;
	MP mp;
	for (int gi = 0; gi < g->ngrids; ++gi) {
		const int cu = g->cu[gi], cv = g->cv[gi];
		const int nk = g->nkeys ? g->nkeys[gi] : 1;
		const long long nv = (long long)(cu + 1) * (cv + 1);
		const long long pb = g->pbase[gi];
		const long long cb = g->cbase[gi];
		const int flags = g->flags ? g->flags[gi] : ORC_GRID_SMOOTH;
		// triangle split line per key (micropolygon.cpp:703-719, 737-746): through the
		// corners cu and cv*(cu+1), ordered so the kept side is positive
		mp.triangular = (flags & ORC_GRID_TRIANGULAR) != 0;
		if (mp.triangular) {
			for (int k = 0; k < nk; ++k) {
				const V3 v0 = loadP(g->P, pb + k * nv), v1 = loadP(g->P, pb + k * nv + cu);
				const V3 v2 = loadP(g->P, pb + k * nv + (long long)cv * (cu + 1));
				if (((v1.x - v0.x) * (v2.y - v0.y) - (v1.y - v0.y) * (v2.x - v0.x)) >= 0) {
					mp.splitA[k] = V2(v1.x, v1.y);
					mp.splitB[k] = V2(v2.x, v2.y);
				} else {
					mp.splitA[k] = V2(v2.x, v2.y);
					mp.splitB[k] = V2(v1.x, v1.y);
				}
			}
		}
		for (int iv = 0; iv < cv; iv++) {
			for (int iu = 0; iu < cu; iu++, mpid++) {
				if (g->culled && g->culled[mpid]) continue;
				const int index = iv * (cu + 1) + iu;
				// trimming in Split (micropolygon.cpp:754-835, 1056-1130)
				mp.trimSet = -1;
				if (g->trim_set && g->trim_set[gi] >= 0) {
					const int set = g->trim_set[gi];
					const long long c = cb + index;
					auto uvAt = [&](long long k) { return V2(g->trim_uv[2 * k], g->trim_uv[2 * k + 1]); };
					const V2 vecA = uvAt(c), vecB = uvAt(c + 1), vecC = uvAt(c + cu + 2), vecD = uvAt(c + cu + 1);
					const bool outside = (flags & ORC_GRID_TRIM_OUTSIDE) != 0;
					bool tA = trimPoint(g, set, vecA), tB = trimPoint(g, set, vecB);
					bool tC = trimPoint(g, set, vecC), tD = trimPoint(g, set, vecD);
					if (outside) {
						tA = !tA;
						tB = !tB;
						tC = !tC;
						tD = !tD;
					}
					if (tA && tB && tC && tD && !trimLine(g, set, vecA, vecB) && !trimLine(g, set, vecB, vecC) &&
					    !trimLine(g, set, vecC, vecD) && !trimLine(g, set, vecD, vecA))
						continue;  // trimmed out: never added
					if (tA || tB || tC || tD) {
						mp.trimSet = set;
						mp.trimOutside = outside;
						mp.trimUV[0] = vecA;
						mp.trimUV[1] = vecB;
						mp.trimUV[2] = vecD;  // index + cu + 1
						mp.trimUV[3] = vecC;  // index + cu + 2
					}
				}
				mp.id = mpid;
				mp.grid = gi;
				mp.index = index;
				mp.cu = cu;
				mp.nkeys = nk;
				mp.keyTimes = (nk > 1) ? g->times + g->tbase[gi] : nullptr;
				for (int k = 0; k < nk; ++k) {
					long long kb = pb + k * nv;
					// AppendKey(aaPtimes[t][i], [i+1], [i+cu+1], [i+cu+2]) (micropolygon.cpp:1136-1137)
					mp.keys[k][0] = loadP(g->P, kb + index);
					mp.keys[k][1] = loadP(g->P, kb + index + 1);
					mp.keys[k][2] = loadP(g->P, kb + index + cu + 1);
					mp.keys[k][3] = loadP(g->P, kb + index + cu + 2);
					// CqMovingMicroPolygonKey::GetBound (micropolygon.cpp:1974-1989)
					const V3* q = mp.keys[k];
					Bound& kbd = mp.keyBound[k];
					kbd.mn = V3(amin(q[0].x, amin(q[1].x, amin(q[2].x, q[3].x))), amin(q[0].y, amin(q[1].y, amin(q[2].y, q[3].y))),
					            amin(q[0].z, amin(q[1].z, amin(q[2].z, q[3].z))));
					kbd.mx = V3(amax(q[0].x, amax(q[1].x, amax(q[2].x, q[3].x))), amax(q[0].y, amax(q[1].y, amax(q[2].y, q[3].y))),
					            amax(q[0].z, amax(q[1].z, amax(q[2].z, q[3].z))));
				}
				mp.indexCode = computeVertexOrder(g->P, pb, index, cu);
				if (nk == 1) {
					// CalculateBound (micropolygon.cpp:1663-1673): min(min(min(A,B),C),D) with C = index+cu+2
					V3 A = mp.keys[0][0], B = mp.keys[0][1], C = mp.keys[0][3], D = mp.keys[0][2];
					mp.bound.mn = vmin(vmin(vmin(A, B), C), D);
					mp.bound.mx = vmax(vmax(vmax(A, B), C), D);
				} else {
					// AppendKey encapsulation (micropolygon.cpp:1952-1967)
					mp.bound = mp.keyBound[0];
					for (int k = 1; k < nk; ++k) mp.bound.encapsulate(mp.keyBound[k]);
				}
				// AddMPG culling (imagebuffer.cpp:514-539)
				{
					Bound B = mp.bound;
					if (usingDof) {
						V2 c1 = fr.ctx.coc(B.mn.z), c2 = fr.ctx.coc(B.mx.z);
						// max(CqVector2D, CqVector2D) is component-wise (vector2d.h)
						V2 maxCoC(amax(c1.x, c2.x), amax(c1.y, c2.y));
						B.mn = B.mn - V3(maxCoC.x, maxCoC.y, 0.0f);
						B.mx = B.mx + V3(maxCoC.x, maxCoC.y, 0.0f);
					}
					if (B.mx.x < f->crop_xmin - f->xfilter / 2.0f || B.mx.y < f->crop_ymin - f->yfilter / 2.0f ||
					    B.mn.x > f->crop_xmax + f->xfilter / 2.0f || B.mn.y > f->crop_ymax + f->yfilter / 2.0f)
						continue;
				}
				// Output cache (micropolygon.cpp:1464-1529)
				mp.smooth = (flags & ORC_GRID_SMOOTH) != 0;
				mp.lodMin = g->lod ? g->lod[2 * gi] : 0.0f;
				mp.lodMax = g->lod ? g->lod[2 * gi + 1] : 1.0f;
				mp.matteFlag = flags & (ORC_GRID_MATTE | ORC_GRID_MATTEALPHA);
				// a micropolygon of a CSG solid is never occlusion-cullable
				// (bucketprocessor.cpp:1074-1080)
				mp.csgNode = (g->csg_node && g->csg_nnodes > 0) ? g->csg_node[gi] : -1;
				mp.isCullable = cullable && mp.csgNode < 0;
				const int vidx[4] = {index, index + 1, index + cu + 1, index + cu + 2};
				const int ncol = mp.smooth ? 4 : 1;
				for (int i = 0; i < ncol; ++i) {
					long long v = cb + vidx[i];
					for (int k = 0; k < 3; ++k) {
						mp.col[i][k] = g->Ci ? g->Ci[4 * v + k] : 1.0f;
						mp.opa[i][k] = g->Oi ? g->Oi[4 * v + k] : 1.0f;
					}
				}
				mp.isOpaque = true;
				for (int i = 0; i < ncol; ++i)
					if (!(mp.opa[i][0] >= 1.0f && mp.opa[i][1] >= 1.0f && mp.opa[i][2] >= 1.0f)) mp.isOpaque = false;
				// RenderMicroPoly (bucketprocessor.cpp:1067-1091)
				const bool isMoving = nk > 1;
				if (isMoving || usingDof) renderMBOrDof(fr, mp, isMoving, usingDof, dofBounds);
				else renderStatic(fr, mp);
			}
		}
	}

	// Per-sample outputs before Combine
	for (size_t i = 0; i < nsamp; ++i) {
		const Sample& sd = fr.samples[i];
		if (out->winner) out->winner[i] = sd.occlValid ? sd.occlMp : -1;
		if (out->occlz) out->occlz[i] = sd.occlZ;
		if (out->nfrag) out->nfrag[i] = (int32_t)sd.data.size();
	}
	// the float64 twin reads each sample before combine() rewrites it
	const bool want64 = out->sdata64 || out->channels64;
	std::vector<Occl64> occl64(want64 ? nsamp : 0);
	if (want64)
		for (size_t i = 0; i < nsamp; ++i) combine64(f, fr.samples[i], g, occl64[i]);
	// CombineElements (bucketprocessor.cpp:365-375)
	for (size_t i = 0; i < nsamp; ++i) combine(f, fr.samples[i], g);
	if (out->sdata64)
		for (size_t i = 0; i < nsamp; ++i)
			for (int k = 0; k < 7; ++k) out->sdata64[7 * i + k] = occl64[i].valid ? occl64[i].d[k] : 0.0;
	for (size_t i = 0; i < nsamp; ++i) {
		const Sample& sd = fr.samples[i];
		if (out->valid) out->valid[i] = sd.occlValid ? 1 : 0;
		if (out->sdata)
			for (int k = 0; k < 7; ++k) out->sdata[7 * i + k] = sd.occl[k];
	}

	// FilterBucket, non-separable path (bucketprocessor.cpp:584-664, 686-707)
	const int naov = (g->aov && g->naov > 0) ? (g->naov < ORC_MAX_AOV ? g->naov : ORC_MAX_AOV) : 0;
	std::vector<int64_t> mpStart((size_t)g->ngrids + 1, 0);
	for (int gi = 0; gi < g->ngrids; ++gi) mpStart[gi + 1] = mpStart[gi] + (int64_t)g->cu[gi] * g->cv[gi];
	const int dw = f->crop_xmax - f->crop_xmin, dh = f->crop_ymax - f->crop_ymin;
	const int xmax = fr.ctx.shiftX, ymax = fr.ctx.shiftY;
	const float xfwo2 = std::ceil(f->xfilter) * 0.5f;
	const float yfwo2 = std::ceil(f->yfilter) * 0.5f;
	const int numSubPixels = spp;
	std::vector<float> chan((size_t)dw * dh * 9);
	for (int y = f->crop_ymin; y < f->crop_ymax; y++) {
		float ycent = y + 0.5f;
		for (int x = f->crop_xmin; x < f->crop_xmax; x++) {
			float xcent = x + 0.5f;
			float gTot = 0.0;
			int SampleCount = 0;
			float samples[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
			// output variables: the hit data past the nine standard floats
			// (StoreExtraData writes vertex A's values, Combine keeps the front
			// entry's), summed with the same weights
			float extra[ORC_MAX_AOV] = {0};
			for (int fy = -ymax; fy <= ymax; fy++) {
				for (int fx = -xmax; fx <= xmax; fx++) {
					int index = ((fy + ymax) * (2 * xmax + 1) + fx + xmax) * numSubPixels;
					int sampleIndex = 0;
					for (int sy = 0; sy < f->ysamples; sy++) {
						for (int sx = 0; sx < f->xsamples; sx++) {
							const Sample& sd = fr.at(x + fx, y + fy, sampleIndex);
							V2 vecS = sd.position - V2(xcent, ycent);
							if (vecS.x >= -xfwo2 && vecS.y >= -yfwo2 && vecS.x <= xfwo2 && vecS.y <= yfwo2) {
								float gw = ftab[index + sampleIndex];
								gTot += gw;
								if (sd.occlValid) {
									// hit data layout: R G B OR OG OB depth coverage alpha; the
									// last two are never written by StoreSample and stay 0.
									for (int k = 0; k < 7; ++k) samples[k] += sd.occl[k] * gw;
									samples[7] += 0.0f * gw;
									samples[8] += 0.0f * gw;
									if (naov > 0 && sd.occlMp >= 0) {
										const float* v = vertexAValues(g, mpStart, sd.occlMp, naov);
										for (int k = 0; k < naov; ++k) extra[k] += v[k] * gw;
									}
									SampleCount++;
								}
							}
							sampleIndex++;
						}
					}
				}
			}
			float* c = &chan[((size_t)(y - f->crop_ymin) * dw + (x - f->crop_xmin)) * 9];
			float coverage;
			if (SampleCount == 0) {
				for (int k = 0; k < 9; ++k) c[k] = 0.0f;
				c[7] = FLT_MAX;
				coverage = 0.0f;
			} else {
				float oneOverGTot = 1.0 / gTot;
				// channel buffer: Ci(0..2) Oi(3..5) a(6) z(7) coverage(8); sample offsets Ci 0, Oi 3, z 6
				for (int k = 0; k < 3; ++k) c[k] = samples[k] * oneOverGTot;
				for (int k = 0; k < 3; ++k) c[3 + k] = samples[3 + k] * oneOverGTot;
				c[6] = samples[8] * oneOverGTot;
				c[7] = samples[6] * oneOverGTot;
				c[8] = samples[7] * oneOverGTot;
				if (SampleCount >= numSubPixels) coverage = 1.0;
				else coverage = (float)SampleCount / (float)(numSubPixels);
			}
			float a = (c[3] + c[4] + c[5]) / 3.0f;
			c[6] = a * coverage;
			c[8] = coverage;
			if (naov > 0 && out->aov_channels) {
				float* o = out->aov_channels + ((size_t)(y - f->crop_ymin) * dw + (x - f->crop_xmin)) * naov;
				const float oneOverGTot = SampleCount ? (float)(1.0 / gTot) : 0.0f;
				for (int k = 0; k < naov; ++k) o[k] = SampleCount ? extra[k] * oneOverGTot : 0.0f;
			}
		}
	}
	exposeChannels(f, chan.data(), (size_t)dw * dh);
	if (out->channels) std::memcpy(out->channels, chan.data(), chan.size() * sizeof(float));
	// Float64 twin of the filter and exposure above: the same window test on
	// the same float sample positions (membership is a selection, not
	// arithmetic), the table weights as exact inputs, sums and the
	// normalisation in double.
	if (out->channels64) {
		for (int y = f->crop_ymin; y < f->crop_ymax; y++) {
			const float ycent = y + 0.5f;
			for (int x = f->crop_xmin; x < f->crop_xmax; x++) {
				const float xcent = x + 0.5f;
				double gTot = 0.0, acc[7] = {0, 0, 0, 0, 0, 0, 0};
				int cnt = 0;
				for (int fy = -ymax; fy <= ymax; fy++)
					for (int fx = -xmax; fx <= xmax; fx++) {
						const int index = ((fy + ymax) * (2 * xmax + 1) + fx + xmax) * numSubPixels;
						for (int si = 0; si < numSubPixels; ++si) {
							const Sample& sd = fr.at(x + fx, y + fy, si);
							const V2 vecS = sd.position - V2(xcent, ycent);
							if (vecS.x >= -xfwo2 && vecS.y >= -yfwo2 && vecS.x <= xfwo2 && vecS.y <= yfwo2) {
								const double gw = ftab[index + si];
								gTot += gw;
								const size_t sidx = (size_t)(&sd - fr.samples.data());
								if (occl64[sidx].valid) {
									for (int k = 0; k < 7; ++k) acc[k] += occl64[sidx].d[k] * gw;
									cnt++;
								}
							}
						}
					}
				double* c = out->channels64 + ((size_t)(y - f->crop_ymin) * dw + (x - f->crop_xmin)) * 9;
				double coverage = 0.0;
				if (cnt == 0) {
					for (int k = 0; k < 9; ++k) c[k] = 0.0;
					c[7] = FLT_MAX;
				} else {
					const double inv = 1.0 / gTot;
					for (int k = 0; k < 6; ++k) c[k] = acc[k] * inv;
					c[7] = acc[6] * inv;
					coverage = cnt >= numSubPixels ? 1.0 : (double)cnt / numSubPixels;
				}
				c[6] = (c[3] + c[4] + c[5]) / 3.0 * coverage;
				c[8] = coverage;
				if (!(f->gain == 1.0f && f->gamma == 1.0f)) {
					for (int k = 0; k < 3; ++k) {
						if (f->gain != 1.0f) c[k] *= f->gain;
						if (f->gamma != 1.0f) c[k] = std::pow(c[k], 1.0 / f->gamma);
					}
				}
			}
		}
	}
	if (out->quantized && out->qchannels)
		quantizeChannels(f, chan.data(), (size_t)dw * dh, s->dither, out->qchannels, out->nqchannels, out->quantized);
	out->spl_count = fr.splCount;
	out->spl_bound_hits = fr.splBoundHits;
	out->spl_hits = fr.splHits;
	return 0;
}

// ---------------------------------------------------------------------------
// The reference's process-global Mersenne Twister (libs/math/random.cpp),
// restated from the published MT19937 algorithm (Matsumoto & Nishimura 1998).
namespace {
const int MT_N = 624, MT_M = 397;
uint32_t mt[MT_N];
int mti = MT_N + 1;
void init_genrand(uint32_t s) {
	mt[0] = s;
	for (mti = 1; mti < MT_N; mti++) mt[mti] = (1812433253u * (mt[mti - 1] ^ (mt[mti - 1] >> 30)) + (uint32_t)mti);
}
uint32_t genrand_int32() {
	static const uint32_t mag01[2] = {0x0u, 0x9908b0dfu};
	uint32_t y;
	if (mti >= MT_N) {
		if (mti == MT_N + 1) init_genrand(5489u);
		int kk;
		for (kk = 0; kk < MT_N - MT_M; kk++) {
			y = (mt[kk] & 0x80000000u) | (mt[kk + 1] & 0x7fffffffu);
			mt[kk] = mt[kk + MT_M] ^ (y >> 1) ^ mag01[y & 1u];
		}
		for (; kk < MT_N - 1; kk++) {
			y = (mt[kk] & 0x80000000u) | (mt[kk + 1] & 0x7fffffffu);
			mt[kk] = mt[kk + (MT_M - MT_N)] ^ (y >> 1) ^ mag01[y & 1u];
		}
		y = (mt[MT_N - 1] & 0x80000000u) | (mt[0] & 0x7fffffffu);
		mt[MT_N - 1] = mt[MT_M - 1] ^ (y >> 1) ^ mag01[y & 1u];
		mti = 0;
	}
	y = mt[mti++];
	y ^= (y >> 11);
	y ^= (y << 7) & 0x9d2c5680u;
	y ^= (y << 15) & 0xefc60000u;
	y ^= (y >> 18);
	return y;
}
// random.cpp:193-205 and 186-190
float randomFloat() { return genrand_int32() * (1.0 / 4294967424.0); }
float randomFloatR(float range) { return range * randomFloat(); }
unsigned randomInt(unsigned range) {
	double n = randomFloatR((float)range);
	return (unsigned)lfloord(n);
}
}  // namespace

extern "C" void orc_mt_seed(uint32_t s) { init_genrand(s); }
extern "C" uint32_t orc_mt_int32(void) { return genrand_int32(); }
extern "C" float orc_mt_float(void) { return randomFloat(); }
extern "C" long orc_lfloor(float x) { return lfloor(x); }
extern "C" long orc_lceil(float x) { return lceil(x); }
extern "C" long orc_lround(double x) { return lroundd(x); }
// CqVector2D::Magnitude2 / Magnitude (vector2d.h:132-147) as the oracle uses
// them (motion divisions, the vertex-order degeneracy test)
extern "C" float orc_mag2(float x, float y) { return mag2(V2(x, y)); }
extern "C" float orc_mag(float x, float y) { return mag(V2(x, y)); }

// multijitter.cpp:83-202, multijitter.h:89-101 (the pattern cache; Reseed(19) is
// left to the caller).
extern "C" void orc_multijitter_tables(int xs, int ys, float* pos, float* t1d, int32_t* shuffle) {
	const int nSamples = xs * ys;
	std::vector<int> indices(2 * nSamples);
	for (int pat = 0; pat < 250; ++pat) {
		const int offset = pat * nSamples;
		if (xs == 1 && ys == 1) {
			// CqVector2D(RandomFloat(), RandomFloat()): GCC evaluates the
			// constructor's arguments right to left, so y draws first.
			float ry = randomFloat();
			float rx = randomFloat();
			pos[2 * offset] = rx;
			pos[2 * offset + 1] = ry;
			t1d[offset] = randomFloat();
		} else {
			// multiJitterIndices
			for (int iy = 0; iy < ys; iy++)
				for (int ix = 0; ix < xs; ix++) {
					int which = 2 * (iy * xs + ix);
					indices[which] = iy;
					indices[which + 1] = ix;
				}
			for (int iy = 0; iy < ys; iy++) {
				int ix = xs;
				while (ix > 1) {
					int ix2 = randomInt(ix);
					--ix;
					std::swap(indices[2 * (iy * xs + ix) + 1], indices[2 * (iy * xs + ix2) + 1]);
				}
			}
			for (int ix = 0; ix < xs; ix++) {
				int iy = ys;
				while (iy > 1) {
					int iy2 = randomInt(iy);
					--iy;
					std::swap(indices[2 * (iy * xs + ix)], indices[2 * (iy2 * xs + ix)]);
				}
			}
			float subPixelHeight = 1.0f / ys;
			float subPixelWidth = 1.0f / xs;
			float subcellWidth = 1.0f / nSamples;
			int which = 0;
			for (int iy = 0; iy < ys; iy++) {
				for (int ix = 0; ix < xs; ix++) {
					int xindex = indices[2 * which];
					int yindex = indices[2 * which + 1];
					// The CqVector2D constructor's two arguments each draw; GCC
					// evaluates them right to left, so the y draw comes first.
					// (Unpinned: the reference cannot be built here to confirm.)
					float ry = randomFloat();
					float rx = randomFloat();
					pos[2 * (offset + which)] = (xindex + rx) * subcellWidth + ix * subPixelWidth;
					pos[2 * (offset + which) + 1] = (yindex + ry) * subcellWidth + iy * subPixelHeight;
					++which;
				}
			}
		}
		float sample1d = 0;
		float delta1d = 1.0f / nSamples;
		float random1d = randomFloatR(delta1d);
		for (int i = 0; i < nSamples; i++) {
			float t = sample1d + random1d;
			t1d[offset + i] = t;
			sample1d += delta1d;
		}
		for (int i = 0; i < nSamples; ++i) shuffle[offset + i] = i;
		int j = nSamples;
		while (j > 1) {
			int j2 = randomInt(j);
			--j;
			std::swap(shuffle[offset + j], shuffle[offset + j2]);
		}
	}
}

// CqMicroPolyGrid::Split projection (micropolygon.cpp:735-745; motion grids
// 1023-1032): each point p becomes matCameraToRaster * p by
// CqMatrix::operator*(const CqVector3D&) (matrix.h:717-750) -- row-vector
// product, x and y (and z, which Split then discards) multiplied by 1/h when
// h != 1 -- and keeps its camera-space z.  m[row*4 + col]; float4 points.
extern "C" void orc_project_points(const float* m, const float* Pin, int64_t n, float* Pout) {
	for (int64_t i = 0; i < n; ++i) {
		const float x = Pin[4 * i], y = Pin[4 * i + 1], z = Pin[4 * i + 2], w = Pin[4 * i + 3];
		const float h = m[0 * 4 + 3] * x + m[1 * 4 + 3] * y + m[2 * 4 + 3] * z + m[3 * 4 + 3];
		float rx = m[0 * 4 + 0] * x + m[1 * 4 + 0] * y + m[2 * 4 + 0] * z + m[3 * 4 + 0];
		float ry = m[0 * 4 + 1] * x + m[1 * 4 + 1] * y + m[2 * 4 + 1] * z + m[3 * 4 + 1];
		if (h != 1) {
			const float invh = 1 / h;
			rx = rx * invh;
			ry = ry * invh;
		}
		Pout[4 * i] = rx;
		Pout[4 * i + 1] = ry;
		Pout[4 * i + 2] = z;
		Pout[4 * i + 3] = w;
	}
}

extern "C" void orc_cull_grid(int cu, int cv, int nkeys, int flags, const float* P, const float* Ng, const float* N,
                              const float* Oi, int zthreshold_black, uint8_t* culled) {
	const int gs = (cu + 1) * (cv + 1);
	std::vector<int> count(gs, 0);
	std::vector<char> cullV(gs, 0);
	const bool bf = (flags & ORC_GRID_CULL_BACKFACING) && Ng;
	if (nkeys <= 1) {
		// CqMicroPolyGrid::Shade: back faces, then the trailing run of black Oi
		if (bf)
			for (int i = gs - 1; i >= 0; i--)
				if (backFacing(P + 4 * i, Ng + 3 * i, N ? N + 3 * i : nullptr)) cullV[i] = 1;
		if ((flags & ORC_GRID_CULL_TRANSPARENT) && Oi && !zthreshold_black)
			for (int i = gs - 1; i >= 0; i--) {
				if (Oi[4 * i] == 0.0f && Oi[4 * i + 1] == 0.0f && Oi[4 * i + 2] == 0.0f) cullV[i] = 1;
				else break;
			}
	} else if (bf) {
		// CqMotionMicroPolyGrid::Split: culled where every key faces away
		for (int k = 0; k < nkeys; ++k)
			for (int i = gs - 1; i >= 0; i--) {
				const long long e = (long long)k * gs + i;
				if (backFacing(P + 4 * e, Ng + 3 * e, N ? N + 3 * e : nullptr)) count[i]++;
			}
		for (int i = 0; i < gs; ++i) cullV[i] = count[i] == nkeys;
	}
	for (int iv = 0; iv < cv; ++iv)
		for (int iu = 0; iu < cu; ++iu)
			if (cullV[iv * (cu + 1) + iu]) culled[iv * cu + iu] = 1;
}
