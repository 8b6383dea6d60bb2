// hider_device.cuh -- per-micropolygon and per-sample arithmetic of the hider.
//
// Every expression keeps the reference's operation order and single-precision
// rounding; the translation units that include this file are compiled with
// -fmad=false so no multiply-add is contracted into an FMA, and with the
// default IEEE division and square root.  References are to aqsis libs/core.
#pragma once

#include <cfloat>
#include <cstdint>

namespace aqh {

// math.h:47-62
__device__ __forceinline__ int lfloor_f(float x) {
	int i = static_cast<int>(x);
	return i - ((x < 0.0f && x != static_cast<float>(i)) ? 1 : 0);
}
__device__ __forceinline__ int lceil_f(float x) {
	int i = static_cast<int>(x);
	return i + ((x > 0.0f && x != static_cast<float>(i)) ? 1 : 0);
}
// Aqsis::min / Aqsis::max (math.h:112-126): a < b ? a : b, a < b ? b : a.
__device__ __forceinline__ float amin(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float amax(float a, float b) { return a < b ? b : a; }

struct V3f { float x, y, z; };

__device__ __forceinline__ V3f ld3(const float4* P, long long i) {
	float4 v = __ldg(P + i);
	return V3f{v.x, v.y, v.z};
}

// CqVector3D::Magnitude2 of a difference (vector3d.h:345-348)
__device__ __forceinline__ float mag2diff(V3f a, V3f b) {
	float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
	return dx * dx + dy * dy + dz * dz;
}

constexpr int kDegeneracyMask = 0x8000000;  // micropolygon.h:791

// CqMicroPolygon::ComputeVertexOrder (micropolygon.cpp:1207-1284).  v[0..3] are
// the grid points at index, index+1, index+cu+1, index+cu+2.
__device__ __forceinline__ int vertex_order(const V3f v[4]) {
	// natural slots: A = v[0], B = v[1], C = v[3] (index+cu+2), D = v[2] (index+cu+1)
	V3f pa = v[0], pb = v[1], pc = v[3], pd = v[2];
	int codeA = 0, codeB = 1, codeC = 3, codeD = 2;
	V3f vA = pa, vB = pb, vC = pc;
	bool degenerate = false;
	if (mag2diff(pa, pb) < 1e-8) {
		// A--B degenerate: B <- C, C <- D
		vB = pc; codeB = codeC; vC = pd; codeC = codeD; degenerate = true;
	} else if (mag2diff(pb, pc) < 1e-8) {
		vB = pc; codeB = codeC; vC = pd; codeC = codeD; degenerate = true;
	} else if (mag2diff(pc, pd) < 1e-8) {
		vC = pd; codeC = codeD; degenerate = true;
	} else if (mag2diff(pd, pa) < 1e-8) {
		degenerate = true;  // the reference only drops D here
	}
	bool flip = ((vA.x - vB.x) * (vB.y - vC.y)) >= ((vA.y - vB.y) * (vB.x - vC.x));
	int code;
	if (!flip) {
		code = degenerate ? ((codeA & 3) | ((codeC & 3) << 2) | ((codeB & 3) << 4) | kDegeneracyMask)
		                  : ((codeA & 3) | ((codeD & 3) << 2) | ((codeC & 3) << 4) | ((codeB & 3) << 6));
	} else {
		code = degenerate ? ((codeA & 3) | ((codeB & 3) << 2) | ((codeC & 3) << 4) | kDegeneracyMask)
		                  : ((codeA & 3) | ((codeB & 3) << 2) | ((codeC & 3) << 4) | ((codeD & 3) << 6));
	}
	return code;
}

// Point-in-polygon coefficients and inverse-bilinear setup: CqHitTestCache as
// filled by CqMicroPolygon::cachePointInPolyTest (micropolygon.cpp:1346-1392)
// and CqInvBilinear::setVertices (bilinear.h:260-275).
struct HitCoeffs {
	float ym[4], xm[4], ex[4], ey[4];
	float ax, ay, e_x, e_y, f_x, f_y, g_x, g_y;
	float z[4];
	bool linear;
};

// CqInvBilinear's "almost rectangular" test `irregularity < 1e-2*patchSize`
// (bilinear.h:271-274), evaluated in double like the reference.  FP64 issues
// slowly on this GPU, so clear cases are decided in float: 0.01f * patch is
// within 2^-22 relative of the double product for normal values, far inside
// the 1e-5 margins, and everything else (near ties, zeros, denormals, inf,
// NaN) takes the double comparison.
__device__ __forceinline__ bool linear_test(float irr, float patch) {
	const float b = 0.01f * patch;
	if (b >= 1e-30f && b <= 1e30f && irr >= 0.0f) {
		if (irr < b * 0.99999f) return true;
		if (irr > b * 1.00001f) return false;
	}
	return static_cast<double>(irr) < 1e-2 * static_cast<double>(patch);
}

__device__ __forceinline__ void hit_setup(const V3f p[4], int code, HitCoeffs& h) {
	h.z[0] = p[0].z; h.z[1] = p[1].z; h.z[2] = p[2].z; h.z[3] = p[3].z;
	// setVertices(A, B, C, D) with A=p0, B=p1, C=p2, D=p3
	h.ax = p[0].x; h.ay = p[0].y;
	h.e_x = p[1].x - p[0].x; h.e_y = p[1].y - p[0].y;
	h.f_x = p[2].x - p[0].x; h.f_y = p[2].y - p[0].y;
	// G = -E - C + D
	h.g_x = ((-h.e_x) - p[2].x) + p[3].x;
	h.g_y = ((-h.e_y) - p[2].y) + p[3].y;
	float patch = amax(amax(fabsf(h.f_x), fabsf(h.f_y)), amax(fabsf(h.e_x), fabsf(h.e_y)));
	float irr = amax(fabsf(h.g_x), fabsf(h.g_y));
	h.linear = linear_test(irr, patch);
	// reorder by the vertex code (selects keep the points in registers)
	auto pick = [&](int k) -> V3f { return k == 0 ? p[0] : (k == 1 ? p[1] : (k == 2 ? p[2] : p[3])); };
	V3f q[4] = {pick((code >> 2) & 3), pick((code >> 4) & 3), pick((code >> 6) & 3), pick(code & 3)};
	int j = 3;
#pragma unroll
	for (int i = 0; i < 4; ++i) {
		h.ym[i] = q[i].x - q[j].x;
		h.xm[i] = q[i].y - q[j].y;
		h.ex[i] = q[j].x;
		h.ey[i] = q[j].y;
		j = i;
	}
	if (code & kDegeneracyMask) {
#pragma unroll
		for (int i = 2; i < 4; ++i) {
			h.ym[i] = q[3].x - q[1].x;
			h.xm[i] = q[3].y - q[1].y;
			h.ex[i] = q[1].x;
			h.ey[i] = q[1].y;
		}
	}
}

// The four edge tests of CqMicroPolygon::fContains (micropolygon.cpp:1295-1332):
// edges 0 and 1 reject on <= 0, edges 2 and 3 on < 0.  The reference's
// starting edge only changes which test fails first, not the answer.
__device__ __forceinline__ bool edges_inside(const float ym[4], const float xm[4], const float ex[4],
                                             const float ey[4], float x, float y) {
	float v0 = ((y - ey[0]) * ym[0]) - ((x - ex[0]) * xm[0]);
	float v1 = ((y - ey[1]) * ym[1]) - ((x - ex[1]) * xm[1]);
	float v2 = ((y - ey[2]) * ym[2]) - ((x - ex[2]) * xm[2]);
	float v3 = ((y - ey[3]) * ym[3]) - ((x - ex[3]) * xm[3]);
	// written as negated rejections so NaN behaves as in the reference
	return !(v0 <= 0.0f) & !(v1 <= 0.0f) & !(v2 < 0.0f) & !(v3 < 0.0f);
}

// CqInvBilinear::operator() (bilinear.h:277-305): one Newton step from the
// centre, a second one unless the micropolygon is almost rectangular.
__device__ __forceinline__ void inv_bilinear(float ax, float ay, float ex, float ey, float fx, float fy, float gx,
                                             float gy, bool linear, float px, float py, float& u, float& v) {
	u = 0.5f;
	v = 0.5f;
#pragma unroll
	for (int it = 0; it < 2; ++it) {
		if (it == 1 && linear) break;
		// M1 = E + G*v, M2 = F + G*u
		float m1x = ex + gx * v, m1y = ey + gy * v;
		float m2x = fx + gx * u, m2y = fy + gy * u;
		// bilinEval(uv) - P = A + E*u + F*v + G*u*v - P
		float bx = (((ax + ex * u) + fx * v) + (gx * u) * v) - px;
		float by = (((ay + ey * u) + fy * v) + (gy * u) * v) - py;
		float det = m1x * m2y - m1y * m2x;
		if (it == 0 || det != 0.0f) det = 1.0f / det;
		float cb2 = bx * m2y - by * m2x;   // cross(b, M2)
		float cb1 = bx * m1y - by * m1x;   // cross(b, M1)
		float du = det * cb2;
		float dv = det * (-cb1);
		u = u - du;
		v = v - dv;
	}
}

// bilerp (bilinear.h:228-236)
__device__ __forceinline__ float bilerp1(float a, float b, float c, float d, float u, float v) {
	float w0 = (1.0f - v) * (1.0f - u);
	float w1 = (1.0f - v) * u;
	float w2 = v * (1.0f - u);
	float w3 = v * u;
	return ((w0 * a + w1 * b) + w2 * c) + w3 * d;
}

// CqMicroPolygon::InterpolateOutputs smooth weights (micropolygon.cpp:1449-1455)
__device__ __forceinline__ void smooth_weights(float u, float v, float w[4]) {
	w[0] = (1.0f - u) * (1.0f - v);
	w[1] = u * (1.0f - v);
	w[2] = (1.0f - u) * v;
	w[3] = u * v;
}

// CqRenderer::GetCircleOfConfusion (renderer.h:401-406)
__device__ __forceinline__ float2 coc(float depth, float mult, float inv_fd, float sx, float sy) {
	float c = mult * fabsf(1.0f / depth - inv_fd);
	return make_float2(sx * c, sy * c);
}

// CqImagePixel::projectToCircle (imagepixel.h:429-436) with CqVector2D::Magnitude
// (vector2d.h:141-147).
__device__ __forceinline__ float2 project_to_circle(float x, float y) {
	float r;
	if (y == 0.0f) r = fabsf(x);
	else if (x == 0.0f) r = fabsf(y);
	else r = sqrtf((x * x) + (y * y));
	if (r == 0.0f) return make_float2(0.0f, 0.0f);
	float adj = amax(fabsf(x), fabsf(y)) / r;
	return make_float2(adj * x, adj * y);
}

// CqTrimLoopArray::TrimPoint (trimcurve.cpp:145-169, 223-237) over the loops
// [l0, l1): per loop the even-odd count of its edges crossing the point's
// row on the left; no loops trims nothing, else a point inside an even
// number of loops is trimmed.
__device__ __forceinline__ bool trim_point(const float2* pts, const int32_t* loop_first, int l0, int l1, float x,
                                           float y) {
	if (l1 == l0) return false;
	int crosses = 0;
	for (int l = l0; l < l1; ++l) {
		const int p0 = __ldg(loop_first + l), n = __ldg(loop_first + l + 1) - p0;
		bool odd = false;
		float2 b = n > 0 ? __ldg(pts + p0 + n - 1) : make_float2(0.0f, 0.0f);
		for (int i = 0; i < n; ++i) {
			const float2 a = __ldg(pts + p0 + i);
			if (((a.y < y) && (b.y >= y)) || ((b.y < y) && (a.y >= y))) {
				if (a.x + (y - a.y) / (b.y - a.y) * (b.x - a.x) < x) odd = !odd;
			}
			b = a;
		}
		crosses += odd ? 1 : 0;
	}
	return !(crosses & 1);
}

// CqTrimLoopArray::LineIntersects (trimcurve.cpp:172-198, 240-253).
__device__ __forceinline__ bool trim_line(const float2* pts, const int32_t* loop_first, int l0, int l1, float2 v1,
                                          float2 v2) {
	const float x1 = v1.x, y1 = v1.y, x2 = v2.x, y2 = v2.y;
	for (int l = l0; l < l1; ++l) {
		const int p0 = __ldg(loop_first + l), n = __ldg(loop_first + l + 1) - p0;
		float2 q4 = n > 0 ? __ldg(pts + p0 + n - 1) : make_float2(0.0f, 0.0f);
		for (int i = 0; i < n; ++i) {
			const float2 q3 = __ldg(pts + p0 + i);
			const float x3 = q3.x, y3 = q3.y, x4 = q4.x, y4 = q4.y;
			q4 = q3;
			const float d = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
			if (d == 0.0f) continue;
			const float r = ((y1 - y3) * (x4 - x3) - (x1 - x3) * (y4 - y3)) / d;
			const float s = ((y1 - y3) * (x2 - x1) - (x1 - x3) * (y2 - y1)) / d;
			if ((r >= 0.0f) && (s >= 0.0f) && (r <= 1.0f) && (s <= 1.0f)) return true;
		}
	}
	return false;
}

// BilinearEvaluate (bilinear.h:189-224) of two-component corners.
__device__ __forceinline__ float2 bilinear_evaluate(float2 A, float2 B, float2 C, float2 D, float s, float t) {
	float2 AB, CD;
	if (s <= 0.0f) {
		AB = A;
		CD = C;
	} else if (s >= 1.0f) {
		AB = B;
		CD = D;
	} else {
		AB = make_float2((B.x - A.x) * s + A.x, (B.y - A.y) * s + A.y);
		CD = make_float2((D.x - C.x) * s + C.x, (D.y - C.y) * s + C.y);
	}
	if (t <= 0.0f) return AB;
	if (t >= 1.0f) return CD;
	return make_float2((CD.x - AB.x) * t + AB.x, (CD.y - AB.y) * t + AB.y);
}

// The triangle split line test of CqMicroPolygon::Sample and
// CqMicroPolygonMotion::Sample (micropolygon.cpp:1630-1654, 1885-1907): line
// (A.x, A.y, B.x, B.y); a hit at (hx, hy) on or behind it misses.
__device__ __forceinline__ bool triangle_keeps(float4 l, float hx, float hy) {
	const float Ax = l.x, Ay = l.y, Bx = l.z, By = l.w;
	const float v = (Ay - By) * hx + (Bx - Ax) * hy + (Ax * By - Bx * Ay);
	return !(v <= 0);
}

// One point of CqMicroPolyGrid::Split's projection (micropolygon.cpp:735-745,
// 1023-1032): matCameraToRaster * P with CqMatrix::operator*(CqVector3D)
// (matrix.h:717-750), x and y divided by h = P.m03 + ... when h != 1; the
// camera-space z is kept.  m: CqMatrix elements m[row*4 + col], points as row
// vectors (x' = x m00 + y m10 + z m20 + m30).
__device__ __forceinline__ float4 project_point(const float* m, float4 p) {
	const float h = ((m[3] * p.x + m[7] * p.y) + m[11] * p.z) + m[15];
	float x = ((m[0] * p.x + m[4] * p.y) + m[8] * p.z) + m[12];
	float y = ((m[1] * p.x + m[5] * p.y) + m[9] * p.z) + m[13];
	if (h != 1.0f) {
		const float invh = 1.0f / h;
		x = x * invh;
		y = y * invh;
	}
	return make_float4(x, y, p.z, p.w);
}


// The motion sampler's staging bound of micropolygon m of grid gi
// (AddMPG, imagebuffer.cpp:514-539): the bound over every key, grown by the
// largest circle of confusion of its depth range, as a conservative pixel
// rectangle [x0, x1) x [y0, y1) with a one-pixel margin over every time slice
// and lens stratum, and its z range.  `keep` is false when the micropolygon
// is culled or outside AddMPG's crop cull window.
struct MbStageBound {
	int x0, x1, y0, y1;
	float mnz, mxz;
	bool keep;
};
__device__ __forceinline__ MbStageBound mb_stage_bound(const FrameParams& fp, const GridsDev& g, int gid, int m) {
	const int cu = __ldg(g.cu + gid), nk = __ldg(g.nkeys + gid);
	const long long nv = (long long)(cu + 1) * (__ldg(g.cv + gid) + 1);
	const long long pb = __ldg(g.pbase + gid);
	const int iv = m / cu, iu = m - iv * cu;
	const int index = iv * (cu + 1) + iu;
	float mnx = FLT_MAX, mny = FLT_MAX, mnz = FLT_MAX, mxx = -FLT_MAX, mxy = -FLT_MAX, mxz = -FLT_MAX;
	for (int k = 0; k < nk; ++k) {
		const long long kb = pb + k * nv + index;
		const V3f a = ld3(g.P, kb), b = ld3(g.P, kb + 1), c = ld3(g.P, kb + cu + 1), d = ld3(g.P, kb + cu + 2);
		mnx = amin(mnx, amin(amin(amin(a.x, b.x), c.x), d.x));
		mny = amin(mny, amin(amin(amin(a.y, b.y), c.y), d.y));
		mnz = amin(mnz, amin(amin(amin(a.z, b.z), c.z), d.z));
		mxx = amax(mxx, amax(amax(amax(a.x, b.x), c.x), d.x));
		mxy = amax(mxy, amax(amax(amax(a.y, b.y), c.y), d.y));
		mxz = amax(mxz, amax(amax(amax(a.z, b.z), c.z), d.z));
	}
	const bool culled = g.culled && g.culled[__ldg(g.mpbase + gid) + m];
	float gx = 0.0f, gy = 0.0f;
	if (fp.use_dof) {
		const float2 c1 = coc(mnz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
		const float2 c2 = coc(mxz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
		gx = amax(c1.x, c2.x);
		gy = amax(c1.y, c2.y);
	}
	const bool cropped = (mxx + gx) < fp.cull_x0 || (mxy + gy) < fp.cull_y0 || (mnx - gx) > fp.cull_x1 ||
	                     (mny - gy) > fp.cull_y1;
	MbStageBound r;
	r.x0 = (int)floorf(mnx - gx) - 1;
	r.x1 = lceil_f(mxx + gx) + 1;
	r.y0 = (int)floorf(mny - gy) - 1;
	r.y1 = lceil_f(mxy + gy) + 1;
	r.mnz = mnz;
	r.mxz = mxz;
	r.keep = !culled && !cropped;
	return r;
}

// The staging bound packed in 16 bytes: the rectangle as int16 pairs
// (clamped to the int16 range, which keeps every comparison with a tile of a
// frame below 32768 pixels), the z range as floats; an empty rectangle when
// the micropolygon is not kept.
__device__ __forceinline__ int4 pack_stage_bound(const MbStageBound& b) {
	auto c16 = [](int v) { return v < -32768 ? -32768 : (v > 32767 ? 32767 : v); };
	int x0 = c16(b.x0), x1 = c16(b.x1), y0 = c16(b.y0), y1 = c16(b.y1);
	if (!b.keep) { x0 = 32767; x1 = -32768; }
	return make_int4((x0 & 0xffff) | (x1 << 16), (y0 & 0xffff) | (y1 << 16), __float_as_int(b.mnz),
	                 __float_as_int(b.mxz));
}
__device__ __forceinline__ MbStageBound unpack_stage_bound(int4 q) {
	MbStageBound b;
	b.x0 = (int)(int16_t)(q.x & 0xffff);
	b.x1 = q.x >> 16;
	b.y0 = (int)(int16_t)(q.y & 0xffff);
	b.y1 = q.y >> 16;
	b.mnz = __int_as_float(q.z);
	b.mxz = __int_as_float(q.w);
	b.keep = b.x0 < b.x1;
	return b;
}

}  // namespace aqh
