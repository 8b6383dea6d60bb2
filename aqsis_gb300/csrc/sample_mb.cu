// sample_mb.cu -- sampling with motion blur and/or depth of field.
//
// Replaces CqBucketProcessor::RenderMPG_MBOrDof (libs/core/bucketprocessor.cpp:
// 1221-1469), CqMicroPolygonMotion::BuildBoundList / Sample
// (micropolygon.cpp:1689-1756, 1768-1914), the depth-of-field branch of
// CqMicroPolygon::Sample (1561-1592) and CqMicroPolygon::dofSampleInBound
// (1531-1550).
//
// The tile's micropolygons are staged into shared-memory records in insertion
// order.  For a moving micropolygon the reference tests a sample once per
// time slice whose window holds the sample's time (and, without depth of
// field, whose sample-index range holds the sample); with depth of field each
// sample belongs to one lens stratum, whose shifted bound decides whether the
// reference visits it.  Frames with transparency (sample_mb_kernel) walk each
// sample's candidates in insertion order, one sample per lane, finding the
// slices by binary search in a per-frame table of the reference's accumulated
// slice times; opaque frames (sample_mbq_kernel) test (slice, sample) pairs in
// parallel and fold the hits (see the section on opaque frames).
#include "aqh_internal.h"
#include "hider_device.cuh"
#include "sample_common.cuh"

namespace aqh {

namespace {


// A candidate's record with room for NK motion keys: frames whose grids have
// at most two keys use two-key records (244 bytes instead of 396), so more
// candidates fit a round.
template <int NK>
struct MbRecT {
	static constexpr int kKeys = NK;
	float bmn[3], bmx[3];          // m_Bound (union of the key bounds for moving micropolygons)
	float key[NK][4][3];           // key vertices in natural order: index, index+1, index+cu+1, index+cu+2
	float kt[NK];                  // key times
	float kbmn[NK][3], kbmx[NK][3];  // per-key bounds
	float cocm[4][2];              // static DoF: CoC multiplier per vertex
	float cocmin[2], cocmax[2];    // DoF: min / max CoC multipliers
	int nkeys, code, id, grid, bits;
};
using MbRec = MbRecT<kMaxKeys>;


struct Bnd {
	float mnx, mny, mnz, mxx, mxy, mxz;
};

template <class R>
__device__ __forceinline__ Bnd key_bound(const R& r, int k) {
	return Bnd{r.kbmn[k][0], r.kbmn[k][1], r.kbmn[k][2], r.kbmx[k][0], r.kbmx[k][1], r.kbmx[k][2]};
}

__device__ __forceinline__ void encapsulate(Bnd& a, const Bnd& b) {
	a.mnx = amin(a.mnx, b.mnx); a.mny = amin(a.mny, b.mny); a.mnz = amin(a.mnz, b.mnz);
	a.mxx = amax(a.mxx, b.mxx); a.mxy = amax(a.mxy, b.mxy); a.mxz = amax(a.mxz, b.mxz);
}

// CqMicroPolygon::dofSampleInBound (micropolygon.cpp:1531-1550)
__device__ __forceinline__ bool dof_in_bound(const Bnd& b, float cminx, float cminy, float cmaxx, float cmaxy,
                                             float px, float py, float dx, float dy) {
	float lox = px + cminx * dx, loy = py + cminy * dy;
	float hix = px + cmaxx * dx, hiy = py + cmaxy * dy;
	if (dx < 0) { float t = lox; lox = hix; hix = t; }
	if (dy < 0) { float t = loy; loy = hiy; hiy = t; }
	// CqBound::Intersects (bound.h:153-160)
	return !(lox > b.mxx || loy > b.mxy || hix < b.mnx || hiy < b.mny);
}

// Hit test of one sample against one micropolygon: CqMicroPolygon::Sample
// (static, with DoF) or CqMicroPolygonMotion::Sample.  On a hit returns depth
// and (u,v).  With `gt`, a static micropolygon marked trimmed also takes the
// trim test (the motion form has none, micropolygon.cpp:1876-1882).
template <class R>
__device__ bool mb_sample(const FrameParams& fp, const R& r, bool moving, bool dof, float px, float py,
                          float time, float dx, float dy, float& D, float& u, float& v, const float4* tri = nullptr,
                          const GridsDev* gt = nullptr) {
	V3f pts[4];
	if (!moving) {
		// dof only (the static no-DoF case never reaches this kernel)
		Bnd b{r.bmn[0], r.bmn[1], r.bmn[2], r.bmx[0], r.bmx[1], r.bmx[2]};
		if (!dof_in_bound(b, r.cocmin[0], r.cocmin[1], r.cocmax[0], r.cocmax[1], px, py, dx, dy)) return false;
#pragma unroll
		for (int i = 0; i < 4; ++i) {
			const float ox = r.cocm[i][0] * dx, oy = r.cocm[i][1] * dy;
			pts[i] = V3f{r.key[0][i][0] - ox, r.key[0][i][1] - oy, r.key[0][i][2] - 0.0f};
		}
	} else {
		int iIndex = 0;
		float Fraction = 0.0f;
		bool Exact = true;
		const int n = r.nkeys;
		if (time > r.kt[0]) {
			if (time >= r.kt[n - 1]) {
				iIndex = n - 1;
			} else {
				iIndex = 0;
				while (time >= r.kt[iIndex + 1]) iIndex += 1;
				Fraction = (time - r.kt[iIndex]) / (r.kt[iIndex + 1] - r.kt[iIndex]);
				Exact = (r.kt[iIndex] == time);
			}
		}
		Bnd tight;
		if (Exact) {
			tight = key_bound(r, iIndex);
		} else {
			const Bnd b1 = key_bound(r, iIndex), b2 = key_bound(r, iIndex + 1);
			const float f1 = 1.0f - Fraction;
			tight.mnx = f1 * b1.mnx + Fraction * b2.mnx;
			tight.mny = f1 * b1.mny + Fraction * b2.mny;
			tight.mnz = f1 * b1.mnz + Fraction * b2.mnz;
			tight.mxx = f1 * b1.mxx + Fraction * b2.mxx;
			tight.mxy = f1 * b1.mxy + Fraction * b2.mxy;
			tight.mxz = f1 * b1.mxz + Fraction * b2.mxz;
		}
		if (dof) {
			if (!dof_in_bound(tight, r.cocmin[0], r.cocmin[1], r.cocmax[0], r.cocmax[1], px, py, dx, dy)) return false;
		} else {
			if ((px < tight.mnx || px > tight.mxx) || (py < tight.mny || py > tight.mxy)) return false;
		}
		if (Exact) {
#pragma unroll
			for (int i = 0; i < 4; ++i)
				pts[i] = V3f{r.key[iIndex][i][0], r.key[iIndex][i][1], r.key[iIndex][i][2]};
		} else {
			const float F1 = 1.0f - Fraction;
#pragma unroll
			for (int i = 0; i < 4; ++i)
				pts[i] = V3f{(F1 * r.key[iIndex][i][0]) + (Fraction * r.key[iIndex + 1][i][0]),
				             (F1 * r.key[iIndex][i][1]) + (Fraction * r.key[iIndex + 1][i][1]),
				             (F1 * r.key[iIndex][i][2]) + (Fraction * r.key[iIndex + 1][i][2])};
		}
		if (dof) {
#pragma unroll
			for (int i = 0; i < 4; ++i) {
				const float2 c = coc(pts[i].z, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
				pts[i].x = pts[i].x - c.x * dx;
				pts[i].y = pts[i].y - c.y * dy;
				pts[i].z = pts[i].z - 0.0f;
			}
		}
	}
	HitCoeffs h;
	hit_setup(pts, r.code, h);
	if (!edges_inside(h.ym, h.xm, h.ex, h.ey, px, py)) return false;
	inv_bilinear(h.ax, h.ay, h.e_x, h.e_y, h.f_x, h.f_y, h.g_x, h.g_y, h.linear, px, py, u, v);
	D = bilerp1(h.z[0], h.z[1], h.z[2], h.z[3], u, v);
	if (gt && !moving && (r.bits & 32) && trim_rejects(*gt, r.id, r.grid, u, v)) return false;
	if (tri && (r.bits & 4)) {
		// triangle split line at the sample time (TriangleSplitPoints,
		// micropolygon.cpp:895-900, over CqMotionSpec::GetMotionObjectInterpolated,
		// motion.h:176-228); with depth of field the hit moves back by the
		// CoC at its depth (micropolygon.cpp:1891-1900)
		const float4* L = tri + (long long)r.grid * kMaxKeys;
		const int n = r.nkeys;
		int i = 0;
		float F = 0.0f;
		bool exact = true;
		if (n > 1) {
			if (time >= r.kt[n - 1]) {
				i = n - 1;
			} else if (time <= r.kt[0]) {
				i = 0;
			} else {
				while (time >= r.kt[i + 1]) i += 1;
				F = (time - r.kt[i]) / (r.kt[i + 1] - r.kt[i]);
				exact = (r.kt[i] == time);
			}
		}
		float4 l = __ldg(L + i);
		if (!exact) {
			const float4 l1 = __ldg(L + i + 1);
			l = make_float4(((1.0f - F) * l.x) + (F * l1.x), ((1.0f - F) * l.y) + (F * l1.y),
			                ((1.0f - F) * l.z) + (F * l1.z), ((1.0f - F) * l.w) + (F * l1.w));
		}
		float hx = px, hy = py;
		if (dof) {
			const float2 c = coc(D, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
			hx = hx + c.x * dx;
			hy = hy + c.y * dy;
		}
		if (!triangle_keeps(l, hx, hy)) return false;
	}
	return true;
}

// Load the record of micropolygon m of grid gi from global memory.
template <class R>
__device__ void load_mb_record(const FrameParams& fp, const GridsDev& g, int gi, int m, R& r) {
	const int cu = __ldg(g.cu + gi), cv = __ldg(g.cv + gi);
	// at most the record's keys (the host sends a frame to two-key records
	// only when no grid has more)
	const int nk = min(__ldg(g.nkeys + gi), R::kKeys);
	const long long nv = (long long)(cu + 1) * (cv + 1);
	const long long pb = __ldg(g.pbase + gi);
	const int iv = m / cu, iu = m - iv * cu;
	const int index = iv * (cu + 1) + iu;
	const int vi[4] = {index, index + 1, index + cu + 1, index + cu + 2};
	r.nkeys = nk;
	for (int k = 0; k < nk; ++k) {
		for (int q = 0; q < 4; ++q) {
			const V3f p = ld3(g.P, pb + k * nv + vi[q]);
			r.key[k][q][0] = p.x; r.key[k][q][1] = p.y; r.key[k][q][2] = p.z;
		}
		// CqMovingMicroPolygonKey::GetBound (micropolygon.cpp:1974-1989)
		for (int c = 0; c < 3; ++c) {
			r.kbmn[k][c] = amin(r.key[k][0][c], amin(r.key[k][1][c], amin(r.key[k][2][c], r.key[k][3][c])));
			r.kbmx[k][c] = amax(r.key[k][0][c], amax(r.key[k][1][c], amax(r.key[k][2][c], r.key[k][3][c])));
		}
		r.kt[k] = (nk > 1) ? __ldg(g.times + __ldg(g.tbase + gi) + k) : 0.0f;
	}
	V3f v0[4];
	for (int q = 0; q < 4; ++q) v0[q] = V3f{r.key[0][q][0], r.key[0][q][1], r.key[0][q][2]};
	r.code = vertex_order(v0);
	if (nk == 1) {
		// CalculateBound: min(min(min(A,B),C),D) with C = index+cu+2 (slot 3), D = index+cu+1 (slot 2)
		for (int c = 0; c < 3; ++c) {
			r.bmn[c] = amin(amin(amin(r.key[0][0][c], r.key[0][1][c]), r.key[0][3][c]), r.key[0][2][c]);
			r.bmx[c] = amax(amax(amax(r.key[0][0][c], r.key[0][1][c]), r.key[0][3][c]), r.key[0][2][c]);
		}
	} else {
		// AppendKey: encapsulate key bounds in key order (micropolygon.cpp:1952-1967)
		for (int c = 0; c < 3; ++c) { r.bmn[c] = r.kbmn[0][c]; r.bmx[c] = r.kbmx[0][c]; }
		for (int k = 1; k < nk; ++k)
			for (int c = 0; c < 3; ++c) { r.bmn[c] = amin(r.bmn[c], r.kbmn[k][c]); r.bmx[c] = amax(r.bmx[c], r.kbmx[k][c]); }
	}
	if (!fp.use_dof) {
		// no lens offsets: a static micropolygon is tested at its own vertices
		for (int q = 0; q < 4; ++q) r.cocm[q][0] = r.cocm[q][1] = 0.0f;
		r.cocmin[0] = r.cocmin[1] = r.cocmax[0] = r.cocmax[1] = 0.0f;
	} else {
		if (nk == 1) {
			// CacheHitTestValues with DoF (micropolygon.cpp:1409-1422)
			for (int q = 0; q < 4; ++q) {
				const float2 c = coc(r.key[0][q][2], fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
				r.cocm[q][0] = c.x;
				r.cocm[q][1] = c.y;
			}
			r.cocmin[0] = amin(amin(r.cocm[0][0], r.cocm[1][0]), amin(r.cocm[2][0], r.cocm[3][0]));
			r.cocmin[1] = amin(amin(r.cocm[0][1], r.cocm[1][1]), amin(r.cocm[2][1], r.cocm[3][1]));
			r.cocmax[0] = amax(amax(r.cocm[0][0], r.cocm[1][0]), amax(r.cocm[2][0], r.cocm[3][0]));
			r.cocmax[1] = amax(amax(r.cocm[0][1], r.cocm[1][1]), amax(r.cocm[2][1], r.cocm[3][1]));
		} else {
			// CqMicroPolygonMotion::CacheHitTestValues (micropolygon.cpp:1916-1940) with
			// CqRenderer::MinCoCForBound (renderer.cpp:1602-1617)
			const float2 c1 = coc(r.bmn[2], fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
			const float2 c2 = coc(r.bmx[2], fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
			const float z1 = r.bmn[2], z2 = r.bmx[2];
			const float focalDist = 1 / fp.dof_inv_fd;
			bool zero;
			if ((z1 - focalDist) * (z2 - focalDist) < 0) {
				zero = true;
			} else {
				const float minBlur = amin(fabsf(1 / z1 - fp.dof_inv_fd), fabsf(1 / z2 - fp.dof_inv_fd));
				zero = (fp.dof_mult * amin(fp.dof_scale_x, fp.dof_scale_y) * minBlur) == 0;
			}
			if (zero) { r.cocmin[0] = 0.0f; r.cocmin[1] = 0.0f; }
			else { r.cocmin[0] = amin(c1.x, c2.x); r.cocmin[1] = amin(c1.y, c2.y); }
			r.cocmax[0] = amax(c1.x, c2.x);
			r.cocmax[1] = amax(c1.y, c2.y);
		}
	}
}

// Record of micropolygon m of grid gi with its occluding flag
// (SqMpgSampleInfo::isOpaque, micropolygon.cpp:1477-1529) and global id.
template <class R>
__device__ __forceinline__ void build_mb_record(const FrameParams& fp, const GridsDev& g, int gi, int m, R& rr) {
	load_mb_record(fp, g, gi, m, rr);
	const int gflags = __ldg(g.flags + gi);
	bool opaque = true;
	const bool smooth = (gflags & 1) != 0;
	if (!(gflags & 8) && g.Oi) {
		const int cu = __ldg(g.cu + gi);
		const int iv = m / cu, iu = m - iv * cu;
		const int index = iv * (cu + 1) + iu;
		const long long cb = __ldg(g.cbase + gi);
		const int vi[4] = {index, index + 1, index + cu + 1, index + cu + 2};
		for (int q = 0; q < (smooth ? 4 : 1); ++q) {
			const float4 o = ld_colour(g, g.Oi, cb + vi[q]);
			opaque = opaque && (o.x >= 1.0f && o.y >= 1.0f && o.z >= 1.0f);
		}
	}
	// bits: 2 occluding, 4 triangular, 8 level-of-detail test, 16 CSG (never
	// occlusion-cullable, never occluding), 32 marked trimmed
	const bool csg = csg_grid(g, gi);
	rr.id = (int)(__ldg(g.mpbase + gi) + m);
	rr.bits = ((!csg && (opaque || (gflags & 4))) ? 2 : 0) | ((gflags & 16) ? 4 : 0) |
	          (lod_active(fp, g, gi) ? 8 : 0) | (csg ? 16 : 0) |
	          ((g.trim.nsets > 0 && __ldg(g.trim.mark + rr.id)) ? 32 : 0);
	rr.grid = gi;
}

// Position, time, lens offset and lens stratum of sample j of pixel (px, py)
// (CqImagePixel::setSamples, imagepixel.cpp:334-359: the lens offset of
// sample j is the one whose shuffled index is j).
__device__ __forceinline__ void mb_sample_attrs(const FrameParams& fp, const SamplerDev& smp, int px, int py, int j,
                                                long long pix, float& x, float& y, float& stime, float& sdx,
                                                float& sdy, int& kinv) {
	const int spp = fp.spp;
	const long long pp = smp.pos_index ? (long long)__ldg(smp.pos_index + pix) : pix;
	const long long tp = smp.time_index ? (long long)__ldg(smp.time_index + pix) : pix;
	const long long dp = smp.dof_index ? (long long)__ldg(smp.dof_index + pix) : pix;
	const long long sp = smp.shuffle_index ? (long long)__ldg(smp.shuffle_index + pix) : pix;
	const float2 o = __ldg(smp.pos + pp * spp + j);
	x = (float)px + o.x;
	y = (float)py + o.y;
	const float tt = smp.time ? __ldg(smp.time + tp * spp + j) : 0.0f;
	stime = (fp.shutter_close - fp.shutter_open) * tt + fp.shutter_open;
	kinv = j;
	if (smp.shuffle)
		for (int q = 0; q < spp; ++q)
			if (__ldg(smp.shuffle + sp * spp + q) == j) kinv = q;
	sdx = 0.0f;
	sdy = 0.0f;
	if (smp.dof) {
		const float2 d = __ldg(smp.dof + dp * spp + kinv);
		const float2 c = project_to_circle(-1.0f + 2.0f * d.x, -1.0f + 2.0f * d.y);
		sdx = c.x;
		sdy = c.y;
	}
}

// Final value of one sample: the occluding hit's colour at its (u,v) --
// the winner's hit test repeated at the sample's time and lens offset -- or
// the Combine of its fragments; written to the sample store.
// (u,v) of a hit that mb_sample reported for micropolygon m of grid gi at
// sample (x, y, time, lens offset dx, dy): the same vertices (the keys around
// the time, interpolated, shifted by the CoC under depth of field), vertex
// order and inverse bilinear, built in registers from the grid's arrays
// rather than from a record.  The bound tests mb_sample makes first passed
// for this sample and change nothing here.
__device__ __forceinline__ void mb_hit_uv(const FrameParams& fp, const GridsDev& g, int gi, int m, float x, float y,
                                          float time, float dx, float dy, float& u, float& v) {
	const int cu = __ldg(g.cu + gi), cv = __ldg(g.cv + gi);
	const int nk = __ldg(g.nkeys + gi);
	const long long nv = (long long)(cu + 1) * (cv + 1);
	const long long pb = __ldg(g.pbase + gi);
	const int iv = m / cu, iu = m - iv * cu;
	const int index = iv * (cu + 1) + iu;
	const int vi[4] = {index, index + 1, index + cu + 1, index + cu + 2};
	V3f k0[4];
#pragma unroll
	for (int q = 0; q < 4; ++q) k0[q] = ld3(g.P, pb + vi[q]);
	V3f pts[4];
	if (nk == 1) {
		// CacheHitTestValues: each vertex moves by its own CoC times the lens offset
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			float cx = 0.0f, cy = 0.0f;
			if (fp.use_dof) {
				const float2 c = coc(k0[q].z, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
				cx = c.x;
				cy = c.y;
			}
			const float ox = cx * dx, oy = cy * dy;
			pts[q] = V3f{k0[q].x - ox, k0[q].y - oy, k0[q].z - 0.0f};
		}
	} else {
		// the key span of CqMicroPolygonMotion::Sample (micropolygon.cpp:1786-1806)
		const float* kt = g.times + __ldg(g.tbase + gi);
		int iIndex = 0;
		float Fraction = 0.0f;
		bool Exact = true;
		if (time > __ldg(kt)) {
			if (time >= __ldg(kt + nk - 1)) {
				iIndex = nk - 1;
			} else {
				while (time >= __ldg(kt + iIndex + 1)) iIndex += 1;
				const float t0 = __ldg(kt + iIndex), t1 = __ldg(kt + iIndex + 1);
				Fraction = (time - t0) / (t1 - t0);
				Exact = (t0 == time);
			}
		}
		V3f a[4];
#pragma unroll
		for (int q = 0; q < 4; ++q) a[q] = ld3(g.P, pb + iIndex * nv + vi[q]);
		if (Exact) {
#pragma unroll
			for (int q = 0; q < 4; ++q) pts[q] = a[q];
		} else {
			const float F1 = 1.0f - Fraction;
#pragma unroll
			for (int q = 0; q < 4; ++q) {
				const V3f b = ld3(g.P, pb + (iIndex + 1) * nv + vi[q]);
				pts[q] = V3f{(F1 * a[q].x) + (Fraction * b.x), (F1 * a[q].y) + (Fraction * b.y),
				             (F1 * a[q].z) + (Fraction * b.z)};
			}
		}
		if (fp.use_dof) {
#pragma unroll
			for (int q = 0; q < 4; ++q) {
				const float2 c = coc(pts[q].z, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
				pts[q].x = pts[q].x - c.x * dx;
				pts[q].y = pts[q].y - c.y * dy;
				pts[q].z = pts[q].z - 0.0f;
			}
		}
	}
	HitCoeffs h;
	hit_setup(pts, vertex_order(k0), h);
	inv_bilinear(h.ax, h.ay, h.e_x, h.e_y, h.f_x, h.f_y, h.g_x, h.g_y, h.linear, x, y, u, v);
}

template <bool TRANSP>
__device__ __forceinline__ void mb_resolve(const FrameParams& fp, const GridsDev& g, const FragPool& pool,
                                           const SampleStore& st, long long sidx, long long aidx, float x, float y,
                                           float stime, float sdx, float sdy, float ozv, int w, int head) {
	float occl[7] = {0, 0, 0, 0, 0, 0, 0};
	int occl_flags = 0;
	if (w >= 0) {
		const int gi = grid_of(g, w);
		const int m = w - (int)__ldg(g.mpbase + gi);
		float u, v;
		mb_hit_uv(fp, g, gi, m, x, y, stime, sdx, sdy, u, v);
		hit_colour(g, gi, m, u, v, occl, occl_flags);
		occl[6] = (TRANSP && fp.midpoint_store) ? st.hitz[sidx] : ozv;
	}
	int nf = 0;
	bool valid = w >= 0;
	int src = w;
	if (TRANSP && head >= 0) {
		bool emptied = false;
		nf = combine_fragments(fp, g, pool, head, w >= 0, ozv, occl, occl_flags, w, src, emptied);
		valid = !emptied;
	}
	if (nf == 0 && valid) {
		if (occl_flags & 1)
			for (int q = 0; q < 6; ++q) occl[q] = 0.0f;
		if (fp.depth_filter == 1) occl[6] = (float)(0.5 * ((double)occl[6] + (double)ozv));
	}
	st.a[aidx] = make_float4(occl[0], occl[1], occl[2], occl[6]);
	st.b[aidx] = make_float4(occl[3], occl[4], occl[5], valid ? 1.0f : 0.0f);
	if (st.aovsrc) st.aovsrc[aidx] = valid ? src : -1;
	if (st.winner) st.winner[sidx] = w;
	if (st.occlz) st.occlz[sidx] = ozv;
	if (st.nfrag) st.nfrag[sidx] = nf;
}

constexpr int kThreadsM = 512;
constexpr int kWarpsM = kThreadsM / 32;
constexpr int kSlotsM = 128;
constexpr int kWordsM = kSlotsM / 32;
constexpr int kTilePixM = 256;
constexpr int kTileSampM = 4096;

struct SmemM {
	MbRec rec[kSlotsM];
	uint32_t mask[kTilePixM][kWordsM];
	int2 pend[kSlotsM];
	int qgrid[kThreadsM];
	int qcum[kThreadsM + 1];
	int qsub[kThreadsM];
	int warp_tot[32];
	int first_reject;
	int qn;
	float dofb[AQH_MAX_SPP_DEV][4];
	float soz[kTileSampM];
	int swin[kTileSampM];
};

__device__ __forceinline__ float warp_max_m(float v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
	return v;
}

// Sub-bound count of a moving micropolygon (CqMicroPolygonMotion::BuildBoundList,
// micropolygon.cpp:1703-1713).
template <class R>
__device__ __forceinline__ int motion_divisions(const R& r, int timeRanges) {
	const float cx = r.kbmx[0][0] - r.kbmn[0][0], cy = r.kbmx[0][1] - r.kbmn[0][1];
	// CqVector2D::Magnitude2 (vector2d.h:132-138)
	const float polyLen2 = (cy == 0.0f) ? cx * cx : ((cx == 0.0f) ? cy * cy : (cx * cx) + (cy * cy));
	const float mx = r.key[0][0][0] - r.key[r.nkeys - 1][0][0];
	const float my = r.key[0][0][1] - r.key[r.nkeys - 1][0][1];
	const float moveDist2 = (my == 0.0f) ? mx * mx : ((mx == 0.0f) ? my * my : (mx * mx) + (my * my));
	// lfloor gives a long that max<TqInt> narrows to int: values beyond int
	// range (an unmoving-sized key bound, inf, NaN) come out as 1
	const float q = sqrtf(moveDist2 / polyLen2);
	const int plm = (q < 2147483648.0f) ? max(1, lfloor_f(q)) : 1;
	return min(plm, timeRanges);
}

// First key index with time >= T (the reference's `endKey` after its while
// loop at time T, micropolygon.cpp:1724-1725).
template <class R>
__device__ __forceinline__ int end_key_at(const R& r, float T) {
	int e = 1;
	while (T > r.kt[e] && e < r.nkeys - 1) ++e;
	return e;
}

// Key bounds interpolated at time T between keys e-1 and e (the `mid` bound).
template <class R>
__device__ __forceinline__ Bnd mid_at(const R& r, int e, float T) {
	const Bnd end0 = key_bound(r, e - 1), end1 = key_bound(r, e);
	const float mix = (T - r.kt[e - 1]) / (r.kt[e] - r.kt[e - 1]);
	Bnd mid = end0;
	mid.mnx = mid.mnx + mix * (end1.mnx - end0.mnx);
	mid.mny = mid.mny + mix * (end1.mny - end0.mny);
	mid.mnz = mid.mnz + mix * (end1.mnz - end0.mnz);
	mid.mxx = mid.mxx + mix * (end1.mxx - end0.mxx);
	mid.mxy = mid.mxy + mix * (end1.mxy - end0.mxy);
	mid.mxz = mid.mxz + mix * (end1.mxz - end0.mxz);
	return mid;
}

// Sub-bound b of a moving micropolygon with `div` slices, computed directly:
// the running bound of BuildBoundList at iteration b is the previous slice's
// `mid` (or key 0's bound) grown by this slice's `mid` and the keys the slice
// passes.  `T` is the per-frame table of the reference's accumulated slice end
// times for `div` slices.
template <class R>
__device__ Bnd sub_bound(const R& r, const float* T, int b) {
	Bnd bound;
	int startKey;
	if (b == 0) {
		bound = key_bound(r, 0);
		startKey = 0;
	} else {
		const int ep = end_key_at(r, T[b - 1]);
		bound = mid_at(r, ep, T[b - 1]);
		startKey = ep - 1;
	}
	const int e = end_key_at(r, T[b]);
	encapsulate(bound, mid_at(r, e, T[b]));
	while (startKey < e - 1) {
		startKey++;
		encapsulate(bound, key_bound(r, startKey));
	}
	return bound;
}

// Phase A of the motion blur / depth of field kernels: stream the
// super-tile's grid list from the cursor (lp, r0, qtotal) and stage, in
// insertion order, the micropolygons whose bound over the whole shutter --
// grown by the largest circle of confusion in their depth range -- meets the
// tile and passes AddMPG's crop cull.  A grid's strips (binning) restrict it
// to the columns and rows of micropolygons that can reach the tile.  With
// `blk` (opaque frames: the largest occluding depth of each row's 4-pixel
// blocks at the round's start), a micropolygon behind every sample its
// rectangle covers is not staged: each of its slices' bounds has a min z at
// or above its own min z less a rounding margin (the slice bounds interpolate
// key bounds; 1e-6 of the largest |z| is several ulps of it), so every one of
// its tests would fail early-z.  Returns true when the list is exhausted.
template <int kSlots, class Smem, int kThreads = kThreadsM>
__device__ __forceinline__ bool stage_mb(const FrameParams& fp, const GridsDev& g, const BinBuffers& bb, Smem& sm,
                                         int tpx0, int tpy0, int tpx1, int tpy1, int lend, int& lp, int& r0,
                                         int& qtotal, int& npend, const float* blk = nullptr) {
	const int t = threadIdx.x;
	const bool usingDof = fp.use_dof != 0;
	while (npend < kSlots) {
		if (r0 >= qtotal) {
			if (lp >= lend) return true;
			const int li = lp + t;
			int gid = -1, nmp = 0, sub = -1;  // sub: first column, first row, width; -1 = whole grid
			bool f = false;
			if (li < lend) {
				gid = bb.st_list[li];
				const int4 rc = bb.grid_rect[gid];
				f = rc.x < rc.y && rc.x < tpx1 && rc.y > tpx0 && rc.z < tpy1 && rc.w > tpy0;
			}
			if (f) {
				const int cu = __ldg(g.cu + gid), cv = __ldg(g.cv + gid);
				nmp = cu * cv;
				if (bb.strips && __ldg(bb.strips + (long long)gid * 64 + 63)) {
					const uint32_t* S = bb.strips + (long long)gid * 64;
					int iu0 = 64, iu1 = -1, iv0 = 64, iv1 = -1;
					for (int k = 0; k < cu; ++k) {
						const uint32_t w = __ldg(S + k);
						if ((int)(int16_t)(w & 0xffffu) < tpx1 && (int)(int16_t)(w >> 16) > tpx0) {
							iu0 = min(iu0, k);
							iu1 = k;
						}
					}
					for (int k = 0; k < cv; ++k) {
						const uint32_t w = __ldg(S + 32 + k);
						if ((int)(int16_t)(w & 0xffffu) < tpy1 && (int)(int16_t)(w >> 16) > tpy0) {
							iv0 = min(iv0, k);
							iv1 = k;
						}
					}
					if (iu1 < 0 || iv1 < 0) {
						f = false;
						nmp = 0;
					} else {
						nmp = (iu1 - iu0 + 1) * (iv1 - iv0 + 1);
						sub = iu0 | (iv0 << 8) | ((iu1 - iu0 + 1) << 16);
					}
				}
			}
			int total, sum;
			const int pos = block_excl_scan(sm.warp_tot, f, total);
			__syncthreads();
			const int pre = block_excl_sum(sm.warp_tot, nmp, sum);
			if (f) {
				sm.qgrid[pos] = gid;
				sm.qcum[pos] = pre;
				sm.qsub[pos] = sub;
			}
			if (t == 0) {
				sm.qcum[total] = sum;
				sm.qn = total;
			}
			__syncthreads();
			qtotal = sm.qcum[sm.qn];
			r0 = 0;
			lp += kThreads;
			continue;
		}
		const int p = r0 + t;
		bool active = false;
		int gid = 0, m = 0;
		if (p < qtotal) {
			int lo = 0, hi = sm.qn - 1;
			while (lo < hi) {
				const int mid = (lo + hi + 1) >> 1;
				if (sm.qcum[mid] <= p) lo = mid; else hi = mid - 1;
			}
			gid = sm.qgrid[lo];
			m = p - sm.qcum[lo];
			const int cu = __ldg(g.cu + gid), nk = __ldg(g.nkeys + gid);
			const int sub = sm.qsub[lo];
			if (sub >= 0) {
				const int w = sub >> 16;
				m = (((sub >> 8) & 0xff) + m / w) * cu + ((sub & 0xff) + m % w);
			}
			(void)nk;
			// conservative pixel rectangle over every time slice and lens stratum
			const MbStageBound sb = bb.mp_bounds ? unpack_stage_bound(bb.mp_bounds[__ldg(g.mpbase + gid) + m])
			                                     : mb_stage_bound(fp, g, gid, m);
			const float mnz = sb.mnz, mxz = sb.mxz;
			const int sX = max(sb.x0, tpx0), eX = min(sb.x1, tpx1);
			const int sY = max(sb.y0, tpy0), eY = min(sb.y1, tpy1);
			active = sb.keep && sX < eX && sY < eY;
			if (active && blk) {
				float zmax = -FLT_MAX;
				for (int y = sY; y < eY; ++y)
					for (int b = (sX - tpx0) >> 2; b <= (eX - 1 - tpx0) >> 2; ++b)
						zmax = fmaxf(zmax, blk[(y - tpy0) * 4 + b]);
				const double margin = 1e-6 * (double)fmaxf(fabsf(mnz), fabsf(mxz));
				if ((double)mnz - margin > (double)zmax) active = false;
			}
		}
		int total;
		const int rank = block_excl_scan(sm.warp_tot, active, total);
		const int navail = kSlots - npend;
		if (t == 0) sm.first_reject = kThreads;
		__syncthreads();
		if (active && rank == navail) sm.first_reject = t;
		if (active && rank < navail) sm.pend[npend + rank] = make_int2(gid, m);
		__syncthreads();
		const int consumed = (total > navail) ? sm.first_reject : min(kThreads, qtotal - r0);
		npend += min(total, navail);
		r0 += consumed;
	}
	return false;
}

template <bool TRANSP>
__global__ void __launch_bounds__(kThreadsM, 1)
sample_mb_kernel(FrameParams fp, GridsDev g, SamplerDev smp, BinBuffers bb, SampleStore st, FragPool pool,
                 const float4* dof_bounds, const float* slice_times) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	SmemM& sm = *reinterpret_cast<SmemM*>(smem_raw);
	int32_t* fhead = reinterpret_cast<int32_t*>(smem_raw + sizeof(SmemM));

	const int tile = blockIdx.x;
	const int tx = tile % fp.ntx, ty = tile / fp.ntx;
	const int tpx0 = fp.sx0 + tx * fp.tile_w, tpy0 = fp.sy0 + ty * fp.tile_h;
	const int tpx1 = min(tpx0 + fp.tile_w, fp.sx0 + fp.sw), tpy1 = min(tpy0 + fp.tile_h, fp.sy0 + fp.sh);
	const int st_idx = (ty / fp.st_tiles) * fp.nstx + (tx / fp.st_tiles);
	const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
	const int spp = fp.spp;
	const int tpix = fp.tile_w * fp.tile_h;
	const int tsamp = tpix * spp;
	const int ngroups = (tsamp + 31) >> 5;
	const int cullable = fp.cullable;
	const bool usingDof = fp.use_dof != 0;
	const float opentime = fp.shutter_open, closetime = fp.shutter_close;
	// isClose (math.h:174-182) and timePerSample (bucketprocessor.cpp:1237-1246)
	const float dclose = fabsf(closetime - opentime);
	const float tol = 10 * FLT_EPSILON;
	const bool fastShutter = dclose <= tol * fabsf(closetime) || dclose <= tol * fabsf(opentime);
	const float timePerSample = fastShutter ? 0.0f : (float)spp / (closetime - opentime);
	const int timeRanges = max(4, spp);

	for (int i = t; i < spp; i += kThreadsM) {
		const float4 b = dof_bounds[i];
		sm.dofb[i][0] = b.x; sm.dofb[i][1] = b.y; sm.dofb[i][2] = b.z; sm.dofb[i][3] = b.w;
	}
	for (int i = t; i < tsamp; i += kThreadsM) {
		sm.soz[i] = FLT_MAX;
		sm.swin[i] = -1;
		if (TRANSP) fhead[i] = -1;
	}
	for (int i = t; i < kTilePixM * kWordsM; i += kThreadsM) (&sm.mask[0][0])[i] = 0u;
	if (t == 0) { sm.qn = 0; sm.qcum[0] = 0; }
	__syncthreads();

	const int lbeg = bb.st_offset[st_idx * bb.nranges];
	const int lend = (int)min((long long)bb.st_offset[(st_idx + 1) * bb.nranges], (long long)bb.list_capacity);
	int lp = lbeg, r0 = 0, qtotal = 0, npend = 0;
	for (;;) {
		// ---- phase A ----
		const bool exhausted =
		    stage_mb<kSlotsM>(fp, g, bb, sm, tpx0, tpy0, tpx1, tpy1, lend, lp, r0, qtotal, npend);
		if (npend == 0) break;

		// ---- records, one per thread ----
		for (int slot = t; slot < npend; slot += kThreadsM) {
			const int2 e = sm.pend[slot];
			MbRec& rr = sm.rec[slot];
			build_mb_record(fp, g, e.x, e.y, rr);
			float gx = 0.0f, gy = 0.0f;
			if (usingDof) {
				const float2 c1 = coc(rr.bmn[2], fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
				const float2 c2 = coc(rr.bmx[2], fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
				gx = amax(c1.x, c2.x);
				gy = amax(c1.y, c2.y);
			}
			const int sX = max((int)floorf(rr.bmn[0] - gx) - 1, tpx0), eX = min(lceil_f(rr.bmx[0] + gx) + 1, tpx1);
			const int sY = max((int)floorf(rr.bmn[1] - gy) - 1, tpy0), eY = min(lceil_f(rr.bmx[1] + gy) + 1, tpy1);
			const uint32_t bit = 1u << (slot & 31);
			const int wd = slot >> 5;
			for (int yy = sY; yy < eY; ++yy)
				for (int xx = sX; xx < eX; ++xx)
					atomicOr(&sm.mask[(yy - tpy0) * fp.tile_w + (xx - tpx0)][wd], bit);
		}
		__syncthreads();

		// ---- phase B: lane per sample, candidates in insertion order ----
		for (int gq = warp; gq < ngroups; gq += kWarpsM) {
			const int s = gq * 32 + lane;
			const int pl = s / spp;
			const int j = s - pl * spp;
			const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
			const bool valid = s < tsamp && px < tpx1 && py < tpy1;
			float x = 0.0f, y = 0.0f, stime = 0.0f, sdx = 0.0f, sdy = 0.0f, oz = -FLT_MAX;
			int w = -1, fh = -1, kinv = 0;
			if (valid) {
				const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
				mb_sample_attrs(fp, smp, px, py, j, pix, x, y, stime, sdx, sdy, kinv);
				oz = sm.soz[s];
				w = sm.swin[s];
				if (TRANSP) fh = fhead[s];
			}
			float gmax = warp_max_m(oz);
#pragma unroll 1
			for (int wd = 0; wd < kWordsM; ++wd) {
				const uint32_t mine = sm.mask[valid ? pl : 0][wd];
				uint32_t bits = __reduce_or_sync(0xffffffffu, valid ? mine : 0u);
				while (bits) {
					const int b = __ffs(bits) - 1;
					bits &= bits - 1u;
					const MbRec& r = sm.rec[wd * 32 + b];
					const bool rcull = cullable && !(r.bits & 16);  // CSG: never occlusion-culled
					if (rcull && r.bmn[2] > gmax) continue;  // behind all 32 samples for the whole shutter
					const bool moving = r.nkeys > 1;
					bool stored = false;
					if (valid) {
						// the slices this sample's time falls in (one, or two on a boundary)
						int div = 1, b0 = 0, b1 = 0;
						const float* T = nullptr;
						float dt = 0.0f;
						if (moving) {
							div = motion_divisions(r, timeRanges);
							dt = (closetime - opentime) / div;
							T = slice_times + (div * (div - 1)) / 2;
							// last slice whose start time0 = T[b] - dt is <= stime
							int lo = 0, hi = div - 1;
							while (lo < hi) {
								const int mid = (lo + hi + 1) >> 1;
								if (T[mid] - dt <= stime) lo = mid; else hi = mid - 1;
							}
							b1 = lo;
							// earlier slices whose end time1 = T[b+1] - dt still reaches stime
							// (one on a boundary; more only if the accumulated times stall)
							b0 = b1;
							while (b0 > 0 && (T[b0] - dt) >= stime) --b0;
						}
						for (int sb = b0; sb <= b1; ++sb) {
							Bnd B;
							float time0 = 0.0f, time1 = 0.0f;
							if (moving) {
								B = sub_bound(r, T, sb);
								time0 = T[sb] - dt;
								time1 = (sb != div - 1) ? (T[sb + 1] - dt) : closetime;
								if (time1 < opentime || time0 > closetime) continue;
								if (stime < time0 || stime > time1) continue;
								if (!usingDof) {
									int indexT0, indexT1;
									if (fastShutter) { indexT0 = 0; indexT1 = spp; }
									else {
										indexT0 = max(0, lfloor_f((time0 - opentime) * timePerSample));
										indexT1 = lceil_f((time1 - opentime) * timePerSample);
									}
									if (indexT1 > spp) indexT1 = spp;
									if (j < indexT0 || j >= max(indexT1, indexT0 + 1)) continue;
								}
							} else {
								B = Bnd{r.bmn[0], r.bmn[1], r.bmn[2], r.bmx[0], r.bmx[1], r.bmx[2]};
							}
							// RenderMPG_MBOrDof's clipping-range cull (FLT_EPSILON, FLT_MAX,
							// options.cpp:296); static micropolygons without depth of field
							// are RenderMPG_Static's and are not culled
							if ((moving || usingDof) && (B.mnz > FLT_MAX || B.mxz < FLT_EPSILON)) continue;
							Bnd TB = B;
							if (usingDof) {
								// the lens stratum of this sample shifts the bound (bucketprocessor.cpp:1299-1321)
								const float2 c1 = coc(B.mnz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
								const float2 c2 = coc(B.mxz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
								const float maxCocX = amax(c1.x, c2.x), maxCocY = amax(c1.y, c2.y);
								TB.mnx = B.mnx - sm.dofb[kinv][2] * maxCocX;
								TB.mxx = B.mxx - sm.dofb[kinv][0] * maxCocX;
								TB.mny = B.mny - sm.dofb[kinv][3] * maxCocY;
								TB.mxy = B.mxy - sm.dofb[kinv][1] * maxCocY;
							}
							// pixels the reference walks for this (slice, stratum)
							if (px < (int)floorf(TB.mnx) || px >= lceil_f(TB.mxx) || py < (int)floorf(TB.mny) ||
							    py >= lceil_f(TB.mxy))
								continue;
							if ((x < TB.mnx || x > TB.mxx) || (y < TB.mny || y > TB.mxy)) continue;
							if (rcull && B.mnz > oz) continue;
							if ((r.bits & 8) && lod_rejects(fp, g, smp, r.grid, px, py, j)) continue;
							float D, u, v;
							if (!mb_sample(fp, r, moving, usingDof, x, y, stime, sdx, sdy, D, u, v, bb.tri, &g)) continue;
							if (rcull && oz <= D) continue;
							if ((r.bits & 2) && rcull) {
								if (TRANSP && fp.midpoint_store) {
									// midpoint filter with a z display (bucketprocessor.cpp:1502-1530)
									const long long hx =
									    ((long long)(py - fp.sy0) * fp.sw + (px - fp.sx0)) * spp + j;
									const float hp = (w >= 0) ? st.hitz[hx] : FLT_MAX;
									if (hp < D) {
										oz = D;
									} else {
										oz = hp;
										st.hitz[hx] = D;
										w = r.id;
									}
								} else {
									oz = D;
									w = r.id;
								}
								stored = true;
							} else if (TRANSP) {
								const unsigned act = __activemask();
								const int leader = __ffs(act) - 1;
								const int lrank = __popc(act & ((1u << lane) - 1u));
								unsigned long long base = 0;
								if (lane == leader) base = atomicAdd(pool.count, (unsigned long long)__popc(act));
								base = __shfl_sync(act, base, leader);
								const long long idx = (long long)base + lrank;
								if (idx < pool.capacity) {
									pool.frag[idx] = make_float4(D, __int_as_float(r.id), u, v);
									pool.next[idx] = fh;
									fh = (int)idx;
								} else {
									atomicOr(pool.overflow, 1);
								}
							}
						}
					}
					if (__any_sync(0xffffffffu, stored)) gmax = warp_max_m(oz);
				}
			}
			if (valid) {
				sm.soz[s] = oz;
				sm.swin[s] = w;
				if (TRANSP) fhead[s] = fh;
			}
		}
		__syncthreads();
		for (int i = t; i < kTilePixM * kWordsM; i += kThreadsM) (&sm.mask[0][0])[i] = 0u;
		__syncthreads();
		npend = 0;
		if (exhausted) break;
	}

	// ---- resolve: repeat the winner's hit test for its (u,v) ----
	// (opaque: consecutive threads take consecutive pixels of one sample index,
	// as the sample store is sample-major; transparent: the samples of one
	// pixel, whose fragments the same warp allocated together)
	for (int q = t; q < tsamp; q += kThreadsM) {
		const int j = TRANSP ? q % spp : q / tpix;
		const int pl = TRANSP ? q / spp : q - j * tpix;
		const int s = pl * spp + j;
		const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
		if (px >= tpx1 || py >= tpy1) continue;
		const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
		const int w = sm.swin[s];
		float x = 0.0f, y = 0.0f, stime = 0.0f, sdx = 0.0f, sdy = 0.0f;
		int kinv = 0;
		if (w >= 0) mb_sample_attrs(fp, smp, px, py, j, pix, x, y, stime, sdx, sdy, kinv);
		mb_resolve<TRANSP>(fp, g, pool, st, pix * spp + j, store_index(pix, j, spp), x, y, stime, sdx, sdy,
		                   sm.soz[s], w, TRANSP ? fhead[s] : -1);
		if (st.wmask) {
			const long long pp = smp.pos_index ? (long long)__ldg(smp.pos_index + pix) : pix;
			const float2 o = __ldg(smp.pos + pp * spp + j);
			st.wmask[store_index(pix, j, spp)] = window_mask(fp, px, py, (float)px + o.x, (float)py + o.y);
		}
	}
}


// ---- opaque frames: parallel (slice, sample) tests with an ordered replay ----
//
// The order argument of the static opaque kernel (sample.cu) carries over:
// RenderMPG_MBOrDof skips a (slice, sample) test when the slice's bound has
// min.z > occlZ and keeps a hit only if D < occlZ, so for every hit with D
// at or above its slice bound's min.z the winner is the least (D, insertion
// order) whatever the order of visits.  Work items are (micropolygon, time
// slice) pairs; each covers the pixels RenderMPG_MBOrDof would visit for
// that slice (with depth of field, the pixels some lens stratum's shifted
// bound covers) times a window of samples that is the same for each of its
// pixels, so that a flat index over all items' (pixel, sample) slots maps to
// its slot with two multiplications.  Each warp takes a contiguous share of
// the slots; a slot's cheap tests (time window, the sample's own stratum
// bound, pixel range, position, early-z against the round's start state)
// queue it for the full hit test, 32 at a time, whose hits fold into a
// 64-bit shared-memory atomicMin.  Hits below their slice's min.z, NaN or
// zero depths flag the sample for an in-order replay from the round's start.
__device__ __forceinline__ unsigned long long depth_key_m(float z, int w) {
	const uint32_t u = __float_as_uint(z);
	const uint32_t o = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
	return ((unsigned long long)o << 32) | (uint32_t)(w + 1);
}
__device__ __forceinline__ float key_depth_m(unsigned long long k) {
	const uint32_t o = (uint32_t)(k >> 32);
	return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
__device__ __forceinline__ int key_winner_m(unsigned long long k) { return (int)(uint32_t)k - 1; }

// Shutter constants of RenderMPG_MBOrDof (bucketprocessor.cpp:1237-1246).
struct Shutter {
	float open, close, timePerSample;
	bool fast;
	int timeRanges;
};

__device__ __forceinline__ Shutter shutter_of(const FrameParams& fp) {
	Shutter sh;
	sh.open = fp.shutter_open;
	sh.close = fp.shutter_close;
	// isClose (math.h:174-182)
	const float dclose = fabsf(sh.close - sh.open);
	const float tol = 10 * FLT_EPSILON;
	sh.fast = dclose <= tol * fabsf(sh.close) || dclose <= tol * fabsf(sh.open);
	sh.timePerSample = sh.fast ? 0.0f : (float)fp.spp / (sh.close - sh.open);
	sh.timeRanges = max(4, fp.spp);
	return sh;
}

// Slice b of micropolygon r: its bound, time window and (without depth of
// field) sample-index window.  False when the reference skips the slice.
template <class R>
__device__ __forceinline__ bool mb_slice(const FrameParams& fp, const Shutter& sh, const R& r, const float* T,
                                         int div, float dt, int b, Bnd& B, float& time0, float& time1, int& j0,
                                         int& j1) {
	const bool moving = r.nkeys > 1;
	j0 = 0;
	j1 = fp.spp;
	time0 = 0.0f;
	time1 = 0.0f;
	if (moving) {
		B = sub_bound(r, T, b);
		time0 = T[b] - dt;
		time1 = (b != div - 1) ? (T[b + 1] - dt) : sh.close;
		if (time1 < sh.open || time0 > sh.close) return false;
		if (!fp.use_dof) {
			int indexT0, indexT1;
			if (sh.fast) {
				indexT0 = 0;
				indexT1 = fp.spp;
			} else {
				indexT0 = max(0, lfloor_f((time0 - sh.open) * sh.timePerSample));
				indexT1 = lceil_f((time1 - sh.open) * sh.timePerSample);
			}
			if (indexT1 > fp.spp) indexT1 = fp.spp;
			j0 = indexT0;
			j1 = min(fp.spp, max(indexT1, indexT0 + 1));
		}
	} else {
		B = Bnd{r.bmn[0], r.bmn[1], r.bmn[2], r.bmx[0], r.bmx[1], r.bmx[2]};
	}
	// The clipping-range cull of RenderMPG_MBOrDof (bucketprocessor.cpp:1294-1296,
	// defaults FLT_EPSILON / FLT_MAX, options.cpp:296).  A micropolygon that
	// neither moves nor sees depth of field is sampled by RenderMPG_Static
	// (bucketprocessor.cpp:1067-1091), which has no such cull.
	if (!moving && !fp.use_dof) return true;
	return !(B.mnz > FLT_MAX || B.mxz < FLT_EPSILON);
}

// The bound of slice B as lens stratum k sees it (bucketprocessor.cpp:1299-1321).
__device__ __forceinline__ Bnd stratum_bound(const FrameParams& fp, const Bnd& B, const float* dofb) {
	const float2 c1 = coc(B.mnz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
	const float2 c2 = coc(B.mxz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
	const float maxCocX = amax(c1.x, c2.x), maxCocY = amax(c1.y, c2.y);
	Bnd TB = B;
	TB.mnx = B.mnx - dofb[2] * maxCocX;
	TB.mxx = B.mxx - dofb[0] * maxCocX;
	TB.mny = B.mny - dofb[3] * maxCocY;
	TB.mxy = B.mxy - dofb[1] * maxCocY;
	return TB;
}

// One (candidate, slice) item of the parallel pass: the slice's bound, time
// and sample-index windows, the largest CoC of its depth range and the tile
// pixels some lens stratum's shifted bound covers (all strata shift by the
// same CoC, so the union takes the extreme shifts).  False when the
// reference skips the slice or no covered pixel is in the tile.
struct MbItem {
	Bnd B;
	float time0, time1, maxCocX, maxCocY;
	int j0, j1, sX, eX, sY, eY;
};

template <class R>
__device__ __forceinline__ bool mb_item(const FrameParams& fp, const Shutter& sh, const R& r,
                                        const float* slice_times, int b, const float* dext, int tpx0, int tpy0,
                                        int tpx1, int tpy1, MbItem& it) {
	const bool moving = r.nkeys > 1;
	const int div = moving ? motion_divisions(r, sh.timeRanges) : 1;
	const float dt = (sh.close - sh.open) / div;
	const float* T = slice_times + (div * (div - 1)) / 2;
	if (!mb_slice(fp, sh, r, T, div, dt, b, it.B, it.time0, it.time1, it.j0, it.j1)) return false;
	const Bnd& B = it.B;
	Bnd U = B;
	it.maxCocX = 0.0f;
	it.maxCocY = 0.0f;
	if (fp.use_dof) {
		const float2 c1 = coc(B.mnz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
		const float2 c2 = coc(B.mxz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
		it.maxCocX = amax(c1.x, c2.x);
		it.maxCocY = amax(c1.y, c2.y);
		U.mnx = B.mnx - dext[2] * it.maxCocX;
		U.mxx = B.mxx - dext[0] * it.maxCocX;
		U.mny = B.mny - dext[3] * it.maxCocY;
		U.mxy = B.mxy - dext[1] * it.maxCocY;
	}
	if (!(U.mnx <= U.mxx && U.mny <= U.mxy)) return false;  // empty or NaN
	it.sX = (int)fmaxf(floorf(U.mnx), (float)tpx0);
	it.eX = (int)fminf(ceilf(U.mxx), (float)tpx1);
	it.sY = (int)fmaxf(floorf(U.mny), (float)tpy0);
	it.eY = (int)fminf(ceilf(U.mxy), (float)tpy1);
	return it.sX < it.eX && it.sY < it.eY && it.j0 < it.j1;
}

// Lens offset of the sample of lens stratum k in lens pattern dp
// (projectToCircle of the pattern's [0,1)^2 lens sample, imagepixel.cpp:338-347).
__device__ __forceinline__ float2 lens_offset(const SamplerDev& smp, int dp, int spp, int k) {
	if (!smp.dof) return make_float2(0.0f, 0.0f);
	const float2 d = __ldg(smp.dof + (long long)dp * spp + k);
	return project_to_circle(-1.0f + 2.0f * d.x, -1.0f + 2.0f * d.y);
}

// Tiles of the opaque kernel hold at most kTileSampQ samples so that two
// 512-thread CTAs fit on an SM (shared memory below half of 228 KB,
// registers at most 64 per thread: 32 warps per SM; measured 212 ms per
// 1080p motion blur + depth of field frame against 223 ms with 384 threads
// and 231 ms with 256).
constexpr int kThreadsQ = 512;
constexpr int kWarpsQ = kThreadsQ / 32;
constexpr int kSlotsQ = 64;      // candidates staged per round
constexpr int kItemsQ = 192;     // kept (candidate, slice) items per pass (at most one per thread)
constexpr int kTileSampQ = 2048;
constexpr int kTilePixQ = 256;
constexpr int kBinsQ = 64;       // time bins of a pixel at most
constexpr int kBinTabQ = kTileSampQ + kTilePixQ;  // (bins + 1) entries per pixel, over the tile

// One kept (candidate, slice) item of a pass.  Its sample slots are the
// product of its pixel rectangle and a window of `width` samples that is the
// same for every pixel: an index window [wbase, wbase + width) (no depth of
// field: RenderMPG_MBOrDof's sample-index range; a static micropolygon under
// depth of field: every sample), or, for a moving micropolygon under depth of
// field, the samples of each pixel whose time bin lies in [q0, q1] -- `wtime`
// slots, the most any pixel of the rectangle has there -- followed by the
// pixel's samples without a time (NaN), which every slice tests.
struct ItemQ {
	Bnd B;
	float time0, time1, maxCocX, maxCocY;
	int sX, sY, rw, npix, width, wtime, wbase;
	int info;  // staged slot | 1 << 8 moving | 1 << 9 time window | q1 << 10
	uint32_t mnpix, mrw;  // ceil(2^32 / npix), ceil(2^32 / rw) (0 for 1): exact quotients of slot indices
};

template <int NK, int SLOTS>
struct SmemQT {
	unsigned long long key[kTileSampQ];   // occluding hit of each tile sample (depth_key_m)
	unsigned long long prev[kTileSampQ];  // ... at the start of the round
	float stime[kTileSampQ];              // time of each tile sample
	uint8_t kinv[kTileSampQ];             // lens stratum of each tile sample
	uint8_t tord[kTileSampQ];             // each pixel's samples by time bin (NaN times last)
	uint16_t tstart[kBinTabQ];            // per pixel: first tord position of each time bin, then the end
	int16_t tval[kTilePixQ];              // samples with a time per pixel
	float pxmax[kTilePixQ];               // per pixel: largest occluding depth at the round's start (NaN: +inf)
	int patidx[kTilePixQ];
	int dofidx[kTilePixQ];                // lens pattern of each tile pixel
	float dofb[AQH_MAX_SPP_DEV][4];
	MbRecT<NK> rec[SLOTS];
	int2 pend[SLOTS];
	int pref[SLOTS + 1];                  // running count of (candidate, slice) items
	ItemQ items[kItemsQ];
	int ipref[kItemsQ + 1];               // running count of the kept items' sample slots
	int qgrid[kThreadsQ];
	int qcum[kThreadsQ + 1];
	int qsub[kThreadsQ];
	float blk[16 * 4];                    // largest occluding depth of each row's 4-pixel blocks (round start)
	uint32_t wq[kWarpsQ][64];             // per-warp queue of (candidate, sample) tests
	float wz[kWarpsQ][64];                // ... with their slice bound's min z
	uint32_t flag[kTileSampQ / 32];
	uint32_t sticky[kTileSampQ / 32];
	int warp_tot[32];
	int first_reject, qn, nsurv, any_nan;
	float dext[4];                        // min dofb[.][0], min [.][1], max [.][2], max [.][3]
};

// candidates per round: 64 four-key records, or 96 two-key ones in less space
constexpr int kSlotsQ2 = 96;
using SmemQ = SmemQT<kMaxKeys, kSlotsQ>;
using SmemQ2 = SmemQT<2, kSlotsQ2>;
// two CTAs per SM: 228 KB of shared memory less 1 KB reserved per CTA
static_assert(sizeof(SmemQ) <= (228 * 1024 - 2 * 1024) / 2, "two opaque motion CTAs must fit on an SM");
static_assert(sizeof(SmemQ2) <= sizeof(SmemQ), "two-key rounds must fit where four-key ones do");
static_assert(kSlotsQ2 <= kThreadsQ && kSlotsQ2 < 256, "one record per thread; slots fit 8 bits");

// One (slice, sample) test as RenderMPG_MBOrDof makes it, given occlZ:
// returns true with D when the sample is hit and not skipped by early-z.
template <class R>
__device__ __forceinline__ bool mb_slice_test(const FrameParams& fp, const R& r, const Bnd& B, bool moving,
                                              float time0, float time1, const float* dofb_k, int px, int py,
                                              float x, float y, float stime, float sdx, float sdy, float oz,
                                              float& D, const float4* tri, const GridsDev* gt) {
	if (moving && (stime < time0 || stime > time1)) return false;
	const Bnd TB = fp.use_dof ? stratum_bound(fp, B, dofb_k) : B;
	if (px < (int)floorf(TB.mnx) || px >= lceil_f(TB.mxx) || py < (int)floorf(TB.mny) || py >= lceil_f(TB.mxy))
		return false;
	if ((x < TB.mnx || x > TB.mxx) || (y < TB.mny || y > TB.mxy)) return false;
	if (B.mnz > oz) return false;
	float u, v;
	return mb_sample(fp, r, moving, fp.use_dof != 0, x, y, stime, sdx, sdy, D, u, v, tri, gt);
}

__device__ __forceinline__ uint32_t quot_magic(int d) {
	return d <= 1 ? 0u : (uint32_t)((0x100000000ull + (unsigned long long)d - 1ull) / (unsigned long long)d);
}
// r / d for 0 <= r, r * d < 2^32, with m = quot_magic(d): floor(r * ceil(2^32 / d) / 2^32)
// is exact there (the rounding up adds less than r * d / 2^32 / d < 1 / d)
__device__ __forceinline__ int quot(int r, uint32_t m) { return m == 0u ? r : (int)__umulhi((unsigned)r, m); }

template <int NK, int SLOTS>
__global__ void __launch_bounds__(kThreadsQ, 2)
sample_mbq_kernel(FrameParams fp, GridsDev g, SamplerDev smp, BinBuffers bb, SampleStore st,
                  const float4* dof_bounds, const float* slice_times) {
	using SmemQ = SmemQT<NK, SLOTS>;
	using MbRec = MbRecT<NK>;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	SmemQ& sm = *reinterpret_cast<SmemQ*>(smem_raw);
	const int tile = blockIdx.x;
	const int tx = tile % fp.ntx, ty = tile / fp.ntx;
	const int tpx0 = fp.sx0 + tx * fp.tile_w, tpy0 = fp.sy0 + ty * fp.tile_h;
	const int tpx1 = min(tpx0 + fp.tile_w, fp.sx0 + fp.sw), tpy1 = min(tpy0 + fp.tile_h, fp.sy0 + fp.sh);
	const int st_idx = (ty / fp.st_tiles) * fp.nstx + (tx / fp.st_tiles);
	const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
	const int spp = fp.spp;
	const int tpix = fp.tile_w * fp.tile_h;
	const int tsamp = tpix * spp;
	const int nflagw = (tsamp + 31) >> 5;
	const bool usingDof = fp.use_dof != 0;
	const Shutter sh = shutter_of(fp);
	const unsigned long long kinit = depth_key_m(FLT_MAX, -1);
	// time bins: only moving micropolygons under depth of field use time
	// windows; the bin of a time is monotone in the time, so a slice's window
	// [time0, time1] holds no sample outside bins [bin(time0), bin(time1)]
	const int Q = (usingDof && fp.any_motion && sh.close > sh.open) ? min(spp, kBinsQ) : 1;
	const float qscale = (Q > 1) ? (float)Q / (sh.close - sh.open) : 0.0f;
	auto tbin = [&](float tm) -> int {
		const float f = (tm - sh.open) * qscale;
		return (Q == 1 || !(f > 0.0f)) ? 0 : (f >= (float)(Q - 1) ? Q - 1 : (int)f);
	};

	for (int i = t; i < spp; i += kThreadsQ) {
		const float4 b = dof_bounds[i];
		sm.dofb[i][0] = b.x; sm.dofb[i][1] = b.y; sm.dofb[i][2] = b.z; sm.dofb[i][3] = b.w;
	}
	for (int i = t; i < tsamp; i += kThreadsQ) {
		sm.key[i] = kinit;
		sm.prev[i] = kinit;
		sm.kinv[i] = (uint8_t)(i % spp);
	}
	for (int i = t; i < kTileSampQ / 32; i += kThreadsQ) {
		sm.flag[i] = 0u;
		sm.sticky[i] = 0u;
	}
	if (t == 0) {
		sm.qn = 0;
		sm.qcum[0] = 0;
		sm.any_nan = 0;
	}
	for (int i = t; i < 16 * 4; i += kThreadsQ) sm.blk[i] = FLT_MAX;
	__syncthreads();
	// pattern of each pixel and the lens stratum of each sample (the shuffle
	// table inverted: the stratum of sample j is the q with shuffle[q] == j)
	for (int pl = t; pl < tpix; pl += kThreadsQ) {
		const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
		int pat = 0;
		if (px < tpx1 && py < tpy1) {
			const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
			pat = smp.pos_index ? (int)__ldg(smp.pos_index + pix) : (int)pix;
			if (smp.shuffle) {
				const long long sp = smp.shuffle_index ? (long long)__ldg(smp.shuffle_index + pix) : pix;
				for (int q = 0; q < spp; ++q) {
					const int j = __ldg(smp.shuffle + sp * spp + q);
					if (j >= 0 && j < spp) sm.kinv[pl * spp + j] = (uint8_t)q;
				}
			}
		}
		sm.patidx[pl] = pat;
	}
	if (t < 32) {
		float a0 = FLT_MAX, a1 = FLT_MAX, a2 = -FLT_MAX, a3 = -FLT_MAX;
		for (int k = lane; k < spp; k += 32) {
			a0 = fminf(a0, sm.dofb[k][0]);
			a1 = fminf(a1, sm.dofb[k][1]);
			a2 = fmaxf(a2, sm.dofb[k][2]);
			a3 = fmaxf(a3, sm.dofb[k][3]);
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			a0 = fminf(a0, __shfl_xor_sync(0xffffffffu, a0, o));
			a1 = fminf(a1, __shfl_xor_sync(0xffffffffu, a1, o));
			a2 = fmaxf(a2, __shfl_xor_sync(0xffffffffu, a2, o));
			a3 = fmaxf(a3, __shfl_xor_sync(0xffffffffu, a3, o));
		}
		if (lane == 0) {
			sm.dext[0] = a0;
			sm.dext[1] = a1;
			sm.dext[2] = a2;
			sm.dext[3] = a3;
		}
	}
	// time of each sample and the lens pattern of each pixel
	for (int s = t; s < tsamp; s += kThreadsQ) {
		const int pl = s / spp, j = s - pl * spp;
		const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
		float tm = 0.0f;
		if (px < tpx1 && py < tpy1) {
			const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
			const long long tp = smp.time_index ? (long long)__ldg(smp.time_index + pix) : pix;
			const float tt = smp.time ? __ldg(smp.time + tp * spp + j) : 0.0f;
			tm = (sh.close - sh.open) * tt + sh.open;
			if (j == 0) sm.dofidx[pl] = smp.dof_index ? (int)__ldg(smp.dof_index + pix) : (int)pix;
		}
		sm.stime[s] = tm;
	}
	__syncthreads();
	// each pixel's samples grouped by time bin (a counting sort; NaN times
	// go last): tstart[pl*(Q+1) + q] is the first position of bin q
	for (int pl = t; pl < tpix; pl += kThreadsQ) {
		uint16_t* row = sm.tstart + pl * (Q + 1);
		const float* tm = sm.stime + pl * spp;
		uint8_t* ord = sm.tord + pl * spp;
		for (int q = 0; q <= Q; ++q) row[q] = 0;
		int nv = 0;
		for (int j = 0; j < spp; ++j) {
			const float v = tm[j];
			if (v != v) continue;
			row[tbin(v) + 1]++;
			++nv;
		}
		for (int q = 1; q <= Q; ++q) row[q] = (uint16_t)(row[q] + row[q - 1]);
		// scatter with row[q] as the cursor of bin q - 1 ... then shift back
		for (int j = 0; j < spp; ++j) {
			const float v = tm[j];
			if (v != v) continue;
			const int q = tbin(v);
			ord[row[q]] = (uint8_t)j;
			row[q] = (uint16_t)(row[q] + 1);
		}
		for (int q = Q; q > 0; --q) row[q] = row[q - 1];
		row[0] = 0;
		int k = nv;
		for (int j = 0; j < spp; ++j)
			if (tm[j] != tm[j]) ord[k++] = (uint8_t)j;
		sm.tval[pl] = (int16_t)nv;
		if (nv < spp) sm.any_nan = 1;
		sm.pxmax[pl] = FLT_MAX;
	}
	__syncthreads();
	const bool any_nan = sm.any_nan != 0;

	const int lbeg = bb.st_offset[st_idx * bb.nranges];
	const int lend = (int)min((long long)bb.st_offset[(st_idx + 1) * bb.nranges], (long long)bb.list_capacity);
	int lp = lbeg, r0 = 0, qtotal = 0, npend = 0;
	for (;;) {
		const bool exhausted =
			stage_mb<SLOTS, SmemQ, kThreadsQ>(fp, g, bb, sm, tpx0, tpy0, tpx1, tpy1, lend, lp, r0, qtotal, npend,
			                                    sm.blk);
		if (npend == 0) break;

		// ---- records and (candidate, slice) items ----
		int nitems = 0;
		if (t < npend) {
			const int2 e = sm.pend[t];
			MbRec& rr = sm.rec[t];
			build_mb_record(fp, g, e.x, e.y, rr);
			nitems = (rr.nkeys > 1) ? motion_divisions(rr, sh.timeRanges) : 1;
		}
		int total;
		const int pre = block_excl_sum(sm.warp_tot, nitems, total);
		if (t < npend) sm.pref[t] = pre;
		__syncthreads();

		for (int base = 0; base < total; base += kItemsQ) {
			// ---- keep the items whose pixel rectangle meets the tile ----
			if (t == 0) sm.nsurv = 0;
			__syncthreads();
			for (int p = base + t; p < min(total, base + kItemsQ); p += kThreadsQ) {
				int lo = 0, hi = npend - 1;
				while (lo < hi) {
					const int mid = (lo + hi + 1) >> 1;
					if (sm.pref[mid] <= p) lo = mid; else hi = mid - 1;
				}
				const MbRec& r = sm.rec[lo];
				MbItem it;
				if (!mb_item(fp, sh, r, slice_times, p - sm.pref[lo], sm.dext, tpx0, tpy0, tpx1, tpy1, it)) continue;
				// early-z of the whole item: behind every sample of its pixels at the
				// round's start, so that every one of its slots would fail the
				// per-sample test below
				float zmax = -FLT_MAX;
				for (int py = it.sY; py < it.eY; ++py)
					for (int px = it.sX; px < it.eX; ++px)
						zmax = fmaxf(zmax, sm.pxmax[(py - tpy0) * fp.tile_w + (px - tpx0)]);
				if (it.B.mnz > zmax) continue;
				const bool moving = r.nkeys > 1;
				const int rw = it.eX - it.sX, npix = rw * (it.eY - it.sY);
				int width, wtime, wbase, info = lo | (moving ? 1 << 8 : 0);
				if (moving && usingDof) {
					const int q0 = tbin(it.time0), q1 = tbin(it.time1);
					int wt = 0, wn = 0;
					for (int py = it.sY; py < it.eY; ++py)
						for (int px = it.sX; px < it.eX; ++px) {
							const int pl = (py - tpy0) * fp.tile_w + (px - tpx0);
							const uint16_t* row = sm.tstart + pl * (Q + 1);
							wt = max(wt, (int)row[q1 + 1] - (int)row[q0]);
							if (any_nan) wn = max(wn, spp - (int)sm.tval[pl]);
						}
					wtime = wt;
					width = wt + wn;
					wbase = q0;
					info |= (1 << 9) | (q1 << 10);
				} else {
					wbase = it.j0;
					width = wtime = it.j1 - it.j0;
				}
				if (width <= 0) continue;
				const int at = atomicAdd(&sm.nsurv, 1);
				ItemQ& q = sm.items[at];
				q.B = it.B;
				q.time0 = it.time0;
				q.time1 = it.time1;
				q.maxCocX = it.maxCocX;
				q.maxCocY = it.maxCocY;
				q.sX = it.sX;
				q.sY = it.sY;
				q.rw = rw;
				q.npix = npix;
				q.width = width;
				q.wtime = wtime;
				q.wbase = wbase;
				q.info = info;
				q.mnpix = quot_magic(npix);
				q.mrw = quot_magic(rw);
			}
			__syncthreads();
			const int nsurv = sm.nsurv;
			const int nslots_t = (t < nsurv) ? sm.items[t].npix * sm.items[t].width : 0;
			int nslots;
			const int ipre = block_excl_sum(sm.warp_tot, nslots_t, nslots);
			if (t < nsurv) sm.ipref[t] = ipre;
			if (t == 0) sm.ipref[nsurv] = nslots;
			__syncthreads();

			// ---- sample slots: each warp a contiguous share, 32 at a time ----
			uint32_t* wq = sm.wq[warp];
			float* wz = sm.wz[warp];
			int qn = 0;
			auto drain = [&](int n) {
				// hit tests of queue entries [0, n), one per lane
				if (lane < n) {
					const uint32_t e = wq[lane];
					const int c = (int)(e & 0xffu), s = (int)(e >> 8);
					const MbRec& r = sm.rec[c];
					const int pl = s / spp, j = s - pl * spp;
					const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
					const float2 o = __ldg(smp.pos + (long long)sm.patidx[pl] * spp + j);
					const float2 d = lens_offset(smp, sm.dofidx[pl], spp, sm.kinv[s]);
					float D, u, v;
					if (!((r.bits & 8) && lod_rejects(fp, g, smp, r.grid, px, py, j)) &&
					    mb_sample(fp, r, r.nkeys > 1, usingDof, (float)px + o.x, (float)py + o.y, sm.stime[s], d.x, d.y,
					              D, u, v, bb.tri, &g)) {
						if (!(D >= wz[lane]) || D == 0.0f)
							atomicOr(&sm.flag[s >> 5], 1u << (s & 31));
						else
							atomicMin(&sm.key[s], depth_key_m(D, r.id));
					}
				}
				__syncwarp();
			};
			const int g0 = (int)((long long)nslots * warp / kWarpsQ);
			const int g1 = (int)((long long)nslots * (warp + 1) / kWarpsQ);
			int cur = advance_item(sm.ipref, nsurv, 0, g0);
			for (int gb = g0; gb < g1; gb += 32) {
				const int gs = gb + lane;
				bool pass = false;
				int s = 0, c = 0;
				float bz = 0.0f;
				int it_l = cur;
				if (gs < g1) {
					it_l = advance_item(sm.ipref, nsurv, cur, gs);
					const ItemQ& it = sm.items[it_l];
					const int r = gs - sm.ipref[it_l];
					const int k = quot(r, it.mnpix);
					const int p = r - k * it.npix;
					const int oy = quot(p, it.mrw);
					const int px = it.sX + (p - oy * it.rw), py = it.sY + oy;
					const int pl = (py - tpy0) * fp.tile_w + (px - tpx0);
					int j = -1;
					if (it.B.mnz > sm.pxmax[pl]) {
						// every sample of the pixel is in front of the slice's bound
					} else if (!(it.info & (1 << 9))) {
						j = it.wbase + k;
					} else if (k < it.wtime) {
						const uint16_t* row = sm.tstart + pl * (Q + 1);
						const int a = row[it.wbase];
						if (k < (int)row[((it.info >> 10) & 0x7f) + 1] - a) j = sm.tord[pl * spp + a + k];
					} else {
						const int kk = k - it.wtime, nv = sm.tval[pl];
						if (kk < spp - nv) j = sm.tord[pl * spp + nv + kk];
					}
					if (j >= 0) {
						s = pl * spp + j;
						c = it.info & 0xff;
						const Bnd& B = it.B;
						bz = B.mnz;
						pass = !(sm.flag[s >> 5] & (1u << (s & 31)));  // else replayed in order below
						if (pass && (it.info & (1 << 8))) {
							const float stime = sm.stime[s];
							pass = !(stime < it.time0 || stime > it.time1);
						}
						if (pass) {
							Bnd TB = B;
							if (usingDof) {
								const float* dk = sm.dofb[sm.kinv[s]];
								TB.mnx = B.mnx - dk[2] * it.maxCocX;
								TB.mxx = B.mxx - dk[0] * it.maxCocX;
								TB.mny = B.mny - dk[3] * it.maxCocY;
								TB.mxy = B.mxy - dk[1] * it.maxCocY;
							}
							const float2 o = __ldg(smp.pos + (long long)sm.patidx[pl] * spp + j);
							const float x = (float)px + o.x, y = (float)py + o.y;
							pass = !(px < (int)floorf(TB.mnx) || px >= lceil_f(TB.mxx) || py < (int)floorf(TB.mny) ||
							         py >= lceil_f(TB.mxy)) &&
							       !((x < TB.mnx || x > TB.mxx) || (y < TB.mny || y > TB.mxy)) &&
							       !(B.mnz > key_depth_m(sm.prev[s]));
						}
					}
				}
				cur = __shfl_sync(0xffffffffu, it_l, 31);
				const uint32_t bal = __ballot_sync(0xffffffffu, pass);
				if (pass) {
					const int at = qn + __popc(bal & ((1u << lane) - 1u));
					wq[at] = (uint32_t)c | ((uint32_t)s << 8);
					wz[at] = bz;
				}
				qn += __popc(bal);
				__syncwarp();
				if (qn >= 32) {
					drain(32);
					if (lane < qn - 32) {  // entries [32, qn) move to the front
						wq[lane] = wq[32 + lane];
						wz[lane] = wz[32 + lane];
					}
					__syncwarp();
					qn -= 32;
				}
			}
			drain(qn);
			__syncthreads();
		}
		int anyf = 0;
		for (int i = t; i < nflagw; i += kThreadsQ) anyf |= (int)(sm.flag[i] != 0u);

		// ---- ordered replay of flagged samples, one thread per sample ----
		if (__syncthreads_or(anyf)) {
			for (int s = t; s < tsamp; s += kThreadsQ) {
				if (!(sm.flag[s >> 5] & (1u << (s & 31)))) continue;
				const int pl = s / spp, j = s - pl * spp;
				const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
				if (px >= tpx1 || py >= tpy1) continue;
				const float2 o = __ldg(smp.pos + (long long)sm.patidx[pl] * spp + j);
				const float x = (float)px + o.x, y = (float)py + o.y;
				const float stime = sm.stime[s];
				const float2 d = lens_offset(smp, sm.dofidx[pl], spp, sm.kinv[s]);
				const float* dk = sm.dofb[sm.kinv[s]];
				float oz = key_depth_m(sm.prev[s]);
				int w = key_winner_m(sm.prev[s]);
				for (int c = 0; c < npend; ++c) {
					const MbRec& r = sm.rec[c];
					const bool moving = r.nkeys > 1;
					const int div = moving ? motion_divisions(r, sh.timeRanges) : 1;
					const float dt = (sh.close - sh.open) / div;
					const float* T = slice_times + (div * (div - 1)) / 2;
					int b0 = 0, b1 = 0;
					if (moving) {
						// slices whose window can hold the sample's time, in slice order
						int blo = 0, bhi = div - 1;
						while (blo < bhi) {
							const int mid = (blo + bhi + 1) >> 1;
							if (T[mid] - dt <= stime) blo = mid; else bhi = mid - 1;
						}
						b1 = blo;
						b0 = b1;
						while (b0 > 0 && (T[b0] - dt) >= stime) --b0;
						if (stime != stime) { b0 = 0; b1 = div - 1; }  // a NaN time passes every window test
					}
					for (int sb = b0; sb <= b1; ++sb) {
						Bnd B;
						float time0, time1;
						int j0, j1;
						if (!mb_slice(fp, sh, r, T, div, dt, sb, B, time0, time1, j0, j1)) continue;
						if (j < j0 || j >= j1) continue;
						if ((r.bits & 8) && lod_rejects(fp, g, smp, r.grid, px, py, j)) continue;
						float D;
						if (!mb_slice_test(fp, r, B, moving, time0, time1, dk, px, py, x, y, stime, d.x, d.y, oz, D, bb.tri, &g))
							continue;
						if (!(oz <= D)) {
							oz = D;
							w = r.id;
						}
					}
				}
				sm.key[s] = depth_key_m(oz, w);
				if (oz != oz || oz == 0.0f) atomicOr(&sm.sticky[s >> 5], 1u << (s & 31));
			}
		}
		__syncthreads();
		for (int i = t; i < tsamp; i += kThreadsQ) sm.prev[i] = sm.key[i];
		for (int i = t; i < nflagw; i += kThreadsQ) sm.flag[i] = sm.sticky[i];
		__syncthreads();
		// largest occluding depth of each pixel (a NaN depth never lets a test be
		// skipped, so it counts as +inf)
		for (int pl = t; pl < tpix; pl += kThreadsQ) {
			float m = -FLT_MAX;
			for (int j = 0; j < spp; ++j) {
				const float z = key_depth_m(sm.prev[pl * spp + j]);
				m = (z != z) ? __int_as_float(0x7f800000) : fmaxf(m, z);
			}
			sm.pxmax[pl] = m;
		}
		__syncthreads();
		for (int i = t; i < fp.tile_h * 4; i += kThreadsQ) {
			const int y = i >> 2, x0 = (i & 3) * 4;
			float m = -FLT_MAX;
			for (int x = x0; x < min(x0 + 4, fp.tile_w); ++x) m = fmaxf(m, sm.pxmax[y * fp.tile_w + x]);
			sm.blk[i] = m;
		}
		__syncthreads();
		npend = 0;
		if (exhausted) break;
	}

	// ---- resolve, pixel-major (a pixel's samples often share a winner, whose
	// loads then merge) ----
	for (int q = t; q < tsamp; q += kThreadsQ) {
		const int j = q % spp;
		const int pl = q / spp;
		const int s = pl * spp + j;
		const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
		if (px >= tpx1 || py >= tpy1) continue;
		const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
		const unsigned long long kk = sm.key[s];
		const float2 o = __ldg(smp.pos + (long long)sm.patidx[pl] * spp + j);
		const float2 d = lens_offset(smp, sm.dofidx[pl], spp, sm.kinv[s]);
		mb_resolve<false>(fp, g, FragPool{}, st, pix * spp + j, store_index(pix, j, spp), (float)px + o.x,
		                  (float)py + o.y, sm.stime[s], d.x, d.y, key_depth_m(kk), key_winner_m(kk), -1);
		if (st.wmask) st.wmask[store_index(pix, j, spp)] = window_mask(fp, px, py, (float)px + o.x, (float)py + o.y);
	}
}

}  // namespace

int sample_mb_opaque_tile_pixels(int spp) { return max(1, min(kTilePixQ, kTileSampQ / max(1, spp))); }

size_t sample_mb_smem(bool transp) {
	return sizeof(SmemM) + (transp ? sizeof(int32_t) * kTileSampM : 0);
}

void launch_sample_mb(const FrameParams& fp, const GridsDev& g, const SamplerDev& sm, const BinBuffers& b,
                      SampleStore st, FragPool pool, const float4* dof_bounds, const float* slice_times,
                      cudaStream_t s) {
	const int ntiles = fp.ntx * fp.nty;
	configure_sample_mb_kernels();
	if (pool.capacity > 0)
		sample_mb_kernel<true><<<ntiles, kThreadsM, sample_mb_smem(true), s>>>(fp, g, sm, b, st, pool, dof_bounds,
		                                                                      slice_times);
	else if (fp.max_keys >= 1 && fp.max_keys <= 2)
		sample_mbq_kernel<2, kSlotsQ2><<<ntiles, kThreadsQ, sizeof(SmemQ2), s>>>(fp, g, sm, b, st, dof_bounds,
		                                                                       slice_times);
	else
		sample_mbq_kernel<kMaxKeys, kSlotsQ><<<ntiles, kThreadsQ, sizeof(SmemQ), s>>>(fp, g, sm, b, st, dof_bounds,
		                                                                             slice_times);
}

void configure_sample_mb_kernels() {
	static std::mutex mu;
	static uint64_t configured = 0;
	if (!first_use_on_device(mu, configured)) return;
	cudaFuncSetAttribute(sample_mbq_kernel<kMaxKeys, kSlotsQ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                     (int)sizeof(SmemQ));
	cudaFuncSetAttribute(sample_mbq_kernel<2, kSlotsQ2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                     (int)sizeof(SmemQ2));
	cudaFuncSetAttribute(sample_mb_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sample_mb_smem(true));
}

}  // namespace aqh
