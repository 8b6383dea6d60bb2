// sample_mb.cu -- sampling with motion blur and/or depth of field.
//
// Replaces CqBucketProcessor::RenderMPG_MBOrDof (libs/core/bucketprocessor.cpp:
// 1221-1469), CqMicroPolygonMotion::BuildBoundList / Sample
// (micropolygon.cpp:1689-1756, 1768-1914), the depth-of-field branch of
// CqMicroPolygon::Sample (1561-1592) and CqMicroPolygon::dofSampleInBound
// (1531-1550).
//
// Same structure as the static kernel (sample.cu): the tile's micropolygons
// are staged into shared-memory records in insertion order and a warp walks
// 32 samples' candidates, one sample per lane.  For a moving micropolygon the
// reference tests a sample once per time slice whose window holds the
// sample's time (and, without depth of field, whose sample-index range holds
// the sample); each lane finds those slices directly -- by binary search in a
// per-frame table of the reference's accumulated slice times -- and builds
// that slice's bound directly, in slice order.  With depth of field each
// sample belongs to one lens stratum, whose shifted bound decides whether the
// reference visits it.
#include "aqh_internal.h"
#include "hider_device.cuh"
#include "sample_common.cuh"

namespace aqh {

namespace {


struct MbRec {
	float bmn[3], bmx[3];          // m_Bound (union of the key bounds for moving micropolygons)
	float key[kMaxKeys][4][3];     // key vertices in natural order: index, index+1, index+cu+1, index+cu+2
	float kt[kMaxKeys];            // key times
	float kbmn[kMaxKeys][3], kbmx[kMaxKeys][3];  // per-key bounds
	float cocm[4][2];              // static DoF: CoC multiplier per vertex
	float cocmin[2], cocmax[2];    // DoF: min / max CoC multipliers
	int nkeys, code, id, grid, bits;
};


struct Bnd {
	float mnx, mny, mnz, mxx, mxy, mxz;
};

__device__ __forceinline__ Bnd key_bound(const MbRec& r, int k) {
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
// and (u,v).
__device__ bool mb_sample(const FrameParams& fp, const MbRec& r, bool moving, bool dof, float px, float py,
                          float time, float dx, float dy, float& D, float& u, float& v) {
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
	return true;
}

// Load the record of micropolygon m of grid gi from global memory.
__device__ void load_mb_record(const FrameParams& fp, const GridsDev& g, int gi, int m, MbRec& r) {
	const int cu = __ldg(g.cu + gi), cv = __ldg(g.cv + gi);
	const int nk = __ldg(g.nkeys + gi);
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
	if (fp.use_dof) {
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
__device__ __forceinline__ int motion_divisions(const MbRec& r, int timeRanges) {
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
__device__ __forceinline__ int end_key_at(const MbRec& r, float T) {
	int e = 1;
	while (T > r.kt[e] && e < r.nkeys - 1) ++e;
	return e;
}

// Key bounds interpolated at time T between keys e-1 and e (the `mid` bound).
__device__ __forceinline__ Bnd mid_at(const MbRec& r, int e, float T) {
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
__device__ Bnd sub_bound(const MbRec& r, const float* T, int b) {
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
		// ---- phase A: stage candidates in insertion order ----
		bool exhausted = false;
		while (npend < kSlotsM) {
			if (r0 >= qtotal) {
				if (lp >= lend) { exhausted = true; break; }
				const int li = lp + t;
				int gid = -1;
				bool f = false;
				if (li < lend) {
					gid = bb.st_list[li];
					const int4 rc = bb.grid_rect[gid];
					f = rc.x < rc.y && rc.x < tpx1 && rc.y > tpx0 && rc.z < tpy1 && rc.w > tpy0;
				}
				int total;
				const int pos = block_excl_scan(sm.warp_tot, f, total);
				if (f) sm.qgrid[pos] = gid;
				__syncthreads();
				if (t == 0) {
					int acc = 0;
					for (int k = 0; k < total; ++k) {
						sm.qcum[k] = acc;
						const int q = sm.qgrid[k];
						acc += __ldg(g.cu + q) * __ldg(g.cv + q);
					}
					sm.qcum[total] = acc;
					sm.qn = total;
				}
				__syncthreads();
				qtotal = sm.qcum[sm.qn];
				r0 = 0;
				lp += kThreadsM;
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
				if (usingDof) {
					const float2 c1 = coc(mnz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
					const float2 c2 = coc(mxz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
					gx = amax(c1.x, c2.x);
					gy = amax(c1.y, c2.y);
				}
				// AddMPG (imagebuffer.cpp:514-539): DoF-grown bound against the crop cull window
				const bool cropped = (mxx + gx) < fp.cull_x0 || (mxy + gy) < fp.cull_y0 || (mnx - gx) > fp.cull_x1 ||
				                     (mny - gy) > fp.cull_y1;
				// conservative pixel rectangle over every time slice and lens stratum
				const int sX = max((int)floorf(mnx - gx) - 1, tpx0), eX = min(lceil_f(mxx + gx) + 1, tpx1);
				const int sY = max((int)floorf(mny - gy) - 1, tpy0), eY = min(lceil_f(mxy + gy) + 1, tpy1);
				active = !culled && !cropped && sX < eX && sY < eY;
			}
			int total;
			const int rank = block_excl_scan(sm.warp_tot, active, total);
			const int navail = kSlotsM - npend;
			if (t == 0) sm.first_reject = kThreadsM;
			__syncthreads();
			if (active && rank == navail) sm.first_reject = t;
			if (active && rank < navail) sm.pend[npend + rank] = make_int2(gid, m);
			__syncthreads();
			const int consumed = (total > navail) ? sm.first_reject : min(kThreadsM, qtotal - r0);
			npend += min(total, navail);
			r0 += consumed;
		}
		if (npend == 0) break;

		// ---- records, one per thread ----
		for (int slot = t; slot < npend; slot += kThreadsM) {
			const int2 e = sm.pend[slot];
			MbRec& rr = sm.rec[slot];
			load_mb_record(fp, g, e.x, e.y, rr);
			const int gflags = __ldg(g.flags + e.x);
			bool opaque = true;
			const bool smooth = (gflags & 1) != 0;
			if (!(gflags & 8) && g.Oi) {
				const int cu = __ldg(g.cu + e.x);
				const int iv = e.y / cu, iu = e.y - iv * cu;
				const int index = iv * (cu + 1) + iu;
				const long long cb = __ldg(g.cbase + e.x);
				const int vi[4] = {index, index + 1, index + cu + 1, index + cu + 2};
				for (int q = 0; q < (smooth ? 4 : 1); ++q) {
					const float4 o = __ldg(g.Oi + cb + vi[q]);
					opaque = opaque && (o.x >= 1.0f && o.y >= 1.0f && o.z >= 1.0f);
				}
			}
			rr.bits = (opaque || (gflags & 4)) ? 2 : 0;
			rr.id = (int)(__ldg(g.mpbase + e.x) + e.y);
			rr.grid = e.x;
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
			float x = 0.0f, y = 0.0f, stime = 0.0f, sdx = 0.0f, sdy = 0.0f, oz = -FLT_MAX, hz = FLT_MAX;
			int w = -1, fh = -1, kinv = 0;
			long long sidx = 0;
			if (valid) {
				const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
				const long long pp = smp.pos_index ? (long long)__ldg(smp.pos_index + pix) : pix;
				const long long tp = smp.time_index ? (long long)__ldg(smp.time_index + pix) : pix;
				const long long dp = smp.dof_index ? (long long)__ldg(smp.dof_index + pix) : pix;
				const long long sp = smp.shuffle_index ? (long long)__ldg(smp.shuffle_index + pix) : pix;
				const float2 o = __ldg(smp.pos + pp * spp + j);
				x = (float)px + o.x;
				y = (float)py + o.y;
				const float tt = smp.time ? __ldg(smp.time + tp * spp + j) : 0.0f;
				stime = (closetime - opentime) * tt + opentime;
				kinv = j;
				if (smp.shuffle)
					for (int q = 0; q < spp; ++q)
						if (__ldg(smp.shuffle + sp * spp + q) == j) kinv = q;
				if (smp.dof) {
					const float2 d = __ldg(smp.dof + dp * spp + kinv);
					const float2 c = project_to_circle(-1.0f + 2.0f * d.x, -1.0f + 2.0f * d.y);
					sdx = c.x;
					sdy = c.y;
				}
				oz = sm.soz[s];
				w = sm.swin[s];
				if (TRANSP) fh = fhead[s];
				sidx = pix * spp + j;
				if (TRANSP && fp.midpoint_store && w >= 0) hz = st.hitz[sidx];
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
					if (cullable && r.bmn[2] > gmax) continue;  // behind all 32 samples for the whole shutter
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
							// Clipping defaults (FLT_EPSILON, FLT_MAX), options.cpp:296
							if (B.mnz > FLT_MAX || B.mxz < FLT_EPSILON) continue;
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
							if (cullable && B.mnz > oz) continue;
							float D, u, v;
							if (!mb_sample(fp, r, moving, usingDof, x, y, stime, sdx, sdy, D, u, v)) continue;
							if (cullable && oz <= D) continue;
							if ((r.bits & 2) && cullable) {
								if (TRANSP && fp.midpoint_store) {
									// midpoint filter with a z display (bucketprocessor.cpp:1502-1530)
									const float hp = (w >= 0) ? hz : FLT_MAX;
									if (hp < D) {
										oz = D;
									} else {
										oz = hp;
										hz = D;
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
				if (TRANSP && fp.midpoint_store && w >= 0) st.hitz[sidx] = hz;
			}
		}
		__syncthreads();
		for (int i = t; i < kTilePixM * kWordsM; i += kThreadsM) (&sm.mask[0][0])[i] = 0u;
		__syncthreads();
		npend = 0;
		if (exhausted) break;
	}

	// ---- resolve: repeat the winner's hit test for its (u,v) ----
	// (consecutive threads take consecutive pixels of one sample index: the
	// sample store is sample-major)
	const long long npix = (long long)fp.sw * fp.sh;
	for (int q = t; q < tsamp; q += kThreadsM) {
		const int j = q / tpix;
		const int pl = q - j * tpix;
		const int s = pl * spp + j;
		const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
		if (px >= tpx1 || py >= tpy1) continue;
		const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
		const long long sidx = pix * spp + j;
		const long long aidx = (long long)j * npix + pix;
		const float ozv = sm.soz[s];
		const int w = sm.swin[s];
		float occl[7] = {0, 0, 0, 0, 0, 0, 0};
		int occl_flags = 0;
		if (w >= 0) {
			const long long pp = smp.pos_index ? (long long)__ldg(smp.pos_index + pix) : pix;
			const long long tp = smp.time_index ? (long long)__ldg(smp.time_index + pix) : pix;
			const long long dp = smp.dof_index ? (long long)__ldg(smp.dof_index + pix) : pix;
			const long long sp = smp.shuffle_index ? (long long)__ldg(smp.shuffle_index + pix) : pix;
			const float2 o = __ldg(smp.pos + pp * spp + j);
			const float x = (float)px + o.x, y = (float)py + o.y;
			const float tt = smp.time ? __ldg(smp.time + tp * spp + j) : 0.0f;
			const float stime = (closetime - opentime) * tt + opentime;
			float sdx = 0.0f, sdy = 0.0f;
			if (smp.dof) {
				int kinv = j;
				if (smp.shuffle)
					for (int q = 0; q < spp; ++q)
						if (__ldg(smp.shuffle + sp * spp + q) == j) kinv = q;
				const float2 d = __ldg(smp.dof + dp * spp + kinv);
				const float2 c = project_to_circle(-1.0f + 2.0f * d.x, -1.0f + 2.0f * d.y);
				sdx = c.x;
				sdy = c.y;
			}
			const int gi = grid_of(g, w);
			const int m = w - (int)__ldg(g.mpbase + gi);
			MbRec rr;
			load_mb_record(fp, g, gi, m, rr);
			float D, u, v;
			mb_sample(fp, rr, rr.nkeys > 1, usingDof, x, y, stime, sdx, sdy, D, u, v);
			hit_colour(g, gi, m, u, v, occl, occl_flags);
			occl[6] = (TRANSP && fp.midpoint_store) ? st.hitz[sidx] : ozv;
		}
		int nf = 0;
		bool valid = w >= 0;
		if (TRANSP) {
			const int head = fhead[s];
			if (head >= 0) {
				nf = combine_fragments(fp, g, pool, head, w >= 0, ozv, occl, occl_flags);
				valid = true;
			}
		}
		if (nf == 0 && valid) {
			if (occl_flags & 1)
				for (int q = 0; q < 6; ++q) occl[q] = 0.0f;
			if (fp.depth_filter == 1) occl[6] = (float)(0.5 * ((double)occl[6] + (double)ozv));
		}
		st.a[aidx] = make_float4(occl[0], occl[1], occl[2], occl[6]);
		st.b[aidx] = make_float4(occl[3], occl[4], occl[5], valid ? 1.0f : 0.0f);
		if (st.winner) st.winner[sidx] = w;
		if (st.occlz) st.occlz[sidx] = ozv;
		if (st.nfrag) st.nfrag[sidx] = nf;
	}
}

}  // namespace

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
	else
		sample_mb_kernel<false><<<ntiles, kThreadsM, sample_mb_smem(false), s>>>(fp, g, sm, b, st, pool, dof_bounds,
		                                                                        slice_times);
}

void configure_sample_mb_kernels() {
	static bool configured = false;
	if (configured) return;
	cudaFuncSetAttribute(sample_mb_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sample_mb_smem(false));
	cudaFuncSetAttribute(sample_mb_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sample_mb_smem(true));
	configured = true;
}

}  // namespace aqh
