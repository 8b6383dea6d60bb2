// sample_mb.cu -- sampling with motion blur and/or depth of field.
//
// Replaces CqBucketProcessor::RenderMPG_MBOrDof (libs/core/bucketprocessor.cpp:
// 1221-1469), CqMicroPolygonMotion::BuildBoundList / Sample
// (micropolygon.cpp:1689-1756, 1768-1914), the depth-of-field branch of
// CqMicroPolygon::Sample (1561-1592) and CqMicroPolygon::dofSampleInBound
// (1531-1550).
//
// Same structure as the static kernel (sample.cu): micropolygons of the tile
// are staged into shared-memory records in insertion order; each thread owns
// up to kMbSamples samples of one pixel and, for every candidate micropolygon
// of its pixel (ascending slot = insertion order), replays the reference's
// loop: the time sub-bounds in order (recomputed exactly, including the
// accumulated shutter times), and per sub-bound either the sample index range
// of that time slice (motion blur) or the one lens stratum each sample belongs
// to (depth of field).  Within one micropolygon the reference visits a sample
// once per sub-bound that admits it, so visiting this thread's samples per
// sub-bound in any order gives the same store sequence.
#include "aqh_internal.h"
#include "hider_device.cuh"
#include "sample_common.cuh"

namespace aqh {

namespace {

constexpr int kMbSamples = 8;   // samples per thread
constexpr int kMbSlots = 128;   // records per pass
constexpr int kMbWords = kMbSlots / 32;

struct MbRec {
	float bmn[3], bmx[3];          // m_Bound (union of the key bounds for moving micropolygons)
	float key[kMaxKeys][4][3];     // key vertices in natural order: index, index+1, index+cu+1, index+cu+2
	float kt[kMaxKeys];            // key times
	float kbmn[kMaxKeys][3], kbmx[kMaxKeys][3];  // per-key bounds
	float cocm[4][2];              // static DoF: CoC multiplier per vertex
	float cocmin[2], cocmax[2];    // DoF: min / max CoC multipliers
	int nkeys, code, id, grid, bits;
};

struct MbSmem {
	MbRec rec[kMbSlots];
	uint32_t mask[kBlock][kMbWords];
	float dofb[AQH_MAX_SPP_DEV][4];  // DoF sub-bounds (CalculateDofBounds): mn.x mn.y mx.x mx.y
	int qgrid[kBlock];
	int warp_tot[32];
	int first_reject;
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

template <bool TRANSP>
__global__ void __launch_bounds__(kBlock, 1)
sample_mb_kernel(FrameParams fp, GridsDev g, SamplerDev smp, BinBuffers bb, SampleStore st, FragPool pool,
                 const float4* dof_bounds) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	MbSmem& sm = *reinterpret_cast<MbSmem*>(smem_raw);
	int32_t* win = reinterpret_cast<int32_t*>(smem_raw + sizeof(MbSmem));
	int32_t* wgrid = win + kBlock * kMbSamples;
	int32_t* fhead = wgrid + kBlock * kMbSamples;

	const int tile = blockIdx.x;
	const int tx = tile % fp.ntx, ty = tile / fp.ntx;
	const int tpx0 = fp.sx0 + tx * fp.tile_w, tpy0 = fp.sy0 + ty * fp.tile_h;
	const int tpx1 = min(tpx0 + fp.tile_w, fp.sx0 + fp.sw), tpy1 = min(tpy0 + fp.tile_h, fp.sy0 + fp.sh);
	const int st_idx = (ty / fp.st_tiles) * fp.nstx + (tx / fp.st_tiles);
	const int t = threadIdx.x;
	const int spp = fp.spp;
	const int spt = (spp + fp.tpp - 1) / fp.tpp;  // samples per thread (<= kMbSamples)

	const int pl = t / fp.tpp;
	const int sg = t - pl * fp.tpp;
	const int lx = pl % fp.tile_w, ly = pl / fp.tile_w;
	const int mypx = tpx0 + lx, mypy = tpy0 + ly;
	const bool own = (pl < fp.tile_w * fp.tile_h) && mypx < tpx1 && mypy < tpy1;
	const int s0 = sg * spt;
	const int nmine = own ? max(0, min(spt, spp - s0)) : 0;
	const long long pix = own ? (long long)(mypy - fp.sy0) * fp.sw + (mypx - fp.sx0) : 0;

	for (int i = t; i < spp; i += blockDim.x) {
		const float4 b = dof_bounds[i];
		sm.dofb[i][0] = b.x; sm.dofb[i][1] = b.y; sm.dofb[i][2] = b.z; sm.dofb[i][3] = b.w;
	}

	// per-sample data (CqImagePixel::setSamples, imagepixel.cpp:334-359)
	float sx[kMbSamples], sy[kMbSamples], stime[kMbSamples], sdx[kMbSamples], sdy[kMbSamples], oz[kMbSamples];
	int kinv[kMbSamples];
	{
		const long long pp = own ? (smp.pos_index ? (long long)smp.pos_index[pix] : pix) : 0;
		const long long tp = own ? (smp.time_index ? (long long)smp.time_index[pix] : pix) : 0;
		const long long dp = own ? (smp.dof_index ? (long long)smp.dof_index[pix] : pix) : 0;
		const long long sp = own ? (smp.shuffle_index ? (long long)smp.shuffle_index[pix] : pix) : 0;
		const float fx = (float)mypx, fy = (float)mypy;
#pragma unroll
		for (int i = 0; i < kMbSamples; ++i) {
			sx[i] = fx; sy[i] = fy; stime[i] = 0.0f; sdx[i] = 0.0f; sdy[i] = 0.0f; oz[i] = FLT_MAX; kinv[i] = 0;
			if (i < nmine) {
				const int j = s0 + i;
				const float2 o = __ldg(smp.pos + pp * spp + j);
				sx[i] = fx + o.x;
				sy[i] = fy + o.y;
				const float tt = smp.time ? __ldg(smp.time + tp * spp + j) : 0.0f;
				stime[i] = (fp.shutter_close - fp.shutter_open) * tt + fp.shutter_open;
				// lens stratum k whose sample is j: m_DofOffsetIndices[k] == j
				int k = j;
				if (smp.shuffle) {
					for (int q = 0; q < spp; ++q)
						if (__ldg(smp.shuffle + sp * spp + q) == j) k = q;
				}
				kinv[i] = k;
				if (smp.dof) {
					const float2 d = __ldg(smp.dof + dp * spp + k);
					// projectToCircle(-1 + 2 * dofOffsets[k])
					const float2 c = project_to_circle(-1.0f + 2.0f * d.x, -1.0f + 2.0f * d.y);
					sdx[i] = c.x;
					sdy[i] = c.y;
				}
			}
		}
	}
#pragma unroll
	for (int i = 0; i < kMbSamples; ++i) {
		win[t * kMbSamples + i] = -1;
		if (TRANSP) fhead[t * kMbSamples + i] = -1;
	}
	for (int i = t; i < kBlock * kMbWords; i += blockDim.x) (&sm.mask[0][0])[i] = 0u;
	__syncthreads();

	const int lbeg = bb.st_offset[st_idx * bb.nranges];
	const int lend = bb.st_offset[(st_idx + 1) * bb.nranges];
	const int cullable = fp.cullable;
	const bool usingDof = fp.use_dof != 0;
	const float opentime = fp.shutter_open, closetime = fp.shutter_close;
	// isClose (math.h:174-182) and timePerSample (bucketprocessor.cpp:1237-1246)
	const float dclose = fabsf(closetime - opentime);
	const float tol = 10 * FLT_EPSILON;
	const bool fastShutter = dclose <= tol * fabsf(closetime) || dclose <= tol * fabsf(opentime);
	const float timePerSample = fastShutter ? 0.0f : (float)spp / (closetime - opentime);
	const int timeRanges = max(4, spp);

	int lp = lbeg, qi = 0, qn = 0, r0 = 0;
	int nslots = 0;
	for (;;) {
		bool exhausted = false;
		while (nslots < kMbSlots) {
			if (qi >= qn) {
				if (lp >= lend) { exhausted = true; break; }
				const int li = lp + t;
				int gid = -1;
				bool f = false;
				if (li < lend && t < kBlock) {
					gid = bb.st_list[li];
					const int4 rc = bb.grid_rect[gid];
					f = rc.x < rc.y && rc.x < tpx1 && rc.y > tpx0 && rc.z < tpy1 && rc.w > tpy0;
				}
				int total;
				const int pos = block_excl_scan(sm.warp_tot, f, total);
				if (f) sm.qgrid[pos] = gid;
				__syncthreads();
				qn = total;
				qi = 0;
				r0 = 0;
				lp += blockDim.x;
				continue;
			}
			const int gi = sm.qgrid[qi];
			const int cu = __ldg(g.cu + gi), cv = __ldg(g.cv + gi);
			const int nmp = cu * cv;
			if (r0 >= nmp) { ++qi; r0 = 0; continue; }
			const int m = r0 + t;
			const long long mpb = __ldg(g.mpbase + gi);
			bool active = false;
			MbRec rr;
			if (m < nmp) {
				load_mb_record(fp, g, gi, m, rr);
				const bool culled = g.culled && g.culled[mpb + m];
				// AddMPG (imagebuffer.cpp:514-539): DoF-grown bound against the crop cull window
				float ax0 = rr.bmn[0], ay0 = rr.bmn[1], ax1 = rr.bmx[0], ay1 = rr.bmx[1];
				float gx = 0.0f, gy = 0.0f;
				if (usingDof) {
					const float2 c1 = coc(rr.bmn[2], fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
					const float2 c2 = coc(rr.bmx[2], fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
					gx = amax(c1.x, c2.x);
					gy = amax(c1.y, c2.y);
				}
				const bool cropped = (ax1 + gx) < fp.cull_x0 || (ay1 + gy) < fp.cull_y0 || (ax0 - gx) > fp.cull_x1 ||
				                     (ay0 - gy) > fp.cull_y1;
				// conservative pixel rectangle over every time slice and lens stratum
				const int sX = max((int)floorf(ax0 - gx) - 1, tpx0), eX = min(lceil_f(ax1 + gx) + 1, tpx1);
				const int sY = max((int)floorf(ay0 - gy) - 1, tpy0), eY = min(lceil_f(ay1 + gy) + 1, tpy1);
				active = !culled && !cropped && sX < eX && sY < eY;
			}
			int total;
			const int rank = block_excl_scan(sm.warp_tot, active, total);
			const int navail = kMbSlots - nslots;
			if (t == 0) sm.first_reject = blockDim.x;
			__syncthreads();
			if (active && rank == navail) sm.first_reject = t;
			if (active && rank < navail) {
				const int slot = nslots + rank;
				const int gflags = __ldg(g.flags + gi);
				bool opaque = true;
				const bool smooth = (gflags & 1) != 0;
				if (!(gflags & 8) && g.Oi) {
					const int iv = m / cu, iu = m - iv * cu;
					const int index = iv * (cu + 1) + iu;
					const long long cb = __ldg(g.cbase + gi);
					const int nvv = smooth ? 4 : 1;
					const int vi[4] = {index, index + 1, index + cu + 1, index + cu + 2};
					for (int q = 0; q < nvv; ++q) {
						const float4 o = __ldg(g.Oi + cb + vi[q]);
						opaque = opaque && (o.x >= 1.0f && o.y >= 1.0f && o.z >= 1.0f);
					}
				}
				int bits = 0;
				if (opaque || (gflags & 4)) bits |= 2;
				rr.bits = bits;
				rr.id = (int)(mpb + m);
				rr.grid = gi;
				sm.rec[slot] = rr;
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
			const int consumed = (total > navail) ? sm.first_reject : min((int)blockDim.x, nmp - r0);
			nslots += min(total, navail);
			r0 += consumed;
		}
		if (nslots == 0) break;

		if (own) {
#pragma unroll 1
			for (int wd = 0; wd < kMbWords; ++wd) {
				uint32_t bits = sm.mask[pl][wd];
				while (bits) {
					const int b = __ffs(bits) - 1;
					bits &= bits - 1u;
					const MbRec& r = sm.rec[wd * 32 + b];
					const bool moving = r.nkeys > 1;
					// time sub-bounds (CqMicroPolygonMotion::BuildBoundList)
					int divisions = 1;
					float dt = 0.0f, time = 0.0f;
					Bnd bound{r.bmn[0], r.bmn[1], r.bmn[2], r.bmx[0], r.bmx[1], r.bmx[2]};
					int startKey = 0, endKey = 1;
					if (moving) {
						const float cx = r.kbmx[0][0] - r.kbmn[0][0], cy = r.kbmx[0][1] - r.kbmn[0][1];
						// CqVector2D::Magnitude2 (vector2d.h:132-138)
						const float polyLen2 = (cy == 0.0f) ? cx * cx : ((cx == 0.0f) ? cy * cy : (cx * cx) + (cy * cy));
						const float mx = r.key[0][0][0] - r.key[r.nkeys - 1][0][0];
						const float my = r.key[0][0][1] - r.key[r.nkeys - 1][0][1];
						const float moveDist2 = (my == 0.0f) ? mx * mx : ((mx == 0.0f) ? my * my : (mx * mx) + (my * my));
						const int plm = max(1, lfloor_f(sqrtf(moveDist2 / polyLen2)));
						divisions = min(plm, timeRanges);
						dt = (closetime - opentime) / divisions;
						time = opentime + dt;
						bound = key_bound(r, 0);
					}
					for (int dv = 0; dv < divisions; ++dv) {
						Bnd B;
						float time0 = 0.0f, time1 = 0.0f;
						if (moving) {
							while (time > r.kt[endKey] && endKey < r.nkeys - 1) ++endKey;
							const int e0 = endKey - 1;
							const Bnd end0 = key_bound(r, e0), end1 = key_bound(r, endKey);
							const float mix = (time - r.kt[e0]) / (r.kt[endKey] - r.kt[e0]);
							Bnd mid = end0;
							mid.mnx = mid.mnx + mix * (end1.mnx - end0.mnx);
							mid.mny = mid.mny + mix * (end1.mny - end0.mny);
							mid.mnz = mid.mnz + mix * (end1.mnz - end0.mnz);
							mid.mxx = mid.mxx + mix * (end1.mxx - end0.mxx);
							mid.mxy = mid.mxy + mix * (end1.mxy - end0.mxy);
							mid.mxz = mid.mxz + mix * (end1.mxz - end0.mxz);
							encapsulate(bound, mid);
							while (startKey < e0) {
								startKey++;
								encapsulate(bound, key_bound(r, startKey));
							}
							B = bound;
							time0 = time - dt;
							const float tnext = time + dt;
							time1 = (dv != divisions - 1) ? (tnext - dt) : closetime;
							bound = mid;
							time = tnext;
						} else {
							B = bound;
						}
						int indexT0 = 0, indexT1 = 0;
						if (moving) {
							if (time1 < opentime || time0 > closetime) continue;
							if (fastShutter) {
								indexT0 = 0;
								indexT1 = spp;
							} else {
								indexT0 = max(0, lfloor_f((time0 - opentime) * timePerSample));
								indexT1 = lceil_f((time1 - opentime) * timePerSample);
							}
							if (indexT1 > spp) indexT1 = spp;
						}
						// Clipping defaults (FLT_EPSILON, FLT_MAX), options.cpp:296
						if (B.mnz > FLT_MAX || B.mxz < FLT_EPSILON) continue;
						float maxCocX = 0.0f, maxCocY = 0.0f;
						if (usingDof) {
							const float2 c1 = coc(B.mnz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
							const float2 c2 = coc(B.mxz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
							maxCocX = amax(c1.x, c2.x);
							maxCocY = amax(c1.y, c2.y);
						}
						// pixel range of the (possibly lens-shifted) bound, for the no-DoF case
						if (!usingDof) {
							const int pX0 = (int)floorf(B.mnx), pX1 = lceil_f(B.mxx);
							const int pY0 = (int)floorf(B.mny), pY1 = lceil_f(B.mxy);
							if (mypx < pX0 || mypx >= pX1 || mypy < pY0 || mypy >= pY1) continue;
						}
						const int lastIdx = max(indexT1, indexT0 + 1);  // the do-while tests indexT0 at least once
#pragma unroll
						for (int i = 0; i < kMbSamples; ++i) {
							if (i >= nmine) continue;
							const int j = s0 + i;
							Bnd TB = B;
							if (usingDof) {
								// lens stratum k of this sample: shift the bound (bucketprocessor.cpp:1309-1321)
								const int k = kinv[i];
								const float leftOffset = sm.dofb[k][2] * maxCocX;
								const float rightOffset = sm.dofb[k][0] * maxCocX;
								const float topOffset = sm.dofb[k][3] * maxCocY;
								const float bottomOffset = sm.dofb[k][1] * maxCocY;
								TB.mnx = B.mnx - leftOffset;
								TB.mxx = B.mxx - rightOffset;
								TB.mny = B.mny - topOffset;
								TB.mxy = B.mxy - bottomOffset;
								const int pX0 = (int)floorf(TB.mnx), pX1 = lceil_f(TB.mxx);
								const int pY0 = (int)floorf(TB.mny), pY1 = lceil_f(TB.mxy);
								if (mypx < pX0 || mypx >= pX1 || mypy < pY0 || mypy >= pY1) continue;
							} else {
								if (j < indexT0 || j >= lastIdx) continue;
							}
							const float x = sx[i], y = sy[i];
							if (moving && (stime[i] < time0 || stime[i] > time1)) continue;
							if ((x < TB.mnx || x > TB.mxx) || (y < TB.mny || y > TB.mxy)) continue;
							if (cullable && B.mnz > oz[i]) continue;
							float D, u, v;
							if (!mb_sample(fp, r, moving, usingDof, x, y, stime[i], sdx[i], sdy[i], D, u, v)) continue;
							if (cullable && oz[i] <= D) continue;
							if ((r.bits & 2) && cullable) {
								oz[i] = D;
								win[t * kMbSamples + i] = r.id;
								wgrid[t * kMbSamples + i] = r.grid;
							} else if (TRANSP) {
								const unsigned act = __activemask();
								const int leader = __ffs(act) - 1;
								const int lrank = __popc(act & ((1u << (threadIdx.x & 31)) - 1u));
								unsigned long long base = 0;
								if ((threadIdx.x & 31) == leader)
									base = atomicAdd(pool.count, (unsigned long long)__popc(act));
								base = __shfl_sync(act, base, leader);
								const long long idx = (long long)base + lrank;
								if (idx < pool.capacity) {
									pool.frag[idx] = make_float4(D, __int_as_float(r.id), u, v);
									pool.next[idx] = fhead[t * kMbSamples + i];
									fhead[t * kMbSamples + i] = (int)idx;
								} else {
									atomicOr(pool.overflow, 1);
								}
							}
						}
					}
				}
			}
		}
		__syncthreads();
		for (int i = t; i < kBlock * kMbWords; i += blockDim.x) (&sm.mask[0][0])[i] = 0u;
		__syncthreads();
		nslots = 0;
		if (exhausted) break;
	}

	// resolve: recompute the winner's (u,v) by repeating its hit test
	__syncthreads();
	if (!own) return;
#pragma unroll
	for (int i = 0; i < kMbSamples; ++i) {
		if (i >= nmine) continue;
		const long long sidx = pix * spp + s0 + i;
		const int w = win[t * kMbSamples + i];
		float occl[7] = {0, 0, 0, 0, 0, 0, 0};
		int occl_flags = 0;
		if (w >= 0) {
			const int gi = wgrid[t * kMbSamples + i];
			MbRec& r = sm.rec[t % kMbSlots];  // scratch: records are no longer read
			(void)r;
			MbRec rr;
			const int m = w - (int)__ldg(g.mpbase + gi);
			load_mb_record(fp, g, gi, m, rr);
			float D, u, v;
			mb_sample(fp, rr, rr.nkeys > 1, usingDof, sx[i], sy[i], stime[i], sdx[i], sdy[i], D, u, v);
			hit_colour(g, gi, m, u, v, occl, occl_flags);
			occl[6] = oz[i];
		}
		int nf = 0;
		bool valid = w >= 0;
		if (TRANSP) {
			const int head = fhead[t * kMbSamples + i];
			if (head >= 0) {
				nf = combine_fragments(fp, g, pool, head, w >= 0, oz[i], occl, occl_flags);
				valid = true;
			}
		}
		if (nf == 0 && valid) {
			if (occl_flags & 1)
				for (int q = 0; q < 6; ++q) occl[q] = 0.0f;
			if (fp.depth_filter == 1) occl[6] = (float)(0.5 * ((double)occl[6] + (double)oz[i]));
		}
		st.a[sidx] = make_float4(occl[0], occl[1], occl[2], occl[6]);
		st.b[sidx] = make_float4(occl[3], occl[4], occl[5], valid ? 1.0f : 0.0f);
		if (st.winner) st.winner[sidx] = w;
		if (st.occlz) st.occlz[sidx] = oz[i];
		if (st.nfrag) st.nfrag[sidx] = nf;
	}
}

}  // namespace

size_t sample_mb_smem(bool transp) {
	return sizeof(MbSmem) + (transp ? 3 : 2) * sizeof(int32_t) * kBlock * kMbSamples;
}

void launch_sample_mb(const FrameParams& fp, const GridsDev& g, const SamplerDev& sm, const BinBuffers& b,
                      SampleStore st, FragPool pool, const float4* dof_bounds, cudaStream_t s) {
	const int ntiles = fp.ntx * fp.nty;
	const size_t so = sample_mb_smem(false), stp = sample_mb_smem(true);
	static bool configured = false;
	if (!configured) {
		cudaFuncSetAttribute(sample_mb_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)so);
		cudaFuncSetAttribute(sample_mb_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stp);
		configured = true;
	}
	const int threads = fp.tile_w * fp.tile_h * fp.tpp;
	const int block = ((threads + 31) / 32) * 32;
	if (pool.capacity > 0)
		sample_mb_kernel<true><<<ntiles, block, stp, s>>>(fp, g, sm, b, st, pool, dof_bounds);
	else
		sample_mb_kernel<false><<<ntiles, block, so, s>>>(fp, g, sm, b, st, pool, dof_bounds);
}

int mb_samples_per_thread() { return kMbSamples; }

}  // namespace aqh
