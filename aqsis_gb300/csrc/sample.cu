// sample.cu -- the sampling stage: subpixel hit tests with depth and opacity
// compositing into the pixel sample store.
//
// Replaces CqBucketProcessor::RenderMicroPoly / RenderMPG_Static /
// RenderMPG_MBOrDof / StoreSample (libs/core/bucketprocessor.cpp:1067-1569),
// CqMicroPolygon::Sample / fContains (micropolygon.cpp:1295-1660, 1768-1914)
// and CqImagePixel::Combine (imagepixel.cpp:144-332).
//
// Layout.  One CTA (16 warps) owns a tile of the sample region holding at
// most 4096 samples (16x16 pixels at 16 samples per pixel).  It walks its
// super-tile's grid list in submission order and expands the grids touching
// the tile into micropolygons, kSlotsS at a time:
//   phase A: one micropolygon per thread tests bound, crop cull and a
//     tile-wide early-z; survivors are compacted in insertion order, then
//     every thread builds one shared-memory record (vertex order, edge and
//     inverse-bilinear coefficients, pixel and sub-sample ranges) and sets a
//     bit per covered pixel in that pixel's candidate mask;
//   phase B: a warp takes 32 consecutive samples of the tile, one per lane,
//     and walks the union of their pixels' masks in ascending slot order --
//     the insertion order -- with warp-uniform control flow: records are
//     shared-memory broadcasts, a candidate behind all 32 samples' occluding
//     depths is skipped by the whole warp, and each lane runs the reference's
//     per-sample sequence (sub-sample range, inclusive bound test, early-z,
//     edge tests, inverse bilinear, depth, store).
// Because each sample is owned by one lane that visits its candidates in
// insertion order, the reference's order-dependent early-z and its "first of
// equal depths wins" rule hold exactly.  Colours are resolved once per sample at the
// end (the reference interpolates them at store time; the values are the
// same because they depend only on the winning micropolygon and (u,v)).
#include "aqh_internal.h"
#include "hider_device.cuh"
#include "sample_common.cuh"

namespace aqh {

namespace {

constexpr int kThreadsS = 512;                   // 16 warps
constexpr int kWarpsS = kThreadsS / 32;
constexpr int kSlotsS = 256;                     // records per pass
constexpr int kWordsS = kSlotsS / 32;
constexpr int kTilePixMax = 256;
constexpr int kTileSampMax = 4096;

// Shared-memory record of one candidate micropolygon (static path).
struct RecS {
	float bminx, bmaxx, bminy, bmaxy, bminz;
	int px0, px1, py0, py1;        // pixels RenderMPG_Static visits: [floor(bmin), lceil(bmax))
	int im, em, in_, en;           // sub-sample starts / ends on the first / last pixel
	float ym[4], xm[4], ex[4], ey[4];
	float ax, ay, e_x, e_y, f_x, f_y, g_x, g_y;
	float z[4];
	int id;                        // global micropolygon id
	int bits;                      // 1 linear, 2 occluding store
};  // 43 words: an odd stride spreads neighbouring records over the banks

// RecS::bits; the grid index sits from bit 6 up.  kRecCsg: a CSG solid's
// micropolygon, never occlusion-cullable; kRecTrim: marked trimmed.
constexpr int kRecLinear = 1, kRecOccluding = 2, kRecTriangular = 4, kRecLod = 8, kRecCsg = 16, kRecTrim = 32;
constexpr int kRecGridShift = 6;

// The tests after fContains that can still reject a static hit at (x, y),
// (u, v): the trim curves of a micropolygon marked trimmed, then the split
// line of a triangular grid (key 0).
__device__ __forceinline__ bool rec_keeps(const GridsDev& g, const BinBuffers& bb, int bits, int id, float x, float y,
                                          float u, float v) {
	if ((bits & kRecTrim) && trim_rejects(g, id, bits >> kRecGridShift, u, v)) return false;
	return !(bits & kRecTriangular) || triangle_keeps(__ldg(bb.tri + (size_t)(bits >> kRecGridShift) * kMaxKeys), x, y);
}

struct SmemS {
	RecS rec[kSlotsS];
	uint32_t mask[kTilePixMax][kWordsS];  // candidate bits per tile pixel
	int2 pend[kSlotsS];                   // (grid, micropolygon) of the staged candidates
	int qgrid[kThreadsS];                 // grids of the current list chunk that touch the tile
	int qcum[kThreadsS + 1];              // running micropolygon counts of those grids
	int qsub[kThreadsS];                  // their micropolygon sub-rectangles (see stage_candidates)
	int warp_tot[32];
	float warp_max[32];
	int first_reject;
	int qn;
	float pixmax[kTilePixMax];            // largest occluding depth over each pixel's samples
	float blkmax[16];                     // ... over each 4x4-pixel block of the tile
	float soz[kTileSampMax];              // occlZ per tile sample
	int swin[kTileSampMax];               // occluding micropolygon per tile sample (-1 none)
};

// Running maximum of occluding depths for the early-z culls.  A NaN depth
// never passes `bminz > occlZ`, so it must never cull: it counts as +inf.
__device__ __forceinline__ float max_depth(float mx, float d) { return (d != d) ? INFINITY : fmaxf(mx, d); }

__device__ __forceinline__ float warp_max_f(float v) {
	v = (v != v) ? INFINITY : v;
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
	return v;
}

// Record of micropolygon m of grid gi: bound (CalculateBound), vertex order
// (ComputeVertexOrder), point-in-polygon and inverse-bilinear coefficients
// (cachePointInPolyTest), opacity (CacheOutputInterpCoeffs*), and the pixel
// and sub-sample ranges RenderMPG_Static walks.
__device__ __forceinline__ void build_record(const FrameParams& fp, const GridsDev& g, int gi, int m, RecS& rec) {
	const int cu = __ldg(g.cu + gi);
	const long long pb = __ldg(g.pbase + gi);
	const int gflags = __ldg(g.flags + gi);
	const int iv = m / cu, iu = m - iv * cu;
	const int index = iv * (cu + 1) + iu;
	V3f v[4];
	v[0] = ld3(g.P, pb + index);
	v[1] = ld3(g.P, pb + index + 1);
	v[2] = ld3(g.P, pb + index + cu + 1);
	v[3] = ld3(g.P, pb + index + cu + 2);
	const float bminx = amin(amin(amin(v[0].x, v[1].x), v[3].x), v[2].x);
	const float bminy = amin(amin(amin(v[0].y, v[1].y), v[3].y), v[2].y);
	const float bminz = amin(amin(amin(v[0].z, v[1].z), v[3].z), v[2].z);
	const float bmaxx = amax(amax(amax(v[0].x, v[1].x), v[3].x), v[2].x);
	const float bmaxy = amax(amax(amax(v[0].y, v[1].y), v[3].y), v[2].y);
	HitCoeffs h;
	hit_setup(v, vertex_order(v), h);
	rec.bminx = bminx; rec.bmaxx = bmaxx; rec.bminy = bminy; rec.bmaxy = bmaxy; rec.bminz = bminz;
	// bucketprocessor.cpp:1119-1138 (the clip to the sample region does not
	// change the range of any pixel inside it)
	const int sX = (int)floorf(bminx), eX = lceil_f(bmaxx);
	const int sY = (int)floorf(bminy), eY = lceil_f(bmaxy);
	rec.px0 = sX; rec.px1 = eX; rec.py0 = sY; rec.py1 = eY;
	rec.im = (int)floorf((bminx - (float)sX) * (float)fp.xs);
	rec.in_ = (int)floorf((bminy - (float)sY) * (float)fp.ys);
	rec.em = lceil_f((bmaxx - (float)(eX - 1)) * (float)fp.xs);
	rec.en = lceil_f((bmaxy - (float)(eY - 1)) * (float)fp.ys);
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		rec.ym[k] = h.ym[k]; rec.xm[k] = h.xm[k]; rec.ex[k] = h.ex[k]; rec.ey[k] = h.ey[k];
		rec.z[k] = h.z[k];
	}
	rec.ax = h.ax; rec.ay = h.ay; rec.e_x = h.e_x; rec.e_y = h.e_y;
	rec.f_x = h.f_x; rec.f_y = h.f_y; rec.g_x = h.g_x; rec.g_y = h.g_y;
	rec.id = (int)(__ldg(g.mpbase + gi) + m);
	// SqMpgSampleInfo::isOpaque (micropolygon.cpp:1477-1529)
	bool opaque = true;
	const bool smooth = (gflags & 1) != 0;
	if (!(gflags & 8) && g.Oi) {
		const long long cb = __ldg(g.cbase + gi);
		const float4 o0 = ld_colour(g, g.Oi, cb + index);
		opaque = o0.x >= 1.0f && o0.y >= 1.0f && o0.z >= 1.0f;
		if (smooth) {
			const float4 o1 = ld_colour(g, g.Oi, cb + index + 1);
			const float4 o2 = ld_colour(g, g.Oi, cb + index + cu + 1);
			const float4 o3 = ld_colour(g, g.Oi, cb + index + cu + 2);
			opaque = opaque && (o1.x >= 1.0f && o1.y >= 1.0f && o1.z >= 1.0f) &&
			         (o2.x >= 1.0f && o2.y >= 1.0f && o2.z >= 1.0f) && (o3.x >= 1.0f && o3.y >= 1.0f && o3.z >= 1.0f);
		}
	}
	int bits = h.linear ? kRecLinear : 0;
	if (opaque || (gflags & 4)) bits |= kRecOccluding;
	if (gflags & 16) bits |= kRecTriangular;
	if (lod_active(fp, g, gi)) bits |= kRecLod;
	if (csg_grid(g, gi)) bits = (bits & ~kRecOccluding) | kRecCsg;
	if (g.trim.nsets > 0 && __ldg(g.trim.mark + rec.id)) bits |= kRecTrim;
	bits |= gi << kRecGridShift;
	rec.bits = bits;
}

// Final value of one sample: the occluding hit's colour at its (u,v), or the
// Combine of its transparent fragments; written to the sample store.
template <bool TRANSP>
__device__ __forceinline__ void resolve_sample(const FrameParams& fp, const GridsDev& g, const FragPool& pool,
                                               const SampleStore& st, long long sidx, long long aidx, float x,
                                               float y, float oz, int w, int head) {
	float occl[7] = {0, 0, 0, 0, 0, 0, 0};
	int occl_flags = 0;
	if (w >= 0) {
		// recompute (u,v) of the winner exactly as when it was stored
		const int wg = grid_of(g, w);
		const int cu = __ldg(g.cu + wg);
		const int m = w - (int)__ldg(g.mpbase + wg);
		const int iv = m / cu, iu = m - iv * cu;
		const int index = iv * (cu + 1) + iu;
		const long long pb = __ldg(g.pbase + wg);
		V3f v[4] = {ld3(g.P, pb + index), ld3(g.P, pb + index + 1), ld3(g.P, pb + index + cu + 1),
		            ld3(g.P, pb + index + cu + 2)};
		HitCoeffs h;
		hit_setup(v, vertex_order(v), h);
		float u, vv;
		inv_bilinear(h.ax, h.ay, h.e_x, h.e_y, h.f_x, h.f_y, h.g_x, h.g_y, h.linear, x, y, u, vv);
		hit_colour(g, wg, m, u, vv, occl, occl_flags);
		occl[6] = (TRANSP && fp.midpoint_store) ? st.hitz[sidx] : oz;
	}
	int nf = 0;
	bool valid = w >= 0;
	int src = w;
	if (TRANSP && head >= 0) {
		bool emptied = false;
		nf = combine_fragments(fp, g, pool, head, w >= 0, oz, occl, occl_flags, w, src, emptied);
		valid = !emptied;
	}
	if (nf == 0 && valid) {
		// imagepixel.cpp:303-330: opaque matte hits become transparent black;
		// the midpoint depth filter averages with occlZ
		if (occl_flags & 1)
			for (int q = 0; q < 6; ++q) occl[q] = 0.0f;
		if (fp.depth_filter == 1) occl[6] = (float)(0.5 * ((double)occl[6] + (double)oz));
	}
	st.a[aidx] = make_float4(occl[0], occl[1], occl[2], occl[6]);
	st.b[aidx] = make_float4(occl[3], occl[4], occl[5], valid ? 1.0f : 0.0f);
	if (st.aovsrc) st.aovsrc[aidx] = valid ? src : -1;
	if (st.winner) st.winner[sidx] = w;
	if (st.occlz) st.occlz[sidx] = oz;
	if (st.nfrag) st.nfrag[sidx] = nf;
}

// Phase A: stream the super-tile's grid list from the cursor (lp, r0,
// qtotal) and append the micropolygons that are candidates of the tile to
// sm.pend, in insertion order, until kSlots are staged or the list ends
// (returns true then).  One micropolygon per thread tests bound, crop cull
// and early-z against the largest occluding depth of every pixel it visits;
// whole grids behind every sample of the 4x4-pixel blocks they overlap are
// skipped.  Survivors are compacted with block scans, so the staged order is
// the insertion order.
// MAY_CSG: the calling kernel can see CSG grids (the opaque kernel never
// does: frames with solids always render with fragments).
template <int kSlots, bool MAY_CSG = true, class Smem>
__device__ __forceinline__ bool stage_candidates(const FrameParams& fp, const GridsDev& g, const BinBuffers& bb,
                                                 Smem& sm, int tpx0, int tpy0, int tpx1, int tpy1, int lend, int& lp,
                                                 int& r0, int& qtotal, int& npend) {
	const int t = threadIdx.x;
	const int cullable = fp.cullable;
	while (npend < kSlots) {
		if (r0 >= qtotal) {
			if (lp >= lend) return true;
			// grids of the next list chunk that touch the tile, in order
			const int li = lp + t;
			int gid = -1, nmp = 0, sub = -1;  // sub: first column, first row, width; -1 = whole grid
			bool f = false;
			if (li < lend) {
				gid = bb.st_list[li];
				const int4 rc = bb.grid_rect[gid];
				f = rc.x < rc.y && rc.x < tpx1 && rc.y > tpx0 && rc.z < tpy1 && rc.w > tpy0;
				if (f && cullable && !(MAY_CSG && csg_grid(g, gid))) {
					// whole grid behind every sample of the 4x4-pixel blocks it overlaps
					const int bx0 = (max(rc.x, tpx0) - tpx0) >> 2, bx1 = (min(rc.y, tpx1) - 1 - tpx0) >> 2;
					const int by0 = (max(rc.z, tpy0) - tpy0) >> 2, by1 = (min(rc.w, tpy1) - 1 - tpy0) >> 2;
					const int nbx = (fp.tile_w + 3) >> 2;
					float mx = -FLT_MAX;
					for (int by = by0; by <= by1; ++by)
						for (int bx = bx0; bx <= bx1; ++bx) mx = fmaxf(mx, sm.blkmax[by * nbx + bx]);
					if (__ldg(bb.grid_minz + gid) > mx) f = false;
				}
				if (f) {
					const int cu = __ldg(g.cu + gid), cv = __ldg(g.cv + gid);
					nmp = cu * cv;
					if (bb.strips && __ldg(bb.strips + (long long)gid * 64 + 63)) {
						// the columns and rows of micropolygons that can meet the tile
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
			}
			int total, sum;
			const int pos = block_excl_scan(sm.warp_tot, f, total);
			__syncthreads();
			// running micropolygon counts of the queued grids
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
			lp += kThreadsS;
			continue;
		}
		// one micropolygon of the stream per thread: is it a candidate of this
		// tile?  Its grid: lane 0 searches for the warp's first position, the
		// other lanes step on from there.
		const int p = r0 + t;
		int lo0 = 0;
		if ((t & 31) == 0 && p < qtotal) {
			int lo = 0, hi = sm.qn - 1;
			while (lo < hi) {
				const int mid = (lo + hi + 1) >> 1;
				if (sm.qcum[mid] <= p) lo = mid; else hi = mid - 1;
			}
			lo0 = lo;
		}
		lo0 = __shfl_sync(0xffffffffu, lo0, 0);
		bool active = false;
		int gid = 0, m = 0;
		if (p < qtotal) {
			const int lo = advance_item(sm.qcum, sm.qn, lo0, p);
			gid = sm.qgrid[lo];
			m = p - sm.qcum[lo];
			const int cu = __ldg(g.cu + gid);
			const int sub = sm.qsub[lo];
			if (sub >= 0) {
				const int w = sub >> 16, jv = m / w;
				m = ((sub >> 8) & 0xff) * cu + jv * cu + (sub & 0xff) + (m - jv * w);
			}
			const long long pb = __ldg(g.pbase + gid);
			const int iv = m / cu, iu = m - iv * cu;
			const int index = iv * (cu + 1) + iu;
			const V3f a = ld3(g.P, pb + index), b = ld3(g.P, pb + index + 1);
			const V3f c = ld3(g.P, pb + index + cu + 1), d = ld3(g.P, pb + index + cu + 2);
			const float bminx = amin(amin(amin(a.x, b.x), d.x), c.x);
			const float bminy = amin(amin(amin(a.y, b.y), d.y), c.y);
			const float bminz = amin(amin(amin(a.z, b.z), d.z), c.z);
			const float bmaxx = amax(amax(amax(a.x, b.x), d.x), c.x);
			const float bmaxy = amax(amax(amax(a.y, b.y), d.y), c.y);
			const bool culled = g.culled && g.culled[__ldg(g.mpbase + gid) + m];
			// AddMPG crop cull (imagebuffer.cpp:533-539)
			const bool cropped =
			    bmaxx < fp.cull_x0 || bmaxy < fp.cull_y0 || bminx > fp.cull_x1 || bminy > fp.cull_y1;
			const int sX = max((int)floorf(bminx), tpx0), eX = min(lceil_f(bmaxx), tpx1);
			const int sY = max((int)floorf(bminy), tpy0), eY = min(lceil_f(bmaxy), tpy1);
			active = !culled && !cropped && sX < eX && sY < eY;
			if (active && cullable && !(MAY_CSG && csg_grid(g, gid))) {
				// early-z for every pixel it visits: behind all their samples' occluding depths
				float mx = -FLT_MAX;
				for (int yy = sY; yy < eY; ++yy)
					for (int xx = sX; xx < eX; ++xx) mx = fmaxf(mx, sm.pixmax[(yy - tpy0) * fp.tile_w + (xx - tpx0)]);
				if (bminz > mx) active = false;
			}
		}
		int total;
		const int rank = block_excl_scan(sm.warp_tot, active, total);
		const int navail = kSlots - npend;
		if (t == 0) sm.first_reject = kThreadsS;
		__syncthreads();
		if (active && rank == navail) sm.first_reject = t;
		if (active && rank < navail) sm.pend[npend + rank] = make_int2(gid, m);
		__syncthreads();
		const int consumed = (total > navail) ? sm.first_reject : min(kThreadsS, qtotal - r0);
		npend += min(total, navail);
		r0 += consumed;
	}
	return false;
}

// PERSIST: a fixed grid of CTAs pulls tiles from a device work queue
// (`queue[0]` counts tiles handed out, `order` lists tiles costliest first);
// otherwise one CTA per tile.
template <bool TRANSP, bool PERSIST>
__global__ void __launch_bounds__(kThreadsS, 2)
sample_static_kernel(FrameParams fp, GridsDev g, SamplerDev smp, BinBuffers bb, SampleStore st, FragPool pool,
                     int* queue, const int* order) {
	// a fragment-only frame without occluders is rendered by sample_frag_kernel
	if (TRANSP && fp.frag_only && !(fp.cullable && *pool.occluders)) return;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	SmemS& sm = *reinterpret_cast<SmemS*>(smem_raw);
	int32_t* fhead = reinterpret_cast<int32_t*>(smem_raw + sizeof(SmemS));  // TRANSP: fragment lists
	__shared__ int next_tile;
	const int ntiles = fp.ntx * fp.nty;
	for (int job = 0;; ++job) {
	int tile;
	if (PERSIST) {
		__syncthreads();
		if (threadIdx.x == 0) next_tile = atomicAdd(queue, 1);
		__syncthreads();
		tile = next_tile;
		if (tile >= ntiles) break;
		if (order) tile = order[tile];
	} else {
		if (job > 0) break;
		tile = blockIdx.x;
	}
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

	for (int i = t; i < tsamp; i += kThreadsS) {
		sm.soz[i] = FLT_MAX;
		sm.swin[i] = -1;
		if (TRANSP) fhead[i] = -1;
	}
	for (int i = t; i < kTilePixMax * kWordsS; i += kThreadsS) (&sm.mask[0][0])[i] = 0u;
	for (int i = t; i < kTilePixMax; i += kThreadsS) sm.pixmax[i] = FLT_MAX;
	if (t < 16) sm.blkmax[t] = FLT_MAX;
	if (t == 0) {
		sm.qn = 0;
		sm.qcum[0] = 0;
	}
	__syncthreads();

	const int lbeg = bb.st_offset[st_idx * bb.nranges];
	const int lend = (int)min((long long)bb.st_offset[(st_idx + 1) * bb.nranges], (long long)bb.list_capacity);

	// Stream cursor (uniform over the block): next list chunk, position in
	// the micropolygon stream of the queued grids.
	int lp = lbeg, r0 = 0, qtotal = 0;
	int npend = 0;
	for (;;) {
		// ---- phase A ----
		const bool exhausted =
		    stage_candidates<kSlotsS>(fp, g, bb, sm, tpx0, tpy0, tpx1, tpy1, lend, lp, r0, qtotal, npend);
		if (npend == 0) break;

		// ---- build the staged records with every thread busy ----
		for (int slot = t; slot < npend; slot += kThreadsS) {
			const int2 e = sm.pend[slot];
			RecS& rec = sm.rec[slot];
			build_record(fp, g, e.x, e.y, rec);
			const int sX = max(rec.px0, tpx0), eX = min(rec.px1, tpx1);
			const int sY = max(rec.py0, tpy0), eY = min(rec.py1, tpy1);
			const uint32_t bit = 1u << (slot & 31);
			const int wd = slot >> 5;
			for (int yy = sY; yy < eY; ++yy)
				for (int xx = sX; xx < eX; ++xx)
					atomicOr(&sm.mask[(yy - tpy0) * fp.tile_w + (xx - tpx0)][wd], bit);
		}
		__syncthreads();

		// ---- phase B: a warp walks 32 samples' candidates in insertion order ----
		float wmax = -FLT_MAX;
		for (int gq = warp; gq < ngroups; gq += kWarpsS) {
			const int s = gq * 32 + lane;
			const int pl = s / spp;
			const int si = s - pl * spp;
			const int lx = pl % fp.tile_w, ly = pl / fp.tile_w;
			const int px = tpx0 + lx, py = tpy0 + ly;
			const bool valid = s < tsamp && px < tpx1 && py < tpy1;
			const int sn = si / fp.xs, smm = si - sn * fp.xs;
			float x = 0.0f, y = 0.0f, oz = -FLT_MAX;
			int w = -1, fh = -1;
			if (valid) {
				const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
				const long long pat = smp.pos_index ? (long long)__ldg(smp.pos_index + pix) : pix;
				const float2 o = __ldg(smp.pos + pat * spp + si);
				x = (float)px + o.x;  // CqImagePixel::setSamples: offset + positions[i]
				y = (float)py + o.y;
				oz = sm.soz[s];
				w = sm.swin[s];
				if (TRANSP) fh = fhead[s];
			}
			float gmax = warp_max_f(oz);
#pragma unroll 1
			for (int wd = 0; wd < kWordsS; ++wd) {
				const uint32_t mine = sm.mask[valid ? pl : 0][wd];  // index stays in bounds for idle lanes
				uint32_t bits = __reduce_or_sync(0xffffffffu, valid ? mine : 0u);
				while (bits) {
					const int b = __ffs(bits) - 1;
					bits &= bits - 1u;
					const RecS& r = sm.rec[wd * 32 + b];
					const bool rcull = cullable && !(r.bits & kRecCsg);  // CSG: never occlusion-culled
					if (rcull && r.bminz > gmax) continue;  // hidden from all 32 samples
					bool ok = valid && px >= r.px0 && px < r.px1 && py >= r.py0 && py < r.py1;
					if (ok) {
						const int m_lo = (px == r.px0) ? r.im : 0;
						const int m_hi = (px == r.px1 - 1) ? r.em : fp.xs;
						const int n_lo = (py == r.py0) ? r.in_ : 0;
						const int n_hi = (py == r.py1 - 1) ? r.en : fp.ys;
						ok = smm >= m_lo && smm < m_hi && sn >= n_lo && sn < n_hi;
					}
					// CqBound::Contains2D (bound.h:144-151) and early-z (bucketprocessor.cpp:1179)
					ok = ok && !((x < r.bminx || x > r.bmaxx) || (y < r.bminy || y > r.bmaxy));
					ok = ok && !(rcull && r.bminz > oz);
					ok = ok && !((r.bits & kRecLod) && lod_rejects(fp, g, smp, r.bits >> kRecGridShift, px, py,
					                                               sn * fp.xs + smm));
					ok = ok && edges_inside(r.ym, r.xm, r.ex, r.ey, x, y);
					bool stored = false;
					if (ok) {
						float u, v;
						inv_bilinear(r.ax, r.ay, r.e_x, r.e_y, r.f_x, r.f_y, r.g_x, r.g_y,
						             (r.bits & kRecLinear) != 0, x, y, u, v);
						const float D = bilerp1(r.z[0], r.z[1], r.z[2], r.z[3], u, v);
						// StoreSample (bucketprocessor.cpp:1471-1569) for a hit the split line keeps
						if (rec_keeps(g, bb, r.bits, r.id, x, y, u, v) && !(rcull && oz <= D)) {
							if ((r.bits & kRecOccluding) && rcull) {
								if (TRANSP && fp.midpoint_store) {
									// midpoint filter with a z display (bucketprocessor.cpp:1502-1530):
									// occlZ follows the second-nearest opaque depth, the hit the nearest
									const long long hx =
									    ((long long)(py - fp.sy0) * fp.sw + (px - fp.sx0)) * spp + si;
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
								// append a fragment {depth, id, u, v}; lists are newest-first
								const unsigned act = __activemask();
								const int leader = __ffs(act) - 1;
								const int rank = __popc(act & ((1u << lane) - 1u));
								unsigned long long base = 0;
								if (lane == leader) base = atomicAdd(pool.count, (unsigned long long)__popc(act));
								base = __shfl_sync(act, base, leader);
								const long long idx = (long long)base + rank;
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
					if (__any_sync(0xffffffffu, stored)) gmax = warp_max_f(oz);
				}
			}
			if (valid) {
				sm.soz[s] = oz;
				sm.swin[s] = w;
				if (TRANSP) fhead[s] = fh;
			}
			wmax = fmaxf(wmax, gmax);
		}
		(void)wmax;
		// largest occluding depth per pixel and per 4x4 block, then clear the masks
		__syncthreads();
		for (int pp = t; pp < tpix; pp += kThreadsS) {
			float mx = -FLT_MAX;
			for (int k = 0; k < spp; ++k) mx = max_depth(mx, sm.soz[pp * spp + k]);
			sm.pixmax[pp] = mx;
		}
		for (int i = t; i < kTilePixMax * kWordsS; i += kThreadsS) (&sm.mask[0][0])[i] = 0u;
		__syncthreads();
		if (t < 16) {
			const int nbx = (fp.tile_w + 3) >> 2;
			const int bx = t % nbx, by = t / nbx;
			float mx = -FLT_MAX;
			if (by * 4 < fp.tile_h)
				for (int yy = by * 4; yy < min(by * 4 + 4, fp.tile_h); ++yy)
					for (int xx = bx * 4; xx < min(bx * 4 + 4, fp.tile_w); ++xx) mx = fmaxf(mx, sm.pixmax[yy * fp.tile_w + xx]);
			sm.blkmax[t] = mx;
		}
		__syncthreads();
		npend = 0;
		if (exhausted) break;
	}

	// ---- resolve: colours of the occluding hits, Combine of fragment lists ----
	// (consecutive threads take the samples of one pixel, whose fragments the
	// same warp allocated together)
	for (int s = t; s < tsamp; s += kThreadsS) {
		const int pl = s / spp;
		const int si = s - pl * spp;
		const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
		if (px >= tpx1 || py >= tpy1) continue;
		const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
		const long long pat = smp.pos_index ? (long long)__ldg(smp.pos_index + pix) : pix;
		const float2 o = __ldg(smp.pos + pat * spp + si);
		resolve_sample<TRANSP>(fp, g, pool, st, pix * spp + si, store_index(pix, si, spp), (float)px + o.x, (float)py + o.y,
		                       sm.soz[s], sm.swin[s], TRANSP ? fhead[s] : -1);
		if (st.wmask) st.wmask[store_index(pix, si, spp)] = window_mask(fp, px, py, (float)px + o.x, (float)py + o.y);
	}
	}  // tile loop
}


// ---- opaque frames: parallel hit tests with an ordered fallback ----------
//
// When every micropolygon is opaque, StoreSample's early-z and store rule
// (bucketprocessor.cpp:1179, 1475: skip if bound.min.z > occlZ, keep the hit
// only if D < occlZ) reduce, for every hit whose depth D is not below its own
// bound's minimum z, to "occlZ = min(occlZ, D), first of equal depths wins":
// such a hit skipped by early-z has D >= min.z > occlZ and would not have
// been kept anyway.  So the winner of a sample is the least (D, insertion
// order) over those hits, which does not depend on the order in which they
// are visited: (candidate, sample) pairs are tested in parallel and folded
// with a 64-bit shared-memory atomicMin on (ordered depth bits, id + 1).
// A hit with D below its bound's minimum (rounding or Newton error), a NaN
// or a zero depth (the signs of zero compare equal) may behave differently
// in order, so the sample is flagged and replayed in insertion order over
// the round's candidates from its state at the start of the round.  A
// sample whose occlZ becomes NaN or zero stays on the ordered replay for
// the rest of the tile.  Early-z in the parallel pass tests the depth at the
// start of the round, which is never below the depth the ordered sequence
// would see, so it only skips what the reference skips.
constexpr int kSlotsO = 192;

// Division of k < 2^16 by 1 <= d < 2^16 with a multiply: m = ceil(2^32 / d)
// makes floor(k * m / 2^32) exact (the error k * (m - 2^32/d) / 2^32 < 2^-16 <
// 1/d); d = 1 has no 32-bit m and is passed through.
__device__ __forceinline__ uint32_t div_magic(int d) { return d > 1 ? 0xffffffffu / (uint32_t)d + 1u : 0u; }
__device__ __forceinline__ int div_small(int k, int d, uint32_t m) { return d > 1 ? (int)__umulhi((uint32_t)k, m) : k; }

__device__ __forceinline__ unsigned long long depth_key(float z, int w) {
	const uint32_t u = __float_as_uint(z);
	const uint32_t o = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
	return ((unsigned long long)o << 32) | (uint32_t)(w + 1);
}
__device__ __forceinline__ float key_depth(unsigned long long k) {
	const uint32_t o = (uint32_t)(k >> 32);
	return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
__device__ __forceinline__ int key_winner(unsigned long long k) { return (int)(uint32_t)k - 1; }

struct SmemO {
	unsigned long long key[kTileSampMax];   // occluding hit of each tile sample (depth_key)
	unsigned long long prev[kTileSampMax];  // ... at the start of the round
	RecS rec[kSlotsO];
	int2 pend[kSlotsO];
	int pref[kSlotsO + 1];                  // running count of (candidate, sample) tests
	int rng[kSlotsO][4];                    // tests in the first column, the first row, per row; divisor magic
	int qgrid[kThreadsS];
	int qcum[kThreadsS + 1];
	int qsub[kThreadsS];
	int patidx[kTilePixMax];                // sample pattern of each tile pixel
	int warp_tot[32];
	int first_reject;
	int qn;
	float pixmax[kTilePixMax];
	float blkmax[16];
	uint32_t flag[kTileSampMax / 32];       // samples replayed in order this round
	uint32_t sticky[kTileSampMax / 32];     // samples replayed in order for the rest of the tile
	uint32_t dirty[kTilePixMax / 32];       // pixels whose samples changed this round
};

template <bool PERSIST>
__global__ void __launch_bounds__(kThreadsS, 2)
sample_opaque_kernel(FrameParams fp, GridsDev g, SamplerDev smp, BinBuffers bb, SampleStore st, int* queue,
                     const int* order) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	SmemO& sm = *reinterpret_cast<SmemO*>(smem_raw);
	__shared__ int next_tile;
	const int ntiles = fp.ntx * fp.nty;
	const FragPool nopool{};
	for (int job = 0;; ++job) {
	int tile;
	if (PERSIST) {
		__syncthreads();
		if (threadIdx.x == 0) next_tile = atomicAdd(queue, 1);
		__syncthreads();
		tile = next_tile;
		if (tile >= ntiles) break;
		if (order) tile = order[tile];
	} else {
		if (job > 0) break;
		tile = blockIdx.x;
	}
	const int tx = tile % fp.ntx, ty = tile / fp.ntx;
	const int tpx0 = fp.sx0 + tx * fp.tile_w, tpy0 = fp.sy0 + ty * fp.tile_h;
	const int tpx1 = min(tpx0 + fp.tile_w, fp.sx0 + fp.sw), tpy1 = min(tpy0 + fp.tile_h, fp.sy0 + fp.sh);
	const int st_idx = (ty / fp.st_tiles) * fp.nstx + (tx / fp.st_tiles);
	const int t = threadIdx.x;
	const int spp = fp.spp, xs = fp.xs, ys = fp.ys;
	const uint32_t mxs = div_magic(xs), mys = div_magic(ys);
	const int tpix = fp.tile_w * fp.tile_h;
	const int tsamp = tpix * spp;
	const int nflagw = (tsamp + 31) >> 5;
	const unsigned long long kinit = depth_key(FLT_MAX, -1);

	for (int i = t; i < tsamp; i += kThreadsS) {
		sm.key[i] = kinit;
		sm.prev[i] = kinit;
	}
	for (int i = t; i < kTileSampMax / 32; i += kThreadsS) {
		sm.flag[i] = 0u;
		sm.sticky[i] = 0u;
	}
	if (t < kTilePixMax / 32) sm.dirty[t] = 0u;
	for (int i = t; i < kTilePixMax; i += kThreadsS) {
		sm.pixmax[i] = FLT_MAX;
		const int px = tpx0 + i % fp.tile_w, py = tpy0 + i / fp.tile_w;
		int pat = 0;
		if (i < tpix && px < tpx1 && py < tpy1) {
			const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
			pat = smp.pos_index ? (int)__ldg(smp.pos_index + pix) : (int)pix;
		}
		sm.patidx[i] = pat;
	}
	if (t < 16) sm.blkmax[t] = FLT_MAX;
	if (t == 0) {
		sm.qn = 0;
		sm.qcum[0] = 0;
	}
	__syncthreads();

	const int lbeg = bb.st_offset[st_idx * bb.nranges];
	const int lend = (int)min((long long)bb.st_offset[(st_idx + 1) * bb.nranges], (long long)bb.list_capacity);
	int lp = lbeg, r0 = 0, qtotal = 0, npend = 0;
	for (;;) {
		const bool exhausted =
		    stage_candidates<kSlotsO, false>(fp, g, bb, sm, tpx0, tpy0, tpx1, tpy1, lend, lp, r0, qtotal, npend);
		if (npend == 0) break;

		// ---- records, and the (candidate, sample) tests RenderMPG_Static makes ----
		// The samples a candidate visits form a product set: columns of the
		// clipped pixel range with their sub-sample ranges (the first and last
		// pixel trimmed, bucketprocessor.cpp:1135-1153) times the same in y.
		int ntests = 0;
		if (t < npend) {
			const int2 e = sm.pend[t];
			RecS& r = sm.rec[t];
			build_record(fp, g, e.x, e.y, r);
			const int sX = max(r.px0, tpx0), eX = min(r.px1, tpx1);
			const int sY = max(r.py0, tpy0), eY = min(r.py1, tpy1);
			// per-axis counts: first pixel, then full pixels, the last one trimmed
			int cx0 = ((sX == r.px1 - 1) ? r.em : xs) - ((sX == r.px0) ? r.im : 0);
			int totx = cx0;
			if (eX - sX > 1) totx += (eX - sX - 2) * xs + ((eX - 1 == r.px1 - 1) ? r.em : xs);
			int cy0 = ((sY == r.py1 - 1) ? r.en : ys) - ((sY == r.py0) ? r.in_ : 0);
			int toty = cy0;
			if (eY - sY > 1) toty += (eY - sY - 2) * ys + ((eY - 1 == r.py1 - 1) ? r.en : ys);
			totx = max(totx, 0);
			toty = max(toty, 0);
			ntests = totx * toty;
			sm.rng[t][0] = cx0;
			sm.rng[t][1] = cy0;
			sm.rng[t][2] = totx;
			sm.rng[t][3] = (int)div_magic(totx);
		}
		int total;
		const int pre = block_excl_sum(sm.warp_tot, ntests, total);
		if (t < npend) sm.pref[t] = pre;
		__syncthreads();

		// ---- parallel pass: one (candidate, sample) test per lane, each warp
		// walking a contiguous run of tests so a lane finds its candidate a
		// step or two on from where the warp's last lane stopped ----
		const int chunk = ((total + kThreadsS - 1) / kThreadsS) * 32;
		const int pw0 = (t >> 5) * chunk, pw1 = min(total, pw0 + chunk);
		int cur = 0;
		for (int p0 = pw0; p0 < pw1; p0 += 32) {
			const int p = p0 + (t & 31);
			const int lo = advance_item(sm.pref, npend, cur, min(p, pw1 - 1));
			cur = __shfl_sync(0xffffffffu, lo, 31);
			if (p >= pw1) continue;
			const RecS& r = sm.rec[lo];
			const int k = p - sm.pref[lo];
			const int cx0 = sm.rng[lo][0], cy0 = sm.rng[lo][1], totx = sm.rng[lo][2];
			const uint32_t mtot = (uint32_t)sm.rng[lo][3];
			const int sX = max(r.px0, tpx0), sY = max(r.py0, tpy0);
			const int ky = div_small(k, totx, mtot), kx = k - ky * totx;
			int px, m, py, n;
			if (kx < cx0) {
				px = sX;
				m = ((sX == r.px0) ? r.im : 0) + kx;
			} else {
				const int q = kx - cx0;
				const int qd = div_small(q, xs, mxs);
				px = sX + 1 + qd;
				m = q - qd * xs;
			}
			if (ky < cy0) {
				py = sY;
				n = ((sY == r.py0) ? r.in_ : 0) + ky;
			} else {
				const int q = ky - cy0;
				const int qd = div_small(q, ys, mys);
				py = sY + 1 + qd;
				n = q - qd * ys;
			}
			const int si = n * xs + m;
			const int pl = (py - tpy0) * fp.tile_w + (px - tpx0);
			const int s = pl * spp + si;
			if (sm.flag[s >> 5] & (1u << (s & 31))) continue;  // replayed in order below
			const float2 o = __ldg(smp.pos + (long long)sm.patidx[pl] * spp + si);
			const float x = (float)px + o.x, y = (float)py + o.y;
			// CqBound::Contains2D (bound.h:144-151), early-z, fContains
			if ((x < r.bminx || x > r.bmaxx) || (y < r.bminy || y > r.bmaxy)) continue;
			if (r.bminz > key_depth(sm.prev[s])) continue;
			if ((r.bits & kRecLod) && lod_rejects(fp, g, smp, r.bits >> kRecGridShift, px, py, si)) continue;
			if (!edges_inside(r.ym, r.xm, r.ex, r.ey, x, y)) continue;
			float u, v;
			inv_bilinear(r.ax, r.ay, r.e_x, r.e_y, r.f_x, r.f_y, r.g_x, r.g_y, (r.bits & kRecLinear) != 0, x, y, u,
			             v);
			const float D = bilerp1(r.z[0], r.z[1], r.z[2], r.z[3], u, v);
			if (!rec_keeps(g, bb, r.bits, r.id, x, y, u, v)) continue;
			if (!(D >= r.bminz) || D == 0.0f) {
				atomicOr(&sm.flag[s >> 5], 1u << (s & 31));
			} else {
				const unsigned long long k = depth_key(D, r.id);
				if (k < atomicMin(&sm.key[s], k)) atomicOr(&sm.dirty[pl >> 5], 1u << (pl & 31));
			}
		}
		__syncthreads();
		int anyf = 0;
		for (int i = t; i < nflagw; i += kThreadsS) anyf |= (int)(sm.flag[i] != 0u);

		// ---- ordered replay of flagged samples: a warp per sample ----
		// Lanes test 32 candidates at a time (the tests do not depend on
		// occlZ); lane order then applies early-z and the store rule in
		// insertion order.
		if (__syncthreads_or(anyf)) {
			const int lane = t & 31, warp = t >> 5;
			for (int wd = warp; wd < nflagw; wd += kWarpsS) {
				uint32_t fb = sm.flag[wd];
				while (fb) {
					const int s = wd * 32 + __ffs(fb) - 1;
					fb &= fb - 1u;
					const int pl = s / spp, si = s - pl * spp;
					const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
					if (px >= tpx1 || py >= tpy1) continue;
					const int sn = si / xs, smm = si - sn * xs;
					const float2 o = __ldg(smp.pos + (long long)sm.patidx[pl] * spp + si);
					const float x = (float)px + o.x, y = (float)py + o.y;
					float oz = key_depth(sm.prev[s]);
					int w = key_winner(sm.prev[s]);
					for (int c0 = 0; c0 < npend; c0 += 32) {
						const int c = c0 + lane;
						bool hit = false;
						float D = 0.0f, bz = 0.0f;
						int id = 0;
						if (c < npend) {
							const RecS& r = sm.rec[c];
							const int m_lo = (px == r.px0) ? r.im : 0, m_hi = (px == r.px1 - 1) ? r.em : xs;
							const int n_lo = (py == r.py0) ? r.in_ : 0, n_hi = (py == r.py1 - 1) ? r.en : ys;
							hit = px >= r.px0 && px < r.px1 && py >= r.py0 && py < r.py1 && smm >= m_lo && smm < m_hi &&
							      sn >= n_lo && sn < n_hi &&
							      !((x < r.bminx || x > r.bmaxx) || (y < r.bminy || y > r.bmaxy)) &&
							      !((r.bits & kRecLod) &&
							        lod_rejects(fp, g, smp, r.bits >> kRecGridShift, px, py, si)) &&
							      edges_inside(r.ym, r.xm, r.ex, r.ey, x, y);
							if (hit) {
								float u, v;
								inv_bilinear(r.ax, r.ay, r.e_x, r.e_y, r.f_x, r.f_y, r.g_x, r.g_y,
								             (r.bits & kRecLinear) != 0, x, y, u, v);
								D = bilerp1(r.z[0], r.z[1], r.z[2], r.z[3], u, v);
								bz = r.bminz;
								id = r.id;
								hit = rec_keeps(g, bb, r.bits, r.id, x, y, u, v);
							}
						}
						uint32_t hb = __ballot_sync(0xffffffffu, hit);
						while (hb) {
							const int b = __ffs(hb) - 1;
							hb &= hb - 1u;
							const float Db = __shfl_sync(0xffffffffu, D, b);
							const float bzb = __shfl_sync(0xffffffffu, bz, b);
							const int idb = __shfl_sync(0xffffffffu, id, b);
							if (!(bzb > oz) && !(oz <= Db)) {
								oz = Db;
								w = idb;
							}
						}
					}
					if (lane == 0) {
						sm.key[s] = depth_key(oz, w);
						atomicOr(&sm.dirty[pl >> 5], 1u << (pl & 31));
						if (oz != oz || oz == 0.0f) atomicOr(&sm.sticky[s >> 5], 1u << (s & 31));
					}
				}
			}
		}
		__syncthreads();

		// ---- end of round: state and largest occluding depth of the pixels
		// whose samples changed (two threads per pixel, even and odd samples;
		// the maximum does not depend on the order, NaN counting as +inf),
		// flags ----
		for (int u0 = 0; u0 < 2 * tpix; u0 += kThreadsS) {
			const int u = u0 + t, pp = u >> 1, half = u & 1;
			const bool act = pp < tpix && (sm.dirty[pp >> 5] & (1u << (pp & 31)));
			float mx = -FLT_MAX;
			if (act)
				for (int k = half; k < spp; k += 2) {
					const unsigned long long kk = sm.key[pp * spp + k];
					sm.prev[pp * spp + k] = kk;
					mx = max_depth(mx, key_depth(kk));
				}
			mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
			if (act && half == 0) sm.pixmax[pp] = mx;
		}
		for (int i = t; i < nflagw; i += kThreadsS) sm.flag[i] = sm.sticky[i];
		__syncthreads();
		if (t < kTilePixMax / 32) sm.dirty[t] = 0u;
		if (t < 16 * 16) {
			// 4x4-pixel block t / 16, one pixel per thread
			const int b = t >> 4, j = t & 15;
			const int nbx = (fp.tile_w + 3) >> 2;
			const int bx = b % nbx, by = b / nbx;
			const int yy = by * 4 + (j >> 2), xx = bx * 4 + (j & 3);
			float mx = (yy < fp.tile_h && xx < fp.tile_w) ? sm.pixmax[yy * fp.tile_w + xx] : -FLT_MAX;
#pragma unroll
			for (int o = 1; o < 16; o <<= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
			if (j == 0) sm.blkmax[b] = mx;
		}
		__syncthreads();
		npend = 0;
		if (exhausted) break;
	}

	// ---- resolve: colours of the occluding hits ----
	if (st.keys) {
		// hand the occluding hits to resolve_opaque_kernel, pixel-major
		// ([pixel][sample index]) like its threads
		for (int q = t; q < tsamp; q += kThreadsS) {
			const int pl = q / spp;
			const int si = q - pl * spp;
			const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
			if (px >= tpx1 || py >= tpy1) continue;
			st.keys[((long long)(py - fp.sy0) * fp.sw + (px - fp.sx0)) * spp + si] = sm.key[pl * spp + si];
		}
		continue;
	}
	// pixel-major: the lanes of a pixel's samples mostly resolve the same
	// winner, whose grid, vertex and colour loads then merge (measured faster
	// than sample-major order, whose store writes coalesce instead)
	for (int q = t; q < tsamp; q += kThreadsS) {
		const int pl = q / spp;
		const int si = q - pl * spp;
		const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
		if (px >= tpx1 || py >= tpy1) continue;
		const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
		const float2 o = __ldg(smp.pos + (long long)sm.patidx[pl] * spp + si);
		const unsigned long long kk = sm.key[pl * spp + si];
		resolve_sample<false>(fp, g, nopool, st, pix * spp + si, store_index(pix, si, spp), (float)px + o.x, (float)py + o.y,
		                      key_depth(kk), key_winner(kk), -1);
		if (st.wmask) st.wmask[store_index(pix, si, spp)] = window_mask(fp, px, py, (float)px + o.x, (float)py + o.y);
	}
	}  // tile loop
}

// Colours of the occluding hits of an opaque frame: one thread per sample,
// pixel-major (consecutive threads, the samples of one pixel, which mostly
// share a winner whose loads then merge).
__global__ void __launch_bounds__(256)
resolve_opaque_kernel(FrameParams fp, GridsDev g, SamplerDev smp, SampleStore st) {
	const long long npix = (long long)fp.sw * fp.sh;
	const long long q0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // pixel * spp + sample index
	if (q0 >= npix * fp.spp) return;
	const long long pix = q0 / fp.spp;
	const int si = (int)(q0 - pix * fp.spp);
	const long long q = store_index(pix, si, fp.spp);
	const int px = fp.sx0 + (int)(pix % fp.sw), py = fp.sy0 + (int)(pix / fp.sw);
	const long long pat = smp.pos_index ? (long long)__ldg(smp.pos_index + pix) : pix;
	const float2 o = __ldg(smp.pos + pat * fp.spp + si);
	const unsigned long long kk = st.keys[q0];
	resolve_sample<false>(fp, g, FragPool{}, st, pix * fp.spp + si, q, (float)px + o.x, (float)py + o.y,
	                      key_depth(kk), key_winner(kk), -1);
	if (st.wmask) st.wmask[q] = window_mask(fp, px, py, (float)px + o.x, (float)py + o.y);
}


// ---- fragment-only frames: parallel hit tests appending fragments --------
//
// When no micropolygon of a static frame can be occluding (none opaque, none
// matte alpha), or samples are not cullable (a z display with the max or
// average depth filter), StoreSample never sets an occluding hit: occlZ stays
// FLT_MAX, early-z skips only bounds with min.z > FLT_MAX, and every hit with
// !(cullable && FLT_MAX <= D) becomes a fragment (bucketprocessor.cpp:
// 1471-1569).  Which hits are kept then does not depend on order, and Combine
// orders fragments by (depth, micropolygon id), so (micropolygon, sample)
// tests run in parallel as on the opaque path and hits are appended to the
// fragment pool in any order: each block iteration reserves its hits' slots
// with one atomic and links them into per-sample lists in shared memory.
constexpr int kSlotsF = 256;
constexpr int kFragRun = 256;  // pool slots a warp reserves at a time

struct SmemF {
	RecS rec[kSlotsF];
	int2 pend[kSlotsF];
	int pref[kSlotsF + 1];
	int rng[kSlotsF][4];
	int qgrid[kThreadsS];
	int qcum[kThreadsS + 1];
	int qsub[kThreadsS];
	int patidx[kTilePixMax];
	int warp_tot[32];
	int first_reject;
	int qn;
	float pixmax[kTilePixMax];  // stay FLT_MAX: no occluding hits
	float blkmax[16];
	int32_t fhead[kTileSampMax];
};

template <bool PERSIST>
__global__ void __launch_bounds__(kThreadsS, 2)
sample_frag_kernel(FrameParams fp, GridsDev g, SamplerDev smp, BinBuffers bb, SampleStore st, FragPool pool,
                   int* queue, const int* order) {
	if (fp.cullable && *pool.occluders) return;  // the ordered kernel renders this frame
	extern __shared__ __align__(16) unsigned char smem_raw[];
	SmemF& sm = *reinterpret_cast<SmemF*>(smem_raw);
	__shared__ int next_tile;
	const int ntiles = fp.ntx * fp.nty;
	const int cullable = fp.cullable;
	unsigned long long rnext = 0, rend = 0;  // this warp's reserved pool slots [rnext, rend)
	for (int job = 0;; ++job) {
	int tile;
	if (PERSIST) {
		__syncthreads();
		if (threadIdx.x == 0) next_tile = atomicAdd(queue, 1);
		__syncthreads();
		tile = next_tile;
		if (tile >= ntiles) break;
		if (order) tile = order[tile];
	} else {
		if (job > 0) break;
		tile = blockIdx.x;
	}
	const int tx = tile % fp.ntx, ty = tile / fp.ntx;
	const int tpx0 = fp.sx0 + tx * fp.tile_w, tpy0 = fp.sy0 + ty * fp.tile_h;
	const int tpx1 = min(tpx0 + fp.tile_w, fp.sx0 + fp.sw), tpy1 = min(tpy0 + fp.tile_h, fp.sy0 + fp.sh);
	const int st_idx = (ty / fp.st_tiles) * fp.nstx + (tx / fp.st_tiles);
	const int t = threadIdx.x;
	const int spp = fp.spp, xs = fp.xs, ys = fp.ys;
	const uint32_t mxs = div_magic(xs), mys = div_magic(ys);
	const int tpix = fp.tile_w * fp.tile_h;
	const int tsamp = tpix * spp;

	for (int i = t; i < tsamp; i += kThreadsS) sm.fhead[i] = -1;
	for (int i = t; i < kTilePixMax; i += kThreadsS) {
		sm.pixmax[i] = FLT_MAX;
		const int px = tpx0 + i % fp.tile_w, py = tpy0 + i / fp.tile_w;
		int pat = 0;
		if (i < tpix && px < tpx1 && py < tpy1) {
			const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
			pat = smp.pos_index ? (int)__ldg(smp.pos_index + pix) : (int)pix;
		}
		sm.patidx[i] = pat;
	}
	if (t < 16) sm.blkmax[t] = FLT_MAX;
	if (t == 0) {
		sm.qn = 0;
		sm.qcum[0] = 0;
	}
	__syncthreads();

	const int lbeg = bb.st_offset[st_idx * bb.nranges];
	const int lend = (int)min((long long)bb.st_offset[(st_idx + 1) * bb.nranges], (long long)bb.list_capacity);
	int lp = lbeg, r0 = 0, qtotal = 0, npend = 0;
	for (;;) {
		const bool exhausted =
		    stage_candidates<kSlotsF>(fp, g, bb, sm, tpx0, tpy0, tpx1, tpy1, lend, lp, r0, qtotal, npend);
		if (npend == 0) break;

		// records and the (candidate, sample) tests, as on the opaque path
		int ntests = 0;
		if (t < npend) {
			const int2 e = sm.pend[t];
			RecS& r = sm.rec[t];
			build_record(fp, g, e.x, e.y, r);
			const int sX = max(r.px0, tpx0), eX = min(r.px1, tpx1);
			const int sY = max(r.py0, tpy0), eY = min(r.py1, tpy1);
			int cx0 = ((sX == r.px1 - 1) ? r.em : xs) - ((sX == r.px0) ? r.im : 0);
			int totx = cx0;
			if (eX - sX > 1) totx += (eX - sX - 2) * xs + ((eX - 1 == r.px1 - 1) ? r.em : xs);
			int cy0 = ((sY == r.py1 - 1) ? r.en : ys) - ((sY == r.py0) ? r.in_ : 0);
			int toty = cy0;
			if (eY - sY > 1) toty += (eY - sY - 2) * ys + ((eY - 1 == r.py1 - 1) ? r.en : ys);
			totx = max(totx, 0);
			toty = max(toty, 0);
			ntests = totx * toty;
			sm.rng[t][0] = cx0;
			sm.rng[t][1] = cy0;
			sm.rng[t][2] = totx;
			sm.rng[t][3] = (int)div_magic(totx);
		}
		int total;
		const int pre = block_excl_sum(sm.warp_tot, ntests, total);
		if (t < npend) sm.pref[t] = pre;
		__syncthreads();

		// each warp walks a contiguous run of tests (a lane finds its candidate
		// a step or two on from where the warp's last lane stopped) and appends
		// its hits into pool slots it reserved in runs of kFragRun: one global
		// atomic per run, no block barrier per batch of tests.  Lists are
		// sorted by (depth, id) in Combine, so their order does not matter;
		// slots left in a warp's last run stay unused.
		{
			const int lane = t & 31;
			const int chunk = ((total + kThreadsS - 1) / kThreadsS) * 32;
			const int pw0 = (t >> 5) * chunk, pw1 = min(total, pw0 + chunk);
			int cur = 0;
			for (int p0 = pw0; p0 < pw1; p0 += 32) {
				const int p = p0 + lane;
				const int lo = advance_item(sm.pref, npend, cur, min(p, pw1 - 1));
				cur = __shfl_sync(0xffffffffu, lo, 31);
				bool hit = false;
				int s = 0, id = 0;
				float D = 0.0f, u = 0.0f, v = 0.0f;
				if (p < pw1) {
					const RecS& r = sm.rec[lo];
					const int k = p - sm.pref[lo];
					const int cx0 = sm.rng[lo][0], cy0 = sm.rng[lo][1], totx = sm.rng[lo][2];
					const uint32_t mtot = (uint32_t)sm.rng[lo][3];
					const int sX = max(r.px0, tpx0), sY = max(r.py0, tpy0);
					const int ky = div_small(k, totx, mtot), kx = k - ky * totx;
					int px, m, py, n;
					if (kx < cx0) {
						px = sX;
						m = ((sX == r.px0) ? r.im : 0) + kx;
					} else {
						const int q = kx - cx0;
						const int qd = div_small(q, xs, mxs);
						px = sX + 1 + qd;
						m = q - qd * xs;
					}
					if (ky < cy0) {
						py = sY;
						n = ((sY == r.py0) ? r.in_ : 0) + ky;
					} else {
						const int q = ky - cy0;
						const int qd = div_small(q, ys, mys);
						py = sY + 1 + qd;
						n = q - qd * ys;
					}
					const int si = n * xs + m;
					const int pl = (py - tpy0) * fp.tile_w + (px - tpx0);
					s = pl * spp + si;
					const float2 o = __ldg(smp.pos + (long long)sm.patidx[pl] * spp + si);
					const float x = (float)px + o.x, y = (float)py + o.y;
					// Contains2D, early-z against occlZ = FLT_MAX, fContains, StoreSample's test
					hit = !((x < r.bminx || x > r.bmaxx) || (y < r.bminy || y > r.bmaxy)) &&
					      !(cullable && !(r.bits & kRecCsg) && r.bminz > FLT_MAX) &&
					      !((r.bits & kRecLod) && lod_rejects(fp, g, smp, r.bits >> kRecGridShift, px, py, si)) &&
					      edges_inside(r.ym, r.xm, r.ex, r.ey, x, y);
					if (hit) {
						inv_bilinear(r.ax, r.ay, r.e_x, r.e_y, r.f_x, r.f_y, r.g_x, r.g_y, (r.bits & kRecLinear) != 0,
						             x, y, u, v);
						D = bilerp1(r.z[0], r.z[1], r.z[2], r.z[3], u, v);
						hit = rec_keeps(g, bb, r.bits, r.id, x, y, u, v) &&
						      !(cullable && !(r.bits & kRecCsg) && FLT_MAX <= D);
						id = r.id;
					}
				}
				const unsigned bal = __ballot_sync(0xffffffffu, hit);
				const int nh = __popc(bal);
				if (nh > 0) {
					if (rnext + nh > rend) {
						unsigned long long b = 0;
						if (lane == 0) b = atomicAdd(pool.count, (unsigned long long)kFragRun);
						rnext = __shfl_sync(0xffffffffu, b, 0);
						rend = rnext + kFragRun;
					}
					if (hit) {
						const long long idx = (long long)(rnext + __popc(bal & ((1u << lane) - 1u)));
						if (idx < pool.capacity) {
							pool.frag[idx] = make_float4(D, __int_as_float(id), u, v);
							pool.next[idx] = atomicExch(&sm.fhead[s], (int)idx);
						} else {
							atomicOr(pool.overflow, 1);
						}
					}
					rnext += nh;
				}
			}
		}
		__syncthreads();
		npend = 0;
		if (exhausted) break;
	}

	// ---- resolve: Combine of each sample's fragments (or the list heads
	// handed to resolve_frag_kernel) ----
	for (int s = t; s < tsamp; s += kThreadsS) {
		const int pl = s / spp;
		const int si = s - pl * spp;
		const int px = tpx0 + pl % fp.tile_w, py = tpy0 + pl / fp.tile_w;
		if (px >= tpx1 || py >= tpy1) continue;
		const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
		if (pool.heads) {
			pool.heads[pix * spp + si] = sm.fhead[s];
			continue;
		}
		const float2 o = __ldg(smp.pos + (long long)sm.patidx[pl] * spp + si);
		resolve_sample<true>(fp, g, pool, st, pix * spp + si, store_index(pix, si, spp), (float)px + o.x,
		                     (float)py + o.y, FLT_MAX, -1, sm.fhead[s]);
		if (st.wmask) st.wmask[store_index(pix, si, spp)] = window_mask(fp, px, py, (float)px + o.x, (float)py + o.y);
	}
	}  // tile loop
}

// Combine of a fragment-only frame's samples from the list heads
// sample_frag_kernel left: one thread per sample, pixel-major, so a warp
// walks lists whose fragments the sampler's warps allocated together.  The
// kernel holds no shared memory, so the sort's local memory stays in L1.
// Returns at once when the frame has occluders (the ordered kernel resolved).
__global__ void __launch_bounds__(256)
resolve_frag_kernel(FrameParams fp, GridsDev g, SamplerDev smp, SampleStore st, FragPool pool) {
	if (fp.cullable && *pool.occluders) return;
	const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // pixel * spp + sample index
	const long long npix = (long long)fp.sw * fp.sh;
	if (q >= npix * fp.spp) return;
	const long long pix = q / fp.spp;
	const int si = (int)(q - pix * fp.spp);
	const int px = fp.sx0 + (int)(pix % fp.sw), py = fp.sy0 + (int)(pix / fp.sw);
	const long long pat = smp.pos_index ? (long long)__ldg(smp.pos_index + pix) : pix;
	const float2 o = __ldg(smp.pos + pat * fp.spp + si);
	resolve_sample<true>(fp, g, pool, st, q, store_index(pix, si, fp.spp), (float)px + o.x, (float)py + o.y, FLT_MAX, -1,
	                     pool.heads[q]);
	if (st.wmask) st.wmask[store_index(pix, si, fp.spp)] = window_mask(fp, px, py, (float)px + o.x, (float)py + o.y);
}

// Whether any micropolygon of the frame may be occluding: a grid flagged
// opaque or matte alpha, no opacity array, or a vertex with every opacity
// channel at 1 or more (a superset of SqMpgSampleInfo::isOpaque).
__global__ void occluder_scan_kernel(GridsDev g, int32_t* flag) {
	const int gi = blockIdx.x;
	if (gi >= g.ngrids) return;
	const int gflags = __ldg(g.flags + gi);
	bool occ = (gflags & (8 | 4)) != 0 || g.Oi == nullptr;
	if (!occ) {
		const long long nv = (long long)(__ldg(g.cu + gi) + 1) * (__ldg(g.cv + gi) + 1);
		const long long cb = __ldg(g.cbase + gi);
		for (long long i = threadIdx.x; i < nv && !occ; i += blockDim.x) {
			const float4 o = ld_colour(g, g.Oi, cb + i);
			occ = o.x >= 1.0f && o.y >= 1.0f && o.z >= 1.0f;
		}
	}
	if (__syncthreads_or(occ) && threadIdx.x == 0) *flag = 1;
}

}  // namespace

void launch_resolve_opaque(const FrameParams& fp, const GridsDev& g, const SamplerDev& sm, SampleStore st,
                           cudaStream_t s) {
	const long long n = (long long)fp.sw * fp.sh * fp.spp;
	if (n > 0) resolve_opaque_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(fp, g, sm, st);
}

void static_tiling(FrameParams& fp, int tile_pixels) {
	int tpix = min(kTilePixMax, max(1, kTileSampMax / fp.spp));
	if (tile_pixels > 0) tpix = min(tpix, tile_pixels);
	int tw = 1;
	while ((tw + 1) * (tw + 1) <= tpix) ++tw;
	fp.tile_w = tw;
	fp.tile_h = min(16, tpix / tw);  // at most 4x4 blocks of 4x4 pixels (blkmax)
	fp.tpp = 1;
}

void launch_sample_tiles(const FrameParams& fp, const GridsDev& g, const SamplerDev& sm, const BinBuffers& b,
                         SampleStore st, FragPool pool, int32_t* err, cudaStream_t s, cudaEvent_t colours_ready,
                         unsigned wait_flags) {
	(void)err;
	launch_sample_tiles_q(fp, g, sm, b, st, pool, nullptr, nullptr, 0, s, colours_ready, wait_flags);
}

void launch_sample_tiles_q(const FrameParams& fp, const GridsDev& g, const SamplerDev& sm, const BinBuffers& b,
                           SampleStore st, FragPool pool, int* queue, const int* order, int nctas, cudaStream_t s,
                           cudaEvent_t colours_ready, unsigned wait_flags) {
	const int ntiles = fp.ntx * fp.nty;
	const size_t smem_transp = sizeof(SmemS) + sizeof(int32_t) * kTileSampMax;
	configure_sample_kernels();
	const bool transp = pool.capacity > 0;
	const bool split = !transp && st.keys;  // the resolve kernel is the first reader of Ci/Oi
	if (colours_ready && !split) cudaStreamWaitEvent(s, colours_ready, wait_flags);
	if (transp && fp.frag_only) {
		// both kernels are queued; each reads the occluder flag and one returns at once
		if (fp.cullable) {
			cudaMemsetAsync(pool.occluders, 0, sizeof(int32_t), s);
			if (g.ngrids > 0) occluder_scan_kernel<<<g.ngrids, 256, 0, s>>>(g, pool.occluders);
		}
		if (queue)
			sample_frag_kernel<true><<<nctas, kThreadsS, sizeof(SmemF), s>>>(fp, g, sm, b, st, pool, queue, order);
		else
			sample_frag_kernel<false><<<ntiles, kThreadsS, sizeof(SmemF), s>>>(fp, g, sm, b, st, pool, nullptr,
			                                                                  nullptr);
		if (pool.heads) {
			const long long n = (long long)fp.sw * fp.sh * fp.spp;
			if (n > 0) resolve_frag_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(fp, g, sm, st, pool);
		}
	}
	if (queue) {
		if (transp)
			sample_static_kernel<true, true><<<nctas, kThreadsS, smem_transp, s>>>(fp, g, sm, b, st, pool, queue, order);
		else
			sample_opaque_kernel<true><<<nctas, kThreadsS, sizeof(SmemO), s>>>(fp, g, sm, b, st, queue, order);
		if (split) {
			if (colours_ready) cudaStreamWaitEvent(s, colours_ready, wait_flags);
			launch_resolve_opaque(fp, g, sm, st, s);
		}
	} else {
		if (transp)
			sample_static_kernel<true, false><<<ntiles, kThreadsS, smem_transp, s>>>(fp, g, sm, b, st, pool, nullptr, nullptr);
		else
			sample_opaque_kernel<false><<<ntiles, kThreadsS, sizeof(SmemO), s>>>(fp, g, sm, b, st, nullptr, nullptr);
		if (split) {
			if (colours_ready) cudaStreamWaitEvent(s, colours_ready, wait_flags);
			launch_resolve_opaque(fp, g, sm, st, s);
		}
	}
}

// Shared-memory limits of the sampling kernels; safe to call repeatedly, and
// done before any graph capture (context creation calls it).
bool first_use_on_device(std::mutex& mu, uint64_t& mask) {
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
	std::lock_guard<std::mutex> lock(mu);
	if (mask >> dev & 1) return false;
	mask |= uint64_t(1) << dev;
	return true;
}

void configure_sample_kernels() {
	static std::mutex mu;
	static uint64_t configured = 0;
	if (!first_use_on_device(mu, configured)) return;
	const int smem_transp = (int)(sizeof(SmemS) + sizeof(int32_t) * kTileSampMax);
	cudaFuncSetAttribute(sample_opaque_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemO));
	cudaFuncSetAttribute(sample_static_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_transp);
	cudaFuncSetAttribute(sample_opaque_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemO));
	cudaFuncSetAttribute(sample_static_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_transp);
	cudaFuncSetAttribute(sample_frag_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemF));
	cudaFuncSetAttribute(sample_frag_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemF));
	configure_sample_mb_kernels();
}

int sample_static_ctas_per_sm(bool transp) {
	int n = 0;
	if (transp)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sample_static_kernel<true, true>, kThreadsS,
		                                              sizeof(SmemS) + sizeof(int32_t) * kTileSampMax);
	else
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sample_opaque_kernel<true>, kThreadsS, sizeof(SmemO));
	return n > 0 ? n : 1;
}

}  // namespace aqh
