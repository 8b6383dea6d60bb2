// sample.cu -- the sampling stage: subpixel hit tests with depth and opacity
// compositing into the pixel sample store.
//
// Replaces CqBucketProcessor::RenderMicroPoly / RenderMPG_Static /
// RenderMPG_MBOrDof / StoreSample (libs/core/bucketprocessor.cpp:1067-1569),
// CqMicroPolygon::Sample / fContains (micropolygon.cpp:1295-1660, 1768-1914)
// and CqImagePixel::Combine (imagepixel.cpp:144-332).
//
// Layout.  One CTA owns a tile of tile_w x tile_h pixels of the sample region;
// each pixel's samples are split over `tpp` threads, a thread holding up to
// kSamplesPerThread samples (position and occluding depth in registers).
// The CTA walks its super-tile's grid list in submission order and expands
// the grids touching the tile into micropolygons, kSlots at a time:
//   phase A (one thread per micropolygon): bound, vertex order, edge and
//     inverse-bilinear coefficients into a shared-memory record, and a bit
//     per covered pixel in that pixel's candidate mask;
//   phase B (pixel-owner threads): each thread walks its pixel's mask in
//     ascending slot order -- the insertion order -- and runs the reference's
//     per-sample sequence (sub-sample range, inclusive bound test, early-z,
//     edge tests, inverse bilinear, depth, store).
// Because one thread owns each sample and visits its candidates in insertion
// order, the reference's order-dependent early-z and its "first of equal
// depths wins" rule hold exactly.  Colours are resolved once per sample at the
// end (the reference interpolates them at store time; the values are the
// same because they depend only on the winning micropolygon and (u,v)).
#include "aqh_internal.h"
#include "hider_device.cuh"
#include "sample_common.cuh"

namespace aqh {

namespace {

// Shared-memory micropolygon record for the static path.
struct MpRec {
	float bminx, bmaxx, bminy, bmaxy, bminz;
	float ym[4], xm[4], ex[4], ey[4];
	float ax, ay, e_x, e_y, f_x, f_y, g_x, g_y;
	float z[4];
	int id;       // global micropolygon id
	int grid;
	int bits;     // 1 linear, 2 occluding store (opaque or matte alpha), 4 smooth, 8 matte, 16 matte alpha
	float pad;    // odd word stride keeps records of different slots on different banks
};

constexpr int kRecLinear = 1, kRecOccluding = 2, kRecSmooth = 4, kRecMatte = 8, kRecMatteAlpha = 16;

struct Smem {
	MpRec rec[kSlots];
	uint32_t mask[kBlock][kSlotWords];  // per tile pixel (tile pixels <= kBlock)
	int qgrid[kBlock];                  // grids of the current list chunk touching the tile
	int warp_tot[kBlock / 32];
	int qn;
	int nslots;
	int consumed;
	int first_reject;
};

// Final value of one sample: the occluding hit's colour at its (u,v), or the
// Combine of its transparent fragments; written to the sample store.
template <bool TRANSP>
__device__ __forceinline__ void resolve_sample(const FrameParams& fp, const GridsDev& g, const FragPool& pool,
                                            const SampleStore& st, long long sidx, float x, float y, float oz,
                                            int w, int wg, int head) {
	float occl[7] = {0, 0, 0, 0, 0, 0, 0};
	int occl_flags = 0;
	if (w >= 0) {
		// recompute (u,v) of the winner exactly as when it was stored
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
		occl[6] = oz;
	}
	int nf = 0;
	bool valid = w >= 0;
	if (TRANSP && head >= 0) {
		nf = combine_fragments(fp, g, pool, head, w >= 0, oz, occl, occl_flags);
		valid = true;
	}
	if (nf == 0 && valid) {
		// imagepixel.cpp:303-330: opaque matte hits become transparent black;
		// the midpoint depth filter averages with occlZ
		if (occl_flags & 1)
			for (int q = 0; q < 6; ++q) occl[q] = 0.0f;
		if (fp.depth_filter == 1) occl[6] = (float)(0.5 * ((double)occl[6] + (double)oz));
	}
	st.a[sidx] = make_float4(occl[0], occl[1], occl[2], occl[6]);
	st.b[sidx] = make_float4(occl[3], occl[4], occl[5], valid ? 1.0f : 0.0f);
	if (st.winner) st.winner[sidx] = w;
	if (st.occlz) st.occlz[sidx] = oz;
	if (st.nfrag) st.nfrag[sidx] = nf;
}

template <bool TRANSP>
__global__ void __launch_bounds__(kBlock, 2)
sample_static_kernel(FrameParams fp, GridsDev g, SamplerDev smp, BinBuffers bb, SampleStore st, FragPool pool,
                     int32_t* err) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
	int32_t* win = reinterpret_cast<int32_t*>(smem_raw + sizeof(Smem));  // [kBlock * kSamplesPerThread]
	int32_t* wgrid = win + kBlock * kSamplesPerThread;                    // grid of the winner
	int32_t* fhead = wgrid + kBlock * kSamplesPerThread;                  // TRANSP: fragment list heads

	const int tile = blockIdx.x;
	const int tx = tile % fp.ntx, ty = tile / fp.ntx;
	const int tpx0 = fp.sx0 + tx * fp.tile_w, tpy0 = fp.sy0 + ty * fp.tile_h;
	const int tpx1 = min(tpx0 + fp.tile_w, fp.sx0 + fp.sw), tpy1 = min(tpy0 + fp.tile_h, fp.sy0 + fp.sh);
	const int st_idx = (ty / fp.st_tiles) * fp.nstx + (tx / fp.st_tiles);
	const int t = threadIdx.x;

	// thread -> (pixel, sample group)
	const int pl = t / fp.tpp;
	const int sg = t - pl * fp.tpp;
	const int lx = pl % fp.tile_w, ly = pl / fp.tile_w;
	const int mypx = tpx0 + lx, mypy = tpy0 + ly;
	const bool own = (pl < fp.tile_w * fp.tile_h) && mypx < tpx1 && mypy < tpy1;
	const int s0 = sg * kSamplesPerThread;
	const int nmine = own ? min(kSamplesPerThread, fp.spp - s0) : 0;
	const long long pix = own ? (long long)(mypy - fp.sy0) * fp.sw + (mypx - fp.sx0) : 0;
	const int n0 = s0 / fp.xs, m0 = s0 - n0 * fp.xs;

	float sx[kSamplesPerThread], sy[kSamplesPerThread], oz[kSamplesPerThread];
	{
		const long long pat = own ? (smp.pos_index ? (long long)smp.pos_index[pix] : pix) : 0;
		const float fx = (float)mypx, fy = (float)mypy;
#pragma unroll
		for (int i = 0; i < kSamplesPerThread; ++i) {
			float2 o = make_float2(0.0f, 0.0f);
			if (i < nmine) o = __ldg(smp.pos + pat * fp.spp + s0 + i);
			sx[i] = fx + o.x;  // CqImagePixel::setSamples: offset + positions[i]
			sy[i] = fy + o.y;
			oz[i] = FLT_MAX;
		}
	}
#pragma unroll
	for (int i = 0; i < kSamplesPerThread; ++i) {
		win[t * kSamplesPerThread + i] = -1;
		if (TRANSP) fhead[t * kSamplesPerThread + i] = -1;
	}
	for (int i = t; i < kBlock * kSlotWords; i += kBlock) (&sm.mask[0][0])[i] = 0u;
	__syncthreads();

	const int lbeg = bb.st_offset[st_idx * bb.nranges];
	const int lend = bb.st_offset[(st_idx + 1) * bb.nranges];
	const int cullable = fp.cullable;

	// Stream cursor (uniform over the block): list position of the next chunk,
	// grid index inside the current chunk, next micropolygon of that grid.
	int lp = lbeg, qi = 0, qn = 0, r0 = 0;
	int nslots = 0;
	for (;;) {
		// ---- phase A: fill up to kSlots records in insertion order ----
		bool exhausted = false;
		while (nslots < kSlots) {
			if (qi >= qn) {
				if (lp >= lend) { exhausted = true; break; }
				// which grids of this chunk of the super-tile list touch the tile?
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
				qn = total;
				qi = 0;
				r0 = 0;
				lp += kBlock;
				continue;
			}
			const int gi = sm.qgrid[qi];
			const int cu = __ldg(g.cu + gi), cv = __ldg(g.cv + gi);
			const int nmp = cu * cv;
			if (r0 >= nmp) { ++qi; r0 = 0; continue; }
			const int gflags = __ldg(g.flags + gi);
			const long long pb = __ldg(g.pbase + gi);
			const long long cb = __ldg(g.cbase + gi);
			const long long mpb = __ldg(g.mpbase + gi);
			// one micropolygon per thread
			const int m = r0 + t;
			bool active = false;
			V3f v[4];
			float bminx = 0, bmaxx = 0, bminy = 0, bmaxy = 0, bminz = 0;
			int index = 0;
			if (m < nmp) {
				const int iv = m / cu, iu = m - iv * cu;
				index = iv * (cu + 1) + iu;
				const bool culled = g.culled && g.culled[mpb + m];
				v[0] = ld3(g.P, pb + index);
				v[1] = ld3(g.P, pb + index + 1);
				v[2] = ld3(g.P, pb + index + cu + 1);
				v[3] = ld3(g.P, pb + index + cu + 2);
				// CalculateBound: min(min(min(A,B),C),D), C = index+cu+2, D = index+cu+1
				bminx = amin(amin(amin(v[0].x, v[1].x), v[3].x), v[2].x);
				bminy = amin(amin(amin(v[0].y, v[1].y), v[3].y), v[2].y);
				bminz = amin(amin(amin(v[0].z, v[1].z), v[3].z), v[2].z);
				bmaxx = amax(amax(amax(v[0].x, v[1].x), v[3].x), v[2].x);
				bmaxy = amax(amax(amax(v[0].y, v[1].y), v[3].y), v[2].y);
				// AddMPG crop cull (imagebuffer.cpp:533-539)
				const bool cropped =
				    bmaxx < fp.cull_x0 || bmaxy < fp.cull_y0 || bminx > fp.cull_x1 || bminy > fp.cull_y1;
				// pixels RenderMPG_Static visits: [floor(bmin), lceil(bmax)) clipped to the tile
				const int sX = max((int)floorf(bminx), tpx0), eX = min(lceil_f(bmaxx), tpx1);
				const int sY = max((int)floorf(bminy), tpy0), eY = min(lceil_f(bmaxy), tpy1);
				active = !culled && !cropped && sX < eX && sY < eY;
			}
			int total;
			const int rank = block_excl_scan(sm.warp_tot, active, total);
			const int navail = kSlots - nslots;
			if (t == 0) sm.first_reject = kBlock;
			__syncthreads();
			if (active && rank == navail) sm.first_reject = t;
			if (active && rank < navail) {
				const int slot = nslots + rank;
				MpRec& rec = sm.rec[slot];
				HitCoeffs h;
				const int code = vertex_order(v);
				hit_setup(v, code, h);
				rec.bminx = bminx; rec.bmaxx = bmaxx; rec.bminy = bminy; rec.bmaxy = bmaxy; rec.bminz = bminz;
#pragma unroll
				for (int k = 0; k < 4; ++k) {
					rec.ym[k] = h.ym[k]; rec.xm[k] = h.xm[k]; rec.ex[k] = h.ex[k]; rec.ey[k] = h.ey[k];
					rec.z[k] = h.z[k];
				}
				rec.ax = h.ax; rec.ay = h.ay; rec.e_x = h.e_x; rec.e_y = h.e_y;
				rec.f_x = h.f_x; rec.f_y = h.f_y; rec.g_x = h.g_x; rec.g_y = h.g_y;
				rec.id = (int)(mpb + m);
				rec.grid = gi;
				// SqMpgSampleInfo::isOpaque (micropolygon.cpp:1477-1529)
				bool opaque = true;
				const bool smooth = (gflags & 1) != 0;
				if (!(gflags & 8) && g.Oi) {
					const float4 o0 = __ldg(g.Oi + cb + index);
					opaque = o0.x >= 1.0f && o0.y >= 1.0f && o0.z >= 1.0f;
					if (smooth) {
						const float4 o1 = __ldg(g.Oi + cb + index + 1);
						const float4 o2 = __ldg(g.Oi + cb + index + cu + 1);
						const float4 o3 = __ldg(g.Oi + cb + index + cu + 2);
						opaque = opaque && (o1.x >= 1.0f && o1.y >= 1.0f && o1.z >= 1.0f) &&
						         (o2.x >= 1.0f && o2.y >= 1.0f && o2.z >= 1.0f) &&
						         (o3.x >= 1.0f && o3.y >= 1.0f && o3.z >= 1.0f);
					}
				}
				int bits = h.linear ? kRecLinear : 0;
				if (opaque || (gflags & 4)) bits |= kRecOccluding;
				if (smooth) bits |= kRecSmooth;
				if (gflags & 2) bits |= kRecMatte;
				if (gflags & 4) bits |= kRecMatteAlpha;
				rec.bits = bits;
				// candidate bit for every tile pixel of the visited range
				const int sX = max((int)floorf(bminx), tpx0), eX = min(lceil_f(bmaxx), tpx1);
				const int sY = max((int)floorf(bminy), tpy0), eY = min(lceil_f(bmaxy), tpy1);
				const uint32_t bit = 1u << (slot & 31);
				const int wd = slot >> 5;
				for (int yy = sY; yy < eY; ++yy)
					for (int xx = sX; xx < eX; ++xx)
						atomicOr(&sm.mask[(yy - tpy0) * fp.tile_w + (xx - tpx0)][wd], bit);
			}
			__syncthreads();
			const int consumed = (total > navail) ? sm.first_reject : min(kBlock, nmp - r0);
			nslots += min(total, navail);
			r0 += consumed;
		}
		if (nslots == 0) break;

		// ---- phase B: walk this pixel's candidates in insertion order ----
		if (own) {
#pragma unroll 1
			for (int wd = 0; wd < kSlotWords; ++wd) {
				uint32_t bits = sm.mask[pl][wd];
				while (bits) {
					const int b = __ffs(bits) - 1;
					bits &= bits - 1u;
					const MpRec& r = sm.rec[wd * 32 + b];
					int m_lo, m_hi, n_lo, n_hi;
					sub_range(mypx, r.bminx, r.bmaxx, fp.xs, m_lo, m_hi);
					sub_range(mypy, r.bminy, r.bmaxy, fp.ys, n_lo, n_hi);
					int m = m0, n = n0;  // sub-pixel column and row of sample s0 + i
#pragma unroll
					for (int i = 0; i < kSamplesPerThread; ++i) {
						const int mi = m, ni = n;
						if (++m == fp.xs) { m = 0; ++n; }
						if (i >= nmine || mi < m_lo || mi >= m_hi || ni < n_lo || ni >= n_hi) continue;
						const float x = sx[i], y = sy[i];
						// CqBound::Contains2D (bound.h:144-151)
						if ((x < r.bminx || x > r.bmaxx) || (y < r.bminy || y > r.bmaxy)) continue;
						// early-z (bucketprocessor.cpp:1179)
						if (cullable && r.bminz > oz[i]) continue;
						if (!edges_inside(r.ym, r.xm, r.ex, r.ey, x, y)) continue;
						float u, v;
						inv_bilinear(r.ax, r.ay, r.e_x, r.e_y, r.f_x, r.f_y, r.g_x, r.g_y, (r.bits & kRecLinear) != 0,
						             x, y, u, v);
						const float D = bilerp1(r.z[0], r.z[1], r.z[2], r.z[3], u, v);
						// StoreSample (bucketprocessor.cpp:1471-1569)
						if (cullable && oz[i] <= D) continue;
						if ((r.bits & kRecOccluding) && cullable) {
							oz[i] = D;
							win[t * kSamplesPerThread + i] = r.id;
							wgrid[t * kSamplesPerThread + i] = r.grid;
						} else if (TRANSP) {
							// append a fragment {depth, id, u, v}; list head is newest-first
							const unsigned act = __activemask();
							const int leader = __ffs(act) - 1;
							const int rank = __popc(act & ((1u << (threadIdx.x & 31)) - 1u));
							unsigned long long base = 0;
							if ((threadIdx.x & 31) == leader)
								base = atomicAdd(pool.count, (unsigned long long)__popc(act));
							base = __shfl_sync(act, base, leader);
							const long long idx = (long long)base + rank;
							if (idx < pool.capacity) {
								pool.frag[idx] = make_float4(D, __int_as_float(r.id), u, v);
								pool.next[idx] = fhead[t * kSamplesPerThread + i];
								fhead[t * kSamplesPerThread + i] = (int)idx;
							} else {
								atomicOr(pool.overflow, 1);
							}
						}
					}
				}
			}
		}
		__syncthreads();
		for (int i = t; i < kBlock * kSlotWords; i += kBlock) (&sm.mask[0][0])[i] = 0u;
		__syncthreads();
		nslots = 0;
		if (exhausted) break;
	}

	// Resolve: colours of the occluding hits, Combine of transparent lists.
	// The record area is free now; park the occluding depths there so the
	// per-sample loop below can index them dynamically without pulling the
	// register arrays into local memory.  Positions are recomputed from the
	// pattern tables, which gives the same values.
	__syncthreads();
	if (!own) return;
	float* ozs = reinterpret_cast<float*>(sm.rec);
#pragma unroll
	for (int i = 0; i < kSamplesPerThread; ++i) ozs[t * kSamplesPerThread + i] = oz[i];
	const long long pat = smp.pos_index ? (long long)smp.pos_index[pix] : pix;
	for (int i = 0; i < nmine; ++i) {
		const float2 o = __ldg(smp.pos + pat * fp.spp + s0 + i);
		resolve_sample<TRANSP>(fp, g, pool, st, pix * fp.spp + s0 + i, (float)mypx + o.x, (float)mypy + o.y,
		                       ozs[t * kSamplesPerThread + i], win[t * kSamplesPerThread + i],
		                       wgrid[t * kSamplesPerThread + i], TRANSP ? fhead[t * kSamplesPerThread + i] : -1);
	}
}

}  // namespace

void launch_sample_tiles(const FrameParams& fp, const GridsDev& g, const SamplerDev& sm, const BinBuffers& b,
                         SampleStore st, FragPool pool, int32_t* err, cudaStream_t s) {
	const int ntiles = fp.ntx * fp.nty;
	const size_t smem_opaque = sizeof(Smem) + 2 * sizeof(int32_t) * kBlock * kSamplesPerThread;
	const size_t smem_transp = smem_opaque + sizeof(int32_t) * kBlock * kSamplesPerThread;
	static bool configured = false;
	if (!configured) {
		cudaFuncSetAttribute(sample_static_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_opaque);
		cudaFuncSetAttribute(sample_static_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_transp);
		configured = true;
	}
	if (pool.capacity > 0)
		sample_static_kernel<true><<<ntiles, kBlock, smem_transp, s>>>(fp, g, sm, b, st, pool, err);
	else
		sample_static_kernel<false><<<ntiles, kBlock, smem_opaque, s>>>(fp, g, sm, b, st, pool, err);
}

}  // namespace aqh
