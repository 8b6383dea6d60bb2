// sample_common.cuh -- pieces shared by the sampling kernels: block scan,
// sub-sample ranges, output interpolation and CqImagePixel::Combine.
#pragma once

#include "aqh_internal.h"
#include "hider_device.cuh"

namespace aqh {

// The level-of-detail test of RenderMPG_Static / RenderMPG_MBOrDof
// (bucketprocessor.cpp:1182-1190, 1404-1412, 1439-1447): a grid whose
// LevelOfDetailBounds minimum is >= 0 (the attribute defaults to 0 1,
// attributes.cpp:127) skips samples whose detail level lies outside
// [min, max).  True when the grid has such a test that can fire this frame.
__device__ __forceinline__ bool lod_active(const FrameParams& fp, const GridsDev& g, int gi) {
	if (!fp.use_lod) return false;
	return g.lod ? __ldg(g.lod + gi).x >= 0.0f : true;
}
// Sample si of sample-region pixel (px, py): is it outside grid gi's bounds?
__device__ __forceinline__ bool lod_rejects(const FrameParams& fp, const GridsDev& g, const SamplerDev& smp, int gi,
                                            int px, int py, int si) {
	const float2 b = g.lod ? __ldg(g.lod + gi) : make_float2(0.0f, 1.0f);
	float level = 0.0f;
	if (smp.lod) {
		const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
		const long long pat = smp.lod_index ? (long long)__ldg(smp.lod_index + pix) : pix;
		level = __ldg(smp.lod + pat * fp.spp + si);
	}
	return b.x > level || level >= b.y;
}

// Does grid gi belong to a CSG solid?  Such micropolygons are never
// occlusion-cullable (bucketprocessor.cpp:1074-1080).
__device__ __forceinline__ bool csg_grid(const GridsDev& g, int gi) {
	return g.csg.nnodes > 0 && __ldg(g.csg.grid_node + gi) >= 0;
}

// CqCSGNode*::EvaluateState (csgtree.cpp:280-351) over the child in/out bits.
__device__ __forceinline__ bool csg_eval(int type, uint32_t st, int nch) {
	if (type == 1) return st != 0u;
	if (type == 2) return st == (nch >= 32 ? 0xffffffffu : ((1u << nch) - 1u));
	if (type == 3) return nch >= 1 && (st & 1u) && !(st & ~1u);
	return false;
}

// The CSG resolve of Combine (imagepixel.cpp:170-190; csgtree.cpp:144-258)
// over a depth-sorted entry list: while an entry still names a node, the
// tree holding the first such entry is processed from its top, node by node
// with children first; at each node the child states start false, every
// entry of a child toggles its state, entries that leave the node's state
// unchanged are dropped and the rest are promoted to the node (to none at
// the top).  A primitive at the top just releases its entries.  Returns
// false if the trees are not processed within the bound (flagged).
template <class E>
__device__ inline bool csg_resolve(const CsgDev& c, E* ent, int* node, int& n) {
	for (int round = 0; round < 64; ++round) {
		int start = -1;
		for (int i = 0; i < n && start < 0; ++i) start = node[i];
		if (start < 0) return true;
		int top = start;
		for (int up = 0; up < c.nnodes && __ldg(c.parent + top) >= 0; ++up) top = __ldg(c.parent + top);
		if (__ldg(c.type + top) == 0) {
			for (int i = 0; i < n; ++i)
				if (node[i] == top) node[i] = -1;
			continue;
		}
		const int pf = __ldg(c.post_first + top), pc = __ldg(c.post_count + top);
		for (int q = 0; q < pc; ++q) {
			const int nd = __ldg(c.post + pf + q);
			const int ty = __ldg(c.type + nd), nch = __ldg(c.nchildren + nd);
			const int promote = __ldg(c.parent + nd) >= 0 ? nd : -1;
			uint32_t st = 0u;
			bool cur = csg_eval(ty, st, nch);
			int w = 0;
			for (int i = 0; i < n; ++i) {
				const int e = node[i];
				if (e < 0 || __ldg(c.parent + e) != nd) {
					ent[w] = ent[i];
					node[w] = e;
					++w;
					continue;
				}
				st ^= 1u << __ldg(c.child_index + e);
				const bool nw = csg_eval(ty, st, nch);
				if (nw == cur) continue;  // no change: the entry goes
				cur = nw;
				ent[w] = ent[i];
				node[w] = promote;
				++w;
			}
			n = w;
		}
	}
	if (c.overflow) atomicOr(c.overflow, 1);
	return false;
}

// The trim test of CqMicroPolygon::Sample (micropolygon.cpp:1592-1627) for a
// hit at (u, v) on micropolygon `id` of grid gi, marked trimmed: the surface
// parameters there inside the grid's trim set reject the hit, with the
// "inside" sense only.
__device__ __forceinline__ bool trim_rejects(const GridsDev& g, int id, int gi, float u, float v) {
	if (g.flags && (__ldg(g.flags + gi) & 64)) return false;  // "outside": no test at the hit
	const int cu = __ldg(g.cu + gi);
	const int m = id - (int)__ldg(g.mpbase + gi);
	const long long c = __ldg(g.cbase + gi) + (long long)(m / cu) * (cu + 1) + (m % cu);
	const float2 A = __ldg(g.trim.uv + c), B = __ldg(g.trim.uv + c + 1);
	const float2 C = __ldg(g.trim.uv + c + cu + 1), D = __ldg(g.trim.uv + c + cu + 2);
	const float2 r = bilinear_evaluate(A, B, C, D, u, v);
	const int set = __ldg(g.trim.grid_set + gi);
	return trim_point(g.trim.pts, g.trim.loop_first, __ldg(g.trim.set_first + set), __ldg(g.trim.set_first + set + 1),
	                  r.x, r.y);
}

// Entry i of a colour array (Ci or Oi): float4, or three packed floats when
// the grids arrived in the three-float host layout.
__device__ __forceinline__ float4 ld_colour(const GridsDev& g, const float4* p, long long i) {
	if (g.colour3) {
		const float* f = reinterpret_cast<const float*>(p) + 3 * i;
		return make_float4(__ldg(f), __ldg(f + 1), __ldg(f + 2), 0.0f);
	}
	return __ldg(p + i);
}

// Exclusive prefix count of `f` over the block (blockDim.x a multiple of 32,
// at most 1024 threads); `warp_tot` is shared scratch of 32 ints.
__device__ __forceinline__ int block_excl_scan(int* warp_tot, bool f, int& total) {
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const unsigned bal = __ballot_sync(0xffffffffu, f);
	if (lane == 0) warp_tot[wid] = __popc(bal);
	__syncthreads();
	int pre = 0, tot = 0;
	for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
		int t = warp_tot[w];
		pre += (w < wid) ? t : 0;
		tot += t;
	}
	total = tot;
	return pre + __popc(bal & ((1u << lane) - 1u));
}

// Exclusive prefix sum of `v` over the block (same layout rules as
// block_excl_scan).
__device__ __forceinline__ int block_excl_sum(int* warp_tot, int v, int& total) {
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	int inc = v;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const int n = __shfl_up_sync(0xffffffffu, inc, o);
		if (lane >= o) inc += n;
	}
	if (lane == 31) warp_tot[wid] = inc;
	__syncthreads();
	int pre = 0, tot = 0;
	for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
		const int t = warp_tot[w];
		pre += (w < wid) ? t : 0;
		tot += t;
	}
	total = tot;
	return pre + inc - v;
}

// The item holding position p of a running count: pref[c] is the first
// position of item c (nondecreasing, pref[0] = 0), n items.  `c` is an item
// already known to start at or before p (pref[c] <= p), typically the one a
// lane of the same warp found for the previous run of positions: a few
// steps forward, then a binary search for long jumps.  Returns the largest c
// with pref[c] <= p.
__device__ __forceinline__ int advance_item(const int* pref, int n, int c, int p) {
#pragma unroll 1
	for (int it = 0; it < 4 && c + 1 < n && pref[c + 1] <= p; ++it) ++c;
	if (c + 1 < n && pref[c + 1] <= p) {
		int lo = c + 1, hi = n - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if (pref[mid] <= p) lo = mid; else hi = mid - 1;
		}
		c = lo;
	}
	return c;
}

// Sub-sample index range of pixel `p` inside [s, e) of a bound edge
// (bucketprocessor.cpp:1119-1138, 1149-1153), for one axis.
__device__ __forceinline__ void sub_range(int p, float bmin, float bmax, int ns, int& lo, int& hi) {
	const int s = (int)floorf(bmin);
	const int e = lceil_f(bmax);
	const int im = (int)floorf((bmin - (float)s) * (float)ns);
	const int em = lceil_f((bmax - (float)(e - 1)) * (float)ns);
	lo = (p == s) ? im : 0;
	hi = (p == e - 1) ? em : ns;
}

// Colour and opacity of micropolygon `m` of grid `gi` at (u,v):
// CqMicroPolygon::InterpolateOutputs (micropolygon.cpp:1443-1462) over the
// cached SqMpgSampleInfo (1464-1529).  Also returns the hit flags
// (Flag_Matte = 1, Flag_MatteAlpha = 2).
__device__ __forceinline__ void hit_colour(const GridsDev& g, int gi, int m, float u, float v, float dat[7],
                                           int& flg) {
	const int cu = __ldg(g.cu + gi);
	const int iv = m / cu, iu = m - iv * cu;
	const int index = iv * (cu + 1) + iu;
	const long long cb = __ldg(g.cbase + gi);
	const int gflags = __ldg(g.flags + gi);
	if (gflags & 1) {
		const int vi[4] = {index, index + 1, index + cu + 1, index + cu + 2};
		float wt[4];
		smooth_weights(u, v, wt);
		float4 c[4], o[4];
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			c[q] = g.Ci ? ld_colour(g, g.Ci, cb + vi[q]) : make_float4(1, 1, 1, 0);
			o[q] = g.Oi ? ld_colour(g, g.Oi, cb + vi[q]) : make_float4(1, 1, 1, 0);
		}
		dat[0] = ((wt[0] * c[0].x + wt[1] * c[1].x) + wt[2] * c[2].x) + wt[3] * c[3].x;
		dat[1] = ((wt[0] * c[0].y + wt[1] * c[1].y) + wt[2] * c[2].y) + wt[3] * c[3].y;
		dat[2] = ((wt[0] * c[0].z + wt[1] * c[1].z) + wt[2] * c[2].z) + wt[3] * c[3].z;
		dat[3] = ((wt[0] * o[0].x + wt[1] * o[1].x) + wt[2] * o[2].x) + wt[3] * o[3].x;
		dat[4] = ((wt[0] * o[0].y + wt[1] * o[1].y) + wt[2] * o[2].y) + wt[3] * o[3].y;
		dat[5] = ((wt[0] * o[0].z + wt[1] * o[1].z) + wt[2] * o[2].z) + wt[3] * o[3].z;
	} else {
		const float4 c = g.Ci ? ld_colour(g, g.Ci, cb + index) : make_float4(1, 1, 1, 0);
		const float4 o = g.Oi ? ld_colour(g, g.Oi, cb + index) : make_float4(1, 1, 1, 0);
		dat[0] = c.x; dat[1] = c.y; dat[2] = c.z;
		dat[3] = o.x; dat[4] = o.y; dat[5] = o.z;
	}
	flg = ((gflags & 2) ? 1 : 0) | ((gflags & 4) ? 2 : 0);
}

// FilterBucket's in-window test (bucketprocessor.cpp:609-614) for one sample
// at (x, y) of pixel (px, py) against every display pixel whose filter
// reaches it, as a bitmask: bit (fy + shiftY) * (2 shiftX + 1) + fx + shiftX
// is set when the sample lies inside the window of display pixel
// (px - fx, py - fy).  The float operations are the filter's own, so the
// filter reads the bit instead of repeating the test per display pixel.
__device__ __forceinline__ uint32_t window_mask(const FrameParams& fp, int px, int py, float x, float y) {
	uint32_t m = 0;
	const int xmax = fp.shiftX, ymax = fp.shiftY;
	for (int fy = -ymax; fy <= ymax; ++fy) {
		const float vy = y - ((float)(py - fy) + 0.5f);
		for (int fx = -xmax; fx <= xmax; ++fx) {
			const float vx = x - ((float)(px - fx) + 0.5f);
			if (vx >= -fp.xfwo2 && vy >= -fp.yfwo2 && vx <= fp.xfwo2 && vy <= fp.yfwo2)
				m |= 1u << ((fy + ymax) * (2 * xmax + 1) + fx + xmax);
		}
	}
	return m;
}

// Grid owning a global micropolygon id: from the id table when there is one,
// else by binary search over the grids' first ids.
__device__ __forceinline__ int grid_of(const GridsDev& g, int id) {
	if (g.id_grid) {
		// the grid holding id & ~255, then forward over grids that start later
		int gi = __ldg(g.id_grid + (id >> 8));
		while (gi + 1 < g.ngrids && __ldg(g.mpbase + gi + 1) <= id) ++gi;
		return gi;
	}
	int lo = 0, hi = g.ngrids - 1;
	while (lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if (__ldg(g.mpbase + mid) <= id) lo = mid; else hi = mid - 1;
	}
	return lo;
}

// Combine's sort order (imagepixel.cpp:155-161, 188-193): the transparent
// fragments followed by the occluding hit, sorted by ascending depth; equal
// depths keep insertion order, which is the micropolygon id order (the
// occluding hit, id INT_MAX, last).  Entries with the same depth and id are
// the same micropolygon hit twice at one sample time (a motion slice
// boundary) and carry the same data.
struct FragKey { float d; int id; int seq; int idx; };

__device__ __forceinline__ bool key_less(float d, int id, int seq, const FragKey& b) {
	return d < b.d || (d == b.d && (id < b.id || (id == b.id && seq < b.seq)));
}
__device__ __forceinline__ bool key_greater(float d, int id, int seq, const FragKey& b) {
	return d > b.d || (d == b.d && (id > b.id || (id == b.id && seq > b.seq)));
}

// Selection form for long lists: the entry after `prev` in ascending order
// (descending: before it), by a walk over the list.
__device__ __forceinline__ FragKey next_key(const FragPool& pool, int head, int n, bool has_occl, float occl_d,
                                            FragKey prev, bool first, bool descending) {
	FragKey best{0.0f, 0, 0, -2};
	bool any = false;
	auto consider = [&](float d, int id, int seq, int idx) {
		bool beyond, better;
		if (descending) {
			beyond = first || key_less(d, id, seq, prev);
			better = !any || key_greater(d, id, seq, best);
		} else {
			beyond = first || key_greater(d, id, seq, prev);
			better = !any || key_less(d, id, seq, best);
		}
		if (beyond && better) { best = FragKey{d, id, seq, idx}; any = true; }
	};
	int seq = n - 1;
	for (int f = head; f >= 0; f = pool.next[f], --seq) {
		const float4 fr = pool.frag[f];
		consider(fr.x, __float_as_int(fr.y), seq, f);
	}
	if (has_occl) consider(occl_d, 0x7fffffff, n, -1);
	return best;
}

__device__ __forceinline__ void key_data(const GridsDev& g, const FragPool& pool, int idx, const float occl[7],
                                         int occl_flags, float dat[7], int& flg) {
	if (idx == -1) {
#pragma unroll
		for (int q = 0; q < 7; ++q) dat[q] = occl[q];
		flg = occl_flags;
	} else {
		const float4 fr = pool.frag[idx];
		const int id = __float_as_int(fr.y);
		const int gi = grid_of(g, id);
		hit_colour(g, gi, id - (int)__ldg(g.mpbase + gi), fr.z, fr.w, dat, flg);
		dat[6] = fr.x;
	}
}

constexpr int kCombineLocal = 24;  // lists up to this long are sorted in local memory

// CqImagePixel::Combine for a sample with transparent fragments
// (imagepixel.cpp:155-301).  Returns the fragment count; writes the collapsed
// sample into occl / occl_flags, and into top_id the micropolygon of the
// front entry, whose output variables the sample keeps (occl_id for the
// occluding hit).  CSG: the frame has CSG trees (compiled out otherwise).
template <bool CSG>
__device__ __forceinline__ int combine_fragments_t(const FrameParams& fp, const GridsDev& g, const FragPool& pool,
                                                   int head, bool has_occl, float occlZ, float occl[7],
                                                   int& occl_flags, int occl_id, int& top_id, bool& emptied) {
	int n = 0;
	bool nan = occl[6] != occl[6];
	bool any_csg = false;
	// One walk over the list (newest first) counts it, checks for NaN depths
	// and, while the entries fit, insertion-sorts them by ascending key.  An
	// entry's sequence number is minus its list position (the occluding hit
	// 1), so of entries with equal depth and id the newer sorts later, as in
	// insertion order.  The walk loads the next fragment before sorting in
	// the current one, so the sort's local-memory traffic overlaps the chase
	// of the links.
	FragKey ent[kCombineLocal];
	int m = 0;
	auto insert = [&](float d, int id, int sq, int idx) {
		int k = m++;
		while (k > 0 && key_less(d, id, sq, ent[k - 1])) {
			ent[k] = ent[k - 1];
			--k;
		}
		ent[k] = FragKey{d, id, sq, idx};
	};
	const int room = kCombineLocal - (has_occl ? 1 : 0);
	float4 fr = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	int nx = -1;
	if (head >= 0) {
		fr = pool.frag[head];
		nx = pool.next[head];
	}
	for (int f = head; f >= 0;) {
		float4 frn = fr;
		int nxn = -1;
		if (nx >= 0) {
			frn = pool.frag[nx];
			nxn = pool.next[nx];
		}
		nan |= fr.x != fr.x;
		if (CSG) any_csg = any_csg || csg_grid(g, grid_of(g, __float_as_int(fr.y)));
		if (n < room) insert(fr.x, __float_as_int(fr.y), -n, f);
		++n;
		f = nx;
		fr = frn;
		nx = nxn;
	}
	int ntot = n + (has_occl ? 1 : 0);
	emptied = false;
	// short lists are now sorted; long ones (or NaN depths) are walked in
	// order by selection
	const bool local = ntot <= kCombineLocal && !nan;
	if (CSG && any_csg && !local && g.csg.overflow) atomicOr(g.csg.overflow, 1);  // CSG needs the sorted list held
	if (local) {
		if (has_occl) insert(occl[6], 0x7fffffff, 1, -1);
		if (CSG && any_csg) {
			// CSG resolve of the sorted list (imagepixel.cpp:170-190); a list it
			// empties leaves the sample as it was (imagepixel.cpp:249)
			int node[kCombineLocal];
			for (int k = 0; k < ntot; ++k)
				node[k] = ent[k].idx < 0 ? -1 : __ldg(g.csg.grid_node + grid_of(g, ent[k].id));
			csg_resolve(g.csg, ent, node, ntot);
			if (ntot == 0) {
				emptied = true;
				return n;
			}
		}
	}
	float sc[3] = {0, 0, 0}, so[3] = {0, 0, 0};
	float opaque0 = occlZ, opaque1 = FLT_MAX, maxOpaque = FLT_MAX;
	float top[7] = {0, 0, 0, 0, 0, 0, 0};
	int top_flags = 0;
	FragKey prev{0.0f, 0, 0, -2};
	// back to front (imagepixel.cpp:196-246)
	for (int k = 0; k < ntot; ++k) {
		int idx;
		if (local) {
			idx = ent[ntot - 1 - k].idx;
		} else {
			prev = next_key(pool, head, n, has_occl, occl[6], prev, k == 0, true);
			idx = prev.idx;
		}
		float dat[7];
		int flg;
		key_data(g, pool, idx, occl, occl_flags, dat, flg);
		if (flg & 1) {
			float nc[3], no[3];
#pragma unroll
			for (int q = 0; q < 3; ++q) nc[q] = (1.0f - dat[3 + q]) * sc[q] + dat[3 + q] * 0.0f;
#pragma unroll
			for (int q = 0; q < 3; ++q) no[q] = (1.0f - dat[q]) * so[q] + dat[q] * 0.0f;
#pragma unroll
			for (int q = 0; q < 3; ++q) { sc[q] = nc[q]; so[q] = no[q]; }
		} else {
#pragma unroll
			for (int q = 0; q < 3; ++q) {
				const float o = dat[3 + q];
				const float cl = o < 0.0f ? 0.0f : (o > 1.0f ? 1.0f : o);
				sc[q] = (sc[q] * (1.0f - cl)) + dat[q];
			}
#pragma unroll
			for (int q = 0; q < 3; ++q) so[q] = ((1.0f - so[q]) * dat[3 + q]) + so[q];
		}
		if (dat[3] >= fp.zthr[0] && dat[4] >= fp.zthr[1] && dat[5] >= fp.zthr[2]) {
			opaque1 = opaque0;
			opaque0 = dat[6];
			if (!(maxOpaque < FLT_MAX)) maxOpaque = dat[6];
		}
		if (k == ntot - 1) {
#pragma unroll
			for (int q = 0; q < 7; ++q) top[q] = dat[q];
			top_flags = flg;
			top_id = idx == -1 ? occl_id : __float_as_int(pool.frag[idx].y);
		}
	}
	float depth = top[6];
	if (fp.depth_filter == 0) {
		depth = opaque0;
	} else if (fp.depth_filter == 1) {
		depth = (ntot > 1) ? ((opaque0 + opaque1) * 0.5f) : FLT_MAX;
	} else if (fp.depth_filter == 2) {
		depth = maxOpaque;
	} else {
		// average over entries with any opacity channel at the threshold, in
		// ascending order (imagepixel.cpp:279-296)
		float tot = 0.0f;
		int cnt = 0;
		FragKey pk{0.0f, 0, 0, -2};
		for (int k = 0; k < ntot; ++k) {
			int idx;
			if (local) {
				idx = ent[k].idx;
			} else {
				pk = next_key(pool, head, n, has_occl, occl[6], pk, k == 0, false);
				idx = pk.idx;
			}
			float dat[7];
			int flg;
			key_data(g, pool, idx, occl, occl_flags, dat, flg);
			if (dat[3] >= fp.zthr[0] || dat[4] >= fp.zthr[1] || dat[5] >= fp.zthr[2]) {
				tot += dat[6];
				cnt++;
			}
		}
		depth = tot / (float)cnt;
	}
	occl[0] = sc[0]; occl[1] = sc[1]; occl[2] = sc[2];
	occl[3] = so[0]; occl[4] = so[1]; occl[5] = so[2];
	occl[6] = depth;
	occl_flags = top_flags;
	return n;
}

__device__ inline int combine_fragments(const FrameParams& fp, const GridsDev& g, const FragPool& pool, int head,
                                        bool has_occl, float occlZ, float occl[7], int& occl_flags, int occl_id,
                                        int& top_id, bool& emptied) {
	if (g.csg.nnodes > 0)
		return combine_fragments_t<true>(fp, g, pool, head, has_occl, occlZ, occl, occl_flags, occl_id, top_id, emptied);
	return combine_fragments_t<false>(fp, g, pool, head, has_occl, occlZ, occl, occl_flags, occl_id, top_id, emptied);
}


}  // namespace aqh
