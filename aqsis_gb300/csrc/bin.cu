// bin.cu -- bound-and-bin stage: per-grid raster rectangles and ordered
// per-super-tile grid lists.
//
// Replaces CqImageBuffer::AddMPG's bucket assignment (libs/core/imagebuffer.cpp:
// 514-591) at grid granularity.  A grid is listed for every super-tile (a
// square of sampling tiles) its pixel rectangle touches, and each list keeps
// grid submission order, so a tile that walks its super-tile's list sees its
// micropolygons in the reference's insertion order (grid order, then iv, iu).
// The exact per-micropolygon tests (bound, AddMPG crop cull) run in the
// sampling kernel; this stage only needs conservative rectangles.
#include "aqh_internal.h"
#include "hider_device.cuh"

namespace aqh {

// One warp per grid: min/max of x, y, z over every vertex of every key, grown
// by the largest circle of confusion in the grid's depth range when depth of
// field is on, turned into the pixel rectangle [floor(min), ceil(max)] + 1
// clipped to the sample region.
// Pixel range [floor(mn), lceil(mx)) packed as two int16, widened to the
// whole int16 range where the floats are out of range or NaN.
__device__ __forceinline__ uint32_t pack_range(float mn, float mx, bool bad) {
	int lo = -32768, hi = 32767;
	if (!bad) {
		if (mn > -32768.0f) lo = (int)floorf(mn);
		if (mx < 32767.0f) hi = lceil_f(mx);
	}
	return (uint32_t)(lo & 0xffff) | ((uint32_t)hi << 16);
}

// Strips: the pixel ranges each micropolygon column and row of a grid can
// touch (x over vertex columns iu, iu+1; y over vertex rows iv, iv+1; every
// motion key), so the sampler streams only the micropolygons whose column and
// row both meet its tile -- a superset of those whose bound does.  In frames
// with motion blur or depth of field the ranges grow by `grow` (the grid's
// largest circle of confusion) and one pixel on each side, which covers the
// staging rectangles of the motion sampler.  Lane = vertex column.
template <int NK>  // NK = 1: one key (its loads pipeline across rows); 0: nk keys
__device__ __forceinline__ void grid_strips(const float4* P, int cu, int cv, int nk, float growx, float growy,
                                            bool margin, int lane, uint32_t* S) {
	if (NK == 1) nk = 1;
	const bool on = lane <= cu;
	const long long nvk = (long long)(cu + 1) * (cv + 1);
	float cmn = FLT_MAX, cmx = -FLT_MAX, pmn = FLT_MAX, pmx = -FLT_MAX;
	bool cbad = false, pbad = false;
	const float mg = margin ? 1.0f : 0.0f;
	for (int j = 0; j <= cv; ++j) {
		float ymn = FLT_MAX, ymx = -FLT_MAX;
		bool ybad = false;
		for (int k = 0; k < nk; ++k) {
			if (on) {
				const float4 p = __ldg(P + k * nvk + j * (cu + 1) + lane);
				cbad |= (p.x != p.x);
				cmn = fminf(cmn, p.x);
				cmx = fmaxf(cmx, p.x);
				ybad |= (p.y != p.y);
				ymn = fminf(ymn, p.y);
				ymx = fmaxf(ymx, p.y);
			}
		}
		if (margin && on) {
			ymn = (ymn - growy) - mg;
			ymx = (ymx + growy) + mg;
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			ymn = fminf(ymn, __shfl_xor_sync(0xffffffffu, ymn, o));
			ymx = fmaxf(ymx, __shfl_xor_sync(0xffffffffu, ymx, o));
		}
		ybad = __any_sync(0xffffffffu, ybad);
		if (j > 0 && lane == 0) S[32 + j - 1] = pack_range(fminf(pmn, ymn), fmaxf(pmx, ymx), pbad || ybad);
		pmn = ymn;
		pmx = ymx;
		pbad = ybad;
	}
	if (margin && on) {
		cmn = (cmn - growx) - mg;
		cmx = (cmx + growx) + mg;
	}
	const float nmn = __shfl_down_sync(0xffffffffu, cmn, 1), nmx = __shfl_down_sync(0xffffffffu, cmx, 1);
	const bool nbad = __shfl_down_sync(0xffffffffu, cbad, 1);
	if (lane < cu) S[lane] = pack_range(fminf(cmn, nmn), fmaxf(cmx, nmx), cbad || nbad);
}

__global__ void grid_rects_kernel(FrameParams fp, GridsDev g, int4* rect, float* minz, uint32_t* strips,
                                  float4* tri) {
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (warp >= g.ngrids) return;
	const int cu = g.cu[warp], cv = g.cv[warp];
	const int nk = g.nkeys[warp];
	const long long nv = (long long)(cu + 1) * (cv + 1) * nk;
	const float4* P = g.P + g.pbase[warp];
	float mnx = FLT_MAX, mny = FLT_MAX, mnz = FLT_MAX, mxx = -FLT_MAX, mxy = -FLT_MAX, mxz = -FLT_MAX;
	// four loads in flight per lane (the pass is bound by loads in flight)
#pragma unroll 4
	for (long long i = lane; i < nv; i += 32) {
		float4 p = __ldg(P + i);
		mnx = fminf(mnx, p.x); mxx = fmaxf(mxx, p.x);
		mny = fminf(mny, p.y); mxy = fmaxf(mxy, p.y);
		mnz = fminf(mnz, p.z); mxz = fmaxf(mxz, p.z);
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
		mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
		mnz = fminf(mnz, __shfl_xor_sync(0xffffffffu, mnz, o));
		mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
		mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
		mxz = fmaxf(mxz, __shfl_xor_sync(0xffffffffu, mxz, o));
	}
	// depth of field: the largest blur AddMPG gives any of the grid's
	// micropolygons, max(CoC(bound min z), CoC(bound max z)) over its own
	// bound (imagebuffer.cpp:520-531).  The grid's depth ends do not bound it
	// when the depth range reaches z = 0, where the blur has its pole.
	float mcx = 0.0f, mcy = 0.0f;
	if (fp.use_dof) {
		const long long nvk = (long long)(cu + 1) * (cv + 1);
		for (int m = lane; m < cu * cv; m += 32) {
			const int iv = m / cu, iu = m - iv * cu;
			const long long idx = (long long)iv * (cu + 1) + iu;
			float zl = FLT_MAX, zh = -FLT_MAX;
			for (int k = 0; k < nk; ++k) {
				const float4* Pk = P + k * nvk;
				const float za = __ldg(Pk + idx).z, zb = __ldg(Pk + idx + 1).z;
				const float zc = __ldg(Pk + idx + cu + 1).z, zd = __ldg(Pk + idx + cu + 2).z;
				zl = amin(zl, amin(amin(amin(za, zb), zc), zd));
				zh = amax(zh, amax(amax(amax(za, zb), zc), zd));
			}
			const float2 c1 = coc(zl, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
			const float2 c2 = coc(zh, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
			mcx = fmaxf(mcx, fmaxf(c1.x, c2.x));
			mcy = fmaxf(mcy, fmaxf(c1.y, c2.y));
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			mcx = fmaxf(mcx, __shfl_xor_sync(0xffffffffu, mcx, o));
			mcy = fmaxf(mcy, __shfl_xor_sync(0xffffffffu, mcy, o));
		}
	}
	if (strips) {
		uint32_t* S = strips + (long long)warp * 64;
		const bool mbdof = fp.use_dof || fp.any_motion;
		const bool has = (nk == 1 || mbdof) && nk <= kMaxKeys && cu <= 31 && cv <= 31;
		if (has) {
			if (nk == 1) grid_strips<1>(P, cu, cv, 1, mcx, mcy, mbdof, lane, S);
			else grid_strips<0>(P, cu, cv, nk, mcx, mcy, mbdof, lane, S);
		}
		if (lane == 0) S[63] = has ? 1u : 0u;
	}
	if (lane != 0) return;
	minz[warp] = mnz;
	if (tri && (g.flags[warp] & 16)) {
		// triangle split line per key (micropolygon.cpp:703-719, 737-746): through
		// corners cu and cv*(cu+1), ordered so that the kept side is positive
		const float4* Pg = g.P + g.pbase[warp];
		for (int k = 0; k < nk && k < kMaxKeys; ++k) {
			const long long kb = (long long)k * (cu + 1) * (cv + 1);
			const float4 v0 = Pg[kb], v1 = Pg[kb + cu], v2 = Pg[kb + (long long)cv * (cu + 1)];
			const bool cw = ((v1.x - v0.x) * (v2.y - v0.y) - (v1.y - v0.y) * (v2.x - v0.x)) >= 0;
			tri[(long long)warp * kMaxKeys + k] = cw ? make_float4(v1.x, v1.y, v2.x, v2.y)
			                                         : make_float4(v2.x, v2.y, v1.x, v1.y);
		}
	}
	if (fp.use_dof) {
		float2 c1 = coc(mnz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
		float2 c2 = coc(mxz, fp.dof_mult, fp.dof_inv_fd, fp.dof_scale_x, fp.dof_scale_y);
		const float cx = fmaxf(fmaxf(c1.x, c2.x), mcx), cy = fmaxf(fmaxf(c1.y, c2.y), mcy);
		mnx -= cx; mxx += cx; mny -= cy; mxy += cy;
	}
	int4 r;
	// one pixel of slack on every side keeps the rectangle conservative
	// against rounding in the per-micropolygon ranges
	float fx0 = floorf(mnx) - 1.0f, fy0 = floorf(mny) - 1.0f;
	float fx1 = ceilf(mxx) + 2.0f, fy1 = ceilf(mxy) + 2.0f;
	const float rx0 = (float)fp.sx0, ry0 = (float)fp.sy0;
	const float rx1 = (float)(fp.sx0 + fp.sw), ry1 = (float)(fp.sy0 + fp.sh);
	fx0 = fmaxf(fx0, rx0); fy0 = fmaxf(fy0, ry0);
	fx1 = fminf(fx1, rx1); fy1 = fminf(fy1, ry1);
	if (!(fx0 < fx1 && fy0 < fy1) || !(mnx <= mxx)) {
		r = make_int4(0, 0, 0, 0);  // empty (also catches NaN)
	} else {
		r = make_int4((int)fx0, (int)fx1, (int)fy0, (int)fy1);
	}
	rect[warp] = r;
}

__device__ __forceinline__ void st_rect(const FrameParams& fp, int st, int& x0, int& x1, int& y0, int& y1) {
	const int stx = st % fp.nstx, sty = st / fp.nstx;
	x0 = fp.sx0 + stx * fp.st_tiles * fp.tile_w;
	y0 = fp.sy0 + sty * fp.st_tiles * fp.tile_h;
	x1 = x0 + fp.st_tiles * fp.tile_w;
	y1 = y0 + fp.st_tiles * fp.tile_h;
}

__device__ __forceinline__ bool rect_hits(int4 r, int x0, int x1, int y0, int y1) {
	return r.x < r.y && r.x < x1 && r.y > x0 && r.z < y1 && r.w > y0;
}

// grid (blockIdx.x = super-tile, blockIdx.y = grid range): count the range's
// grids that touch the super-tile.
__global__ void st_count_kernel(FrameParams fp, int ngrids, const int4* rect, int nranges, int range_size,
                                int32_t* count) {
	const int st = blockIdx.x, r = blockIdx.y;
	int x0, x1, y0, y1;
	st_rect(fp, st, x0, x1, y0, y1);
	const int g0 = r * range_size, g1 = min(ngrids, g0 + range_size);
	int c = 0;
	for (int gi = g0 + threadIdx.x; gi < g1; gi += blockDim.x) c += rect_hits(rect[gi], x0, x1, y0, y1) ? 1 : 0;
	__shared__ int red[32];
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
	__syncthreads();
	if (threadIdx.x < 32) {
		int v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
		if (threadIdx.x == 0) count[st * nranges + r] = v;
	}
}

// Ordered compaction: write the range's touching grids at the super-tile's
// offset, in grid order.
__global__ void st_write_kernel(FrameParams fp, int ngrids, const int4* rect, int nranges, int range_size,
                                const int32_t* offset, int32_t* list, long long capacity) {
	const int st = blockIdx.x, r = blockIdx.y;
	int x0, x1, y0, y1;
	st_rect(fp, st, x0, x1, y0, y1);
	const int g0 = r * range_size, g1 = min(ngrids, g0 + range_size);
	__shared__ int warp_tot[32];
	__shared__ int base;
	if (threadIdx.x == 0) base = offset[st * nranges + r];
	__syncthreads();
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
	for (int c0 = g0; c0 < g1; c0 += blockDim.x) {
		const int gi = c0 + threadIdx.x;
		const bool f = gi < g1 && rect_hits(rect[gi], x0, x1, y0, y1);
		const unsigned bal = __ballot_sync(0xffffffffu, f);
		if (lane == 0) warp_tot[wid] = __popc(bal);
		__syncthreads();
		int pre = 0, tot = 0;
		for (int w = 0; w < nw; ++w) {
			int t = warp_tot[w];
			pre += (w < wid) ? t : 0;
			tot += t;
		}
		const long long idx = (long long)base + pre + __popc(bal & ((1u << lane) - 1u));
		if (f && idx < capacity) list[idx] = gi;  // a short list is detected by the host and re-binned
		__syncthreads();
		if (threadIdx.x == 0) base += tot;
		__syncthreads();
	}
}

// Single-block exclusive scan with the grand total appended at out[n].
__global__ void scan_i32_kernel(const int32_t* in, int32_t* out, int n) {
	__shared__ int warp_sum[32];
	__shared__ int carry;
	if (threadIdx.x == 0) carry = 0;
	__syncthreads();
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
	for (int c0 = 0; c0 < n; c0 += blockDim.x) {
		const int i = c0 + threadIdx.x;
		int v = i < n ? in[i] : 0;
		int x = v;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			int y = __shfl_up_sync(0xffffffffu, x, o);
			if (lane >= o) x += y;
		}
		if (lane == 31) warp_sum[wid] = x;
		__syncthreads();
		int pre = 0, tot = 0;
		for (int w = 0; w < nw; ++w) {
			pre += (w < wid) ? warp_sum[w] : 0;
			tot += warp_sum[w];
		}
		if (i < n) out[i] = carry + pre + x - v;
		__syncthreads();
		if (threadIdx.x == 0) carry += tot;
		__syncthreads();
	}
	if (threadIdx.x == 0) out[n] = carry;
}

// Lookup table from micropolygon id to grid: entry k is the grid holding id
// k * 256 (thread per grid writes the entries whose id falls in it).
__global__ void id_grid_kernel(GridsDev g, int64_t nmps, int32_t* table) {
	const int gi = blockIdx.x * blockDim.x + threadIdx.x;
	if (gi >= g.ngrids) return;
	const int64_t s = g.mpbase[gi];
	const int64_t e = (gi + 1 < g.ngrids) ? g.mpbase[gi + 1] : nmps;
	for (int64_t k = (s + 255) >> 8; (k << 8) < e; ++k) table[k] = gi;
}

// Split's projection for grids flagged AQH_GRID_CAMERA: block per grid, every
// key's points replaced in place by their hybrid raster form, then the flag
// cleared so a later pass over the same arrays leaves them alone.
__global__ void project_grids_kernel(GridsDev g, float4* P, int32_t* flags, CamMatrix M) {
	const int gi = blockIdx.x;
	if (!(__ldg(g.flags + gi) & AQH_GRID_CAMERA)) return;
	const int64_t nv = (int64_t)(__ldg(g.cu + gi) + 1) * (__ldg(g.cv + gi) + 1);
	const int64_t n = nv * __ldg(g.nkeys + gi);
	float4* p = P + __ldg(g.pbase + gi);
	for (int64_t i = threadIdx.x; i < n; i += blockDim.x) p[i] = project_point(M.m, p[i]);
	__syncthreads();
	if (threadIdx.x == 0) flags[gi] &= ~AQH_GRID_CAMERA;
}

void launch_project_grids(const GridsDev& g, float4* P, int32_t* flags, const CamMatrix& m, cudaStream_t s) {
	if (g.ngrids == 0) return;
	project_grids_kernel<<<g.ngrids, 256, 0, s>>>(g, P, flags, m);
}

// CqBasicVec3 dot product (vector3d.h:602-606) and the back-face test of one
// vertex (micropolygon.cpp:451-459, 1013-1017).
__device__ __forceinline__ bool back_facing(float4 p, const float* ng, const float* n) {
	const float gx = __ldg(ng), gy = __ldg(ng + 1), gz = __ldg(ng + 2);
	float s = 1.0f;
	if (n) s = ((__ldg(n) * gx + __ldg(n + 1) * gy) + __ldg(n + 2) * gz < 0.0f) ? -1.0f : 1.0f;
	return ((s * gx) * p.x + (s * gy) * p.y) + (s * gz) * p.z >= 0.0f;
}

// CqMicroPolyGrid::Shade's and CqMotionMicroPolyGrid::Split's culling, one
// block per flagged grid, on camera-space P before projection.
__global__ void cull_grids_kernel(GridsDev g, const float* Ng, const float* N, long long nng, int zthr_black,
                                  uint8_t* culled, int32_t* err) {
	__shared__ int last_visible;
	const int gi = blockIdx.x;
	const int flags = __ldg(g.flags + gi);
	if (!(flags & (AQH_GRID_CULL_BACKFACING | AQH_GRID_CULL_TRANSPARENT))) return;
	const int cu = __ldg(g.cu + gi), cv = __ldg(g.cv + gi), nk = __ldg(g.nkeys + gi);
	const int nv = (cu + 1) * (cv + 1);
	const long long pb = __ldg(g.pbase + gi), cb = __ldg(g.cbase + gi), mb = __ldg(g.mpbase + gi);
	// the back-face test needs camera-space P: a grid already projected (a
	// device-resident grid after its first frame) keeps the result of none
	const bool bf = (flags & AQH_GRID_CULL_BACKFACING) && (flags & AQH_GRID_CAMERA);
	if (bf && (!Ng || pb < 0 || pb + (long long)nk * nv > nng)) {
		if (threadIdx.x == 0) atomicOr(err, 1);
		return;
	}
	// the trailing run of black Oi starts after the last vertex that is not black
	const bool tr = nk == 1 && (flags & AQH_GRID_CULL_TRANSPARENT) && g.Oi && !zthr_black;
	if (threadIdx.x == 0) last_visible = -1;
	__syncthreads();
	if (tr) {
		int mx = -1;
		for (int i = threadIdx.x; i < nv; i += blockDim.x) {
			float r, gg, b;
			if (g.colour3) {
				const float* o = reinterpret_cast<const float*>(g.Oi) + 3 * (cb + i);
				r = __ldg(o); gg = __ldg(o + 1); b = __ldg(o + 2);
			} else {
				const float4 o = __ldg(g.Oi + cb + i);
				r = o.x; gg = o.y; b = o.z;
			}
			if (!(r == 0.0f && gg == 0.0f && b == 0.0f)) mx = i;
		}
		atomicMax(&last_visible, mx);
	}
	__syncthreads();
	const int run_start = tr ? last_visible + 1 : nv;
	for (int m = threadIdx.x; m < cu * cv; m += blockDim.x) {
		const int ia = (m / cu) * (cu + 1) + (m % cu);
		bool c = false;
		if (bf) {
			int facing_away = 0;
			for (int k = 0; k < nk; ++k) {
				const long long e = pb + (long long)k * nv + ia;
				facing_away += back_facing(__ldg(g.P + e), Ng + 3 * e, N ? N + 3 * e : nullptr) ? 1 : 0;
			}
			c = facing_away == nk;
		}
		c = c || ia >= run_start;
		if (c) culled[mb + m] = 1;
	}
}

void launch_cull_grids(const GridsDev& g, const float* Ng, const float* N, long long nng, int zthr_black,
                       uint8_t* culled, int32_t* err, cudaStream_t s) {
	if (g.ngrids == 0) return;
	cull_grids_kernel<<<g.ngrids, 256, 0, s>>>(g, Ng, N, nng, zthr_black, culled, err);
}

// CqMicroPolyGrid::Split / CqMotionMicroPolyGrid::Split trimming
// (micropolygon.cpp:754-835, 1056-1130), one block per grid: the corners'
// surface parameters (index, index+1, index+cu+2, index+cu+1) are classified
// against the grid's trim set, inverted for the "outside" sense; all four
// trimmed with no edge crossing a loop drops the micropolygon, any trimmed
// marks it for the per-hit test.
__global__ void trim_mark_kernel(GridsDev g, long long nuv, uint8_t* mark, uint8_t* culled, int32_t* err) {
	const int gi = blockIdx.x;
	const int set = __ldg(g.trim.grid_set + gi);
	if (set < 0) return;
	const int cu = __ldg(g.cu + gi), cv = __ldg(g.cv + gi);
	const long long cb = __ldg(g.cbase + gi);
	if (cb < 0 || cb + (long long)(cu + 1) * (cv + 1) > nuv) {
		if (threadIdx.x == 0) atomicOr(err, 1);
		return;
	}
	const bool outside = (__ldg(g.flags + gi) & 64) != 0;
	const int l0 = __ldg(g.trim.set_first + set), l1 = __ldg(g.trim.set_first + set + 1);
	const long long mb = __ldg(g.mpbase + gi);
	const int nm = cu * cv;
	for (int m = threadIdx.x; m < nm; m += blockDim.x) {
		if (culled[mb + m]) continue;
		const long long c = cb + (long long)(m / cu) * (cu + 1) + (m % cu);
		const float2 A = __ldg(g.trim.uv + c), B = __ldg(g.trim.uv + c + 1);
		const float2 C = __ldg(g.trim.uv + c + cu + 2), D = __ldg(g.trim.uv + c + cu + 1);
		const bool tA = trim_point(g.trim.pts, g.trim.loop_first, l0, l1, A.x, A.y) != outside;
		const bool tB = trim_point(g.trim.pts, g.trim.loop_first, l0, l1, B.x, B.y) != outside;
		const bool tC = trim_point(g.trim.pts, g.trim.loop_first, l0, l1, C.x, C.y) != outside;
		const bool tD = trim_point(g.trim.pts, g.trim.loop_first, l0, l1, D.x, D.y) != outside;
		if (tA && tB && tC && tD && !trim_line(g.trim.pts, g.trim.loop_first, l0, l1, A, B) &&
		    !trim_line(g.trim.pts, g.trim.loop_first, l0, l1, B, C) &&
		    !trim_line(g.trim.pts, g.trim.loop_first, l0, l1, C, D) &&
		    !trim_line(g.trim.pts, g.trim.loop_first, l0, l1, D, A)) {
			culled[mb + m] = 1;
			continue;
		}
		if (tA || tB || tC || tD) mark[mb + m] = 1;
	}
}

void launch_trim_mark(const GridsDev& g, long long nuv, uint8_t* mark, uint8_t* culled, int32_t* err, cudaStream_t s) {
	if (g.ngrids == 0) return;
	trim_mark_kernel<<<g.ngrids, 128, 0, s>>>(g, nuv, mark, culled, err);
}

void launch_id_grid(const GridsDev& g, int64_t nmps, int32_t* table, cudaStream_t s) {
	if (g.ngrids == 0) return;
	id_grid_kernel<<<(g.ngrids + 255) / 256, 256, 0, s>>>(g, nmps, table);
}

void launch_grid_rects(const FrameParams& fp, const GridsDev& g, const BinBuffers& b, cudaStream_t s) {
	if (g.ngrids == 0) return;
	const int wpb = kBlock / 32;
	grid_rects_kernel<<<(g.ngrids + wpb - 1) / wpb, kBlock, 0, s>>>(fp, g, b.grid_rect, b.grid_minz, b.strips, b.tri);
}

void launch_st_count(const FrameParams& fp, const GridsDev& g, BinBuffers& b, cudaStream_t s) {
	dim3 grid(fp.nstx * fp.nsty, b.nranges);
	st_count_kernel<<<grid, kBlock, 0, s>>>(fp, g.ngrids, b.grid_rect, b.nranges, b.range_size, b.st_count);
}

void launch_scan_i32(const int32_t* in, int32_t* out, int n, int32_t*, cudaStream_t s) {
	scan_i32_kernel<<<1, 1024, 0, s>>>(in, out, n);
}

void launch_st_write(const FrameParams& fp, const GridsDev& g, BinBuffers& b, cudaStream_t s) {
	dim3 grid(fp.nstx * fp.nsty, b.nranges);
	st_write_kernel<<<grid, kBlock, 0, s>>>(fp, g.ngrids, b.grid_rect, b.nranges, b.range_size, b.st_offset,
	                                        b.st_list, (long long)b.list_capacity);
}

// One warp per grid: the staging bound of each of its micropolygons, read by
// every motion sampling tile the micropolygon may reach instead of its key
// vertices.
__global__ void mb_stage_bounds_kernel(FrameParams fp, GridsDev g, int4* out) {
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (warp >= g.ngrids) return;
	const int n = __ldg(g.cu + warp) * __ldg(g.cv + warp);
	int4* o = out + __ldg(g.mpbase + warp);
	for (int m = lane; m < n; m += 32) o[m] = pack_stage_bound(mb_stage_bound(fp, g, warp, m));
}

void launch_mb_stage_bounds(const FrameParams& fp, const GridsDev& g, int4* out, cudaStream_t s) {
	if (g.ngrids <= 0) return;
	const int wpb = kBlock / 32;
	mb_stage_bounds_kernel<<<(g.ngrids + wpb - 1) / wpb, kBlock, 0, s>>>(fp, g, out);
}

}  // namespace aqh
