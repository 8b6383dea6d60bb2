// api.cu -- host runtime behind include/aqh.h.
//
// Owns the device buffers of a frame, stages host-submitted grids in pinned
// memory, resolves the frame options the way SqOptionCache/CqRenderer do, and
// runs the stages on the context's stream:
//   bin      grid rectangles -> ordered super-tile grid lists   (bin.cu)
//   sample   hit tests, early-z, store, Combine                 (sample.cu)
//   filter   reconstruction filter, exposure (+ quantize)       (filter.cu)
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <list>
#include <vector>

#include "../../include/aqh.h"
#include "aqh_internal.h"

using namespace aqh;

namespace {

struct DevBuf {
	void* p = nullptr;
	size_t cap = 0;
	~DevBuf() { release(); }
	void release() {
		if (p) cudaFree(p);
		p = nullptr;
		cap = 0;
	}
	cudaError_t ensure(size_t bytes) {
		if (bytes <= cap) return cudaSuccess;
		// grow by at least half: a context that sees frames of many sizes (a
		// server slot) settles after a few frees, each of which stalls the device
		const size_t grown = cap ? cap + cap / 2 : 0;
		release();
		size_t want = std::max<size_t>(std::max(bytes, grown), 256);
		cudaError_t e = cudaMalloc(&p, want);
		if (e == cudaErrorMemoryAllocation && want > bytes) {
			cudaGetLastError();
			want = std::max<size_t>(bytes, 256);
			e = cudaMalloc(&p, want);
		}
		if (e != cudaSuccess) {
			p = nullptr;
			cap = 0;
			return e;
		}
		cap = want;
		return cudaSuccess;
	}
	template <class T> T* as() const { return static_cast<T*>(p); }
};

struct PinnedBuf {
	void* p = nullptr;
	size_t cap = 0, used = 0;
	~PinnedBuf() { if (p) cudaFreeHost(p); }
	cudaError_t reserve(size_t bytes) {
		if (bytes <= cap) return cudaSuccess;
		size_t want = std::max(bytes, cap * 2 + (1u << 20));
		void* q = nullptr;
		cudaError_t e = cudaMallocHost(&q, want);
		if (e != cudaSuccess) return e;
		if (p) {
			std::memcpy(q, p, used);
			cudaFreeHost(p);
		}
		p = q;
		cap = want;
		return cudaSuccess;
	}
	cudaError_t append(const void* src, size_t bytes) {
		cudaError_t e = reserve(used + bytes);
		if (e != cudaSuccess) return e;
		std::memcpy(static_cast<char*>(p) + used, src, bytes);
		used += bytes;
		return cudaSuccess;
	}
};

// Host copies of the RI filter functions (libs/core/filters.cpp), restated from
// the RenderMan Interface 3.2 forms the reference implements.
float filter_eval(int filter, float x, float y, float xwidth, float ywidth) {
	auto fmin_ = [](float a, float b) { return a < b ? a : b; };
	switch (filter) {
	case AQH_FILTER_GAUSSIAN:
		x /= xwidth;
		y /= ywidth;
		return std::exp(-8.0 * (x * x + y * y));
	case AQH_FILTER_BOX:
		return fmin_((std::fabs(x) <= xwidth / 2.0 ? 1.0f : 0.0f), (std::fabs(y) <= ywidth / 2.0 ? 1.0f : 0.0f));
	case AQH_FILTER_TRIANGLE: {
		float hx = xwidth / 2.0, hy = ywidth / 2.0;
		float ax = std::fabs(x), ay = std::fabs(y);
		return fmin_((ax <= hx ? (hx - ax) / hx : 0.0f), (ay <= hy ? (hy - ay) / hy : 0.0f));
	}
	case AQH_FILTER_CATMULLROM: {
		float r2 = (x * x + y * y);
		float r = std::sqrt(r2);
		return (r >= 2.0) ? 0.0 : (r < 1.0) ? (3.0 * r * r2 - 5.0 * r2 + 2.0) : (-r * r2 + 5.0 * r2 - 8.0 * r + 4.0);
	}
	case AQH_FILTER_SINC: {
		const double pi = 3.14159265358979323846;
		if (x != 0.0) { x *= pi; x = std::cos(0.5 * x / xwidth) * std::sin(x) / x; } else x = 1.0;
		if (y != 0.0) { y *= pi; y = std::cos(0.5 * y / ywidth) * std::sin(y) / y; } else y = 1.0;
		return x * y;
	}
	case AQH_FILTER_DISK: {
		double xx = x * x, yy = y * y;
		xwidth *= 0.5; ywidth *= 0.5;
		double d = xx / (xwidth * xwidth) + yy / (ywidth * ywidth);
		return d < 1.0 ? 1.0f : 0.0f;
	}
	case AQH_FILTER_BESSEL: {
		const double pi = 3.14159265358979323846;
		double xx = x * x, yy = y * y;
		xwidth *= 0.5; ywidth *= 0.5;
		double w = xx / (xwidth * xwidth) + yy / (ywidth * ywidth);
		if (w < 1.0) {
			double d = std::sqrt(xx + yy);
			if (d != 0.0) {
				w = std::cos(0.5 * pi * std::sqrt(w));
				return w * 2 * j1(pi * d) / d;
			}
			return pi;
		}
		return 0.0f;
	}
	case AQH_FILTER_MITCHELL: {
		const float B = 1 / 3.0f, C = 1 / 3.0f;
		const float ixw = 1.0f / xwidth, iyw = 1.0f / ywidth;
		auto ev = [&](float t) {
			t = std::fabs(2.f * t);
			if (t > 1.f)
				return ((-B - 6 * C) * t * t * t + (6 * B + 30 * C) * t * t + (-12 * B - 48 * C) * t + (8 * B + 24 * C)) *
				       (1.f / 6.f);
			return ((12 - 9 * B - 6 * C) * t * t * t + (-18 + 12 * B + 6 * C) * t * t + (6 - 2 * B)) * (1.f / 6.f);
		};
		return ev(x * ixw) * ev(y * iyw);
	}
	}
	return 0.0f;
}

int lfloor_h(float x) { int i = (int)x; return i - ((x < 0 && x != (float)i) ? 1 : 0); }

}  // namespace

namespace aqh {

// Tile grid and super-tiles over the sample region.  The tile shape is the
// static kernel's (every sampler shares it), optionally narrowed to
// `tile_pixels`; a super-tile is about `supertile_px` pixels on a side.
void set_tiling(FrameParams& fp, int tile_pixels, int supertile_px) {
	static_tiling(fp, tile_pixels);
	const int tw = fp.tile_w, th = fp.tile_h;
	fp.ntx = (fp.sw + tw - 1) / tw;
	fp.nty = (fp.sh + th - 1) / th;
	fp.st_tiles = std::max(1, (supertile_px > 0 ? supertile_px : 128) / std::max(tw, th));
	fp.nstx = (fp.ntx + fp.st_tiles - 1) / fp.st_tiles;
	fp.nsty = (fp.nty + fp.st_tiles - 1) / fp.st_tiles;
}

// CqImagePixel::projectToCircle (imagepixel.h:429-436)
void project_to_circle_h(float x, float y, float& ox, float& oy) {
	float r;
	if (y == 0.0f) r = std::fabs(x);
	else if (x == 0.0f) r = std::fabs(y);
	else r = std::sqrt((x * x) + (y * y));
	if (r == 0.0f) { ox = 0.0f; oy = 0.0f; return; }
	const float ax = std::fabs(x), ay = std::fabs(y);
	const float adj = (ax < ay ? ay : ax) / r;
	ox = adj * x;
	oy = adj * y;
}

// Accumulated slice end times of CqMicroPolygonMotion::BuildBoundList
// (micropolygon.cpp:1714-1752) for every slice count d in 1..max(4, spp):
// dt = (close - open) / d, time = open + dt, then time += dt per slice.
void slice_times_h(float open, float close, int spp, std::vector<float>& out) {
	const int maxd = std::max(4, spp);
	out.assign((size_t)maxd * (maxd + 1) / 2, 0.0f);
	for (int d = 1; d <= maxd; ++d) {
		const float dt = (close - open) / d;
		float time = open + dt;
		float* T = out.data() + (size_t)d * (d - 1) / 2;
		for (int b = 0; b < d; ++b) {
			T[b] = time;
			time += dt;
		}
	}
}

// CqBucketProcessor::CalculateDofBounds (bucketprocessor.cpp:858-913): the
// region of the lens each sub-pixel stratum's offsets fall in, as
// {min.x, min.y, max.x, max.y}.
void dof_bounds_h(int xs, int ys, std::vector<float4>& out) {
	out.resize((size_t)xs * ys);
	const float dx = 2.0 / xs, dy = 2.0 / ys;
	float minX = -1.0, minY = -1.0;
	int which = 0;
	for (int j = 0; j < ys; ++j) {
		for (int i = 0; i < xs; ++i) {
			float tlx, tly, trx, try_, blx, bly, brx, bry;
			project_to_circle_h(minX, minY, tlx, tly);
			project_to_circle_h(minX + dx, minY, trx, try_);
			project_to_circle_h(minX, minY + dy, blx, bly);
			project_to_circle_h(minX + dx, minY + dy, brx, bry);
			if ((tly > 0.0 && bly < 0.0) || (tly < 0.0 && bly > 0.0)) {
				tlx = minX; blx = minX; trx = minX + dx; brx = minX + dx;
			}
			if ((tlx > 0.0 && trx < 0.0) || (tlx < 0.0 && trx > 0.0)) {
				tly = minY; bly = minY + dy; try_ = minY; bry = minY + dy;
			}
			float mnx = tlx, mny = tly, mxx = tlx, mxy = tly;
			auto enc = [&](float x, float y) {
				mnx = x < mnx ? x : mnx; mny = y < mny ? y : mny;
				mxx = mxx < x ? x : mxx; mxy = mxy < y ? y : mxy;
			};
			enc(trx, try_);
			enc(blx, bly);
			enc(brx, bry);
			out[which++] = make_float4(mnx, mny, mxx, mxy);
			minX += dx;
		}
		minX = -1.0;
		minY += dy;
	}
}


// Frame options resolved the way SqOptionCache / CqRenderer / CqBucketProcessor
// derive them (optioncache.cpp:48-118, renderer.h:368-377,
// bucketprocessor.cpp:36-37, 811-856, imagebuffer.cpp:533-539).
aqh_status resolve_frame(const aqh_frame_desc& dd, FrameParams& fp, std::vector<float>& ftab, std::string& err) {
	const aqh_frame_desc* d = &dd;
	char buf[256];
	if (d->width <= 0 || d->height <= 0) {
		snprintf(buf, sizeof buf, "bad resolution %dx%d", d->width, d->height);
		err = buf;
		return AQH_EINVAL;
	}
	if (d->xsamples <= 0 || d->ysamples <= 0 || d->xsamples * d->ysamples > AQH_MAX_SPP) {
		snprintf(buf, sizeof buf, "PixelSamples %d %d outside 1..%d samples", d->xsamples, d->ysamples, AQH_MAX_SPP);
		err = buf;
		return AQH_ELIMIT;
	}
	if (!(d->xfilter > 0) || !(d->yfilter > 0) || d->xfilter > 64 || d->yfilter > 64) {
		err = "bad filter width";
		return AQH_EINVAL;
	}
	std::memset(&fp, 0, sizeof fp);
	int cx0 = d->crop_xmin, cx1 = d->crop_xmax, cy0 = d->crop_ymin, cy1 = d->crop_ymax;
	if (cx0 == 0 && cx1 == 0 && cy0 == 0 && cy1 == 0) { cx1 = d->width; cy1 = d->height; }
	if (cx0 < 0 || cy0 < 0 || cx1 > d->width || cy1 > d->height || cx0 >= cx1 || cy0 >= cy1) {
		err = "bad crop window";
		return AQH_EINVAL;
	}
	fp.crop_x0 = cx0; fp.crop_x1 = cx1; fp.crop_y0 = cy0; fp.crop_y1 = cy1;
	fp.xs = d->xsamples; fp.ys = d->ysamples; fp.spp = fp.xs * fp.ys;
	fp.shiftX = lfloor_h(d->xfilter / 2.0f);
	fp.shiftY = lfloor_h(d->yfilter / 2.0f);
	fp.xfwo2 = std::ceil(d->xfilter) * 0.5f;
	fp.yfwo2 = std::ceil(d->yfilter) * 0.5f;
	fp.sx0 = cx0 - fp.shiftX; fp.sy0 = cy0 - fp.shiftY;
	fp.sw = (cx1 - cx0) + 2 * fp.shiftX; fp.sh = (cy1 - cy0) + 2 * fp.shiftY;
	fp.cull_x0 = cx0 - d->xfilter / 2.0f; fp.cull_x1 = cx1 + d->xfilter / 2.0f;
	fp.cull_y0 = cy0 - d->yfilter / 2.0f; fp.cull_y1 = cy1 + d->yfilter / 2.0f;
	fp.use_dof = (d->fstop > 0.0f && d->fstop < FLT_MAX) ? 1 : 0;
	if (fp.use_dof) {
		// CqRenderer::SetDepthOfFieldData (renderer.h:368-377)
		float lensDiameter = d->focal_length / d->fstop;
		fp.dof_mult = 0.5 * lensDiameter * d->focal_distance / (d->focal_distance + lensDiameter);
		fp.dof_inv_fd = 1.0 / d->focal_distance;
		fp.dof_scale_x = d->dof_scale_x;
		fp.dof_scale_y = d->dof_scale_y;
	}
	fp.shutter_open = d->shutter_open;
	fp.shutter_close = d->shutter_close;
	fp.depth_filter = d->depth_filter;
	fp.cullable = !(d->display_z && (d->depth_filter == AQH_DEPTH_MAX || d->depth_filter == AQH_DEPTH_AVERAGE));
	fp.midpoint_store = (d->display_z && d->depth_filter == AQH_DEPTH_MIDPOINT) ? 1 : 0;
	for (int k = 0; k < 3; ++k) fp.zthr[k] = d->zthreshold[k];
	fp.gain = d->gain; fp.gamma = d->gamma;
	fp.q_one = d->q_one; fp.q_min = d->q_min; fp.q_max = d->q_max; fp.q_dither = d->q_dither;
	set_tiling(fp, 0);
	const int n = aqh_filter_table(d->filter, d->xfilter, d->yfilter, fp.xs, fp.ys, nullptr, 0);
	ftab.assign(-n, 0.0f);
	aqh_filter_table(d->filter, d->xfilter, d->yfilter, fp.xs, fp.ys, ftab.data(), -n);
	fp.ftab_n = -n;
	return AQH_OK;
}

}  // namespace aqh

struct aqh_ctx {
	int device = 0;
	cudaStream_t stream = nullptr;
	cudaEvent_t ev[6] = {};
	// packed host grids: Ci/Oi go up on their own stream so the sampler, which
	// reads only P, overlaps the copy; `ev_cioi` marks them resident
	cudaStream_t cstream = nullptr;
	cudaEvent_t ev_before_up = nullptr, ev_cioi = nullptr;
	bool cioi_pending = false;
	std::string err;
	bool frame_open = false;
	aqh_frame_desc desc{};
	FrameParams fp{};
	std::vector<float> ftab;

	// host-submitted grids
	std::vector<int32_t> h_cu, h_cv, h_nkeys, h_flags, h_tbase;
	std::vector<int64_t> h_pbase, h_cbase, h_mpbase;
	std::vector<float> h_times;
	std::vector<uint8_t> h_culled;
	bool any_culled = false;
	PinnedBuf hP, hCi, hOi;
	int64_t h_verts_p = 0, h_verts_c = 0, h_mps = 0;
	bool h_has_ci = true, h_has_oi = true;
	bool any_transparent = false;
	// Split's projection: grids flagged AQH_GRID_CAMERA and the frame's matrix
	bool any_camera = false;
	int host_copy = AQH_HOST_COPY_AUTO;
	bool camera_set = false;
	aqh::CamMatrix camera{};
	// output variables: count, per-vertex values staged for host grids, the
	// packed host or device arrays, and the device copies
	int naov = 0;
	std::vector<float> h_aov;
	const float* hp_aov = nullptr;
	size_t hp_naov_vertices = 0;
	const float* dev_aov = nullptr;
	DevBuf d_aov, d_aovsrc, d_aovchan;
	// level-of-detail bounds per grid (min, max), host copy
	std::vector<float> h_lod;
	bool lod_set = false;
	DevBuf d_lod;
	// CSG: the tree and each grid's node, host arrays laid out for CsgDev
	int csg_n = 0;
	std::vector<int32_t> csg_grid_node, csg_type, csg_parent, csg_child, csg_nch, csg_pfirst, csg_pcount, csg_post;
	DevBuf d_csg, d_csg_overflow;
	// trim curves: host copies of the sets, the grids' sets and the uv array
	int trim_nsets = 0;
	bool cull_on = false;
	bool imager = false;        // aqh_set_imager: frames stop after the filter
	bool imager_pending = false; // the last frame waits for aqh_apply_imager
	DevBuf d_imager;
	std::vector<float> cull_Ng, cull_N;
	DevBuf d_cull_n;
	std::vector<int32_t> trim_grid_set, trim_loop_first, trim_set_first;
	std::vector<float> trim_pts, trim_uv;
	DevBuf d_trim_i, d_trim_f, d_trim_mark, d_trim_cull, d_trim_err;

	// host-submitted packed arrays (caller-owned, uploaded at render)
	bool host_packed = false;
	struct {
		int ngrids;
		const int32_t *cu, *cv, *nkeys, *flags, *tbase;
		const int64_t *pbase, *cbase;
		const float *times, *P, *Ci, *Oi;
		const uint8_t* culled;
		size_t ntimes, nP, nC;
		int comps;  // floats per P / Ci / Oi entry in the host arrays: 4, or 3 (CqVector3D / CqColor)
	} hp{};
	cudaStream_t own_stream = nullptr;
	// device-submitted grids (caller-owned)
	bool dev_grids = false;
	GridsDev dg{};
	int64_t dev_mps = 0;

	// device buffers
	DevBuf d_cu, d_cv, d_nkeys, d_flags, d_tbase, d_pbase, d_cbase, d_mpbase, d_times, d_culled, d_P, d_Ci, d_Oi;
	DevBuf d_mpcount;
	DevBuf d_rect, d_minz, d_strips, d_tri, d_stcount, d_stoffset, d_stlist, d_idgrid, d_mpb;
	DevBuf d_sa, d_sb, d_win, d_oz, d_nf, d_hz, d_keys, d_wmask;
	DevBuf d_frag, d_next, d_fcount, d_foverflow, d_err, d_occl, d_fheads;
	DevBuf d_ftab, d_chan, d_q8, d_qchan, d_dofb, d_disp, d_dither_req;
	DevBuf d_q8_req;          // quantized reads with other channel lists
	DevBuf d_P3, d_C3, d_O3;  // three-float host entries before widening
	bool q8_default = false;  // d_q8 holds the last frame's r g b a display
	bool dev_motion = false;
	int dev_max_keys = 0;
	DevBuf d_queue, d_slices;
	std::vector<float4> h_dofb;
	std::vector<float> h_slices;
	int mode = AQH_MODE_PLAIN;
	aqh_tuning tune{};  // launch shape of the sampling stage (zeros: defaults)
	// batched mode: instantiated frame graphs keyed by every kernel argument of
	// the frame, most recently used first (a server slot sees many job shapes)
	struct GraphEntry {
		std::vector<unsigned char> key;
		cudaGraphExec_t exec;
	};
	std::list<GraphEntry> graphs;
	bool graph_valid = true;  // false: buffers moved, drop every cached graph
	int64_t graphs_built = 0, overflow_rerenders = 0;
	bool pending_check = false;
	aqh::RenderPlan pending_plan{};
	// sampler
	DevBuf s_pos, s_time, s_dof, s_shuffle, s_lod, s_ipos, s_idof, s_itime, s_ishuf, s_ilod, s_dither;
	SamplerDev smp{};
	bool samples_set = false;
	int64_t frag_capacity = 0;
	bool debug_samples = true;
	aqh_frame_stats stats{};
	int64_t st_list_cap = 0;

	aqh_status fail(aqh_status s, const char* fmt, ...) {
		char buf[512];
		va_list ap;
		va_start(ap, fmt);
		vsnprintf(buf, sizeof buf, fmt, ap);
		va_end(ap);
		err = buf;
		return s;
	}
	aqh_status cuda_fail(cudaError_t e, const char* what) {
		return fail(e == cudaErrorMemoryAllocation ? AQH_ENOMEM : AQH_EDEVICE, "%s: %s", what, cudaGetErrorString(e));
	}
};

#define AQH_TRY(expr, what)                                   \
	do {                                                      \
		cudaError_t e_ = (expr);                              \
		if (e_ != cudaSuccess) return ctx->cuda_fail(e_, what); \
	} while (0)

extern "C" {

const char* aqh_status_string(aqh_status s) {
	switch (s) {
	case AQH_OK: return "ok";
	case AQH_EINVAL: return "invalid argument";
	case AQH_ENOMEM: return "out of memory";
	case AQH_EDEVICE: return "device error";
	case AQH_ETIMEDOUT: return "timed out";
	case AQH_EREJECTED: return "rejected";
	case AQH_ENOTREADY: return "not ready";
	case AQH_ELIMIT: return "limit exceeded";
	}
	return "unknown";
}

void aqh_frame_desc_defaults(aqh_frame_desc* d) {
	std::memset(d, 0, sizeof *d);
	d->width = 640;
	d->height = 480;
	d->bucket_x = d->bucket_y = 16;
	d->xsamples = d->ysamples = 2;
	d->xfilter = d->yfilter = 2.0f;
	d->filter = AQH_FILTER_GAUSSIAN;
	d->gain = d->gamma = 1.0f;
	d->q_one = 255.0f;
	d->q_min = 0.0f;
	d->q_max = 255.0f;
	d->q_dither = 0.5f;
	d->fstop = FLT_MAX;
	d->dof_scale_x = d->dof_scale_y = 1.0f;
	d->zthreshold[0] = d->zthreshold[1] = d->zthreshold[2] = 1.0f;
}

aqh_status aqh_create(const aqh_device_opts* opts, aqh_ctx** out) {
	if (!out) return AQH_EINVAL;
	*out = nullptr;
	aqh_ctx* ctx = new aqh_ctx();
	ctx->device = opts ? opts->device : 0;
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
	ctx->own_stream = ctx->stream;
	if (e == cudaSuccess) aqh::configure_sample_kernels();
	for (int i = 0; e == cudaSuccess && i < 6; ++i) e = cudaEventCreate(&ctx->ev[i]);
	if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->cstream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_before_up, cudaEventDisableTiming);
	if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_cioi, cudaEventDisableTiming);
	if (e != cudaSuccess) {
		delete ctx;
		return e == cudaErrorMemoryAllocation ? AQH_ENOMEM : AQH_EDEVICE;
	}
	*out = ctx;
	return AQH_OK;
}

void aqh_destroy(aqh_ctx* ctx) {
	if (!ctx) return;
	cudaSetDevice(ctx->device);
	if (ctx->stream) cudaStreamSynchronize(ctx->stream);
	if (ctx->own_stream && ctx->own_stream != ctx->stream) cudaStreamSynchronize(ctx->own_stream);
	if (ctx->cstream) cudaStreamSynchronize(ctx->cstream);
	for (auto& ev : ctx->ev)
		if (ev) cudaEventDestroy(ev);
	if (ctx->ev_before_up) cudaEventDestroy(ctx->ev_before_up);
	if (ctx->ev_cioi) cudaEventDestroy(ctx->ev_cioi);
	if (ctx->cstream) cudaStreamDestroy(ctx->cstream);
	for (auto& ge : ctx->graphs) cudaGraphExecDestroy(ge.exec);
	if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
	delete ctx;
}

const char* aqh_last_error(const aqh_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int aqh_filter_table(int filter, float xw, float yw, int xs, int ys, float* out, int max_out) {
	// CqBucketProcessor::InitialiseFilterValues (bucketprocessor.cpp:811-856)
	const int nsub = xs * ys;
	const int xmax = lfloor_h(xw / 2.0f), ymax = lfloor_h(yw / 2.0f);
	const int n = (2 * xmax + 1) * (2 * ymax + 1) * nsub;
	if (!out || n > max_out) return -n;
	const float xfwo2 = std::ceil(xw) * 0.5f, yfwo2 = std::ceil(yw) * 0.5f;
	for (int py = -ymax; py <= ymax; py++)
		for (int px = -xmax; px <= xmax; px++) {
			int idx = ((py + ymax) * (2 * xmax + 1) + px + xmax) * nsub;
			for (int sy = 0; sy < ys; sy++)
				for (int sx = 0; sx < xs; sx++, ++idx) {
					float fx = (sx + 0.5f) / xs + px - 0.5f;
					float fy = (sy + 0.5f) / ys + py - 0.5f;
					float w = 0;
					if (fx >= -xfwo2 && fy >= -yfwo2 && fx <= xfwo2 && fy <= yfwo2)
						w = filter_eval(filter, fx, fy, std::ceil(xw), std::ceil(yw));
					out[idx] = w;
				}
		}
	return n;
}

aqh_status aqh_frame_begin(aqh_ctx* ctx, const aqh_frame_desc* d) {
	if (!ctx || !d) return AQH_EINVAL;
	FrameParams fp{};
	std::string err;
	const aqh_status st = aqh::resolve_frame(*d, fp, ctx->ftab, err);
	if (st != AQH_OK) return ctx->fail(st, "%s", err.c_str());
	ctx->desc = *d;
	ctx->fp = fp;
	// reset grid stream
	ctx->h_cu.clear(); ctx->h_cv.clear(); ctx->h_nkeys.clear(); ctx->h_flags.clear(); ctx->h_tbase.clear();
	ctx->h_pbase.clear(); ctx->h_cbase.clear(); ctx->h_mpbase.clear(); ctx->h_times.clear(); ctx->h_culled.clear();
	ctx->any_culled = false;
	ctx->hP.used = ctx->hCi.used = ctx->hOi.used = 0;
	ctx->h_verts_p = ctx->h_verts_c = ctx->h_mps = 0;
	ctx->h_has_ci = ctx->h_has_oi = true;
	ctx->any_transparent = false;
	ctx->any_camera = false;
	ctx->camera_set = false;
	ctx->naov = 0;
	ctx->h_aov.clear();
	ctx->h_lod.clear();
	ctx->lod_set = false;
	ctx->csg_n = 0;
	ctx->trim_nsets = 0;
	ctx->cull_on = false;
	ctx->hp_aov = nullptr;
	ctx->hp_naov_vertices = 0;
	ctx->dev_aov = nullptr;
	ctx->dev_grids = false;
	ctx->dev_motion = false;
	ctx->dev_max_keys = 0;
	ctx->host_packed = false;
	ctx->dev_mps = 0;
	ctx->samples_set = false;
	ctx->frame_open = true;
	return AQH_OK;
}

aqh_status aqh_set_samples(aqh_ctx* ctx, const aqh_samples* s) {
	if (!ctx || !s || !s->pos || s->npatterns <= 0) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	cudaSetDevice(ctx->device);
	const FrameParams& fp = ctx->fp;
	const size_t np = (size_t)s->npatterns * fp.spp;
	const size_t npix = (size_t)fp.sw * fp.sh;
	const size_t ndisp = (size_t)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	// every table is read at (pattern of the pixel) * spp: a table without a
	// per-pixel choice needs one pattern per pixel, and every choice must name
	// an existing pattern
	struct Table { const void* data; const uint32_t* index; const char* name; };
	const Table tables[5] = {{s->pos, s->pos_index, "positions"}, {s->time, s->time_index, "times"},
	                         {s->dof, s->dof_index, "lens positions"}, {s->shuffle, s->shuffle_index, "lens shuffles"},
	                         {s->lod, s->lod_index, "detail levels"}};
	for (const Table& t : tables) {
		if (!t.data) continue;
		if (!t.index && (size_t)s->npatterns < npix)
			return ctx->fail(AQH_EINVAL, "sample %s without pattern choices need one pattern per pixel of the %dx%d "
			                 "sample region", t.name, fp.sw, fp.sh);
		if (t.index)
			for (size_t i = 0; i < npix; ++i)
				if (t.index[i] >= (uint32_t)s->npatterns)
					return ctx->fail(AQH_EINVAL, "pattern choice %u for sample %s at pixel %zu; %d patterns",
					                 t.index[i], t.name, i, s->npatterns);
	}
	if (s->shuffle) {
		for (size_t i = 0; i < np; ++i)
			if (s->shuffle[i] < 0 || s->shuffle[i] >= fp.spp)
				return ctx->fail(AQH_EINVAL, "lens shuffle entry %d out of range", s->shuffle[i]);
	}
	SamplerDev& m = ctx->smp;
	std::memset(&m, 0, sizeof m);
	m.npatterns = s->npatterns;
	auto up = [&](DevBuf& b, const void* src, size_t bytes) -> cudaError_t {
		if (!src) return cudaSuccess;
		cudaError_t e = b.ensure(bytes);
		if (e != cudaSuccess) return e;
		return cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
	};
	AQH_TRY(up(ctx->s_pos, s->pos, np * sizeof(float2)), "upload sample positions");
	AQH_TRY(up(ctx->s_time, s->time, np * sizeof(float)), "upload sample times");
	AQH_TRY(up(ctx->s_dof, s->dof, np * sizeof(float2)), "upload lens samples");
	AQH_TRY(up(ctx->s_shuffle, s->shuffle, np * sizeof(int32_t)), "upload lens shuffles");
	AQH_TRY(up(ctx->s_lod, s->lod, np * sizeof(float)), "upload lod samples");
	AQH_TRY(up(ctx->s_ipos, s->pos_index, npix * sizeof(uint32_t)), "upload pattern choices");
	AQH_TRY(up(ctx->s_idof, s->dof_index, npix * sizeof(uint32_t)), "upload pattern choices");
	AQH_TRY(up(ctx->s_itime, s->time_index, npix * sizeof(uint32_t)), "upload pattern choices");
	AQH_TRY(up(ctx->s_ishuf, s->shuffle_index, npix * sizeof(uint32_t)), "upload pattern choices");
	AQH_TRY(up(ctx->s_ilod, s->lod_index, npix * sizeof(uint32_t)), "upload pattern choices");
	AQH_TRY(up(ctx->s_dither, s->dither, ndisp * sizeof(float)), "upload dither");
	m.pos = ctx->s_pos.as<float2>();
	m.pos_unit = 1;
	for (size_t i = 0; i < np && m.pos_unit; ++i)
		m.pos_unit = s->pos[2 * i] >= 0.0f && s->pos[2 * i] <= 1.0f && s->pos[2 * i + 1] >= 0.0f && s->pos[2 * i + 1] <= 1.0f;
	m.time = s->time ? ctx->s_time.as<float>() : nullptr;
	m.dof = s->dof ? ctx->s_dof.as<float2>() : nullptr;
	m.shuffle = s->shuffle ? ctx->s_shuffle.as<int32_t>() : nullptr;
	m.lod = s->lod ? ctx->s_lod.as<float>() : nullptr;
	m.pos_index = s->pos_index ? ctx->s_ipos.as<uint32_t>() : nullptr;
	m.dof_index = s->dof_index ? ctx->s_idof.as<uint32_t>() : nullptr;
	m.time_index = s->time_index ? ctx->s_itime.as<uint32_t>() : nullptr;
	m.shuffle_index = s->shuffle_index ? ctx->s_ishuf.as<uint32_t>() : nullptr;
	m.lod_index = s->lod_index ? ctx->s_ilod.as<uint32_t>() : nullptr;
	m.dither = s->dither ? ctx->s_dither.as<float>() : nullptr;
	ctx->samples_set = true;
	return AQH_OK;
}

aqh_status aqh_submit_grid(aqh_ctx* ctx, const aqh_grid* gr) {
	if (!ctx || !gr || !gr->P) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	if (ctx->dev_grids || ctx->host_packed) return ctx->fail(AQH_EINVAL, "frame already holds packed grids");
	if (gr->cu <= 0 || gr->cv <= 0) return ctx->fail(AQH_EINVAL, "empty grid %dx%d", gr->cu, gr->cv);
	if (gr->nkeys < 1 || gr->nkeys > AQH_MAX_KEYS)
		return ctx->fail(AQH_ELIMIT, "grid has %d motion keys; 1..%d supported", gr->nkeys, AQH_MAX_KEYS);
	if (gr->nkeys > 1 && !gr->key_times) return ctx->fail(AQH_EINVAL, "motion grid without key times");
	const int64_t nv = (int64_t)(gr->cu + 1) * (gr->cv + 1);
	const int64_t nmp = (int64_t)gr->cu * gr->cv;
	if (ctx->h_mps + nmp > INT32_MAX) return ctx->fail(AQH_ELIMIT, "more than 2^31 micropolygons in one frame");
	ctx->h_cu.push_back(gr->cu);
	ctx->h_cv.push_back(gr->cv);
	ctx->h_nkeys.push_back(gr->nkeys);
	int flags = gr->flags;
	ctx->h_pbase.push_back(ctx->h_verts_p);
	ctx->h_cbase.push_back(ctx->h_verts_c);
	ctx->h_mpbase.push_back(ctx->h_mps);
	ctx->h_tbase.push_back((int32_t)ctx->h_times.size());
	if (gr->nkeys > 1)
		ctx->h_times.insert(ctx->h_times.end(), gr->key_times, gr->key_times + gr->nkeys);
	else
		ctx->h_times.push_back(0.0f);
	cudaError_t e = ctx->hP.append(gr->P, (size_t)nv * gr->nkeys * 16);
	if (e == cudaSuccess) {
		if (gr->Ci) e = ctx->hCi.append(gr->Ci, (size_t)nv * 16);
		else {
			std::vector<float> w((size_t)nv * 4, 1.0f);
			e = ctx->hCi.append(w.data(), w.size() * 4);
		}
	}
	if (e == cudaSuccess) {
		if (gr->Oi) {
			e = ctx->hOi.append(gr->Oi, (size_t)nv * 16);
			if (!(flags & AQH_GRID_OPAQUE)) ctx->any_transparent = true;
		} else {
			std::vector<float> w((size_t)nv * 4, 1.0f);
			e = ctx->hOi.append(w.data(), w.size() * 4);
			flags |= AQH_GRID_OPAQUE;
		}
	}
	if (e != cudaSuccess) return ctx->cuda_fail(e, "stage grid");
	if (ctx->naov > 0) {
		if (gr->aov) ctx->h_aov.insert(ctx->h_aov.end(), gr->aov, gr->aov + (size_t)nv * ctx->naov);
		else ctx->h_aov.insert(ctx->h_aov.end(), (size_t)nv * ctx->naov, 0.0f);
	}
	if (flags & AQH_GRID_CAMERA) ctx->any_camera = true;
	ctx->h_flags.push_back(flags);
	if (gr->culled) {
		if (!ctx->any_culled) {
			ctx->h_culled.assign((size_t)ctx->h_mps, 0);
			ctx->any_culled = true;
		}
		ctx->h_culled.insert(ctx->h_culled.end(), gr->culled, gr->culled + nmp);
	} else if (ctx->any_culled) {
		ctx->h_culled.insert(ctx->h_culled.end(), (size_t)nmp, 0);
	}
	ctx->h_verts_p += nv * gr->nkeys;
	ctx->h_verts_c += nv;
	ctx->h_mps += nmp;
	return AQH_OK;
}

namespace {
__global__ void mpcount_kernel(int n, const int32_t* cu, const int32_t* cv, int32_t* out) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) out[i] = cu[i] * cv[i];
}
__global__ void widen_kernel(int n, const int32_t* in, int64_t* out) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i <= n) out[i] = in[i];
}
// Packed three-float host entries (P, Ci, Oi as CqVector3D / CqColor) to
// the float4 device layout.
__global__ void widen3_kernel(const float* __restrict__ in, float4* __restrict__ out, long long n) {
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		out[i] = make_float4(in[3 * i], in[3 * i + 1], in[3 * i + 2], 0.0f);
}
void launch_widen3(const float* in, float4* out, size_t n, cudaStream_t s) {
	if (n == 0) return;
	const long long blocks = std::min<long long>(((long long)n + 255) / 256, 152LL * 16);
	widen3_kernel<<<(unsigned)blocks, 256, 0, s>>>(in, out, (long long)n);
}
__global__ void any_transparent_kernel(int n, const int32_t* flags, const int32_t* nkeys, int32_t* out) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n && !(flags[i] & AQH_GRID_OPAQUE)) out[0] = 1;
	if (i < n && nkeys[i] > 1) out[1] = 1;
	if (i < n && (flags[i] & AQH_GRID_CAMERA)) out[2] = 1;
	if (i < n) atomicMax(out + 3, nkeys[i]);
}
}  // namespace

aqh_status aqh_set_stream(aqh_ctx* ctx, void* stream) {
	if (!ctx) return AQH_EINVAL;
	cudaSetDevice(ctx->device);
	AQH_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
	ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
	return AQH_OK;
}

void* aqh_host_alloc(size_t bytes) {
	void* p = nullptr;
	if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
	return p;
}

void aqh_host_free(void* p) {
	if (p) cudaFreeHost(p);
}

static aqh_status submit_grids_host(aqh_ctx* ctx, int comps, int ngrids, const int32_t* cu, const int32_t* cv,
                                    const int32_t* nkeys, const int32_t* flags, const int64_t* pbase,
                                    const int64_t* cbase, const int32_t* tbase, const float* times, size_t ntimes,
                                    const float* P, size_t nP, const float* Ci, const float* Oi, size_t nC,
                                    const uint8_t* culled, int64_t total_mps) {
	if (!ctx || ngrids < 0 || !cu || !cv || !nkeys || !flags || !pbase || !cbase || !tbase || !P) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	if (!ctx->h_cu.empty() || ctx->dev_grids || ctx->host_packed) return ctx->fail(AQH_EINVAL, "frame already holds grids");
	if (total_mps > INT32_MAX) return ctx->fail(AQH_ELIMIT, "more than 2^31 micropolygons in one frame");
	int64_t mps = 0;
	bool transp = false;
	for (int i = 0; i < ngrids; ++i) {
		if (cu[i] <= 0 || cv[i] <= 0 || nkeys[i] < 1 || nkeys[i] > AQH_MAX_KEYS)
			return ctx->fail(AQH_EINVAL, "grid %d: bad size or key count", i);
		const int64_t nv = (int64_t)(cu[i] + 1) * (cv[i] + 1);
		if (pbase[i] < 0 || (size_t)(pbase[i] + nv * nkeys[i]) > nP || cbase[i] < 0 || (size_t)(cbase[i] + nv) > nC)
			return ctx->fail(AQH_EINVAL, "grid %d: vertices out of range", i);
		if (nkeys[i] > 1 && (tbase[i] < 0 || (size_t)(tbase[i] + nkeys[i]) > ntimes))
			return ctx->fail(AQH_EINVAL, "grid %d: key times out of range", i);
		mps += (int64_t)cu[i] * cv[i];
		if (!(flags[i] & AQH_GRID_OPAQUE)) transp = true;
		if (flags[i] & AQH_GRID_CAMERA) ctx->any_camera = true;
	}
	if (mps != total_mps) return ctx->fail(AQH_EINVAL, "total_micropolygons %lld != %lld", (long long)total_mps, (long long)mps);
	ctx->hp.ngrids = ngrids;
	ctx->hp.cu = cu; ctx->hp.cv = cv; ctx->hp.nkeys = nkeys; ctx->hp.flags = flags; ctx->hp.tbase = tbase;
	ctx->hp.pbase = pbase; ctx->hp.cbase = cbase; ctx->hp.times = times; ctx->hp.ntimes = ntimes;
	ctx->hp.P = P; ctx->hp.nP = nP; ctx->hp.Ci = Ci; ctx->hp.Oi = Oi; ctx->hp.nC = nC;
	ctx->hp.comps = comps;
	ctx->hp.culled = culled;
	ctx->h_mpbase.resize(ngrids);
	int64_t acc = 0;
	for (int i = 0; i < ngrids; ++i) { ctx->h_mpbase[i] = acc; acc += (int64_t)cu[i] * cv[i]; }
	ctx->h_mps = mps;
	ctx->any_transparent = transp && Oi;
	ctx->host_packed = true;
	return AQH_OK;
}

aqh_status aqh_submit_grids_host(aqh_ctx* ctx, int ngrids, const int32_t* cu, const int32_t* cv,
                                 const int32_t* nkeys, const int32_t* flags, const int64_t* pbase,
                                 const int64_t* cbase, const int32_t* tbase, const float* times, size_t ntimes,
                                 const float* P, size_t nP, const float* Ci, const float* Oi, size_t nC,
                                 const uint8_t* culled, int64_t total_mps) {
	return submit_grids_host(ctx, 4, ngrids, cu, cv, nkeys, flags, pbase, cbase, tbase, times, ntimes, P, nP, Ci, Oi,
	                         nC, culled, total_mps);
}

aqh_status aqh_submit_grids_host3(aqh_ctx* ctx, int ngrids, const int32_t* cu, const int32_t* cv,
                                  const int32_t* nkeys, const int32_t* flags, const int64_t* pbase,
                                  const int64_t* cbase, const int32_t* tbase, const float* times, size_t ntimes,
                                  const float* P, size_t nP, const float* Ci, const float* Oi, size_t nC,
                                  const uint8_t* culled, int64_t total_mps) {
	return submit_grids_host(ctx, 3, ngrids, cu, cv, nkeys, flags, pbase, cbase, tbase, times, ntimes, P, nP, Ci, Oi,
	                         nC, culled, total_mps);
}

aqh_status aqh_submit_grids_device(aqh_ctx* ctx, int ngrids, const int32_t* d_cu, const int32_t* d_cv,
                                   const int32_t* d_nkeys, const int32_t* d_flags, const int64_t* d_pbase,
                                   const int64_t* d_cbase, const int32_t* d_tbase, const float* d_times,
                                   const float* d_P, const float* d_Ci, const float* d_Oi, const uint8_t* d_culled,
                                   int64_t total_mps) {
	if (!ctx || ngrids < 0 || !d_cu || !d_cv || !d_nkeys || !d_flags || !d_pbase || !d_cbase || !d_P)
		return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	if (!ctx->h_cu.empty() || ctx->dev_grids || ctx->host_packed) return ctx->fail(AQH_EINVAL, "frame already holds grids");
	if (total_mps > INT32_MAX) return ctx->fail(AQH_ELIMIT, "more than 2^31 micropolygons in one frame");
	cudaSetDevice(ctx->device);
	GridsDev& g = ctx->dg;
	g.ngrids = ngrids;
	g.cu = d_cu; g.cv = d_cv; g.nkeys = d_nkeys; g.flags = d_flags;
	g.pbase = d_pbase; g.cbase = d_cbase; g.tbase = d_tbase; g.times = d_times;
	g.P = reinterpret_cast<const float4*>(d_P);
	g.Ci = reinterpret_cast<const float4*>(d_Ci);
	g.Oi = reinterpret_cast<const float4*>(d_Oi);
	g.colour3 = 0;
	g.culled = d_culled;
	// first micropolygon id of every grid
	AQH_TRY(ctx->d_mpcount.ensure(sizeof(int32_t) * (ngrids + 1) * 2 + 64), "alloc");
	AQH_TRY(ctx->d_mpbase.ensure(sizeof(int64_t) * (ngrids + 1)), "alloc");
	int32_t* cnt = ctx->d_mpcount.as<int32_t>();
	int32_t* off = cnt + (ngrids + 1);
	if (ngrids > 0) mpcount_kernel<<<(ngrids + 255) / 256, 256, 0, ctx->stream>>>(ngrids, d_cu, d_cv, cnt);
	launch_scan_i32(cnt, off, ngrids, nullptr, ctx->stream);
	widen_kernel<<<(ngrids + 256) / 256, 256, 0, ctx->stream>>>(ngrids, off, ctx->d_mpbase.as<int64_t>());
	g.mpbase = ctx->d_mpbase.as<int64_t>();
	// does any grid need the transparency path?
	AQH_TRY(ctx->d_err.ensure(64), "alloc");
	AQH_TRY(cudaMemsetAsync(ctx->d_err.p, 0, 64, ctx->stream), "memset");
	if (ngrids > 0)
		any_transparent_kernel<<<(ngrids + 255) / 256, 256, 0, ctx->stream>>>(ngrids, d_flags, d_nkeys,
		                                                                    ctx->d_err.as<int32_t>() + 8);
	int32_t anyt[4] = {0, 0, 0, 0};
	AQH_TRY(cudaMemcpyAsync(anyt, ctx->d_err.as<int32_t>() + 8, 16, cudaMemcpyDeviceToHost, ctx->stream), "readback");
	AQH_TRY(cudaStreamSynchronize(ctx->stream), "sync");
	ctx->any_transparent = anyt[0] != 0;
	ctx->dev_motion = anyt[1] != 0;
	ctx->any_camera = anyt[2] != 0;
	ctx->dev_max_keys = anyt[3];
	ctx->dev_grids = true;
	ctx->dev_mps = total_mps;
	return AQH_OK;
}

static aqh_status upload_packed_grids(aqh_ctx* ctx) {
	auto& hp = ctx->hp;
	const int G = hp.ngrids;
	auto up = [&](DevBuf& b, const void* src, size_t bytes) -> cudaError_t {
		cudaError_t e = b.ensure(bytes);
		if (e != cudaSuccess || bytes == 0 || !src) return e;
		return cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
	};
	AQH_TRY(up(ctx->d_cu, hp.cu, G * 4), "upload grids");
	AQH_TRY(up(ctx->d_cv, hp.cv, G * 4), "upload grids");
	AQH_TRY(up(ctx->d_nkeys, hp.nkeys, G * 4), "upload grids");
	AQH_TRY(up(ctx->d_flags, hp.flags, G * 4), "upload grids");
	AQH_TRY(up(ctx->d_tbase, hp.tbase, G * 4), "upload grids");
	AQH_TRY(up(ctx->d_pbase, hp.pbase, G * 8), "upload grids");
	AQH_TRY(up(ctx->d_cbase, hp.cbase, G * 8), "upload grids");
	AQH_TRY(up(ctx->d_mpbase, ctx->h_mpbase.data(), G * 8), "upload grids");
	AQH_TRY(up(ctx->d_times, hp.times, std::max<size_t>(hp.ntimes, 1) * 4), "upload grids");
	const bool packed3 = hp.comps == 3;
	// Ci/Oi go up on the copy stream, after everything already queued on the
	// main stream (the previous frame may still read the old colours); with
	// the copy engines moving P as well they start at once, beside P, so a
	// widening kernel that waits for another context's frame to leave the
	// SMs does not hold them back; otherwise after P's widening kernel, which
	// reads the host array over the same link
	DevBuf& dCi = packed3 ? ctx->d_C3 : ctx->d_Ci;
	DevBuf& dOi = packed3 ? ctx->d_O3 : ctx->d_Oi;
	const size_t csz = packed3 ? 12 : 16;
	AQH_TRY(dCi.ensure(std::max<size_t>(hp.nC, 1) * csz), "upload Ci");
	AQH_TRY(dOi.ensure(std::max<size_t>(hp.nC, 1) * csz), "upload Oi");
	auto colours_up = [&]() -> aqh_status {
		AQH_TRY(cudaEventRecord(ctx->ev_before_up, ctx->stream), "upload Ci");
		AQH_TRY(cudaStreamWaitEvent(ctx->cstream, ctx->ev_before_up, 0), "upload Ci");
		if (hp.Ci && hp.nC)
			AQH_TRY(cudaMemcpyAsync(dCi.p, hp.Ci, hp.nC * csz, cudaMemcpyHostToDevice, ctx->cstream), "upload Ci");
		if (hp.Oi && hp.nC)
			AQH_TRY(cudaMemcpyAsync(dOi.p, hp.Oi, hp.nC * csz, cudaMemcpyHostToDevice, ctx->cstream), "upload Oi");
		AQH_TRY(cudaEventRecord(ctx->ev_cioi, ctx->cstream), "upload Ci");
		ctx->cioi_pending = true;
		return AQH_OK;
	};
	const bool colours_first = ctx->host_copy == AQH_HOST_COPY_ENGINES;
	if (colours_first) {
		const aqh_status st = colours_up();
		if (st != AQH_OK) return st;
	}
	if (packed3) {
		// three-float P: widened to float4 by a kernel that reads the host
		// array itself when it is page-locked (as fast as the copy engines
		// over this link, and no second pass), else copied up and widened
		AQH_TRY(ctx->d_P.ensure(std::max<size_t>(hp.nP, 1) * 16), "upload P");
		cudaPointerAttributes pa{};
		const bool mapped = ctx->host_copy == AQH_HOST_COPY_AUTO && hp.nP &&
		                    cudaPointerGetAttributes(&pa, hp.P) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
		                    pa.devicePointer;
		cudaGetLastError();
		if (mapped) {
			launch_widen3(static_cast<const float*>(pa.devicePointer), ctx->d_P.as<float4>(), hp.nP, ctx->stream);
		} else {
			AQH_TRY(up(ctx->d_P3, hp.P, hp.nP * 12), "upload P");
			launch_widen3(ctx->d_P3.as<float>(), ctx->d_P.as<float4>(), hp.nP, ctx->stream);
		}
	} else {
		AQH_TRY(up(ctx->d_P, hp.P, hp.nP * 16), "upload P");
	}
	// three-float colours stay packed on the device (GridsDev::colour3)
	if (!colours_first) {
		const aqh_status st = colours_up();
		if (st != AQH_OK) return st;
	}
	if (hp.culled) AQH_TRY(up(ctx->d_culled, hp.culled, (size_t)ctx->h_mps), "upload culled");
	GridsDev& g = ctx->dg;
	g.ngrids = G;
	g.cu = ctx->d_cu.as<int32_t>(); g.cv = ctx->d_cv.as<int32_t>(); g.nkeys = ctx->d_nkeys.as<int32_t>();
	g.flags = ctx->d_flags.as<int32_t>(); g.tbase = ctx->d_tbase.as<int32_t>();
	g.pbase = ctx->d_pbase.as<int64_t>(); g.cbase = ctx->d_cbase.as<int64_t>(); g.mpbase = ctx->d_mpbase.as<int64_t>();
	g.times = hp.times ? ctx->d_times.as<float>() : nullptr;
	g.P = ctx->d_P.as<float4>();
	g.Ci = hp.Ci ? dCi.as<float4>() : nullptr;
	g.Oi = hp.Oi ? dOi.as<float4>() : nullptr;
	g.colour3 = packed3 ? 1 : 0;
	g.culled = hp.culled ? ctx->d_culled.as<uint8_t>() : nullptr;
	g.naov = 0;
	g.aov = nullptr;
	if (ctx->naov > 0) {
		const size_t n = hp.nC * (size_t)ctx->naov;
		AQH_TRY(ctx->d_aov.ensure(std::max<size_t>(n, 1) * 4), "alloc output variables");
		if (ctx->hp_aov && ctx->hp_naov_vertices >= hp.nC)
			AQH_TRY(cudaMemcpyAsync(ctx->d_aov.p, ctx->hp_aov, n * 4, cudaMemcpyHostToDevice, ctx->stream), "upload aov");
		else
			AQH_TRY(cudaMemsetAsync(ctx->d_aov.p, 0, n * 4, ctx->stream), "clear aov");
		g.aov = ctx->d_aov.as<float>();
		g.naov = ctx->naov;
	}
	return AQH_OK;
}

static aqh_status upload_host_grids(aqh_ctx* ctx) {
	const int G = (int)ctx->h_cu.size();
	auto up = [&](DevBuf& b, const void* src, size_t bytes) -> cudaError_t {
		cudaError_t e = b.ensure(bytes);
		if (e != cudaSuccess || bytes == 0) return e;
		return cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
	};
	AQH_TRY(up(ctx->d_cu, ctx->h_cu.data(), G * 4), "upload grids");
	AQH_TRY(up(ctx->d_cv, ctx->h_cv.data(), G * 4), "upload grids");
	AQH_TRY(up(ctx->d_nkeys, ctx->h_nkeys.data(), G * 4), "upload grids");
	AQH_TRY(up(ctx->d_flags, ctx->h_flags.data(), G * 4), "upload grids");
	AQH_TRY(up(ctx->d_tbase, ctx->h_tbase.data(), G * 4), "upload grids");
	AQH_TRY(up(ctx->d_pbase, ctx->h_pbase.data(), G * 8), "upload grids");
	AQH_TRY(up(ctx->d_cbase, ctx->h_cbase.data(), G * 8), "upload grids");
	AQH_TRY(up(ctx->d_mpbase, ctx->h_mpbase.data(), G * 8), "upload grids");
	AQH_TRY(up(ctx->d_times, ctx->h_times.data(), ctx->h_times.size() * 4), "upload grids");
	AQH_TRY(up(ctx->d_P, ctx->hP.p, ctx->hP.used), "upload P");
	AQH_TRY(up(ctx->d_Ci, ctx->hCi.p, ctx->hCi.used), "upload Ci");
	AQH_TRY(up(ctx->d_Oi, ctx->hOi.p, ctx->hOi.used), "upload Oi");
	if (ctx->any_culled) AQH_TRY(up(ctx->d_culled, ctx->h_culled.data(), ctx->h_culled.size()), "upload culled");
	GridsDev& g = ctx->dg;
	g.ngrids = G;
	g.cu = ctx->d_cu.as<int32_t>(); g.cv = ctx->d_cv.as<int32_t>(); g.nkeys = ctx->d_nkeys.as<int32_t>();
	g.flags = ctx->d_flags.as<int32_t>(); g.tbase = ctx->d_tbase.as<int32_t>();
	g.pbase = ctx->d_pbase.as<int64_t>(); g.cbase = ctx->d_cbase.as<int64_t>(); g.mpbase = ctx->d_mpbase.as<int64_t>();
	g.times = ctx->d_times.as<float>();
	g.P = ctx->d_P.as<float4>(); g.Ci = ctx->d_Ci.as<float4>(); g.Oi = ctx->d_Oi.as<float4>();
	g.colour3 = 0;
	g.culled = ctx->any_culled ? ctx->d_culled.as<uint8_t>() : nullptr;
	g.naov = 0;
	g.aov = nullptr;
	if (ctx->naov > 0) {
		AQH_TRY(up(ctx->d_aov, ctx->h_aov.data(), ctx->h_aov.size() * 4), "upload aov");
		g.aov = ctx->d_aov.as<float>();
		g.naov = ctx->naov;
	}
	return AQH_OK;
}


static aqh_status plan_render(aqh_ctx* ctx, RenderPlan& P) {
	FrameParams& fp = ctx->fp;
	cudaStream_t s = ctx->stream;
	aqh_status st = AQH_OK;
	if (ctx->host_packed) {
		st = upload_packed_grids(ctx);
		if (st != AQH_OK) return st;
	} else if (!ctx->dev_grids) {
		st = upload_host_grids(ctx);
		if (st != AQH_OK) return st;
	}
	const GridsDev& g = ctx->dg;
	if (ctx->any_camera && !ctx->camera_set && !ctx->dev_grids)
		return ctx->fail(AQH_EINVAL, "grids flagged AQH_GRID_CAMERA but no camera-to-raster matrix is set");
	P.project = ctx->any_camera && ctx->camera_set;
	P.imager = ctx->imager;
	P.cam = ctx->camera;
	P.nmps = ctx->dev_grids ? ctx->dev_mps : ctx->h_mps;
	bool motion = false;
	int max_keys = 0;
	if (ctx->host_packed) {
		for (int i = 0; i < ctx->hp.ngrids; ++i) max_keys = std::max(max_keys, (int)ctx->hp.nkeys[i]);
	} else if (!ctx->dev_grids) {
		for (int k : ctx->h_nkeys) max_keys = std::max(max_keys, k);
	}
	motion = max_keys > 1;
	if (ctx->dev_grids) {
		motion = ctx->dev_motion;
		max_keys = ctx->dev_max_keys;
	}
	fp.max_keys = max_keys;
	fp.any_motion = motion ? 1 : 0;
	P.mbdof = fp.use_dof || fp.any_motion;
	// opaque motion blur / depth of field frames sample smaller tiles (two
	// CTAs share an SM); frames that keep fragments use the default size
	const bool frags = ctx->any_transparent || !fp.cullable || fp.midpoint_store || ctx->csg_n > 0;
	int tile_pixels = ctx->tune.tile_pixels;
	if (P.mbdof && !frags) {
		const int cap = sample_mb_opaque_tile_pixels(fp.spp);
		tile_pixels = tile_pixels > 0 ? std::min(tile_pixels, cap) : cap;
	}
	set_tiling(fp, tile_pixels, ctx->tune.supertile_pixels);
	fp.filter_ctas = ctx->tune.filter_ctas_per_sm;
	fp.use_lod = (ctx->smp.lod != nullptr || ctx->lod_set) ? 1 : 0;
	if (P.mbdof) {
		ctx->h_dofb.clear();
		dof_bounds_h(fp.xs, fp.ys, ctx->h_dofb);
		AQH_TRY(ctx->d_dofb.ensure(ctx->h_dofb.size() * sizeof(float4)), "alloc");
		AQH_TRY(cudaMemcpyAsync(ctx->d_dofb.p, ctx->h_dofb.data(), ctx->h_dofb.size() * sizeof(float4),
		                        cudaMemcpyHostToDevice, s),
		        "upload lens bounds");
		slice_times_h(fp.shutter_open, fp.shutter_close, fp.spp, ctx->h_slices);
		AQH_TRY(ctx->d_slices.ensure(ctx->h_slices.size() * sizeof(float)), "alloc");
		AQH_TRY(cudaMemcpyAsync(ctx->d_slices.p, ctx->h_slices.data(), ctx->h_slices.size() * sizeof(float),
		                        cudaMemcpyHostToDevice, s),
		        "upload slice times");
	}
	const int G = g.ngrids;
	// the sampling records keep the grid index above six flag bits
	if (G > (1 << 25)) return ctx->fail(AQH_ELIMIT, "%d grids in one frame; at most 2^25", G);
	P.nsamp = (size_t)fp.sw * fp.sh * fp.spp;
	P.nst = fp.nstx * fp.nsty;
	BinBuffers& bb = P.bb;
	bb = BinBuffers{};
	bb.range_size = 4096;
	bb.nranges = std::max(1, (G + bb.range_size - 1) / bb.range_size);
	AQH_TRY(ctx->d_rect.ensure(sizeof(int4) * std::max(G, 1)), "alloc rects");
	AQH_TRY(ctx->d_minz.ensure(sizeof(float) * std::max(G, 1)), "alloc rects");
	AQH_TRY(ctx->d_stcount.ensure(sizeof(int32_t) * ((size_t)P.nst * bb.nranges + 1)), "alloc bins");
	AQH_TRY(ctx->d_stoffset.ensure(sizeof(int32_t) * ((size_t)P.nst * bb.nranges + 1)), "alloc bins");
	bb.grid_rect = ctx->d_rect.as<int4>();
	bb.grid_minz = ctx->d_minz.as<float>();
	AQH_TRY(ctx->d_strips.ensure(sizeof(uint32_t) * 64 * std::max(G, 1)), "alloc strips");
	bb.strips = ctx->d_strips.as<uint32_t>();
	AQH_TRY(ctx->d_tri.ensure(sizeof(float4) * kMaxKeys * std::max(G, 1)), "alloc split lines");
	bb.tri = ctx->d_tri.as<float4>();
	bb.st_count = ctx->d_stcount.as<int32_t>();
	bb.st_offset = ctx->d_stoffset.as<int32_t>();
	if (P.mbdof && P.nmps > 0) {
		// each micropolygon's staging bound, computed once instead of in every tile it may reach
		AQH_TRY(ctx->d_mpb.ensure(sizeof(int4) * (size_t)P.nmps), "alloc staging bounds");
		bb.mp_bounds = ctx->d_mpb.as<int4>();
	}
	const size_t nstore = store_size((long long)fp.sw * fp.sh, fp.spp);
	AQH_TRY(ctx->d_sa.ensure(nstore * sizeof(float4)), "alloc sample store");
	AQH_TRY(ctx->d_sb.ensure(nstore * sizeof(float4)), "alloc sample store");
	// window masks pay off where positions vary across the filter window and
	// pixels hold few samples (measured: 16 samples, 3x3 pixels)
	const bool wmask = fp.spp <= 16 && (fp.shiftX > 0 || fp.shiftY > 0) &&
	                   (2 * fp.shiftX + 1) * (2 * fp.shiftY + 1) <= 32;
	if (wmask) AQH_TRY(ctx->d_wmask.ensure(nstore * sizeof(uint32_t)), "alloc window masks");
	SampleStore& store = P.store;
	store = SampleStore{};
	store.a = ctx->d_sa.as<float4>();
	store.b = ctx->d_sb.as<float4>();
	if (wmask) store.wmask = ctx->d_wmask.as<uint32_t>();
	if (ctx->debug_samples) {
		AQH_TRY(ctx->d_win.ensure(P.nsamp * 4), "alloc");
		AQH_TRY(ctx->d_oz.ensure(P.nsamp * 4), "alloc");
		AQH_TRY(ctx->d_nf.ensure(P.nsamp * 4), "alloc");
		store.winner = ctx->d_win.as<int32_t>();
		store.occlz = ctx->d_oz.as<float>();
		store.nfrag = ctx->d_nf.as<int32_t>();
	}
	if (fp.midpoint_store) {
		AQH_TRY(ctx->d_hz.ensure(P.nsamp * 4), "alloc");
		store.hitz = ctx->d_hz.as<float>();
	}
	AQH_TRY(ctx->d_ftab.ensure(ctx->ftab.size() * 4), "alloc");
	AQH_TRY(cudaMemcpyAsync(ctx->d_ftab.p, ctx->ftab.data(), ctx->ftab.size() * 4, cudaMemcpyHostToDevice, s), "ftab");
	const size_t ndisp = (size_t)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	AQH_TRY(ctx->d_chan.ensure(ndisp * 9 * 4), "alloc channels");
	AQH_TRY(ctx->d_q8.ensure(ndisp * 4), "alloc quantized");
	AQH_TRY(ctx->d_qchan.ensure(64), "alloc");
	AQH_TRY(ctx->d_err.ensure(64), "alloc");
	AQH_TRY(ctx->d_queue.ensure(64), "alloc");
	FragPool& pool = P.pool;
	pool = FragPool{};
	fp.frag_only = 0;
	if (ctx->any_transparent || !fp.cullable || fp.midpoint_store || ctx->csg_n > 0) {
		// fragment links are int32: the pool indexes at most INT32_MAX fragments
		if (ctx->frag_capacity == 0)
			ctx->frag_capacity = std::min<int64_t>(INT32_MAX, std::max<int64_t>(1 << 20, (int64_t)P.nsamp * 2));
		AQH_TRY(ctx->d_frag.ensure(ctx->frag_capacity * sizeof(float4)), "alloc fragments");
		AQH_TRY(ctx->d_next.ensure(ctx->frag_capacity * sizeof(int32_t)), "alloc fragments");
		AQH_TRY(ctx->d_fcount.ensure(16), "alloc");
		AQH_TRY(ctx->d_foverflow.ensure(16), "alloc");
		pool.frag = ctx->d_frag.as<float4>();
		pool.next = ctx->d_next.as<int32_t>();
		pool.count = ctx->d_fcount.as<unsigned long long>();
		pool.overflow = ctx->d_foverflow.as<int32_t>();
		pool.capacity = ctx->frag_capacity;
		AQH_TRY(ctx->d_occl.ensure(16), "alloc");
		pool.occluders = ctx->d_occl.as<int32_t>();
		fp.frag_only = (!P.mbdof && !fp.midpoint_store) ? 1 : 0;
		if (fp.frag_only) {
			// the fragment-only sampler hands its list heads to a separate
			// Combine kernel, whose sort gets the L1 the sampler's shared memory
			// leaves too small
			AQH_TRY(ctx->d_fheads.ensure(P.nsamp * sizeof(int32_t)), "alloc list heads");
			pool.heads = ctx->d_fheads.as<int32_t>();
		}
	}
	if (pool.capacity == 0 && !P.mbdof && ctx->host_packed) {
		// colours still on their way from the host: the sampler hands its
		// hits to a separate resolve kernel, which alone waits for Ci/Oi
		AQH_TRY(ctx->d_keys.ensure(nstore * sizeof(unsigned long long)), "alloc hit keys");
		store.keys = ctx->d_keys.as<unsigned long long>();
	}
	int nsm = 0;
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
	int resident = nsm * sample_static_ctas_per_sm(pool.capacity > 0);
	if (ctx->tune.persistent_ctas > 0) resident = std::min(resident, ctx->tune.persistent_ctas);
	P.nctas = std::max(1, std::min(fp.ntx * fp.nty, resident));
	P.fp = fp;
	P.g = g;
	AQH_TRY(ctx->d_idgrid.ensure(sizeof(int32_t) * (size_t)((P.nmps + 255) / 256 + 1)), "alloc id table");
	P.g.id_grid = ctx->d_idgrid.as<int32_t>();
	P.g.csg = CsgDev{};
	if (ctx->csg_n > 0) {
		// one buffer: grid nodes (G, -1 past the given ones), then the node tables
		const int N = ctx->csg_n;
		std::vector<int32_t> buf;
		buf.reserve((size_t)G + 7 * N + ctx->csg_post.size());
		for (int i = 0; i < G; ++i) buf.push_back(i < (int)ctx->csg_grid_node.size() ? ctx->csg_grid_node[i] : -1);
		const size_t o_type = buf.size();
		buf.insert(buf.end(), ctx->csg_type.begin(), ctx->csg_type.end());
		const size_t o_parent = buf.size();
		buf.insert(buf.end(), ctx->csg_parent.begin(), ctx->csg_parent.end());
		const size_t o_child = buf.size();
		buf.insert(buf.end(), ctx->csg_child.begin(), ctx->csg_child.end());
		const size_t o_nch = buf.size();
		buf.insert(buf.end(), ctx->csg_nch.begin(), ctx->csg_nch.end());
		const size_t o_pf = buf.size();
		buf.insert(buf.end(), ctx->csg_pfirst.begin(), ctx->csg_pfirst.end());
		const size_t o_pc = buf.size();
		buf.insert(buf.end(), ctx->csg_pcount.begin(), ctx->csg_pcount.end());
		const size_t o_post = buf.size();
		buf.insert(buf.end(), ctx->csg_post.begin(), ctx->csg_post.end());
		buf.push_back(0);
		AQH_TRY(ctx->d_csg.ensure(buf.size() * 4), "alloc CSG tree");
		AQH_TRY(cudaMemcpyAsync(ctx->d_csg.p, buf.data(), buf.size() * 4, cudaMemcpyHostToDevice, s), "upload CSG tree");
		AQH_TRY(ctx->d_csg_overflow.ensure(16), "alloc");
		AQH_TRY(cudaMemsetAsync(ctx->d_csg_overflow.p, 0, 4, s), "memset");
		AQH_TRY(cudaStreamSynchronize(s), "upload CSG tree");
		const int32_t* b = ctx->d_csg.as<int32_t>();
		CsgDev& c = P.g.csg;
		c.nnodes = N;
		c.grid_node = b;
		c.type = b + o_type;
		c.parent = b + o_parent;
		c.child_index = b + o_child;
		c.nchildren = b + o_nch;
		c.post_first = b + o_pf;
		c.post_count = b + o_pc;
		c.post = b + o_post;
		c.overflow = ctx->d_csg_overflow.as<int32_t>();
	}
	P.g.lod = nullptr;
	if (ctx->lod_set && G > 0) {
		// grids past the given bounds keep the attribute default (0, 1)
		std::vector<float> b((size_t)G * 2);
		for (int i = 0; i < G; ++i) {
			const bool have = (size_t)(2 * i + 1) < ctx->h_lod.size();
			b[2 * i] = have ? ctx->h_lod[2 * i] : 0.0f;
			b[2 * i + 1] = have ? ctx->h_lod[2 * i + 1] : 1.0f;
		}
		AQH_TRY(ctx->d_lod.ensure(b.size() * 4), "alloc detail bounds");
		AQH_TRY(cudaMemcpyAsync(ctx->d_lod.p, b.data(), b.size() * 4, cudaMemcpyHostToDevice, s), "upload detail bounds");
		AQH_TRY(cudaStreamSynchronize(s), "upload detail bounds");
		P.g.lod = ctx->d_lod.as<float2>();
	}
	if (ctx->dev_grids) {
		if (ctx->naov > 0 && !ctx->dev_aov)
			return ctx->fail(AQH_EINVAL, "output variables are set but aqh_submit_aov_device was not called");
		P.g.aov = ctx->dev_aov;
		P.g.naov = ctx->dev_aov ? ctx->naov : 0;
	}
	P.g.trim = TrimDev{};
	if ((ctx->trim_nsets > 0 || ctx->cull_on) && G > 0) {
		// the frame's own culled mask: the caller's (or none) plus what Shade /
		// Split culling and trimming drop
		const size_t nm = (size_t)std::max<int64_t>(P.nmps, 1);
		AQH_TRY(ctx->d_trim_cull.ensure(nm), "alloc culled mask");
		AQH_TRY(ctx->d_trim_err.ensure(16), "alloc");
		AQH_TRY(cudaMemsetAsync(ctx->d_trim_err.p, 0, 4, s), "memset");
		if (P.g.culled && P.nmps > 0)
			AQH_TRY(cudaMemcpyAsync(ctx->d_trim_cull.p, P.g.culled, (size_t)P.nmps, cudaMemcpyDeviceToDevice, s), "copy");
		else
			AQH_TRY(cudaMemsetAsync(ctx->d_trim_cull.p, 0, nm, s), "memset");
	}
	if (ctx->cull_on && G > 0) {
		const size_t n3 = ctx->cull_Ng.size();
		AQH_TRY(ctx->d_cull_n.ensure((n3 + ctx->cull_N.size() + 4) * 4), "alloc normals");
		float* dn = ctx->d_cull_n.as<float>();
		if (n3) AQH_TRY(cudaMemcpyAsync(dn, ctx->cull_Ng.data(), n3 * 4, cudaMemcpyHostToDevice, s), "upload Ng");
		if (!ctx->cull_N.empty())
			AQH_TRY(cudaMemcpyAsync(dn + n3, ctx->cull_N.data(), ctx->cull_N.size() * 4, cudaMemcpyHostToDevice, s),
			        "upload N");
		const int zblack = fp.zthr[0] == 0.0f && fp.zthr[1] == 0.0f && fp.zthr[2] == 0.0f;
		launch_cull_grids(P.g, n3 ? dn : nullptr, ctx->cull_N.empty() ? nullptr : dn + n3, (long long)(n3 / 3), zblack,
		                  ctx->d_trim_cull.as<uint8_t>(), ctx->d_trim_err.as<int32_t>(), s);
		AQH_TRY(cudaGetLastError(), "cull kernel launch");
	}
	if (ctx->trim_nsets > 0 && G > 0) {
		// ints: grid sets (G, -1 past the given ones), loop starts, set starts;
		// floats: loop points, then uv
		std::vector<int32_t> bi;
		bi.reserve((size_t)G + ctx->trim_loop_first.size() + ctx->trim_set_first.size());
		for (int i = 0; i < G; ++i) bi.push_back(i < (int)ctx->trim_grid_set.size() ? ctx->trim_grid_set[i] : -1);
		const size_t o_lf = bi.size();
		bi.insert(bi.end(), ctx->trim_loop_first.begin(), ctx->trim_loop_first.end());
		const size_t o_sf = bi.size();
		bi.insert(bi.end(), ctx->trim_set_first.begin(), ctx->trim_set_first.end());
		const size_t npf = ctx->trim_pts.size();
		AQH_TRY(ctx->d_trim_i.ensure(bi.size() * 4), "alloc trim sets");
		AQH_TRY(ctx->d_trim_f.ensure((npf + ctx->trim_uv.size() + 2) * 4), "alloc trim sets");
		AQH_TRY(cudaMemcpyAsync(ctx->d_trim_i.p, bi.data(), bi.size() * 4, cudaMemcpyHostToDevice, s), "upload trim sets");
		float* df = ctx->d_trim_f.as<float>();
		if (npf) AQH_TRY(cudaMemcpyAsync(df, ctx->trim_pts.data(), npf * 4, cudaMemcpyHostToDevice, s), "upload trim sets");
		if (!ctx->trim_uv.empty())
			AQH_TRY(cudaMemcpyAsync(df + npf, ctx->trim_uv.data(), ctx->trim_uv.size() * 4, cudaMemcpyHostToDevice, s),
			        "upload trim uv");
		const size_t nm = (size_t)std::max<int64_t>(P.nmps, 1);
		AQH_TRY(ctx->d_trim_mark.ensure(nm), "alloc trim marks");
		AQH_TRY(cudaMemsetAsync(ctx->d_trim_mark.p, 0, nm, s), "memset");
		const int32_t* b = ctx->d_trim_i.as<int32_t>();
		TrimDev& t = P.g.trim;
		t.nsets = ctx->trim_nsets;
		t.grid_set = b;
		t.loop_first = b + o_lf;
		t.set_first = b + o_sf;
		t.pts = reinterpret_cast<const float2*>(df);
		t.uv = reinterpret_cast<const float2*>(df + npf);
		t.mark = ctx->d_trim_mark.as<uint8_t>();
		launch_trim_mark(P.g, (long long)(ctx->trim_uv.size() / 2), ctx->d_trim_mark.as<uint8_t>(),
		                 ctx->d_trim_cull.as<uint8_t>(), ctx->d_trim_err.as<int32_t>(), s);
		AQH_TRY(cudaGetLastError(), "trim kernel launch");
	}
	if ((ctx->trim_nsets > 0 || ctx->cull_on) && G > 0) {
		int32_t err = 0;
		AQH_TRY(cudaMemcpyAsync(&err, ctx->d_trim_err.p, 4, cudaMemcpyDeviceToHost, s), "readback");
		AQH_TRY(cudaStreamSynchronize(s), "culling");
		if (err)
			return ctx->fail(AQH_EINVAL, "culling: a grid's vertices run past the uv array (trim curves) or the "
			                 "normal arrays (back faces), or back-face culling without Ng");
		P.g.culled = ctx->d_trim_cull.as<uint8_t>();
	}
	if (P.g.naov > 0) {
		AQH_TRY(ctx->d_aovsrc.ensure(nstore * sizeof(int32_t)), "alloc output variable sources");
		AQH_TRY(ctx->d_aovchan.ensure(ndisp * P.g.naov * sizeof(float)), "alloc output variables");
		P.store.aovsrc = ctx->d_aovsrc.as<int32_t>();
	}
	return AQH_OK;
}

static const int kDefaultDisplay[4] = {0, 1, 2, 6};  // r, g, b, a

// The device work of one frame after binning's list capacity is known.
// `batched`: persistent sampling kernel fed from a work queue; no host
// synchronization anywhere, so the sequence can be captured in a CUDA graph.
static aqh_status enqueue_frame(aqh_ctx* ctx, RenderPlan& P, bool batched, bool timing) {
	cudaStream_t s = ctx->stream;
	FrameParams& fp = P.fp;
	// inside a graph capture the stage events must be external record nodes to
	// be usable for timing after the graph runs
	auto mark = [&](cudaEvent_t e) {
		if (batched) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
		else cudaEventRecord(e, s);
	};
	if (timing) mark(ctx->ev[0]);
	if (P.project)
		launch_project_grids(P.g, const_cast<float4*>(P.g.P), const_cast<int32_t*>(P.g.flags), P.cam, s);
	if (P.g.ngrids > 0) {
		launch_id_grid(P.g, P.nmps, const_cast<int32_t*>(P.g.id_grid), s);
		launch_grid_rects(fp, P.g, P.bb, s);
		launch_st_count(fp, P.g, P.bb, s);
		launch_scan_i32(P.bb.st_count, P.bb.st_offset, P.nst * P.bb.nranges, nullptr, s);
		launch_st_write(fp, P.g, P.bb, s);
		if (P.bb.mp_bounds) launch_mb_stage_bounds(fp, P.g, P.bb.mp_bounds, s);
	} else {
		AQH_TRY(cudaMemsetAsync(P.bb.st_offset, 0, sizeof(int32_t) * ((size_t)P.nst * P.bb.nranges + 1), s), "memset");
	}
	if (P.pool.capacity > 0) {
		AQH_TRY(cudaMemsetAsync(P.pool.count, 0, 8, s), "memset");
		AQH_TRY(cudaMemsetAsync(P.pool.overflow, 0, 4, s), "memset");
	}
	if (timing) mark(ctx->ev[1]);
	// host-packed colours arrive on the copy stream (ev_cioi); inside a
	// capture the wait is an external-event node, so every replay waits for
	// the latest upload
	const unsigned wflags = batched ? cudaEventWaitExternal : cudaEventWaitDefault;
	if (P.mbdof) {
		AQH_TRY(cudaStreamWaitEvent(s, ctx->ev_cioi, wflags), "wait for colours");
		launch_sample_mb(fp, P.g, ctx->smp, P.bb, P.store, P.pool, ctx->d_dofb.as<float4>(), ctx->d_slices.as<float>(), s);
	} else if (batched) {
		AQH_TRY(cudaMemsetAsync(ctx->d_queue.p, 0, 4, s), "memset");
		launch_sample_tiles_q(fp, P.g, ctx->smp, P.bb, P.store, P.pool, ctx->d_queue.as<int>(), nullptr, P.nctas, s,
		                      ctx->ev_cioi, wflags);
	} else {
		launch_sample_tiles(fp, P.g, ctx->smp, P.bb, P.store, P.pool, ctx->d_err.as<int32_t>(), s, ctx->ev_cioi, wflags);
	}
	AQH_TRY(cudaGetLastError(), "sample kernel launch");
	if (timing) mark(ctx->ev[2]);
	// the frame's r g b a display is quantized in the filter pass when it fits 8 bits
	const bool fuse_q8 = fp.q_one == 0.0f || (fp.q_min >= 0.0f && fp.q_max <= 255.0f);
	// with an imager the channels stay as FilterBucket leaves them (no
	// exposure, no display) until aqh_apply_imager
	FrameParams ffp = fp;
	if (P.imager) ffp.gain = ffp.gamma = 1.0f;
	launch_filter(ffp, ctx->smp, P.store, ctx->d_ftab.as<float>(), ctx->d_chan.as<float>(),
	              (fuse_q8 && !P.imager) ? ctx->d_q8.as<uint8_t>() : nullptr, s);
	ctx->q8_default = fuse_q8 && !P.imager;
	ctx->imager_pending = P.imager;
	if (P.g.naov > 0) launch_filter_aov(fp, ctx->smp, P.store, P.g, ctx->d_ftab.as<float>(), ctx->d_aovchan.as<float>(), s);
	AQH_TRY(cudaGetLastError(), "filter kernel launch");
	if (timing) mark(ctx->ev[3]);
	return AQH_OK;
}

static void read_stage_times(aqh_ctx* ctx) {
	float a = 0, b = 0, c = 0;
	if (cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]) != cudaSuccess) a = 0;
	if (cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]) != cudaSuccess) b = 0;
	if (cudaEventElapsedTime(&c, ctx->ev[2], ctx->ev[3]) != cudaSuccess) c = 0;
	cudaGetLastError();  // a failed timing query is not an error of the next launch
	ctx->stats.ms_bin = a;
	ctx->stats.ms_sample = b;
	ctx->stats.ms_filter = c;
	ctx->stats.ms_total = a + b + c;
}

// One frame, one launch per stage, with the host reading binning's list size
// and the fragment count back between stages (the plain path).
static aqh_status render_plain(aqh_ctx* ctx, RenderPlan& P, bool sync) {
	cudaStream_t s = ctx->stream;
	const FrameParams& fp = P.fp;
	cudaEventRecord(ctx->ev[0], s);
	int32_t total = 0;
	if (P.project)
		launch_project_grids(P.g, const_cast<float4*>(P.g.P), const_cast<int32_t*>(P.g.flags), P.cam, s);
	if (P.g.ngrids > 0) {
		launch_id_grid(P.g, P.nmps, const_cast<int32_t*>(P.g.id_grid), s);
		launch_grid_rects(fp, P.g, P.bb, s);
		launch_st_count(fp, P.g, P.bb, s);
		launch_scan_i32(P.bb.st_count, P.bb.st_offset, P.nst * P.bb.nranges, nullptr, s);
		AQH_TRY(cudaMemcpyAsync(&total, P.bb.st_offset + (size_t)P.nst * P.bb.nranges, 4, cudaMemcpyDeviceToHost, s),
		        "readback");
		AQH_TRY(cudaStreamSynchronize(s), "bin");
	}
	AQH_TRY(ctx->d_stlist.ensure(sizeof(int32_t) * std::max<int64_t>(total, 1)), "alloc tile lists");
	ctx->st_list_cap = std::max<int64_t>(ctx->st_list_cap, ctx->d_stlist.cap / sizeof(int32_t));
	P.bb.st_list = ctx->d_stlist.as<int32_t>();
	P.bb.list_capacity = ctx->d_stlist.cap / sizeof(int32_t);
	if (P.g.ngrids > 0) launch_st_write(fp, P.g, P.bb, s);
	if (P.g.ngrids > 0 && P.bb.mp_bounds) launch_mb_stage_bounds(fp, P.g, P.bb.mp_bounds, s);
	if (P.g.ngrids <= 0) AQH_TRY(cudaMemsetAsync(P.bb.st_offset, 0, sizeof(int32_t) * ((size_t)P.nst * P.bb.nranges + 1), s), "memset");
	for (int attempt = 0; attempt < 4; ++attempt) {
		if (P.pool.capacity > 0) {
			AQH_TRY(cudaMemsetAsync(P.pool.count, 0, 8, s), "memset");
			AQH_TRY(cudaMemsetAsync(P.pool.overflow, 0, 4, s), "memset");
		}
		if (P.g.csg.nnodes > 0) AQH_TRY(cudaMemsetAsync(P.g.csg.overflow, 0, 4, s), "memset");
		cudaEventRecord(ctx->ev[1], s);
		if (P.mbdof) {
			if (ctx->cioi_pending) AQH_TRY(cudaStreamWaitEvent(s, ctx->ev_cioi, 0), "wait for colours");
			launch_sample_mb(fp, P.g, ctx->smp, P.bb, P.store, P.pool, ctx->d_dofb.as<float4>(), ctx->d_slices.as<float>(), s);
		} else {
			launch_sample_tiles(fp, P.g, ctx->smp, P.bb, P.store, P.pool, ctx->d_err.as<int32_t>(), s,
			                    ctx->cioi_pending ? ctx->ev_cioi : nullptr);
		}
		ctx->cioi_pending = false;
		AQH_TRY(cudaGetLastError(), "sample kernel launch");
		if (P.pool.capacity == 0) break;
		int32_t ovf = 0;
		unsigned long long used = 0;
		AQH_TRY(cudaMemcpyAsync(&ovf, P.pool.overflow, 4, cudaMemcpyDeviceToHost, s), "readback");
		AQH_TRY(cudaMemcpyAsync(&used, P.pool.count, 8, cudaMemcpyDeviceToHost, s), "readback");
		AQH_TRY(cudaStreamSynchronize(s), "sample");
		ctx->stats.fragments = (int64_t)used;
		if (!ovf) break;
		// grow the fragment pool to what this frame needed and sample again
		if (used > (unsigned long long)INT32_MAX)
			return ctx->fail(AQH_ELIMIT,
			                 "the frame needs %llu transparent fragments; the fragment pool indexes at most %d "
			                 "(render it in smaller crop windows)",
			                 used, INT32_MAX);
		ctx->frag_capacity = std::min<int64_t>(INT32_MAX, (int64_t)used + (int64_t)used / 4 + 1024);
		AQH_TRY(ctx->d_frag.ensure(ctx->frag_capacity * sizeof(float4)), "alloc fragments");
		AQH_TRY(ctx->d_next.ensure(ctx->frag_capacity * sizeof(int32_t)), "alloc fragments");
		P.pool.frag = ctx->d_frag.as<float4>();
		P.pool.next = ctx->d_next.as<int32_t>();
		P.pool.capacity = ctx->frag_capacity;
		ctx->graph_valid = false;
	}
	if (P.g.csg.nnodes > 0) {
		int32_t co = 0;
		AQH_TRY(cudaMemcpyAsync(&co, P.g.csg.overflow, 4, cudaMemcpyDeviceToHost, s), "readback");
		AQH_TRY(cudaStreamSynchronize(s), "sample");
		if (co)
			return ctx->fail(AQH_ELIMIT, "CSG: a sample holds more than %d fragments, or a NaN depth, or the tree "
			                 "needed more than 64 resolve rounds", 24);
	}
	cudaEventRecord(ctx->ev[2], s);
	// the frame's r g b a display is quantized in the filter pass when it fits 8 bits
	const bool fuse_q8 = fp.q_one == 0.0f || (fp.q_min >= 0.0f && fp.q_max <= 255.0f);
	// with an imager the channels stay as FilterBucket leaves them (no
	// exposure, no display) until aqh_apply_imager
	FrameParams ffp = fp;
	if (P.imager) ffp.gain = ffp.gamma = 1.0f;
	launch_filter(ffp, ctx->smp, P.store, ctx->d_ftab.as<float>(), ctx->d_chan.as<float>(),
	              (fuse_q8 && !P.imager) ? ctx->d_q8.as<uint8_t>() : nullptr, s);
	ctx->q8_default = fuse_q8 && !P.imager;
	ctx->imager_pending = P.imager;
	if (P.g.naov > 0) launch_filter_aov(fp, ctx->smp, P.store, P.g, ctx->d_ftab.as<float>(), ctx->d_aovchan.as<float>(), s);
	AQH_TRY(cudaGetLastError(), "filter kernel launch");
	cudaEventRecord(ctx->ev[3], s);
	ctx->stats.tile_grid_pairs = total;
	if (sync) {
		AQH_TRY(cudaStreamSynchronize(s), "render");
		read_stage_times(ctx);
	}
	return AQH_OK;
}

// Batched path: the list and fragment capacities come from the previous
// frame (or a bound), overflow is detected on the device, and the whole frame
// is one CUDA graph replayed while its arguments stay the same.
constexpr size_t kMaxGraphs = 16;

static aqh_status render_batched(aqh_ctx* ctx, RenderPlan& P, bool sync) {
	cudaStream_t s = ctx->stream;
	// list room for 16 super-tiles per grid: a frame that needs more is caught
	// on the device and rendered again on the plain path
	const int64_t want = std::max<int64_t>(ctx->st_list_cap, (int64_t)P.g.ngrids * 16 + 4096);
	AQH_TRY(ctx->d_stlist.ensure(sizeof(int32_t) * want), "alloc tile lists");
	ctx->st_list_cap = ctx->d_stlist.cap / sizeof(int32_t);
	P.bb.st_list = ctx->d_stlist.as<int32_t>();
	P.bb.list_capacity = ctx->st_list_cap;
	// graph key: every kernel argument of the frame
	std::vector<unsigned char> key(sizeof(RenderPlan) + sizeof(SamplerDev) + sizeof(void*) * 9);
	unsigned char* k = key.data();
	std::memcpy(k, &P, sizeof(RenderPlan));
	k += sizeof(RenderPlan);
	std::memcpy(k, &ctx->smp, sizeof(SamplerDev));
	k += sizeof(SamplerDev);
	void* ptrs[9] = {ctx->d_ftab.p, ctx->d_chan.p, ctx->d_q8.p, ctx->d_qchan.p, ctx->d_queue.p, ctx->d_dofb.p,
	                 ctx->d_err.p, ctx->d_aovchan.p, (void*)s};
	std::memcpy(k, ptrs, sizeof ptrs);
	if (!ctx->graph_valid) {
		for (auto& ge : ctx->graphs) cudaGraphExecDestroy(ge.exec);
		ctx->graphs.clear();
		ctx->graph_valid = true;
	}
	auto hit = std::find_if(ctx->graphs.begin(), ctx->graphs.end(), [&](const aqh_ctx::GraphEntry& ge) { return ge.key == key; });
	if (hit != ctx->graphs.end()) {
		ctx->graphs.splice(ctx->graphs.begin(), ctx->graphs, hit);
	} else {
		cudaGraph_t graph = nullptr;
		AQH_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
		aqh_status st = enqueue_frame(ctx, P, true, true);
		cudaError_t e = cudaStreamEndCapture(s, &graph);
		if (st != AQH_OK) {
			if (graph) cudaGraphDestroy(graph);
			return st;
		}
		AQH_TRY(e, "end capture");
		cudaGraphExec_t exec = nullptr;
		e = cudaGraphInstantiate(&exec, graph, 0);
		cudaGraphDestroy(graph);
		AQH_TRY(e, "instantiate graph");
		ctx->graphs.push_front(aqh_ctx::GraphEntry{key, exec});
		while (ctx->graphs.size() > kMaxGraphs) {
			cudaGraphExecDestroy(ctx->graphs.back().exec);
			ctx->graphs.pop_back();
		}
		ctx->graphs_built++;
	}
	ctx->cioi_pending = false;  // the graph waits for ev_cioi itself
	AQH_TRY(cudaGraphLaunch(ctx->graphs.front().exec, s), "launch graph");
	ctx->pending_check = true;
	ctx->pending_plan = P;
	if (sync) return aqh_synchronize(ctx);
	return AQH_OK;
}

aqh_status aqh_render(aqh_ctx* ctx, int sync) {
	if (!ctx) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	if (!ctx->samples_set) return ctx->fail(AQH_EINVAL, "aqh_set_samples was not called");
	cudaSetDevice(ctx->device);
	RenderPlan P;
	aqh_status st = plan_render(ctx, P);
	if (st != AQH_OK) return st;
	ctx->stats.micropolygons = P.nmps;
	ctx->stats.samples = (int64_t)P.nsamp;
	ctx->stats.grids = P.g.ngrids;
	// CSG frames take the plain path, which reads the resolve's overflow flag;
	// so do frames with trim curves (their micropolygon marks are per frame)
	if (ctx->mode == AQH_MODE_BATCHED && P.g.csg.nnodes == 0 && P.g.trim.nsets == 0 && !ctx->cull_on)
		return render_batched(ctx, P, sync != 0);
	return render_plain(ctx, P, sync != 0 || P.g.csg.nnodes > 0);
}

aqh_status aqh_synchronize(aqh_ctx* ctx) {
	if (!ctx) return AQH_EINVAL;
	cudaSetDevice(ctx->device);
	AQH_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
	if (ctx->pending_check) {
		// batched frame: did binning or the fragment pool outgrow its capacity?
		ctx->pending_check = false;
		RenderPlan& P = ctx->pending_plan;
		int32_t total = 0;
		if (P.g.ngrids > 0)
			AQH_TRY(cudaMemcpy(&total, P.bb.st_offset + (size_t)P.nst * P.bb.nranges, 4, cudaMemcpyDeviceToHost), "readback");
		int32_t ovf = 0;
		if (P.pool.capacity > 0) {
			unsigned long long used = 0;
			AQH_TRY(cudaMemcpy(&ovf, P.pool.overflow, 4, cudaMemcpyDeviceToHost), "readback");
			AQH_TRY(cudaMemcpy(&used, P.pool.count, 8, cudaMemcpyDeviceToHost), "readback");
			ctx->stats.fragments = (int64_t)used;
		}
		ctx->stats.tile_grid_pairs = total;
		read_stage_times(ctx);
		if (total > ctx->st_list_cap || ovf) {
			// render this frame again on the plain path, which sizes both exactly
			ctx->st_list_cap = std::max<int64_t>(ctx->st_list_cap, total + total / 8 + 1024);
			ctx->graph_valid = false;
			ctx->overflow_rerenders++;
			return render_plain(ctx, P, true);
		}
	}
	return AQH_OK;
}

aqh_status aqh_dspy_geometry_of(aqh_ctx* ctx, aqh_dspy_geometry* g) {
	if (!ctx || !g) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	const FrameParams& fp = ctx->fp;
	g->width = fp.crop_x1 - fp.crop_x0;
	g->height = fp.crop_y1 - fp.crop_y0;
	g->origin_x = fp.crop_x0;
	g->origin_y = fp.crop_y0;
	g->full_width = ctx->desc.width;
	g->full_height = ctx->desc.height;
	g->bucket_x = ctx->desc.bucket_x > 0 ? ctx->desc.bucket_x : 16;
	g->bucket_y = ctx->desc.bucket_y > 0 ? ctx->desc.bucket_y : 16;
	return AQH_OK;
}

aqh_status aqh_set_csg(aqh_ctx* ctx, const int32_t* node_type, const int32_t* node_parent, int nnodes,
                       const int32_t* grid_node, int ngrids) {
	if (!ctx || nnodes < 0 || ngrids < 0 || (nnodes > 0 && (!node_type || !node_parent)) || (ngrids > 0 && !grid_node))
		return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	ctx->csg_n = 0;
	if (nnodes == 0) return AQH_OK;
	std::vector<int32_t> nch(nnodes, 0), child(nnodes, 0);
	for (int i = 0; i < nnodes; ++i) {
		if (node_type[i] < 0 || node_type[i] > 3) return ctx->fail(AQH_EINVAL, "CSG node %d: bad type %d", i, node_type[i]);
		const int p = node_parent[i];
		if (p < -1 || p >= nnodes) return ctx->fail(AQH_EINVAL, "CSG node %d: bad parent %d", i, p);
		if (p >= 0) {
			if (node_type[p] == 0) return ctx->fail(AQH_EINVAL, "CSG node %d: a primitive cannot have children", p);
			child[i] = nch[p]++;
			if (nch[p] > 32) return ctx->fail(AQH_ELIMIT, "CSG node %d: more than 32 children", p);
		}
		// no cycles: the walk up ends within nnodes steps
		int up = p, steps = 0;
		while (up >= 0 && steps <= nnodes) { up = node_parent[up]; ++steps; }
		if (up >= 0) return ctx->fail(AQH_EINVAL, "CSG node %d: its parents form a cycle", i);
	}
	for (int i = 0; i < ngrids; ++i)
		if (grid_node[i] < -1 || grid_node[i] >= nnodes) return ctx->fail(AQH_EINVAL, "grid %d: bad CSG node", i);
	// per node, the non-primitive nodes of its subtree with children first
	// (children in index order, as CqCSGTreeNode::ProcessSampleList recurses)
	std::vector<std::vector<int>> kids(nnodes);
	for (int i = 0; i < nnodes; ++i)
		if (node_parent[i] >= 0) kids[node_parent[i]].push_back(i);
	std::vector<int32_t> pfirst(nnodes), pcount(nnodes), post;
	for (int n = 0; n < nnodes; ++n) {
		pfirst[n] = (int32_t)post.size();
		std::vector<std::pair<int, size_t>> stack{{n, 0}};
		while (!stack.empty()) {
			auto& top = stack.back();
			if (top.second < kids[top.first].size()) {
				const int c = kids[top.first][top.second++];
				if (node_type[c] != 0) stack.push_back({c, 0});
			} else {
				if (node_type[top.first] != 0) post.push_back(top.first);
				stack.pop_back();
			}
		}
		pcount[n] = (int32_t)post.size() - pfirst[n];
	}
	ctx->csg_type.assign(node_type, node_type + nnodes);
	ctx->csg_parent.assign(node_parent, node_parent + nnodes);
	ctx->csg_child = child;
	ctx->csg_nch = nch;
	ctx->csg_pfirst = pfirst;
	ctx->csg_pcount = pcount;
	ctx->csg_post = post;
	ctx->csg_grid_node.assign(grid_node, grid_node + ngrids);
	ctx->csg_n = nnodes;
	return AQH_OK;
}

aqh_status aqh_set_trim(aqh_ctx* ctx, const int32_t* grid_set, int ngrids, const float* uv, size_t nuv,
                        const float* points, int npoints, const int32_t* loop_first, int nloops,
                        const int32_t* set_first, int nsets) {
	if (!ctx || ngrids < 0 || npoints < 0 || nloops < 0 || nsets < 0) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	ctx->trim_nsets = 0;
	if (nsets == 0) return AQH_OK;
	if ((ngrids > 0 && !grid_set) || (nuv > 0 && !uv) || (npoints > 0 && !points) || !loop_first || !set_first)
		return ctx->fail(AQH_EINVAL, "trim curves: missing array");
	if (loop_first[0] < 0 || loop_first[nloops] > npoints)
		return ctx->fail(AQH_EINVAL, "trim curves: loop starts outside the point array");
	for (int l = 0; l < nloops; ++l)
		if (loop_first[l + 1] < loop_first[l]) return ctx->fail(AQH_EINVAL, "trim curves: loop starts decrease");
	if (set_first[0] < 0 || set_first[nsets] > nloops)
		return ctx->fail(AQH_EINVAL, "trim curves: set starts outside the loop array");
	for (int k = 0; k < nsets; ++k)
		if (set_first[k + 1] < set_first[k]) return ctx->fail(AQH_EINVAL, "trim curves: set starts decrease");
	for (int i = 0; i < ngrids; ++i)
		if (grid_set[i] < -1 || grid_set[i] >= nsets) return ctx->fail(AQH_EINVAL, "grid %d: bad trim set %d", i, grid_set[i]);
	ctx->trim_grid_set.assign(grid_set, grid_set + ngrids);
	ctx->trim_uv.assign(uv, uv + 2 * nuv);
	ctx->trim_pts.assign(points, points + 2 * (size_t)npoints);
	ctx->trim_loop_first.assign(loop_first, loop_first + nloops + 1);
	ctx->trim_set_first.assign(set_first, set_first + nsets + 1);
	ctx->trim_nsets = nsets;
	return AQH_OK;
}

aqh_status aqh_set_cull_normals(aqh_ctx* ctx, const float* Ng, const float* N, size_t n) {
	if (!ctx) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	if (!Ng && N) return ctx->fail(AQH_EINVAL, "N without Ng");
	ctx->cull_Ng.assign(Ng ? Ng : nullptr, Ng ? Ng + 3 * n : nullptr);
	ctx->cull_N.assign(N ? N : nullptr, N ? N + 3 * n : nullptr);
	ctx->cull_on = true;
	return AQH_OK;
}

aqh_status aqh_set_host_copy(aqh_ctx* ctx, int mode) {
	if (!ctx) return AQH_EINVAL;
	if (mode != AQH_HOST_COPY_AUTO && mode != AQH_HOST_COPY_ENGINES) return ctx->fail(AQH_EINVAL, "bad host copy mode %d", mode);
	ctx->host_copy = mode;
	return AQH_OK;
}

aqh_status aqh_set_lod_bounds(aqh_ctx* ctx, const float* bounds, int ngrids) {
	if (!ctx || ngrids < 0 || (ngrids > 0 && !bounds)) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	ctx->h_lod.assign(bounds, bounds + (size_t)ngrids * 2);
	ctx->lod_set = ngrids > 0;
	return AQH_OK;
}

aqh_status aqh_set_aov_count(aqh_ctx* ctx, int n) {
	if (!ctx) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	if (n < 0 || n > AQH_MAX_AOV) return ctx->fail(AQH_ELIMIT, "%d output variables; 0..%d supported", n, AQH_MAX_AOV);
	if (!ctx->h_cu.empty() || ctx->host_packed || ctx->dev_grids)
		return ctx->fail(AQH_EINVAL, "the output variable count is set before grids are submitted");
	ctx->naov = n;
	return AQH_OK;
}

aqh_status aqh_submit_aov_host(aqh_ctx* ctx, const float* aov, size_t nvertices) {
	if (!ctx || !aov) return AQH_EINVAL;
	if (ctx->naov == 0) return ctx->fail(AQH_EINVAL, "no output variables set");
	ctx->hp_aov = aov;
	ctx->hp_naov_vertices = nvertices;
	return AQH_OK;
}

aqh_status aqh_submit_aov_device(aqh_ctx* ctx, const float* d_aov) {
	if (!ctx || !d_aov) return AQH_EINVAL;
	if (ctx->naov == 0) return ctx->fail(AQH_EINVAL, "no output variables set");
	ctx->dev_aov = d_aov;
	return AQH_OK;
}

aqh_status aqh_read_aov(aqh_ctx* ctx, float* out, size_t out_floats) {
	if (!ctx || !out) return AQH_EINVAL;
	const FrameParams& fp = ctx->fp;
	const size_t n = (size_t)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0) * ctx->naov;
	if (ctx->naov == 0) return ctx->fail(AQH_EINVAL, "no output variables set");
	if (out_floats < n) return ctx->fail(AQH_EINVAL, "output holds %zu floats, %zu needed", out_floats, n);
	cudaSetDevice(ctx->device);
	AQH_TRY(cudaMemcpyAsync(out, ctx->d_aovchan.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "read aov");
	AQH_TRY(cudaStreamSynchronize(ctx->stream), "read aov");
	return AQH_OK;
}

aqh_status aqh_set_camera_to_raster(aqh_ctx* ctx, const float* m) {
	if (!ctx) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	ctx->camera_set = m != nullptr;
	if (m) std::memcpy(ctx->camera.m, m, sizeof ctx->camera.m);
	return AQH_OK;
}

aqh_status aqh_set_tuning(aqh_ctx* ctx, const aqh_tuning* t) {
	if (!ctx || !t) return AQH_EINVAL;
	if (t->tile_pixels < 0 || t->tile_pixels > 256 || t->supertile_pixels < 0 || t->supertile_pixels > 65536 ||
	    t->persistent_ctas < 0 || t->filter_ctas_per_sm < 0 || t->filter_ctas_per_sm > 8)
		return ctx->fail(AQH_EINVAL, "tuning out of range (tile %d, super-tile %d, ctas %d)", t->tile_pixels,
		                 t->supertile_pixels, t->persistent_ctas);
	ctx->tune = *t;
	ctx->tune.ms = 0.0f;
	return AQH_OK;
}

aqh_status aqh_get_tuning(aqh_ctx* ctx, aqh_tuning* t) {
	if (!ctx || !t) return AQH_EINVAL;
	*t = ctx->tune;
	return AQH_OK;
}

aqh_status aqh_autotune(aqh_ctx* ctx, int repeats, aqh_tuning* best) {
	if (!ctx) return AQH_EINVAL;
	if (!ctx->frame_open) return ctx->fail(AQH_EINVAL, "no frame");
	if (!ctx->samples_set) return ctx->fail(AQH_EINVAL, "aqh_set_samples was not called");
	repeats = std::max(1, std::min(repeats, 64));
	const int t0 = std::min(256, std::max(1, 4096 / std::max(1, ctx->fp.spp)));
	std::vector<int> tiles = {0};
	for (int div : {2, 4})
		if (t0 / div >= 16) tiles.push_back(t0 / div);
	std::vector<int> ctas = {0};
	if (ctx->mode == AQH_MODE_BATCHED) {
		int nsm = 0;
		cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
		const int half = nsm * std::max(1, sample_static_ctas_per_sm(ctx->any_transparent)) / 2;
		if (half >= 1) ctas.push_back(half);
	}
	const aqh_tuning keep = ctx->tune;
	aqh_tuning pick{};
	float pick_ms = 0.0f;
	bool have = false;
	for (int c : ctas)
		for (int tp : tiles)
			for (int stp : {128, 64, 256}) {
				aqh_tuning t{};
				t.tile_pixels = tp;
				t.supertile_pixels = stp == 128 ? 0 : stp;
				t.persistent_ctas = c;
				ctx->tune = t;
				float ms = 0.0f;
				for (int r = 0; r < repeats; ++r) {
					const aqh_status st = aqh_render(ctx, 1);
					if (st != AQH_OK) {
						ctx->tune = keep;
						return st;
					}
					const float m = ctx->stats.ms_total;
					if (r == 0 || m < ms) ms = m;
				}
				if (!have || ms < pick_ms * 0.99f) {
					pick = t;
					pick_ms = ms;
					have = true;
				}
			}
	// the filter's tiles in flight, with the sampling shape chosen above
	// (device time of the filter and quantize stage)
	auto filter_ms = [&](int fc, float& out) -> aqh_status {
		ctx->tune = pick;
		ctx->tune.filter_ctas_per_sm = fc;
		for (int r = 0; r < repeats; ++r) {
			const aqh_status st = aqh_render(ctx, 1);
			if (st != AQH_OK) return st;
			const float m = ctx->stats.ms_filter;
			if (r == 0 || m < out) out = m;
		}
		return AQH_OK;
	};
	float fbest = 0.0f;
	aqh_status fst = filter_ms(0, fbest);
	int fpick = 0;
	for (int fc : {3, 4, 5}) {
		if (fst != AQH_OK) break;
		float m = 0.0f;
		fst = filter_ms(fc, m);
		if (fst == AQH_OK && m < fbest * 0.99f) {
			fbest = m;
			fpick = fc;
		}
	}
	if (fst != AQH_OK) {
		ctx->tune = keep;
		return fst;
	}
	pick.filter_ctas_per_sm = fpick;
	ctx->tune = pick;
	pick.ms = pick_ms;
	if (best) *best = pick;
	return AQH_OK;
}

aqh_status aqh_set_mode(aqh_ctx* ctx, int mode) {
	if (!ctx || (mode != AQH_MODE_PLAIN && mode != AQH_MODE_BATCHED)) return AQH_EINVAL;
	cudaSetDevice(ctx->device);
	AQH_TRY(cudaStreamSynchronize(ctx->stream), "synchronize");
	ctx->mode = mode;
	return AQH_OK;
}

aqh_status aqh_set_imager(aqh_ctx* ctx, int enabled) {
	if (!ctx) return AQH_EINVAL;
	ctx->imager = enabled != 0;
	return AQH_OK;
}

aqh_status aqh_apply_imager(aqh_ctx* ctx, const float* ci_oi, size_t n_floats) {
	if (!ctx || !ci_oi) return AQH_EINVAL;
	if (!ctx->imager_pending) return ctx->fail(AQH_EINVAL, "no frame rendered with an imager is waiting");
	const FrameParams& fp = ctx->fp;
	const size_t n = (size_t)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0) * 6;
	if (n_floats < n) return ctx->fail(AQH_EINVAL, "imager values hold %zu floats, %zu needed", n_floats, n);
	cudaSetDevice(ctx->device);
	AQH_TRY(ctx->d_imager.ensure(n * 4), "alloc imager values");
	AQH_TRY(cudaMemcpyAsync(ctx->d_imager.p, ci_oi, n * 4, cudaMemcpyHostToDevice, ctx->stream), "upload imager");
	const bool fuse_q8 = fp.q_one == 0.0f || (fp.q_min >= 0.0f && fp.q_max <= 255.0f);
	launch_imager(fp, ctx->smp, ctx->d_imager.as<float>(), ctx->d_chan.as<float>(),
	              fuse_q8 ? ctx->d_q8.as<uint8_t>() : nullptr, ctx->stream);
	AQH_TRY(cudaGetLastError(), "imager launch");
	AQH_TRY(cudaStreamSynchronize(ctx->stream), "imager");  // the host array may go away on return
	ctx->q8_default = fuse_q8;
	ctx->imager_pending = false;
	return AQH_OK;
}

aqh_status aqh_read_channels(aqh_ctx* ctx, float* out, size_t out_floats) {
	if (!ctx || !out) return AQH_EINVAL;
	const FrameParams& fp = ctx->fp;
	const size_t n = (size_t)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0) * 9;
	if (out_floats < n) return ctx->fail(AQH_EINVAL, "output holds %zu floats, %zu needed", out_floats, n);
	cudaSetDevice(ctx->device);
	AQH_TRY(cudaMemcpyAsync(out, ctx->d_chan.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "read channels");
	AQH_TRY(cudaStreamSynchronize(ctx->stream), "read channels");
	return AQH_OK;
}

aqh_status aqh_read_bucket(aqh_ctx* ctx, int bx, int by, float* out, size_t out_floats, int* bw, int* bh) {
	if (!ctx || !out) return AQH_EINVAL;
	const FrameParams& fp = ctx->fp;
	const int bsx = ctx->desc.bucket_x > 0 ? ctx->desc.bucket_x : 16;
	const int bsy = ctx->desc.bucket_y > 0 ? ctx->desc.bucket_y : 16;
	const int cw = fp.crop_x1 - fp.crop_x0, ch = fp.crop_y1 - fp.crop_y0;
	const int x0 = bx * bsx, y0 = by * bsy;
	if (bx < 0 || by < 0 || x0 >= cw || y0 >= ch) return ctx->fail(AQH_EINVAL, "bucket (%d,%d) outside the image", bx, by);
	const int w = std::min(bsx, cw - x0), h = std::min(bsy, ch - y0);
	if (out_floats < (size_t)w * h * 9) return ctx->fail(AQH_EINVAL, "bucket buffer too small");
	cudaSetDevice(ctx->device);
	AQH_TRY(cudaMemcpy2DAsync(out, (size_t)w * 9 * 4, ctx->d_chan.as<float>() + ((size_t)y0 * cw + x0) * 9,
	                          (size_t)cw * 9 * 4, (size_t)w * 9 * 4, h, cudaMemcpyDeviceToHost, ctx->stream),
	        "read bucket");
	AQH_TRY(cudaStreamSynchronize(ctx->stream), "read bucket");
	if (bw) *bw = w;
	if (bh) *bh = h;
	return AQH_OK;
}

aqh_status aqh_read_quantized_u8(aqh_ctx* ctx, const int* channels, int nchan, uint8_t* out, size_t out_bytes) {
	if (!ctx || !channels || nchan <= 0 || nchan > 16 || !out) return AQH_EINVAL;
	const FrameParams& fp = ctx->fp;
	if (fp.q_one != 0.0f && (fp.q_min < 0.0f || fp.q_max > 255.0f))
		return ctx->fail(AQH_EINVAL, "quantize range [%g,%g] does not fit 8 bits", fp.q_min, fp.q_max);
	const size_t npix = (size_t)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	if (out_bytes < npix * nchan) return ctx->fail(AQH_EINVAL, "output too small");
	for (int c = 0; c < nchan; ++c)
		if (channels[c] < 0 || channels[c] >= AQH_NCHANNELS) return ctx->fail(AQH_EINVAL, "bad channel %d", channels[c]);
	cudaSetDevice(ctx->device);
	const bool rgba = nchan == 4 && channels[0] == kDefaultDisplay[0] && channels[1] == kDefaultDisplay[1] &&
	                  channels[2] == kDefaultDisplay[2] && channels[3] == kDefaultDisplay[3];
	if (rgba && ctx->q8_default) {
		// quantized by the frame's filter pass already
		AQH_TRY(cudaMemcpyAsync(out, ctx->d_q8.p, npix * 4, cudaMemcpyDeviceToHost, ctx->stream), "read quantized");
		AQH_TRY(cudaStreamSynchronize(ctx->stream), "read quantized");
		return AQH_OK;
	}
	AQH_TRY(ctx->d_qchan.ensure(64), "alloc");
	AQH_TRY(ctx->d_q8_req.ensure(npix * nchan), "alloc");
	AQH_TRY(cudaMemcpyAsync(ctx->d_qchan.p, channels, nchan * 4, cudaMemcpyHostToDevice, ctx->stream), "upload");
	cudaGetLastError();
	launch_quantize_u8(fp, ctx->smp, ctx->d_chan.as<float>(), ctx->d_qchan.as<int>(), nchan,
	                   ctx->d_q8_req.as<uint8_t>(), ctx->stream);
	AQH_TRY(cudaGetLastError(), "quantize launch");
	AQH_TRY(cudaMemcpyAsync(out, ctx->d_q8_req.p, npix * nchan, cudaMemcpyDeviceToHost, ctx->stream), "read quantized");
	AQH_TRY(cudaStreamSynchronize(ctx->stream), "read quantized");
	return AQH_OK;
}

int aqh_display_format(float one, float min, float max) {
	if (one == 0.0f) return AQH_DSPY_FLOAT32;
	if (min >= 0.0f) {
		if (max <= 255.0f) return AQH_DSPY_UNSIGNED8;
		if (max <= 65535.0f) return AQH_DSPY_UNSIGNED16;
		return AQH_DSPY_UNSIGNED32;
	}
	if (min >= -128.0f && max <= 127.0f) return AQH_DSPY_SIGNED8;
	if (min >= -32768.0f && max <= 32767.0f) return AQH_DSPY_SIGNED16;
	return AQH_DSPY_SIGNED32;
}

aqh_status aqh_read_display(aqh_ctx* ctx, const aqh_display* d, void* out, size_t out_bytes, int* format_used) {
	if (!ctx || !d || !out || d->nchan <= 0 || d->nchan > 16) return AQH_EINVAL;
	const FrameParams& fp = ctx->fp;
	for (int c = 0; c < d->nchan; ++c)
		if (d->channels[c] < 0 || d->channels[c] >= AQH_NCHANNELS + ctx->naov)
			return ctx->fail(AQH_EINVAL, "bad channel %d", d->channels[c]);
	const int fmt = d->format ? d->format : aqh_display_format(d->q_one, d->q_min, d->q_max);
	if (fmt < AQH_DSPY_FLOAT32 || fmt > AQH_DSPY_SIGNED8) return ctx->fail(AQH_EINVAL, "bad display format %d", fmt);
	static const size_t kSize[8] = {0, 4, 4, 4, 2, 2, 1, 1};
	const size_t npix = (size_t)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	const size_t bytes = npix * d->nchan * kSize[fmt];
	if (out_bytes < bytes) return ctx->fail(AQH_EINVAL, "output holds %zu bytes, %zu needed", out_bytes, bytes);
	cudaSetDevice(ctx->device);
	cudaStream_t s = ctx->stream;
	AQH_TRY(ctx->d_qchan.ensure(64), "alloc");
	AQH_TRY(ctx->d_disp.ensure(std::max<size_t>(bytes, 16)), "alloc display");
	AQH_TRY(cudaMemcpyAsync(ctx->d_qchan.p, d->channels, d->nchan * 4, cudaMemcpyHostToDevice, s), "upload");
	const float* dither = ctx->smp.dither;
	if (d->dither) {
		AQH_TRY(ctx->d_dither_req.ensure(npix * 4), "alloc dither");
		AQH_TRY(cudaMemcpyAsync(ctx->d_dither_req.p, d->dither, npix * 4, cudaMemcpyHostToDevice, s), "upload dither");
		dither = ctx->d_dither_req.as<float>();
	}
	const QuantizeParams q{d->q_zero, d->q_one, d->q_min, d->q_max, d->q_dither};
	cudaGetLastError();
	launch_display(fp, q, dither, ctx->d_chan.as<float>(), ctx->d_aovchan.as<float>(), ctx->naov,
	               ctx->d_qchan.as<int>(), d->nchan, fmt, ctx->d_disp.p, s);
	AQH_TRY(cudaGetLastError(), "display launch");
	AQH_TRY(cudaMemcpyAsync(out, ctx->d_disp.p, bytes, cudaMemcpyDeviceToHost, s), "read display");
	AQH_TRY(cudaStreamSynchronize(s), "read display");
	if (format_used) *format_used = fmt;
	return AQH_OK;
}

aqh_status aqh_read_samples(aqh_ctx* ctx, int32_t* winner, float* occlz, int32_t* nfrag, uint8_t* valid,
                            float* sdata, size_t nsamples) {
	if (!ctx) return AQH_EINVAL;
	const FrameParams& fp = ctx->fp;
	const size_t n = (size_t)fp.sw * fp.sh * fp.spp;
	if (nsamples < n) return ctx->fail(AQH_EINVAL, "buffers hold %zu samples, %zu needed", nsamples, n);
	if (!ctx->debug_samples && (winner || occlz || nfrag)) return ctx->fail(AQH_EINVAL, "debug sample outputs are off");
	cudaSetDevice(ctx->device);
	cudaStream_t s = ctx->stream;
	if (winner) AQH_TRY(cudaMemcpyAsync(winner, ctx->d_win.p, n * 4, cudaMemcpyDeviceToHost, s), "read");
	if (occlz) AQH_TRY(cudaMemcpyAsync(occlz, ctx->d_oz.p, n * 4, cudaMemcpyDeviceToHost, s), "read");
	if (nfrag) AQH_TRY(cudaMemcpyAsync(nfrag, ctx->d_nf.p, n * 4, cudaMemcpyDeviceToHost, s), "read");
	if (valid || sdata) {
		const size_t ns = store_size((long long)fp.sw * fp.sh, fp.spp);
		std::vector<float4> a(ns), b(ns);
		AQH_TRY(cudaMemcpyAsync(a.data(), ctx->d_sa.p, ns * 16, cudaMemcpyDeviceToHost, s), "read");
		AQH_TRY(cudaMemcpyAsync(b.data(), ctx->d_sb.p, ns * 16, cudaMemcpyDeviceToHost, s), "read");
		AQH_TRY(cudaStreamSynchronize(s), "read");
		// the device store is in 32-pixel blocks (store_index)
		const size_t spp = (size_t)fp.spp;
		for (size_t i = 0; i < n; ++i) {
			const size_t j = (size_t)store_index((long long)(i / spp), (int)(i % spp), (int)spp);
			if (valid) valid[i] = b[j].w != 0.0f ? 1 : 0;
			if (sdata) {
				float* d = sdata + 7 * i;
				d[0] = a[j].x; d[1] = a[j].y; d[2] = a[j].z;
				d[3] = b[j].x; d[4] = b[j].y; d[5] = b[j].z; d[6] = a[j].w;
			}
		}
	}
	AQH_TRY(cudaStreamSynchronize(s), "read");
	return AQH_OK;
}

aqh_status aqh_get_stats(aqh_ctx* ctx, aqh_frame_stats* st) {
	if (!ctx || !st) return AQH_EINVAL;
	*st = ctx->stats;
	st->graphs_built = ctx->graphs_built;
	st->rerenders = ctx->overflow_rerenders;
	return AQH_OK;
}

aqh_status aqh_test_invbilinear(const float* quad8, const float* P, int n, float* uv) {
	if (!quad8 || !P || !uv || n < 0) return AQH_EINVAL;
	float* dq = nullptr;
	float2 *dp = nullptr, *du = nullptr;
	cudaError_t e = cudaMalloc(&dq, 8 * 4);
	if (e == cudaSuccess) e = cudaMalloc(&dp, sizeof(float2) * std::max(n, 1));
	if (e == cudaSuccess) e = cudaMalloc(&du, sizeof(float2) * std::max(n, 1));
	if (e == cudaSuccess) e = cudaMemcpy(dq, quad8, 32, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(dp, P, sizeof(float2) * n, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) {
		launch_test_invbilinear(dq, dp, n, du, 0);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpy(uv, du, sizeof(float2) * n, cudaMemcpyDeviceToHost);
	cudaFree(dq);
	cudaFree(dp);
	cudaFree(du);
	return e == cudaSuccess ? AQH_OK : AQH_EDEVICE;
}

}  // extern "C"
