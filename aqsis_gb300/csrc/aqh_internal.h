// aqh_internal.h -- device-side frame layout shared by the host runtime and
// the CUDA kernels of the hider.  Not part of the public C-ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/aqh.h"

namespace aqh {

// Samples a thread owns.  A pixel with spp samples is split over
// ceil(spp / kSamplesPerThread) threads; per-sample depth and position live in
// that thread's registers while it walks the pixel's candidate micropolygons.
constexpr int kSamplesPerThread = 16;
// Micropolygon records staged in shared memory per sampling pass.
constexpr int kSlots = 256;
constexpr int kSlotWords = kSlots / 32;
constexpr int kMaxKeys = 4;
constexpr int kBlock = 256;
#define AQH_MAX_SPP_DEV 256

// Frame options resolved for the device (SqOptionCache + CqRenderer state).
struct FrameParams {
	int crop_x0, crop_x1, crop_y0, crop_y1;  // display region (crop window)
	int sx0, sy0, sw, sh;                    // sample region = crop grown by the shift
	int xs, ys, spp;                         // PixelSamples
	int tpp;                                 // threads per pixel
	int shiftX, shiftY;                      // lfloor(filterwidth / 2)
	float xfwo2, yfwo2;                      // ceil(filterwidth) * 0.5f
	float cull_x0, cull_x1, cull_y0, cull_y1;  // AddMPG crop cull window (crop -/+ filterwidth / 2)
	int use_dof;
	float dof_mult, dof_inv_fd, dof_scale_x, dof_scale_y;
	float shutter_open, shutter_close;
	int cullable;                            // samples are occlusion cullable (depth filter min/midpoint)
	int depth_filter;
	int midpoint_store;                      // display_z && depth_filter == midpoint
	int frag_only;                           // static frame whose hits all become fragments when no
	                                         // micropolygon occludes (FragPool::occluders == 0) or
	                                         // samples are not cullable: parallel fragment kernel
	float zthr[3];
	float gain, gamma;
	float q_one, q_min, q_max, q_dither;
	// tiling of the sample region
	int tile_w, tile_h, ntx, nty;
	int st_tiles;                            // tiles per super-tile side
	int nstx, nsty;
	int any_motion;
	int max_keys;  // the most motion keys any grid of the frame has (0: not known)
	int use_lod;                             // level-of-detail tests can reject samples (sample detail
	                                         // levels or grid bounds were given)
	int ftab_n;                              // floats in the filter table
	int filter_ctas;                         // filter CTAs per SM (0: by the samples' L2 footprint)
};

// CSG trees (RiSolidBegin / RiSolidEnd) in device memory.  Node types:
// 0 primitive, 1 union, 2 intersection, 3 difference.
struct CsgDev {
	int nnodes;                  // 0: no CSG in the frame
	const int32_t* grid_node;    // per grid: its primitive node, -1 none
	const int32_t* type;         // per node
	const int32_t* parent;       // per node, -1 for a root
	const int32_t* child_index;  // per node: its place among its parent's children
	const int32_t* nchildren;    // per node
	const int32_t* post_first;   // per node: the non-primitive nodes of its subtree, children
	const int32_t* post_count;   //   before parents, at post[post_first .. + post_count)
	const int32_t* post;
	int32_t* overflow;           // set when a sample's CSG list exceeds what Combine holds
};

// Grid stream in device memory (aqh_submit_grids_device layout).
// Trim curves of NURBS grids (CqTrimLoopArray, trimcurve.h:110-160):
// prepared loops as point lists, grouped in sets; each grid names a set or -1.
struct TrimDev {
	int nsets;                  // 0: nothing is trimmed this frame
	const int32_t* grid_set;    // per grid: its set, -1 = not trimmable
	const float2* uv;           // surface (u, v) per vertex, indexed like Ci
	const float2* pts;          // loop points
	const int32_t* loop_first;  // [nloops + 1]
	const int32_t* set_first;   // [nsets + 1]
	const uint8_t* mark;        // per micropolygon: 1 = trimmed (tested at each hit)
};

struct GridsDev {
	int ngrids;
	const int32_t* cu;
	const int32_t* cv;
	const int32_t* nkeys;
	const int32_t* flags;
	const int64_t* pbase;
	const int64_t* cbase;
	const int32_t* tbase;
	const int64_t* mpbase;   // first global micropolygon id of each grid
	const float* times;
	const float4* P;
	const float4* Ci;
	const float4* Oi;
	const uint8_t* culled;   // per global micropolygon id, may be null
	const int32_t* id_grid;  // grid holding micropolygon id k * 256, for each k; may be null
	const float* aov;        // output variables, float[vertex][naov] indexed like Ci; null when naov == 0
	int naov;
	int colour3;             // Ci / Oi hold packed three-float entries (float[3 n]) rather than float4
	const float2* lod;       // LevelOfDetailBounds (min, max) per grid, or null: (0, 1) for every grid
	CsgDev csg;
	TrimDev trim;
};

// Sample pattern caches (aqh_samples) in device memory.
struct SamplerDev {
	int npatterns;
	const float2* pos;
	const float* time;
	const float2* dof;       // raw lens samples in [0,1)^2
	const int32_t* shuffle;
	const float* lod;
	const uint32_t* pos_index;
	const uint32_t* dof_index;
	const uint32_t* time_index;
	const uint32_t* shuffle_index;
	const uint32_t* lod_index;
	const float* dither;
	int pos_unit;  // every position offset is a number in [0, 1] (checked on the host)
};

// Per-sample resolved store (after Combine): R G B depth / OR OG OB flags.
// Sample store layout: sample-region pixels in blocks of 32 consecutive ones,
// each block holding its samples sample-index-major ([block][sample][32]).
// Loads of one sample index over neighbouring pixels coalesce, and all of a
// pixel's samples stay within one block of 512 * spp bytes.
__host__ __device__ inline long long store_index(long long pix, int si, int spp) {
	return ((pix >> 5) * spp + si) * 32 + (pix & 31);
}
__host__ __device__ inline size_t store_size(long long npix, int spp) {
	return (size_t)((npix + 31) >> 5) * 32 * (size_t)spp;
}

// a and b in the store layout above; the debug arrays are pixel-major
// ([pixel][sample index]).
struct SampleStore {
	float4* a;        // r, g, b, depth
	float4* b;        // or, og, ob, valid (1.0f / 0.0f)
	int32_t* winner;  // debug: occluding hit id before Combine (or null)
	float* occlz;     // debug: occlZ (or null)
	int32_t* nfrag;   // debug: transparent fragment count (or null)
	float* hitz;      // depth of the occluding hit when occlZ tracks the second-nearest
	                  // depth (midpoint depth filter with a z display), else null
	uint32_t* wmask;  // per sample (store layout): bit (fy + shiftY) * (2 shiftX + 1) + fx + shiftX set
	                  // when the sample is inside the filter window of the display pixel at
	                  // offset (-fx, -fy); null: the filter tests sample positions itself
	unsigned long long* keys;  // opaque frames: (ordered depth, id + 1) of each sample's occluding
	                           // hit, pixel-major ([pixel][sample index]), resolved by a separate
	                           // kernel; null: the sampler resolves in place
	int32_t* aovsrc;  // micropolygon whose output variables the sample carries after Combine
	                  // (store layout; -1 none), or null without output variables
};

// Transparent fragment pool: {depth, micropolygon id bits, u, v} + next link.
struct FragPool {
	float4* frag;
	int32_t* next;
	unsigned long long* count;
	int64_t capacity;
	int32_t* overflow;
	int32_t* occluders;  // nonzero when some micropolygon may be occluding (opaque or matte alpha)
	int32_t* heads;      // fragment-only frames: each sample's list head, pixel-major ([pixel][sample
	                     // index]), handed to resolve_frag_kernel; null: the sampler resolves in place
};

struct BinBuffers {
	int4* grid_rect;       // pixel rectangle [x0,x1) x [y0,y1) touched by each grid (empty: x0 >= x1)
	float* grid_minz;      // smallest camera z over each grid's vertices (all keys)
	int32_t* st_count;     // [nst][nranges]
	int32_t* st_offset;    // exclusive scan of st_count, plus total at the end
	int32_t* st_list;      // grid ids per super-tile, in grid order
	float4* tri;           // per grid and motion key (kMaxKeys each): the triangle split line
	                       // (A.x, A.y, B.x, B.y) of triangular grids; may be null (no such grids)
	uint32_t* strips;      // per grid 64 words, or null: [0, 32) the pixel range [lo, hi) of each
	                       // micropolygon column, [32, 63) of each row (lo | hi << 16, int16 each);
	                       // word 63 = 1 when present (one motion key, cu and cv at most 31)
	int4* mp_bounds;       // motion frames, per micropolygon: its staging bound (pack_stage_bound), or null
	int nranges;
	int range_size;
	int64_t list_capacity;
};

// Camera-to-raster matrix of the frame in CqMatrix element order m[row*4 + col].
struct CamMatrix {
	float m[16];
};

// Everything one render of a context needs: uploads done, buffers sized, kernel arguments filled.
struct RenderPlan {
	FrameParams fp;
	GridsDev g;
	BinBuffers bb;
	SampleStore store;
	FragPool pool;
	bool mbdof;
	int nst;
	int nctas;     // persistent sampling CTAs (batched form)
	size_t nsamp;
	int64_t nmps;
	bool project;  // AQH_GRID_CAMERA grids to project before binning (with cam)
	CamMatrix cam;
	bool imager;   // stop after FilterBucket: no exposure or 8-bit display until aqh_apply_imager
};

// Kernel launchers (implemented in the .cu files).
void launch_grid_rects(const FrameParams& fp, const GridsDev& g, const BinBuffers& b, cudaStream_t s);
void launch_id_grid(const GridsDev& g, int64_t nmps, int32_t* table, cudaStream_t s);
// Split's camera-to-raster projection of AQH_GRID_CAMERA grids, in place in
// P (the grids' point array, g.P made writable) and clearing the flag.
// Split's trimming of every micropolygon of a trimmable grid: trimmed out
// ones are set in `culled`, ones to test at each hit in `mark`; a grid whose
// vertices run past `nuv` uv entries sets *err and is skipped.
// Shade / Split culling of the flagged grids, before projection: sets
// `culled` per micropolygon; a grid that cannot be culled as asked sets *err.
void launch_cull_grids(const GridsDev& g, const float* Ng, const float* N, long long nng, int zthr_black,
                       uint8_t* culled, int32_t* err, cudaStream_t s);
void launch_trim_mark(const GridsDev& g, long long nuv, uint8_t* mark, uint8_t* culled, int32_t* err, cudaStream_t s);
void launch_project_grids(const GridsDev& g, float4* P, int32_t* flags, const CamMatrix& m, cudaStream_t s);
void launch_st_count(const FrameParams& fp, const GridsDev& g, BinBuffers& b, cudaStream_t s);
void launch_scan_i32(const int32_t* in, int32_t* out, int n, int32_t* scratch, cudaStream_t s);
void launch_st_write(const FrameParams& fp, const GridsDev& g, BinBuffers& b, cudaStream_t s);
// `colours_ready`, when given, is an event the first kernel that reads Ci/Oi
// waits for (on an opaque frame, the resolve after the sampler), with
// cudaStreamWaitEvent flags `wait_flags` (cudaEventWaitExternal in a capture).
// Staging bound of every micropolygon of a motion blur / depth of field frame.
void launch_mb_stage_bounds(const FrameParams& fp, const GridsDev& g, int4* out, cudaStream_t s);
void launch_sample_tiles(const FrameParams& fp, const GridsDev& g, const SamplerDev& sm, const BinBuffers& b,
                         SampleStore st, FragPool pool, int32_t* err, cudaStream_t s,
                         cudaEvent_t colours_ready = nullptr, unsigned wait_flags = 0);
// Persistent form: `nctas` CTAs pull tiles from queue[0] (zeroed by the
// caller), in `order` when given.
void launch_sample_tiles_q(const FrameParams& fp, const GridsDev& g, const SamplerDev& sm, const BinBuffers& b,
                           SampleStore st, FragPool pool, int* queue, const int* order, int nctas, cudaStream_t s,
                           cudaEvent_t colours_ready = nullptr, unsigned wait_flags = 0);
int sample_static_ctas_per_sm(bool transp);
// Kernel attributes (dynamic shared memory above 48 KB) apply to the current
// device's context: both set them once per device.
void configure_sample_kernels();
void configure_sample_mb_kernels();
// True the first time it is called for the current device with this `mask`
// (one static bitmask per caller); false afterwards or without a device.
bool first_use_on_device(std::mutex& mu, uint64_t& mask);
// `slice_times`: for every slice count d in 1..max(4, spp), the d accumulated
// slice end times of CqMicroPolygonMotion::BuildBoundList, at offset d*(d-1)/2.
void launch_sample_mb(const FrameParams& fp, const GridsDev& g, const SamplerDev& sm, const BinBuffers& b,
                      SampleStore st, FragPool pool, const float4* dof_bounds, const float* slice_times,
                      cudaStream_t s);
void slice_times_h(float open, float close, int spp, std::vector<float>& out);
// Largest sampling tile (pixels) of opaque motion blur / depth of field frames.
int sample_mb_opaque_tile_pixels(int spp);
void static_tiling(FrameParams& fp, int tile_pixels);
// Frame options resolved from an aqh_frame_desc (plus the host filter table).
aqh_status resolve_frame(const aqh_frame_desc& d, FrameParams& fp, std::vector<float>& ftab, std::string& err);
// Tile grid, super-tiles and the MB/DoF lens-stratum bounds (api.cu).
// tile_pixels: pixels per sampling tile (0: the most a CTA holds, min(256,
// 4096 / samples per pixel)); supertile_px: side of a binning super-tile
// (0: 128 pixels).  Neither changes any result.
void set_tiling(FrameParams& fp, int tile_pixels = 0, int supertile_px = 0);
void dof_bounds_h(int xs, int ys, std::vector<float4>& out);
// `q8` (may be null): the frame's r g b a display quantized to 8 bits,
// written in the same pass (the quantize of quantize_u8 with channels 0 1 2 6).
void launch_filter(const FrameParams& fp, const SamplerDev& sm, const SampleStore& st, const float* ftab,
                   float* channels, uint8_t* q8, cudaStream_t s);
// The imager's Ci and Oi (float[pixel][6]) into the channels, alpha from
// that opacity, then exposure and (q8 non-null) the 8-bit r g b a display.
void launch_imager(const FrameParams& fp, const SamplerDev& sm, const float* ci_oi, float* channels, uint8_t* q8,
                   cudaStream_t s);
// Output variables of the crop window, float[pixel][g.naov], filtered like Ci.
void launch_filter_aov(const FrameParams& fp, const SamplerDev& sm, const SampleStore& st, const GridsDev& g,
                       const float* ftab, float* aov_channels, cudaStream_t s);
void launch_quantize_u8(const FrameParams& fp, const SamplerDev& sm, const float* channels, const int* chans,
                        int nchan, uint8_t* out, cudaStream_t s);
// Quantize settings of one display request (CqDisplayRequest, ddmanager.cpp:428-457).
struct QuantizeParams {
	float zero, one, min, max, dither;
};
void launch_display(const FrameParams& fp, const QuantizeParams& q, const float* dither, const float* channels,
                    const float* aov_channels, int naov, const int* chans, int nchan, int format, void* out,
                    cudaStream_t s);
void launch_test_invbilinear(const float* quad8, const float2* P, int n, float2* uv, cudaStream_t s);

}  // namespace aqh
