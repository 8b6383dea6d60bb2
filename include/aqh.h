/*
 * aqh.h -- C-ABI of the GB300-native REYES hider ("aqh").
 *
 * This is the drop-in boundary for the aqsis hider path: the part of
 * aqsis libs/core that runs after shading (bin micropolygons into buckets,
 * sample them with depth/opacity compositing into the pixel sample store,
 * reconstruct pixels with the pixel filter, expose and quantize).  The
 * reference's RI front end, CPU dicer and shading VM keep producing shaded
 * grids; its CqImageBuffer hands them to this library instead of splitting
 * them into CqMicroPolygon objects, and its display manager reads finished
 * buckets back through an IqChannelBuffer view of aqh_read_bucket().
 *
 * Plain C types only; no exceptions cross this boundary.  Every call returns
 * an aqh_status; aqh_last_error() gives the message of the last failure on
 * a context.  One host thread per context.
 *
 * Insertion order: micropolygons are ordered by grid submission order, then
 * by row (iv), then column (iu), exactly the order in which
 * CqMicroPolyGrid::Split feeds CqImageBuffer::AddMPG
 * (libs/core/micropolygon.cpp:770-880).  Opaque sample ties are resolved by
 * that order, as in the reference.
 */
#ifndef AQH_H
#define AQH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AQH_VERSION_MAJOR 0
#define AQH_VERSION_MINOR 1

typedef enum {
	AQH_OK = 0,
	AQH_EINVAL = 1,      /* bad argument or state */
	AQH_ENOMEM = 2,      /* device or host allocation failed */
	AQH_EDEVICE = 3,     /* CUDA error */
	AQH_ETIMEDOUT = 4,   /* a bounded device wait ran out */
	AQH_EREJECTED = 5,   /* admission refused (serving) */
	AQH_ENOTREADY = 6,   /* job still running (serving) */
	AQH_ELIMIT = 7       /* a documented size limit was exceeded */
} aqh_status;

/* RiPixelFilter filter functions (libs/core/filters.cpp). */
typedef enum {
	AQH_FILTER_BOX = 0,
	AQH_FILTER_TRIANGLE = 1,
	AQH_FILTER_GAUSSIAN = 2,
	AQH_FILTER_CATMULLROM = 3,
	AQH_FILTER_SINC = 4,
	AQH_FILTER_DISK = 5,
	AQH_FILTER_BESSEL = 6,
	AQH_FILTER_MITCHELL = 7
} aqh_filter;

/* Hider "depthfilter" (libs/core/optioncache.h:34). */
typedef enum { AQH_DEPTH_MIN = 0, AQH_DEPTH_MIDPOINT = 1, AQH_DEPTH_MAX = 2, AQH_DEPTH_AVERAGE = 3 } aqh_depth_filter;

/* Per-grid flags (SqGridInfo, libs/core/micropolygon.h:57-63). */
enum {
	AQH_GRID_SMOOTH = 1,      /* ShadingInterpolation "smooth": bilinear Ci/Oi across the micropolygon */
	AQH_GRID_MATTE = 2,       /* Matte 1 (SqImageSample::Flag_Matte) */
	AQH_GRID_MATTEALPHA = 4,  /* aqsis "matte alpha" (Flag_MatteAlpha) */
	AQH_GRID_OPAQUE = 8,      /* caller guarantees Oi >= 1 on every vertex (skips reading Oi while sampling) */
	AQH_GRID_TRIANGULAR = 16, /* CqMicroPolyGridBase::fTriangular (micropolygon.h:139-147): hits on or behind
	                             the line through corners cu and cv*(cu+1) miss (micropolygon.cpp:1630-1654) */
	AQH_GRID_CAMERA = 32,     /* P holds camera-space points: projected on the device with the frame's
	                             camera-to-raster matrix (aqh_set_camera_to_raster) */
	AQH_GRID_TRIM_OUTSIDE = 64, /* "trimcurve" "sense" "outside" (micropolygon.cpp:754-759) */
	AQH_GRID_CULL_BACKFACING = 128, /* Sides 1, outside any solid, "cull" "backfacing" 1: back-facing
	                                   micropolygons are culled (camera-space grids, aqh_set_cull_normals) */
	AQH_GRID_CULL_TRANSPARENT = 256 /* the surface shader uses Oi: a static grid's trailing run of vertices
	                                   with black Oi is culled (micropolygon.cpp:486-506) */
};

typedef struct aqh_ctx aqh_ctx;

typedef struct {
	int device;                 /* CUDA device ordinal */
	size_t vertex_capacity;     /* initial device capacity in vertices (0 = grow on demand) */
	size_t grid_capacity;       /* initial device capacity in grids (0 = grow on demand) */
} aqh_device_opts;

/*
 * Frame options.  Replaces the hider's reads of SqOptionCache::cacheOptions
 * (libs/core/optioncache.cpp:48-118) and CqRenderer state set by the RI
 * option calls RiFormat / RiCropWindow / RiPixelSamples (api/ri.cpp:852-858) /
 * RiPixelFilter (:862-867) / RiExposure (:873-877) / RiQuantize (:902-930) /
 * RiShutter (:832-836) / RiDepthOfField (:821-826) / RiHider (:1014-1038) and
 * Option "limits" "bucketsize" / "zthreshold".
 */
typedef struct {
	int width, height;                 /* Format */
	int crop_xmin, crop_xmax;          /* raster crop window in pixels (CqRenderer::initialiseCropWindow); */
	int crop_ymin, crop_ymax;          /*   all zero = whole image */
	int bucket_x, bucket_y;            /* Option "limits" "bucketsize" (0 = 16) */
	int xsamples, ysamples;            /* PixelSamples */
	float xfilter, yfilter;            /* PixelFilter widths */
	int filter;                        /* aqh_filter */
	float gain, gamma;                 /* Exposure */
	float q_one, q_min, q_max, q_dither; /* Quantize "rgba" one min max dither */
	float shutter_open, shutter_close; /* Shutter */
	float fstop, focal_length, focal_distance; /* DepthOfField (fstop >= FLT_MAX or 0 = off) */
	float dof_scale_x, dof_scale_y;    /* raster size of a unit camera-space vector at z=-1 (options.cpp:162-171) */
	int depth_filter;                  /* aqh_depth_filter */
	float zthreshold[3];               /* Option "limits" "zthreshold" (default 1 1 1) */
	int display_z;                     /* nonzero when a display asks for z (DMode_Z) */
} aqh_frame_desc;

/* Fill `d` with the reference defaults (libs/core/options.cpp:273-310):
 * 640x480, PixelSamples 2 2, gaussian 2x2, Exposure 1 1, Quantize 255 0 255 0.5. */
void aqh_frame_desc_defaults(aqh_frame_desc* d);

/*
 * One shaded grid.  Replaces the per-micropolygon CqImageBuffer::AddMPG()
 * calls made by CqMicroPolyGrid::Split / CqMotionMicroPolyGrid::Split
 * (libs/core/micropolygon.cpp:641-892, 946-1156; imagebuffer.cpp:514-591).
 * P is in the hybrid raster space Split produces (raster x, raster y,
 * camera-space z), or in camera space with AQH_GRID_CAMERA.  The library
 * copies the arrays before returning.
 */
typedef struct {
	int cu, cv;                  /* micropolygons along u and v; (cu+1)*(cv+1) vertices */
	int nkeys;                   /* motion keys (1 = static, at most AQH_MAX_KEYS) */
	const float* key_times;      /* nkeys shutter times, ascending (NULL when nkeys == 1) */
	const float* P;              /* float4[nkeys][(cu+1)*(cv+1)]: x, y, z, unused */
	const float* Ci;             /* float4[(cu+1)*(cv+1)]: r, g, b, unused; NULL = white */
	const float* Oi;             /* float4[(cu+1)*(cv+1)]: r, g, b, unused; NULL = opaque */
	const uint8_t* culled;       /* cu*cv bytes, nonzero = culled micropolygon (m_CulledPolys); may be NULL */
	int flags;                   /* AQH_GRID_* */
	const float* aov;            /* float[(cu+1)*(cv+1)][n] output variables when aqh_set_aov_count(n > 0);
	                                NULL = zeros */
} aqh_grid;

#define AQH_MAX_KEYS 4
#define AQH_MAX_SPP 256

/*
 * Sample patterns.  Mirrors IqSampler (libs/core/isampler.h:42-78) and
 * CqImagePixel::setSamples (imagepixel.cpp:334-359): each pixel picks a
 * position pattern, a lens pattern, a time pattern and a lens-shuffle table
 * out of pattern caches.  Explicit per-pixel samples are the special case of
 * one pattern per pixel with NULL index arrays.
 *
 * The sample region is the crop window grown by floor(filterwidth/2) pixels
 * on every side (bucketprocessor.cpp:112-125); pixel indices are row-major
 * over that region.
 */
typedef struct {
	int npatterns;                /* patterns in each table */
	const float* pos;             /* float2[npatterns][spp]: offsets inside the pixel (added to x, y) */
	const float* time;            /* float[npatterns][spp] in [0,1): scaled to the shutter; NULL = 0 */
	const float* dof;             /* float2[npatterns][spp]: lens positions in [0,1)^2 (projected to the
	                                 unit disc by the library); NULL = no lens offsets */
	const int32_t* shuffle;       /* int[npatterns][spp] lens-shuffle tables; NULL = identity */
	const float* lod;             /* float[npatterns][spp] detail levels; NULL = 0 */
	/* per-pixel pattern choices over the sample region; NULL = pattern index == pixel index */
	const uint32_t* pos_index;
	const uint32_t* dof_index;
	const uint32_t* time_index;
	const uint32_t* shuffle_index;
	const uint32_t* lod_index;
	/* per display pixel (crop window, row-major) dither value s in [0,1); NULL = 0 */
	const float* dither;
} aqh_samples;

/* ---- context ------------------------------------------------------------ */
aqh_status aqh_create(const aqh_device_opts* opts, aqh_ctx** out);
void aqh_destroy(aqh_ctx* ctx);
const char* aqh_last_error(const aqh_ctx* ctx);
const char* aqh_status_string(aqh_status s);

/* ---- frame (RiWorldBegin ... RiWorldEnd) --------------------------------- */
/* Validate options and reset the frame's grid stream.  RiWorldBegin's
 * CqImageBuffer::SetImage (imagebuffer.cpp:174-228). */
aqh_status aqh_frame_begin(aqh_ctx* ctx, const aqh_frame_desc* desc);
/* Upload sample patterns; required before aqh_render.  Copies the arrays. */
aqh_status aqh_set_samples(aqh_ctx* ctx, const aqh_samples* samples);
/* The projection step of CqMicroPolyGrid::Split / CqMotionMicroPolyGrid::Split
 * (micropolygon.cpp:649-651, 735-745, 1023-1032) on the device.  Grids flagged
 * AQH_GRID_CAMERA carry camera-space P for every key; before binning each
 * point becomes matCameraToRaster * P (CqMatrix::operator*(CqVector3D),
 * matrix.h:717-750: x and y divided by h when h != 1) with its camera-space z
 * kept.  `m` is the matrix in CqMatrix element order m[row*4 + col], points
 * as row vectors (x' = x m[0] + y m[4] + z m[8] + m[12], h = x m[3] + y m[7] +
 * z m[11] + m[15]); NULL clears it.  Reset by aqh_frame_begin.  Host grids
 * flagged AQH_GRID_CAMERA without a matrix are rejected at aqh_render.
 * Device-submitted grids are projected in place, as Split overwrites the
 * grid's P, and their AQH_GRID_CAMERA flag is cleared in d_flags (without a
 * matrix they are taken as already projected). */
aqh_status aqh_set_camera_to_raster(aqh_ctx* ctx, const float* m);
/* Append one grid (host arrays) in insertion order: CqImageBuffer::AddMPG. */
aqh_status aqh_submit_grid(aqh_ctx* ctx, const aqh_grid* grid);
/* Append many grids whose arrays already live in device memory, packed:
 *   cu, cv, nkeys, flags: per grid;  vbase: first vertex of each grid in P/Ci/Oi
 *   (key k of grid g starts at vbase[g] + k*(cu+1)*(cv+1) in P; Ci/Oi are indexed
 *   by cbase[g]); times: key times at tbase[g].  All pointers are device pointers
 *   that must stay valid until aqh_render returns.  Used by callers that dice
 *   and shade on the device or that keep a scene resident between frames. */
aqh_status aqh_submit_grids_device(aqh_ctx* ctx, int ngrids,
                                   const int32_t* d_cu, const int32_t* d_cv, const int32_t* d_nkeys,
                                   const int32_t* d_flags, const int64_t* d_pbase, const int64_t* d_cbase,
                                   const int32_t* d_tbase, const float* d_times,
                                   const float* d_P, const float* d_Ci, const float* d_Oi,
                                   const uint8_t* d_culled, int64_t total_micropolygons);
/* Append many grids from packed HOST arrays (same layout as
 * aqh_submit_grids_device).  Nothing is copied until aqh_render, which
 * uploads them in one transfer per array; the arrays must stay valid until
 * then.  Page-locked memory (aqh_host_alloc) transfers fastest. */
aqh_status aqh_submit_grids_host(aqh_ctx* ctx, int ngrids,
                                 const int32_t* cu, const int32_t* cv, const int32_t* nkeys,
                                 const int32_t* flags, const int64_t* pbase, const int64_t* cbase,
                                 const int32_t* tbase, const float* times, size_t ntimes,
                                 const float* P, size_t nP, const float* Ci, const float* Oi, size_t nC,
                                 const uint8_t* culled, int64_t total_micropolygons);
/* The same with P, Ci and Oi as packed three-float entries -- the memory
 * layout of the reference's CqVector3D / CqColor grid arrays -- so they go
 * up 25% smaller and are widened to float4 on the device; nP and nC count
 * entries.  The fourth P component is 0. */
aqh_status aqh_submit_grids_host3(aqh_ctx* ctx, int ngrids,
                                  const int32_t* cu, const int32_t* cv, const int32_t* nkeys,
                                  const int32_t* flags, const int64_t* pbase, const int64_t* cbase,
                                  const int32_t* tbase, const float* times, size_t ntimes,
                                  const float* P, size_t nP, const float* Ci, const float* Oi, size_t nC,
                                  const uint8_t* culled, int64_t total_micropolygons);
/* How aqh_render moves three-float P from page-locked host memory:
 * AQH_HOST_COPY_AUTO (default) widens it with a kernel that reads the host
 * array directly (fastest for one frame at a time); AQH_HOST_COPY_ENGINES
 * copies it with the copy engines and widens it on the device, so the
 * transfer overlaps another context's frame in flight. */
enum { AQH_HOST_COPY_AUTO = 0, AQH_HOST_COPY_ENGINES = 1 };
aqh_status aqh_set_host_copy(aqh_ctx* ctx, int mode);
/* Page-locked host memory for grid arrays. */
void* aqh_host_alloc(size_t bytes);
void aqh_host_free(void* p);
/* Issue the context's work on a caller-owned CUDA stream (cudaStream_t passed
 * as void*; NULL restores the context's own stream). */
aqh_status aqh_set_stream(aqh_ctx* ctx, void* stream);
/* Run the hider over every submitted grid: CqImageBuffer::RenderImage
 * (imagebuffer.cpp:605-772) with the per-bucket preProcess/process/postProcess
 * (bucketprocessor.cpp:95-359) done on the device.  Asynchronous on the
 * context's stream unless `sync` is nonzero. */
aqh_status aqh_render(aqh_ctx* ctx, int sync);
/* Execution form of aqh_render.  PLAIN: one launch per stage, the host reads
 * binning's list size and the fragment count back between stages.  BATCHED:
 * a persistent sampling kernel pulls tiles from a device work queue, nothing
 * synchronizes with the host inside a frame, and the frame's whole
 * bin -> sample -> filter -> quantize sequence is one CUDA graph, captured on
 * the first render and replayed while the frame's arguments are unchanged;
 * capacities come from the previous frame and an overflow found at
 * aqh_synchronize re-renders that frame on the plain path.  Same pixels. */
enum { AQH_MODE_PLAIN = 0, AQH_MODE_BATCHED = 1 };
aqh_status aqh_set_mode(aqh_ctx* ctx, int mode);
aqh_status aqh_synchronize(aqh_ctx* ctx);

/* ---- launch-shape tuning ---------------------------------------------------- */
/* The device counterpart of the reference's bucket size (CqImageBuffer's
 * bucket loop, imagebuffer.cpp): how the sample region is cut for the
 * sampling kernels.  tile_pixels: pixels per sampling tile (0: the most one
 * CTA holds, min(256, 4096 / samples per pixel); tiles stay within 16x16
 * pixels).  supertile_pixels: side of a binning super-tile in pixels (0: 128).
 * persistent_ctas: CTAs of the batched form's persistent sampling kernel (0:
 * every CTA that fits on the device at once).  filter_ctas_per_sm: 16x16
 * display tiles the filter keeps in flight per SM (0: as many as fit, else
 * 1..8).  No setting changes a result:
 * each sample meets its candidate micropolygons in the same order under any
 * tiling.  `ms` is only written by aqh_autotune. */
typedef struct {
	int tile_pixels;
	int supertile_pixels;
	int persistent_ctas;
	int filter_ctas_per_sm;  /* filter tiles in flight per SM (0: as many as fit) */
	float ms;  /* device time of the frame with this tuning (sum of the stage times) */
} aqh_tuning;
aqh_status aqh_set_tuning(aqh_ctx* ctx, const aqh_tuning* t);
aqh_status aqh_get_tuning(aqh_ctx* ctx, aqh_tuning* t);
/* Render the open frame `repeats` times under each candidate tuning (tile
 * sizes of 1, 1/2 and 1/4 of the default, super-tiles of 64, 128 and 256
 * pixels, and in the batched form half the persistent CTAs), in the context's
 * current mode, and keep the one with the least device time, best of its
 * repeats; the default is kept unless another is at least 1% faster.  The
 * choice stays set for later frames and is written to `best` (may be NULL).
 * The open frame's results are those of its last render, which are the same
 * under every candidate. */
aqh_status aqh_autotune(aqh_ctx* ctx, int repeats, aqh_tuning* best);

/* ---- results ------------------------------------------------------------- */
/* Channel-buffer layout of one display pixel, CqBucketProcessor::FilterBucket
 * (bucketprocessor.cpp:385-398): Ci r g b, Oi r g b, a, z, coverage. */
#define AQH_NCHANNELS 9
/* Copy the whole crop window's channel buffer (float[h][w][9]) to host memory. */
aqh_status aqh_read_channels(aqh_ctx* ctx, float* out, size_t out_floats);
/* One bucket as CqDDManager::DisplayBucket receives it (iddmanager.h:99):
 * float[bh][bw][9] for bucket (bx, by) of the crop window, bucket size from
 * the frame.  Returns the bucket's width and height. */
aqh_status aqh_read_bucket(aqh_ctx* ctx, int bx, int by, float* out, size_t out_floats, int* bw, int* bh);
/* Quantized display data, CqDisplayRequest::FormatBucketForDisplay
 * (ddmanager.cpp:1022-1119): for each pixel of the crop window and each of
 * `nchan` channel-buffer indices in `channels` (e.g. {6,0,1,2} for the
 * reference's a,r,g,b), lround(v*one + dither*s) clamped to [min,max], stored
 * as uint8 when the range fits (selectDataFormat, ddmanager.cpp:249-285). */
aqh_status aqh_read_quantized_u8(aqh_ctx* ctx, const int* channels, int nchan, uint8_t* out, size_t out_bytes);

/* Display element types: the PkDspy* codes of ndspy.h:70-76, so a Dspy
 * driver receives them unchanged. */
enum {
	AQH_DSPY_FLOAT32 = 1, AQH_DSPY_UNSIGNED32 = 2, AQH_DSPY_SIGNED32 = 3, AQH_DSPY_UNSIGNED16 = 4,
	AQH_DSPY_SIGNED16 = 5, AQH_DSPY_UNSIGNED8 = 6, AQH_DSPY_SIGNED8 = 7
};
/* selectDataFormat (ddmanager.cpp:249-285): float32 when one == 0, else the
 * narrowest unsigned (min >= 0) or signed type holding [min, max]. */
int aqh_display_format(float one, float min, float max);
/* One display request (CqDisplayRequest) with its own channels and quantize
 * settings -- an rgba display and a z display of the same frame are two. */
typedef struct {
	int nchan;                   /* channels per pixel, at most 16 */
	int channels[16];            /* channel-buffer indices in display order, e.g. {6,0,1,2} = a,r,g,b */
	float q_zero, q_one, q_min, q_max, q_dither;  /* the request's quantize; q_one == 0: unquantized */
	int format;                  /* AQH_DSPY_*; 0 = aqh_display_format(q_one, q_min, q_max) */
	const float* dither;         /* per display pixel random s in [0,1) (crop window, row-major);
	                                NULL = the frame's aqh_samples dither (or 0) */
} aqh_display;
/* FormatBucketForDisplay (ddmanager.cpp:1022-1119) over the whole crop window
 * on the device: value = lround(zero + v*(one-zero) + dither*s) in double,
 * clamped to [min, max] (unsigned/signed 32-bit also to the type's range),
 * then converted to the element type; with q_one == 0 the channel value as
 * is.  `out` gets width x height x nchan elements, row-major; `format_used`
 * (may be NULL) the element type written. */
aqh_status aqh_read_display(aqh_ctx* ctx, const aqh_display* d, void* out, size_t out_bytes, int* format_used);
/* Per-sample results for parity checks, over the sample region (pixel-major,
 * sample-minor): occluding-hit micropolygon id before Combine (-1 none), occlZ,
 * transparent fragment count, valid flag after Combine, and the combined
 * 7-float sample (R G B OR OG OB depth).  Any pointer may be NULL. */
aqh_status aqh_read_samples(aqh_ctx* ctx, int32_t* winner, float* occlz, int32_t* nfrag,
                            uint8_t* valid, float* sdata, size_t nsamples);

/* ---- level of detail ------------------------------------------------------------ */
/* LevelOfDetailBounds per grid (RiDetailRange; attribute default 0 1,
 * attributes.cpp:127): float[ngrids][2] (min, max) in submission order,
 * copied; grids beyond `ngrids` keep 0 1.  A grid whose min is >= 0 is not
 * sampled by samples whose detail level (aqh_samples.lod, 0 when NULL) lies
 * outside [min, max) (RenderMPG_Static / _MBOrDof, bucketprocessor.cpp:
 * 1182-1190, 1404-1412, 1439-1447).  Reset by aqh_frame_begin. */
aqh_status aqh_set_lod_bounds(aqh_ctx* ctx, const float* bounds, int ngrids);

/* ---- constructive solid geometry ------------------------------------------------- */
/* The frame's CSG trees (RiSolidBegin / RiSolidEnd; CqCSGTreeNode,
 * libs/core/csgtree.h:64-260) and each grid's primitive node.  node_type[n]
 * is AQH_CSG_*; node_parent[n] is its parent node or -1 for a root; the
 * children of a node are the nodes naming it as parent, in index order (at
 * most 32).  grid_node[i] is the primitive node of grid i in submission order,
 * -1 for a grid outside any solid; grids beyond `ngrids` are outside.  At each
 * sample the depth-sorted hit list passes through the tree of every solid it
 * holds (CqImagePixel::Combine, imagepixel.cpp:166-188; ProcessSampleList /
 * EvaluateState, csgtree.cpp:166-350): a hit survives where it changes its
 * tree's inside/outside state; a list left empty leaves the sample unwritten.
 * CSG grids are never depth-culled.  A sample with a CSG hit and more than 24
 * hits, or a NaN depth, fails the render with AQH_ELIMIT.  nnodes = 0 clears
 * the trees.  Reset by aqh_frame_begin. */
enum { AQH_CSG_PRIMITIVE = 0, AQH_CSG_UNION = 1, AQH_CSG_INTERSECTION = 2, AQH_CSG_DIFFERENCE = 3 };
aqh_status aqh_set_csg(aqh_ctx* ctx, const int32_t* node_type, const int32_t* node_parent, int nnodes,
                       const int32_t* grid_node, int ngrids);

/* ---- culling ------------------------------------------------------------------------ */
/* The culling of CqMicroPolyGrid::Shade and CqMotionMicroPolyGrid::Split done
 * on the device before projection (micropolygon.cpp:431-506, 957-1020,
 * 1075-1080), for grids flagged AQH_GRID_CULL_*: Ng (and N, which may be
 * NULL) are camera-space float[n][3] indexed like P, every key.  A static
 * grid culls the micropolygons whose first vertex faces away (P . Ng >= 0,
 * Ng flipped to N's side) and, with AQH_GRID_CULL_TRANSPARENT unless
 * zthreshold is black, those whose first vertex lies in the trailing run of
 * vertices with black Oi; a moving grid culls a micropolygon whose first
 * vertex faces away at every key.  Calling this turns the culling on for the
 * frame (Ng may be NULL when no grid asks for back faces); the arrays are
 * copied.  The back-face test applies to AQH_GRID_CAMERA grids only (P still
 * in camera space; a device-resident grid is projected in place by its first
 * frame).  A flagged camera grid whose P entries run past `n`, or with no
 * Ng, fails aqh_render with AQH_EINVAL.  Reset by aqh_frame_begin. */
aqh_status aqh_set_cull_normals(aqh_ctx* ctx, const float* Ng, const float* N, size_t n);

/* ---- trim curves ----------------------------------------------------------------- */
/* Trim curves of NURBS grids (CqTrimLoopArray, trimcurve.h:110-160).  A set
 * is a list of loops, a loop a closed polyline of prepared curve points
 * (CqTrimLoop::Prepare's m_aCurvePoints, trimcurve.cpp:110-133):
 * points float[npoints][2]; loop l runs over points [loop_first[l],
 * loop_first[l+1]); set k over loops [set_first[k], set_first[k+1]).
 * grid_set[i] is the set of grid i in submission order, -1 for a grid that
 * cannot be trimmed (grids beyond `ngrids` cannot); uv float[nuv][2] holds
 * the surface (u, v) of every vertex, indexed like Ci.  As Split does
 * (micropolygon.cpp:754-835, 1056-1130), a micropolygon whose four corners
 * are all trimmed (in the grid's sense, AQH_GRID_TRIM_OUTSIDE inverting) and
 * whose edges cross no loop is dropped, one with any corner trimmed is
 * tested at each static hit (micropolygon.cpp:1592-1627: the "inside" sense
 * rejects a hit whose bilinear (u, v) is trimmed; moving micropolygons take
 * no test).  The arrays are copied; nsets = 0 turns trimming off.  A grid
 * whose vertices run past `nuv` fails aqh_render with AQH_EINVAL.  Reset by
 * aqh_frame_begin. */
aqh_status aqh_set_trim(aqh_ctx* ctx, const int32_t* grid_set, int ngrids, const float* uv, size_t nuv,
                        const float* points, int npoints, const int32_t* loop_first, int nloops,
                        const int32_t* set_first, int nsets);

/* ---- arbitrary output variables ----------------------------------------------- */
/* Extra float channels per vertex: the shader outputs a display asks for
 * (CqRenderer's output data map).  Each stored hit carries its
 * micropolygon's vertex-A values (CqBucketProcessor::StoreExtraData,
 * bucketprocessor.cpp:1573-1643, GetIndex), Combine keeps the values of the
 * front entry (imagepixel.cpp:253-262) and FilterBucket averages them with
 * the same weights as Ci, 0 where a pixel has no valid sample
 * (bucketprocessor.cpp:620-660).  n = 0..AQH_MAX_AOV floats, set after
 * aqh_frame_begin and before any grid is submitted.  Unlike the reference,
 * a grid without values contributes zeros rather than leaving earlier
 * values in the sample. */
#define AQH_MAX_AOV 16
aqh_status aqh_set_aov_count(aqh_ctx* ctx, int n);
/* Values for packed grids, float[vertices][n] indexed like Ci (cbase):
 * host arrays (kept by the caller until aqh_render returns) or device. */
aqh_status aqh_submit_aov_host(aqh_ctx* ctx, const float* aov, size_t nvertices);
aqh_status aqh_submit_aov_device(aqh_ctx* ctx, const float* d_aov);
/* The filtered output variables of the crop window: float[h][w][n].  In
 * aqh_read_display, channel 9 + k is output variable k. */
aqh_status aqh_read_aov(aqh_ctx* ctx, float* out, size_t out_floats);

/* ---- display drivers ------------------------------------------------------------ */
/* A frame sent to a RenderMan display driver library (the Dspy plugin ABI:
 * DspyImageOpen / DspyImageData / DspyImageClose), as CqDDManager and
 * CqDisplayRequest do (ddmanager.cpp:560-640, 930-952, 984-1176): the
 * driver gets the crop window's size, one format per channel of the request
 * (the request's element type) and the "origin" / "OriginalSize"
 * parameters; if it reorders the formats the host follows by channel name;
 * data go out bucket by bucket in row order, or a scanline at a time when the
 * driver sets PkDspyFlagsWantsScanLineOrder.  Host-only apart from
 * aqh_dspy_send, which reads the request from a rendered context.  The
 * library also builds a capture driver (libaqh_dspy_capture.so) that writes
 * PPM files. */
typedef struct {
	int width, height;            /* the image the driver receives: the crop window */
	int origin_x, origin_y;       /* the crop window's origin in the full image */
	int full_width, full_height;  /* the full resolution */
	int bucket_x, bucket_y;       /* bucket size of bucket-order delivery */
} aqh_dspy_geometry;
typedef struct aqh_dspy aqh_dspy;
aqh_status aqh_dspy_geometry_of(aqh_ctx* ctx, aqh_dspy_geometry* g);
aqh_status aqh_dspy_open(const char* driver_path, const char* filename, const aqh_dspy_geometry* g,
                         const aqh_display* d, const char* const* channel_names, aqh_dspy** out);
/* The request's channels of the context's last render (aqh_read_display). */
aqh_status aqh_dspy_send(aqh_dspy* dd, aqh_ctx* ctx);
/* A host image in the request's channel order, width x height x nchan elements. */
aqh_status aqh_dspy_send_image(aqh_dspy* dd, const void* image, size_t bytes);
aqh_status aqh_dspy_close(aqh_dspy* dd);
const char* aqh_dspy_last_error(void);

/* ---- micropolygon dump files ----------------------------------------------- */
/* The files CqMPDump writes when Option "mpdump" "enabled" is set
 * (libs/core/mpdump.cpp:40-210; records dumped by CqImageBuffer::AddMPG,
 * imagebuffer.cpp:541-545, and per bucket by dumpPixelSamples): a stream of
 * micropolygons in insertion order, each with vertex A's colour and opacity,
 * plus pixel sample positions and the image resolution.  Host-only; no
 * context.  Only dumps with sizeof(TqFloat) == 4 are read. */
typedef struct {
	int width, height;        /* the image information record (-1 when absent) */
	int64_t micropolygons;    /* id 1 records */
	int64_t samples;          /* id 2 records */
} aqh_mpdump_info;
aqh_status aqh_mpdump_scan(const char* path, aqh_mpdump_info* info);
/* Read a scanned file.  P: float4[micropolygons][4] in one-micropolygon grid
 * order (index, index+1, index+cu+1, index+cu+2; the file's circular order
 * is undone), Ci / Oi: float4[micropolygons], sample_pix: int[samples][3]
 * (pixel x, y, sample index), sample_pos: float[samples][2] raster
 * positions.  Any output may be NULL. */
aqh_status aqh_mpdump_read(const char* path, const aqh_mpdump_info* info, float* P, float* Ci, float* Oi,
                           int32_t* sample_pix, float* sample_pos);
/* Write a dump in the same layout (image record first, then the
 * micropolygons, then the samples); Ci / Oi NULL write CqMPDump's (0.9, 0.9, 1). */
aqh_status aqh_mpdump_write(const char* path, int width, int height, int64_t micropolygons, const float* P,
                            const float* Ci, const float* Oi, int64_t samples, const int32_t* sample_pix,
                            const float* sample_pos);
const char* aqh_mpdump_last_error(void);

/* ---- statistics and timing ------------------------------------------------ */
typedef struct {
	int64_t micropolygons;        /* micropolygons submitted this frame */
	int64_t samples;              /* samples in the sample region */
	int64_t grids;
	int64_t tile_grid_pairs;      /* grid references the tile lists hold */
	int64_t fragments;            /* transparent fragments stored */
	float ms_bin, ms_sample, ms_filter, ms_total;  /* device time per stage of the last render */
	int64_t graphs_built;         /* batched mode: frame graphs captured by this context so far */
	int64_t rerenders;            /* batched mode: frames rendered again on the plain path because
	                                 a device list outgrew its capacity */
} aqh_frame_stats;
aqh_status aqh_get_stats(aqh_ctx* ctx, aqh_frame_stats* st);

/* ---- serving --------------------------------------------------------------- */
/* No counterpart in the reference, which renders one frame per process.  A
 * server keeps `slots` contexts resident on one GPU, each with its own
 * stream and device buffers reused from job to job; jobs are admitted (in
 * the order `admission` names) when a slot is free and their estimated HBM footprint fits
 * in the budget the running jobs leave, and jobs on different slots run
 * concurrently on the device.  A job that can never fit is rejected at
 * submission (AQH_EREJECTED). */
typedef struct aqh_server aqh_server;
typedef struct {
	int device;
	size_t hbm_budget;   /* bytes the admitted jobs may hold together; 0 = 80% of free memory */
	int slots;           /* jobs in flight at once (1..64) */
	int mode;            /* AQH_MODE_BATCHED or AQH_MODE_PLAIN for every slot */
	int admission;       /* AQH_ADMIT_ARRIVAL (0) or AQH_ADMIT_SMALLEST */
} aqh_server_opts;
/* Admission order among pending jobs whose footprint fits: arrival order, or
 * the smallest footprint first (shorter jobs finish sooner, which lowers the
 * median latency of a mixed stream); under AQH_ADMIT_SMALLEST a job pending
 * for more than AQH_ADMIT_MAX_WAIT_MS goes first, in arrival order, so large
 * jobs are not starved. */
#define AQH_ADMIT_ARRIVAL 0
#define AQH_ADMIT_SMALLEST 1
#define AQH_ADMIT_MAX_WAIT_MS 250
/* One render request.  Every pointer is host memory that must stay valid
 * until the job completes; grids use the aqh_submit_grids_host layout. */
typedef struct {
	aqh_frame_desc frame;
	aqh_samples samples;
	int ngrids;
	const int32_t *cu, *cv, *nkeys, *flags;
	const int64_t *pbase, *cbase;
	const int32_t* tbase;
	const float* times;
	size_t ntimes;
	const float* P;
	size_t nP;
	const float *Ci, *Oi;
	size_t nC;
	const uint8_t* culled;   /* one byte per micropolygon, nonzero = culled; may be NULL */
	int64_t micropolygons;
	uint8_t* rgba;       /* out: crop window x 4 bytes (r, g, b, a quantized), or NULL */
	float* channels;     /* out: crop window x AQH_NCHANNELS floats, or NULL */
} aqh_job;
typedef struct {
	int64_t id;
	int status;          /* aqh_status of the job once done */
	int state;           /* 0 pending, 1 running, 2 done, 3 failed, 4 cancelled */
	double t_submit, t_admit, t_done;  /* seconds on the server's clock */
	size_t footprint;    /* estimated HBM bytes while running */
	float ms_device;     /* device time of the frame */
	int slot;
	/* host time of the job's phases on its slot: frame options, sample
	 * patterns and grids in; render to completion; results out */
	float ms_prepare, ms_render, ms_read;
} aqh_job_info;
typedef struct {
	size_t budget, in_use, peak_in_use;
	int64_t pending, completed;
	int running, peak_running;
	int64_t graphs_built, rerenders;  /* summed over the slots (see aqh_frame_stats) */
} aqh_server_info;
aqh_status aqh_server_create(const aqh_server_opts* opts, aqh_server** out);
void aqh_server_destroy(aqh_server* s);
aqh_status aqh_server_submit(aqh_server* s, const aqh_job* job, int64_t* id);
/* AQH_ENOTREADY while pending or running; the job's status once finished. */
aqh_status aqh_server_poll(aqh_server* s, int64_t id, aqh_job_info* info);
/* Waits up to timeout_ms; AQH_ETIMEDOUT if the job has not finished. */
aqh_status aqh_server_wait(aqh_server* s, int64_t id, int timeout_ms, aqh_job_info* info);
/* Removes a job that has not been admitted yet (AQH_ENOTREADY if it has). */
aqh_status aqh_server_cancel(aqh_server* s, int64_t id);
const char* aqh_server_job_error(aqh_server* s, int64_t id);
aqh_status aqh_server_stats(aqh_server* s, aqh_server_info* info);
/* Estimated HBM footprint of a job (host arithmetic, no GPU needed); 0 if invalid. */
size_t aqh_job_footprint(const aqh_job* job);

/* ---- imager shaders --------------------------------------------------------- */
/* RiImager (bucketprocessor.cpp:712-743): the imager shader runs on the
 * host's shading VM over the filtered display pixels, after FilterBucket and
 * before ExposeBucket.  With aqh_set_imager(ctx, 1), aqh_render stops after
 * the filter: aqh_read_channels / aqh_read_bucket then give the channels
 * before exposure (the shader's input, as InitialiseColorImager sees them).
 * The host runs the shader and hands its colour and opacity back with
 * aqh_apply_imager (float[pixel][6]: Ci r g b, Oi r g b, crop-window pixels in
 * raster order), which writes them, sets alpha to the mean of that opacity,
 * and then applies exposure (bucketprocessor.cpp:766-806) and the frame's
 * 8-bit display.  Reads of the frame before aqh_apply_imager see the
 * unexposed channels. */
aqh_status aqh_set_imager(aqh_ctx* ctx, int enabled);
aqh_status aqh_apply_imager(aqh_ctx* ctx, const float* ci_oi, size_t n_floats);

/* ---- rendering without allocation ---------------------------------------- */
/* No counterpart in the reference (aqsis renders into memory it allocates
 * per bucket).  For callers that cannot allocate device memory: a host whose
 * device memory belongs to another allocator, a plugin running inside
 * someone else's CUDA context, or code that must not grow the process's
 * footprint.  Renders one small, static, opaque frame with no cudaMalloc,
 * cudaFree or other allocation: the caller passes the grids (table on the
 * host, P/Ci/Oi in device memory) and a device output of
 * (crop width x crop height x AQH_NCHANNELS) floats; all intermediate data
 * lives in fixed device arrays of about 19 MB that every GPU loading this
 * library holds until the process exits.  Limits: AQH_NOALLOC_MAX_GRIDS
 * grids of at most 65535 x 65535 micropolygons, AQH_NOALLOC_MAX_REGION_PIXELS
 * pixels and AQH_NOALLOC_MAX_SAMPLES samples in the sample region (at most
 * 16 super-tiles of 128x128 pixels), AQH_NOALLOC_MAX_PATTERN_SAMPLES pattern
 * entries; no motion blur, no depth of field; every grid AQH_GRID_OPAQUE in
 * raster space, with no flags but AQH_GRID_SMOOTH, _MATTE, _MATTEALPHA and
 * _OPAQUE (camera-space grids, culling and trim curves need the context
 * path).  Larger or unsupported inputs return AQH_ELIMIT, bad ones AQH_EINVAL,
 * with a message in `err`; every check runs on the host before anything is
 * queued.
 * Sizes: `nP` is the number of float4 vertices in d_P, `nC` that of d_Ci and
 * d_Oi; pbase[i] + (cu[i]+1)*(cv[i]+1) must not exceed nP, nor cbase[i] + the
 * same count nC.  d_Ci or d_Oi may be NULL (white colour, full opacity, as on
 * the context path).  `channels_floats` is the size of d_channels in floats.
 * `pos`/`pos_index` follow aqh_samples (host arrays): every pattern choice
 * must be below `npatterns`.
 * The first call on a device looks up the arrays' device addresses with that
 * device current, so make it before any stream capture.  Each call queues its
 * work on `stream` (a cudaStream_t, NULL = default stream) and waits for that
 * stream once, after copying its small host tables into the arrays, before
 * queueing the kernels.  Calls share the arrays: calls whose work overlaps on
 * the GPU (other streams, other threads) race. */
#define AQH_NOALLOC_MAX_GRIDS 65536
#define AQH_NOALLOC_MAX_REGION_PIXELS 36864
#define AQH_NOALLOC_MAX_SAMPLES 300000
#define AQH_NOALLOC_MAX_PATTERN_SAMPLES 65536
aqh_status aqh_render_noalloc(const aqh_frame_desc* desc, const float* pos, int npatterns,
                              const uint32_t* pos_index, int ngrids, const int32_t* cu, const int32_t* cv,
                              const int32_t* flags, const int64_t* pbase, const int64_t* cbase,
                              const float* d_P, size_t nP, const float* d_Ci, const float* d_Oi, size_t nC,
                              float* d_channels, size_t channels_floats, void* stream, char* err,
                              size_t err_len);

/* ---- weight table and test hooks ----------------------------------------- */
/* Host-side filter weight table [(2*sy+1)*(2*sx+1)][spp] evaluated at sub-pixel
 * centres (CqBucketProcessor::InitialiseFilterValues, bucketprocessor.cpp:811-856).
 * Returns the number of floats written, or -needed when max_out is too small. */
int aqh_filter_table(int filter, float xw, float yw, int xs, int ys, float* out, int max_out);
/* Device CqInvBilinear (libs/core/bilinear.h:260-305) for n points against one quad. */
aqh_status aqh_test_invbilinear(const float* quad8, const float* P, int n, float* uv);

#ifdef __cplusplus
}
#endif
#endif /* AQH_H */
