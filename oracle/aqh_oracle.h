/*
 * aqh_oracle.h -- C interface of the CPU oracle for the aqsis REYES hider.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a plain C++17 restatement of the
 * reference hider (aqsis libs/core) used by tests/, __graft_entry__.smoke()
 * and the cpu_baseline leg of bench.py as the checker.  No product code path
 * may call it.
 *
 * All arrays are plain host memory.  Layouts match the ones the product's
 * C-ABI (include/aqh.h) consumes, so a test can hand the same buffers to both.
 */
#ifndef AQH_ORACLE_H
#define AQH_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
	ORC_FILTER_BOX = 0,
	ORC_FILTER_TRIANGLE = 1,
	ORC_FILTER_GAUSSIAN = 2,
	ORC_FILTER_CATMULLROM = 3,
	ORC_FILTER_SINC = 4,
	ORC_FILTER_DISK = 5,
	ORC_FILTER_BESSEL = 6,
	ORC_FILTER_MITCHELL = 7
};

enum { ORC_DEPTH_MIN = 0, ORC_DEPTH_MIDPOINT = 1, ORC_DEPTH_MAX = 2, ORC_DEPTH_AVERAGE = 3 };

/* Grid flags (SqGridInfo, micropolygon.h:57-63). */
enum {
	ORC_GRID_SMOOTH = 1,      /* ShadingInterpolation "smooth" */
	ORC_GRID_MATTE = 2,       /* SqImageSample::Flag_Matte */
	ORC_GRID_MATTEALPHA = 4,  /* SqImageSample::Flag_MatteAlpha */
	ORC_GRID_TRIANGULAR = 16, /* CqMicroPolyGridBase::fTriangular: split line through corners cu, cv*(cu+1) */
	ORC_GRID_CAMERA = 32,     /* P in camera space: orc_project_points first (orc_render itself ignores it) */
	ORC_GRID_TRIM_OUTSIDE = 64, /* "trimcurve" "sense" "outside" */
	ORC_GRID_CULL_BACKFACING = 128, /* Sides 1, outside any solid, "cull" "backfacing" 1 */
	ORC_GRID_CULL_TRANSPARENT = 256 /* the surface shader uses Oi */
};

typedef struct {
	int32_t width, height;                  /* Format */
	int32_t crop_xmin, crop_xmax;           /* raster crop window, CqRenderer::initialiseCropWindow */
	int32_t crop_ymin, crop_ymax;
	int32_t xsamples, ysamples;             /* PixelSamples */
	float xfilter, yfilter;                 /* PixelFilter widths */
	float gain, gamma;                      /* Exposure */
	float q_zero, q_one, q_min, q_max, q_dither; /* Quantize (ddmanager.cpp:428-457) */
	float shutter_open, shutter_close;      /* Shutter */
	int32_t use_dof;                        /* CqRenderer::UsingDepthOfField */
	float dof_mult, dof_inv_fd;             /* m_DofMultiplier, m_OneOverFocalDistance (renderer.h:368-377) */
	float dof_scale_x, dof_scale_y;         /* SetDepthOfFieldScale (options.cpp:162-171) */
	int32_t depth_filter;                   /* Hider "depthfilter" */
	float zthreshold[3];                    /* Option "limits" "zthreshold" */
	int32_t display_z;                      /* DisplayMode includes DMode_Z */
} OrcFrame;

#define ORC_MAX_AOV 16

typedef struct {
	int32_t ngrids;
	const int32_t* cu;        /* micropolygons along u, per grid */
	const int32_t* cv;        /* micropolygons along v, per grid */
	const int32_t* nkeys;     /* motion keys per grid (1 = static) */
	const int64_t* pbase;     /* first vertex of key 0 in P (float4 units); key k at pbase + k*(cu+1)*(cv+1) */
	const int64_t* cbase;     /* first vertex in Ci/Oi (float4 units) */
	const int64_t* tbase;     /* first key time in `times` */
	const float* times;       /* motion key times */
	const float* P;           /* float4: raster x, raster y, camera z, unused */
	const float* Ci;          /* float4: r g b unused (NULL = white) */
	const float* Oi;          /* float4: r g b unused (NULL = opaque white) */
	const int32_t* flags;     /* ORC_GRID_* */
	const uint8_t* culled;    /* per micropolygon (global mp id) 1 = culled, or NULL */
	const float* aov;         /* output variables float[vertex][naov] indexed like Ci, or NULL */
	int32_t naov;
	const float* lod;         /* LevelOfDetailBounds float[grid][2] (min, max), or NULL = (0, 1) */
	/* CSG (RiSolidBegin / RiSolidEnd): the primitive node of each grid (-1: none)
	 * and the tree: per node its type (ORC_CSG_*) and parent (-1: a root); the
	 * children of a node are the nodes naming it as parent, in index order */
	const int32_t* csg_node;
	int32_t csg_nnodes;
	const int32_t* csg_type;
	const int32_t* csg_parent;
	/* trim curves (NURBS surfaces, CqTrimLoopArray, trimcurve.h:110-160): the
	 * trim set of each grid (-1: not trimmable) and the sets as loops of
	 * prepared curve points; uv float[vertex][2] indexed like Ci */
	const int32_t* trim_set;
	const float* trim_uv;
	const float* trim_points;      /* float[point][2] */
	const int32_t* trim_loop_first; /* [nloops + 1] first point of each loop */
	const int32_t* trim_set_first;  /* [nsets + 1] first loop of each set */
} OrcGrids;

enum { ORC_CSG_PRIMITIVE = 0, ORC_CSG_UNION = 1, ORC_CSG_INTERSECTION = 2, ORC_CSG_DIFFERENCE = 3 };

typedef struct {
	int32_t x0, y0, w, h;     /* sample region in pixels: [x0,x0+w) x [y0,y0+h) */
	/* Pattern caches and per-pixel choices, as IqSampler / CqImagePixel::setSamples
	 * use them (isampler.h:42-78, imagepixel.cpp:334-359).  NULL index = pixel index. */
	int32_t npatterns;
	const float* pos;         /* float2[npatterns][spp] offsets within the pixel */
	const float* time;        /* float[npatterns][spp] in [0,1) (NULL = 0) */
	const float* dof;         /* float2[npatterns][spp] lens samples in [0,1)^2 (NULL = none) */
	const int32_t* shuffle;   /* int[npatterns][spp] (NULL = identity) */
	const float* lod;         /* float[npatterns][spp] (NULL = 0) */
	const uint32_t* pos_index;
	const uint32_t* dof_index;
	const uint32_t* time_index;
	const uint32_t* shuffle_index;
	const uint32_t* lod_index;
	const float* dither;      /* per display pixel (crop window, row-major) random float s */
} OrcSamples;

typedef struct {
	/* per sample of the sample region (pixel-major, sample-minor) */
	int32_t* winner;          /* occluding hit micropolygon id before Combine, -1 if none */
	float* occlz;             /* occlZ after sampling */
	int32_t* nfrag;           /* transparent fragments stored */
	uint8_t* valid;           /* occludingHit valid after Combine */
	float* sdata;             /* 7 floats after Combine: R G B OR OG OB depth */
	/* per display pixel of the crop window: Ci(3) Oi(3) a z coverage (channelbuffer order) */
	float* channels;
	/* per display pixel: quantized value of each requested channel, as double */
	double* quantized;
	const int32_t* qchannels; /* channel-buffer indices to quantize, in display order */
	int32_t nqchannels;
	/* statistics */
	int64_t spl_count, spl_bound_hits, spl_hits;
	/* per display pixel: the filtered output variables (naov floats), or NULL */
	float* aov_channels;
	/* Float64 twin (NULL = not computed): Combine's composite and FilterBucket /
	 * ExposeBucket re-evaluated in double from the same per-sample entries
	 * (the float hit data StoreSample wrote, taken as exact inputs) and the
	 * same filter table.  Per sample 7 doubles after Combine (as sdata; a
	 * sample without a valid entry is all zero), per display pixel 9 doubles
	 * (as channels).  Used to state the float path's rounding error. */
	double* sdata64;
	double* channels64;
} OrcOut;

/* Weight table [(2*shiftY+1)*(2*shiftX+1)][spp] (bucketprocessor.cpp:811-856). */
int orc_filter_table(int filter, float xw, float yw, int xs, int ys, float* out, int max_out);
/* Evaluate one RI filter function (filters.cpp). */
float orc_filter_eval(int filter, float x, float y, float xw, float yw);

/* CqInvBilinear lookup (bilinear.h:260-305) for n points against one quad A B C D. */
void orc_invbilinear(const float* quad8, const float* P, int n, float* uv);
/* bilerp (bilinear.h:228-236) of 2D vertices at n (u,v). */
void orc_bilerp2(const float* quad8, const float* uv, int n, float* P);

/* Whole-frame hider: sample, combine, filter, expose, quantize. */
int orc_render(const OrcFrame* f, const OrcGrids* g, const OrcSamples* s,
               const float* filter_table, OrcOut* out);

/* The imager shader's write-back (bucketprocessor.cpp:712-743) then
 * ExposeBucket (766-806), on n display pixels' channels as FilterBucket left
 * them: Ci, Oi from ci_oi [pixel][6], alpha = the mean of that opacity. */
void orc_imager(const OrcFrame* f, float* chan, const float* ci_oi, int64_t n);
/* FormatBucketForDisplay's quantize (ddmanager.cpp:1022-1119) of channels qch. */
void orc_quantize(const OrcFrame* f, const float* chan, int64_t n, const float* dither, const int32_t* qch, int nq,
                  double* out);

/* The reference's global MT19937 (libs/math/random.cpp) and its multi-jittered
 * sample tables, for regenerating aqsis' own sample patterns. */
void orc_mt_seed(uint32_t s);
uint32_t orc_mt_int32(void);
float orc_mt_float(void);
/* Fill the 250-pattern caches of CqMultiJitteredSampler (multijitter.cpp:130-202).
 * pos: [250*spp*2], t1d: [250*spp], shuffle: [250*spp]. Consumes the global MT. */
void orc_multijitter_tables(int xs, int ys, float* pos, float* t1d, int32_t* shuffle);

/* Split's camera-to-raster projection of n float4 points (micropolygon.cpp:
 * 735-745, 1023-1032; CqMatrix::operator*(CqVector3D), matrix.h:717-750):
 * raster x, y and the camera-space z.  m: CqMatrix elements m[row*4 + col]. */
void orc_project_points(const float* m, const float* Pin, int64_t n, float* Pout);

/* The culling of CqMicroPolyGrid::Shade (micropolygon.cpp:431-506) and
 * CqMotionMicroPolyGrid::Split (micropolygon.cpp:957-1020, 1075-1080) for
 * one grid in camera space: P float4 and Ng / N (N may be NULL) float3 per
 * P entry, every key; Oi float4 per vertex or NULL.  Sets culled[mp] for
 * the grid's cu*cv micropolygons (never clears). */
void orc_cull_grid(int cu, int cv, int nkeys, int flags, const float* P, const float* Ng, const float* N,
                   const float* Oi, int zthreshold_black, uint8_t* culled);

/* The rounding helpers of libs/math/math.h:46-70 as the oracle uses them
 * (lfloor/lceil of a float, lround of a double). */
long orc_lfloor(float x);
long orc_lceil(float x);
long orc_lround(double x);

/* CqVector2D::Magnitude2 and Magnitude (libs/math/vector2d.h:132-147). */
float orc_mag2(float x, float y);
float orc_mag(float x, float y);

#ifdef __cplusplus
}
#endif
#endif
