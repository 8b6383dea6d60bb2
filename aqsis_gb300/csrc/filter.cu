// filter.cu -- pixel reconstruction filter, exposure and quantize.
//
// Replaces CqBucketProcessor::FilterBucket (non-separable path,
// libs/core/bucketprocessor.cpp:584-664, 686-707), ExposeBucket (766-806) and
// the quantize of CqDisplayRequest::FormatBucketForDisplay
// (ddmanager/ddmanager.cpp:1022-1119).  One thread per display pixel walks
// the (2*shift+1)^2 neighbouring pixels and their samples in the reference's
// loop order (fy, fx, sy, sx), so the float sums round identically.
#include <algorithm>
#include <type_traits>

#include "aqh_internal.h"
#include "hider_device.cuh"
#include "sample_common.cuh"

namespace aqh {

namespace {

// aqsis lround (math.h:67-70) in double: lfloor(x - 0.5) + 1
__device__ __forceinline__ double lround_d(double x) {
	const double y = x - 0.5;
	long long i = (long long)y;
	i -= (y < 0.0 && y != (double)i) ? 1 : 0;
	return (double)(i + 1);
}

__device__ __forceinline__ void finish_pixel(const FrameParams& fp, const SamplerDev& smp, int spp, float gTot,
                                             int count, const float acc[7], float* __restrict__ chan,
                                             uint8_t* __restrict__ q8, int x, int y);
__device__ __forceinline__ void expose_store(const FrameParams& fp, const SamplerDev& smp, float c[9],
                                             float* __restrict__ chan, uint8_t* __restrict__ q8, int x, int y);

// One display pixel (x, y).  SPP > 0: samples per pixel known at compile
// time (the sample loop is unrolled by four so its loads issue together); 0:
// read from fp.
template <int SPP>
__device__ __forceinline__ void filter_pixel(const FrameParams& fp, const SamplerDev& smp, const SampleStore& st,
                                             const float* __restrict__ ftab, float* __restrict__ chan,
                                             uint8_t* __restrict__ q8, int x, int y) {
	const float xcent = x + 0.5f, ycent = y + 0.5f;
	const int xmax = fp.shiftX, ymax = fp.shiftY;
	const int spp = SPP > 0 ? SPP : fp.spp;
	float gTot = 0.0f;
	int count = 0;
	float acc[7] = {0, 0, 0, 0, 0, 0, 0};
	for (int fy = -ymax; fy <= ymax; fy++) {
		const int py = y + fy;
		for (int fx = -xmax; fx <= xmax; fx++) {
			const int px = x + fx;
			const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
			const long long pat = (st.wmask || !smp.pos_index) ? pix : (long long)__ldg(smp.pos_index + pix);
			const int bit = (fy + ymax) * (2 * xmax + 1) + fx + xmax;
			const int index = bit * spp;
			const float fpx = (float)px, fpy = (float)py;
			// samples in groups of four: the window tests of a group first, then
			// the sample data of the samples inside it, so each group costs two
			// memory round trips; the sums still run in sample order
			for (int i0 = 0; i0 < spp; i0 += 4) {
				bool in[4];
				float gv[4];
#pragma unroll
				for (int j = 0; j < 4; ++j) {
					const int i = i0 + j;
					const bool ok = (SPP > 0 && SPP % 4 == 0) || i < spp;
					const int ic = ok ? i : i0;
					if (st.wmask) {
						in[j] = ok && ((__ldg(st.wmask + store_index(pix, ic, spp)) >> bit) & 1u);
					} else {
						const float2 o = __ldg(smp.pos + pat * spp + ic);
						const float vx = (fpx + o.x) - xcent;
						const float vy = (fpy + o.y) - ycent;
						in[j] = ok && vx >= -fp.xfwo2 && vy >= -fp.yfwo2 && vx <= fp.xfwo2 && vy <= fp.yfwo2;
					}
					gv[j] = __ldg(ftab + index + ic);
				}
				float4 av[4], bv[4];
#pragma unroll
				for (int j = 0; j < 4; ++j) {
					const long long si = store_index(pix, in[j] ? i0 + j : i0, spp);
					bv[j] = in[j] ? __ldg(st.b + si) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
					av[j] = in[j] ? __ldg(st.a + si) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
				}
#pragma unroll
				for (int j = 0; j < 4; ++j) {
					if (in[j]) {
						const float gw = gv[j];
						gTot += gw;
						if (bv[j].w != 0.0f) {
							const float4 a = av[j], b = bv[j];
							acc[0] += a.x * gw;
							acc[1] += a.y * gw;
							acc[2] += a.z * gw;
							acc[3] += b.x * gw;
							acc[4] += b.y * gw;
							acc[5] += b.z * gw;
							acc[6] += a.w * gw;
							count++;
						}
					}
				}
			}
		}
	}
	finish_pixel(fp, smp, spp, gTot, count, acc, chan, q8, x, y);
}

// The end of FilterBucket for one display pixel from its sums: normalisation
// by the weight total (1/gTot in double, rounded to float), coverage and
// alpha; then ExposeBucket, the channel-buffer write and the frame's fused
// 8-bit r g b a display.
__device__ __forceinline__ void finish_pixel(const FrameParams& fp, const SamplerDev& smp, int spp, float gTot,
                                             int count, const float acc[7], float* __restrict__ chan,
                                             uint8_t* __restrict__ q8, int x, int y) {
	float c[9];
	float coverage;
	if (count == 0) {
#pragma unroll
		for (int k = 0; k < 9; ++k) c[k] = 0.0f;
		c[7] = FLT_MAX;
		coverage = 0.0f;
	} else {
		const float inv = (float)(1.0 / (double)gTot);
		c[0] = acc[0] * inv; c[1] = acc[1] * inv; c[2] = acc[2] * inv;
		c[3] = acc[3] * inv; c[4] = acc[4] * inv; c[5] = acc[5] * inv;
		c[7] = acc[6] * inv;
		coverage = (count >= spp) ? 1.0f : (float)count / (float)spp;
	}
	const float a = (c[3] + c[4] + c[5]) / 3.0f;
	c[6] = a * coverage;
	c[8] = coverage;
	expose_store(fp, smp, c, chan, q8, x, y);
}

// ExposeBucket (bucketprocessor.cpp:766-806) on one display pixel's channels,
// then the channel-buffer write and the frame's fused 8-bit r g b a display.
__device__ __forceinline__ void expose_store(const FrameParams& fp, const SamplerDev& smp, float c[9],
                                             float* __restrict__ chan, uint8_t* __restrict__ q8, int x, int y) {
	// ExposeBucket: color = (color * gain) ^ (1 / gamma)
	if (!(fp.gain == 1.0f && fp.gamma == 1.0f)) {
		const float oneovergamma = 1.0f / fp.gamma;
		if (fp.gain != 1.0f) { c[0] *= fp.gain; c[1] *= fp.gain; c[2] *= fp.gain; }
		if (fp.gamma != 1.0f) {
			c[0] = (float)pow((double)c[0], (double)oneovergamma);
			c[1] = (float)pow((double)c[1], (double)oneovergamma);
			c[2] = (float)pow((double)c[2], (double)oneovergamma);
		}
	}
	const long long p = (long long)(y - fp.crop_y0) * (fp.crop_x1 - fp.crop_x0) + (x - fp.crop_x0);
	float* out = chan + p * 9;
#pragma unroll
	for (int k = 0; k < 9; ++k) out[k] = c[k];
	if (q8) {
		// the frame's own display, r g b a, quantized as quantize_u8_kernel does
		const double s = smp.dither ? (double)__ldg(smp.dither + p) : 0.0;
		const float src[4] = {c[0], c[1], c[2], c[6]};
		uchar4 q;
		unsigned char* qb = reinterpret_cast<unsigned char*>(&q);
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			double value = src[k];
			if (fp.q_one != 0.0f) {
				value = lround_d(0.0 + value * (double)(fp.q_one - 0.0f) + ((double)fp.q_dither * s));
				value = value < (double)fp.q_min ? (double)fp.q_min : (value > (double)fp.q_max ? (double)fp.q_max : value);
			}
			qb[k] = (uint8_t)(int)value;
		}
		reinterpret_cast<uchar4*>(q8)[p] = q;
	}
}

// 16x16-pixel tiles of the crop window in raster order, `gridDim.x` of them
// in flight at once.
template <int SPP>
__global__ void __launch_bounds__(256)
filter_kernel(FrameParams fp, SamplerDev smp, SampleStore st, const float* __restrict__ ftab,
              float* __restrict__ chan, uint8_t* __restrict__ q8) {
	const int ntx = (fp.crop_x1 - fp.crop_x0 + 15) >> 4, nty = (fp.crop_y1 - fp.crop_y0 + 15) >> 4;
	for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
		const int x = fp.crop_x0 + (tile % ntx) * 16 + (threadIdx.x & 15);
		const int y = fp.crop_y0 + (tile / ntx) * 16 + (threadIdx.x >> 4);
		if (x < fp.crop_x1 && y < fp.crop_y1) filter_pixel<SPP>(fp, smp, st, ftab, chan, q8, x, y);
	}
}

// ---- 3x3 windows (filter widths in [2, 4), shift 1): a rolling window ----
//
// One thread owns a display column and a run of rows.  It reads each row of
// input pixels once and adds every sample to the three output rows whose
// windows hold that row: the row below (fy = -1), its own row (fy = 0) and
// the row above (fy = +1).  Output row y takes its fy = -1 terms from input
// row y - 1, its fy = 0 terms from row y and its fy = +1 terms from row y + 1;
// input rows ascend, and within an input row the columns ascend (fx = -1, 0,
// 1) and then the samples -- the reference's (fy, fx, sy, sx) order, so every
// sum rounds exactly as in filter_pixel.  Each sample is
// loaded by three threads (the neighbouring columns, which read it back to
// back) instead of nine, once per run of rows plus the two rows around it.
struct FiltSum {
	float acc[7];
	float gTot;
	int count;
};
__device__ __forceinline__ void fsum_reset(FiltSum& f) {
#pragma unroll
	for (int k = 0; k < 7; ++k) f.acc[k] = 0.0f;
	f.gTot = 0.0f;
	f.count = 0;
}
__device__ __forceinline__ void fsum_add(FiltSum& f, bool in, float gw, const float4& a, const float4& b) {
	if (!in) return;
	f.gTot += gw;
	if (b.w != 0.0f) {
		f.acc[0] += a.x * gw;
		f.acc[1] += a.y * gw;
		f.acc[2] += a.z * gw;
		f.acc[3] += b.x * gw;
		f.acc[4] += b.y * gw;
		f.acc[5] += b.z * gw;
		f.acc[6] += a.w * gw;
		f.count++;
	}
}

// Input row r of display column x: its three pixels' samples into the sums
// of output rows r + 1 (B, window row fy = -1), r (M, fy = 0) and r - 1 (A,
// fy = +1), each only when that row is the thread's (uB, uM, uA).  `allin`:
// every sample of the three pixels is inside all three windows (see
// filter_roll_kernel), so the window tests are not evaluated.
template <int SPP>
__device__ __forceinline__ void roll_row(const FrameParams& fp, const SamplerDev& smp, const SampleStore& st,
                                         const float* __restrict__ ftab, int x, int r, FiltSum& B, FiltSum& M,
                                         FiltSum& A, bool uB, bool uM, bool uA, bool allin) {
	const int spp = SPP > 0 ? SPP : fp.spp;
	const float xcent = x + 0.5f;
	const float ycB = (r + 1) + 0.5f, ycM = r + 0.5f, ycA = (r - 1) + 0.5f;
	for (int fx = -1; fx <= 1; ++fx) {
		const int px = x + fx;
		const long long pix = (long long)(r - fp.sy0) * fp.sw + (px - fp.sx0);
		const long long pat =
		    (st.wmask || allin || !smp.pos_index) ? pix : (long long)__ldg(smp.pos_index + pix);
		const float fpx = (float)px, fpy = (float)r;
		const int bB = fx + 1, bM = 3 + fx + 1, bA = 6 + fx + 1;  // window bits (fy + 1) * 3 + fx + 1
		for (int i0 = 0; i0 < spp; i0 += 4) {
			bool iB[4], iM[4], iA[4];
			float gB[4], gM[4], gA[4];
#pragma unroll
			for (int j = 0; j < 4; ++j) {
				const int i = i0 + j;
				const bool ok = (SPP > 0 && SPP % 4 == 0) || i < spp;
				const int ic = ok ? i : i0;
				if (st.wmask) {
					const uint32_t mk = ok ? __ldg(st.wmask + store_index(pix, ic, spp)) : 0u;
					iB[j] = uB && ((mk >> bB) & 1u);
					iM[j] = uM && ((mk >> bM) & 1u);
					iA[j] = uA && ((mk >> bA) & 1u);
				} else if (allin) {
					iB[j] = uB && ok;
					iM[j] = uM && ok;
					iA[j] = uA && ok;
				} else {
					const float2 o = __ldg(smp.pos + pat * spp + ic);
					const float vx = (fpx + o.x) - xcent;
					const bool inx = ok && vx >= -fp.xfwo2 && vx <= fp.xfwo2;
					const float vB = (fpy + o.y) - ycB, vM = (fpy + o.y) - ycM, vA = (fpy + o.y) - ycA;
					iB[j] = uB && inx && vB >= -fp.yfwo2 && vB <= fp.yfwo2;
					iM[j] = uM && inx && vM >= -fp.yfwo2 && vM <= fp.yfwo2;
					iA[j] = uA && inx && vA >= -fp.yfwo2 && vA <= fp.yfwo2;
				}
				gB[j] = ftab[bB * spp + ic];
				gM[j] = ftab[bM * spp + ic];
				gA[j] = ftab[bA * spp + ic];
			}
			float4 av[4], bv[4];
#pragma unroll
			for (int j = 0; j < 4; ++j) {
				const bool any = iB[j] || iM[j] || iA[j];
				const long long si = store_index(pix, any ? i0 + j : i0, spp);
				bv[j] = any ? __ldg(st.b + si) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
				av[j] = any ? __ldg(st.a + si) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			}
#pragma unroll
			for (int j = 0; j < 4; ++j) {
				fsum_add(B, iB[j], gB[j], av[j], bv[j]);
				fsum_add(M, iM[j], gM[j], av[j], bv[j]);
				fsum_add(A, iA[j], gA[j], av[j], bv[j]);
			}
		}
	}
}

constexpr int kRollThreads = 128;  // display columns per CTA
constexpr int kRollRows = 8;       // display rows per CTA (8 measured faster than 16)

// Input row q (0 .. R+1) of a run: r = y0 - 1 + q feeds output rows y0 + q
// (B), y0 + q - 1 (M) and y0 + q - 2 (A); row y0 + q - 2 is then complete.
#define AQH_ROLL_STEP(QQ, SB, SM, SA)                                                                     \
	{                                                                                                     \
		const int q = (QQ);                                                                               \
		if (q < R + 2) {                                                                                  \
			if (q < R) fsum_reset(SB);                                                                    \
			roll_row<SPP>(fp, smp, st, ftab_s, x, y0 - 1 + q, SB, SM, SA, q < R, q >= 1 && q <= R, q >= 2, allin); \
			if (q >= 2) finish_pixel(fp, smp, spp, SA.gTot, SA.count, SA.acc, chan, q8, x, y0 + q - 2);  \
		}                                                                                                 \
	}

template <int SPP>
__global__ void __launch_bounds__(kRollThreads)
filter_roll_kernel(FrameParams fp, SamplerDev smp, SampleStore st, const float* __restrict__ ftab,
                   float* __restrict__ chan, uint8_t* __restrict__ q8) {
	__shared__ float ftab_s[9 * AQH_MAX_SPP_DEV];
	const int spp = SPP > 0 ? SPP : fp.spp;
	for (int i = threadIdx.x; i < 9 * spp; i += kRollThreads) ftab_s[i] = ftab[i];
	__syncthreads();
	const int x = fp.crop_x0 + blockIdx.x * kRollThreads + threadIdx.x;
	const int y0 = fp.crop_y0 + blockIdx.y * kRollRows;
	const int R = min(kRollRows, fp.crop_y1 - y0);
	if (x >= fp.crop_x1 || R <= 0) return;
	// With every sample offset in [0, 1] and half-widths of at least 1.5,
	// every sample of the 3x3 neighbourhood passes the window test in float:
	// for fx = -1, (px + o) >= px rounds to at least x - 1 and x + 0.5 is
	// exact below 2^22, so v >= -1.5; for fx = +1, px + o <= x + 2, so v <=
	// 1.5; fx = 0 and the rows alike.  The test then decides nothing.
	const int lim = 1 << 22;
	const bool allin = smp.pos_unit && fp.xfwo2 >= 1.5f && fp.yfwo2 >= 1.5f && fp.sx0 > -lim && fp.sy0 > -lim &&
	                   fp.sx0 + fp.sw < lim && fp.sy0 + fp.sh < lim;
	FiltSum S0, S1, S2;
	fsum_reset(S0);
	fsum_reset(S1);
	fsum_reset(S2);
	// slots rotate with the input row: B = S[q % 3], M = S[(q + 2) % 3], A = S[(q + 1) % 3]
	for (int q0 = 0; q0 < R + 2; q0 += 3) {
		AQH_ROLL_STEP(q0, S0, S2, S1)
		AQH_ROLL_STEP(q0 + 1, S1, S0, S2)
		AQH_ROLL_STEP(q0 + 2, S2, S1, S0)
	}
}
#undef AQH_ROLL_STEP

// Output variables of one display pixel: FilterBucket's weighted sum over
// the same window, weights and order as filter_pixel (gTot included), of the
// vertex-A values of each valid sample's front micropolygon.
template <int SPP>
__global__ void __launch_bounds__(256)
filter_aov_kernel(FrameParams fp, SamplerDev smp, SampleStore st, GridsDev g, const float* __restrict__ ftab,
                  float* __restrict__ out) {
	const int ntx = (fp.crop_x1 - fp.crop_x0 + 15) >> 4, nty = (fp.crop_y1 - fp.crop_y0 + 15) >> 4;
	const int spp = SPP > 0 ? SPP : fp.spp;
	const int naov = g.naov;
	for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
		const int x = fp.crop_x0 + (tile % ntx) * 16 + (threadIdx.x & 15);
		const int y = fp.crop_y0 + (tile / ntx) * 16 + (threadIdx.x >> 4);
		if (x >= fp.crop_x1 || y >= fp.crop_y1) continue;
		const float xcent = x + 0.5f, ycent = y + 0.5f;
		const int xmax = fp.shiftX, ymax = fp.shiftY;
		float gTot = 0.0f;
		int count = 0;
		float acc[AQH_MAX_AOV];
#pragma unroll
		for (int k = 0; k < AQH_MAX_AOV; ++k) acc[k] = 0.0f;
		for (int fy = -ymax; fy <= ymax; fy++) {
			const int py = y + fy;
			for (int fx = -xmax; fx <= xmax; fx++) {
				const int px = x + fx;
				const long long pix = (long long)(py - fp.sy0) * fp.sw + (px - fp.sx0);
				const long long pat = (st.wmask || !smp.pos_index) ? pix : (long long)__ldg(smp.pos_index + pix);
				const int bit = (fy + ymax) * (2 * xmax + 1) + fx + xmax;
				const int index = bit * spp;
				const float fpx = (float)px, fpy = (float)py;
				for (int i = 0; i < spp; ++i) {
					bool inside;
					if (st.wmask) {
						inside = (__ldg(st.wmask + store_index(pix, i, spp)) >> bit) & 1u;
					} else {
						const float2 o = __ldg(smp.pos + pat * spp + i);
						const float vx = (fpx + o.x) - xcent;
						const float vy = (fpy + o.y) - ycent;
						inside = vx >= -fp.xfwo2 && vy >= -fp.yfwo2 && vx <= fp.xfwo2 && vy <= fp.yfwo2;
					}
					if (!inside) continue;
					const float gw = __ldg(ftab + index + i);
					gTot += gw;
					const long long si = store_index(pix, i, spp);
					if (__ldg(st.b + si).w == 0.0f) continue;
					count++;
					const int id = __ldg(st.aovsrc + si);
					if (id < 0) continue;
					const int gi = grid_of(g, id);
					const int cu = __ldg(g.cu + gi);
					const int m = id - (int)__ldg(g.mpbase + gi);
					const int iv = m / cu, iu = m - iv * cu;
					const float* v = g.aov + (__ldg(g.cbase + gi) + iv * (cu + 1) + iu) * naov;
#pragma unroll
					for (int k = 0; k < AQH_MAX_AOV; ++k)
						if (k < naov) acc[k] += __ldg(v + k) * gw;
				}
			}
		}
		float* o = out + ((long long)(y - fp.crop_y0) * (fp.crop_x1 - fp.crop_x0) + (x - fp.crop_x0)) * naov;
		const float inv = count == 0 ? 0.0f : (float)(1.0 / (double)gTot);
#pragma unroll
		for (int k = 0; k < AQH_MAX_AOV; ++k)
			if (k < naov) o[k] = count == 0 ? 0.0f : acc[k] * inv;
	}
}


// The imager's write-back (bucketprocessor.cpp:712-743): Ci and Oi of each
// display pixel from the imager shader's output (the shading VM runs on the
// host), alpha = the mean of that opacity (no coverage factor), then
// ExposeBucket and the 8-bit display as after the filter.
__global__ void imager_kernel(FrameParams fp, SamplerDev smp, const float* __restrict__ ci_oi,
                              float* __restrict__ chan, uint8_t* __restrict__ q8) {
	const int w = fp.crop_x1 - fp.crop_x0;
	const long long npix = (long long)w * (fp.crop_y1 - fp.crop_y0);
	const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= npix) return;
	float c[9];
#pragma unroll
	for (int k = 0; k < 9; ++k) c[k] = chan[p * 9 + k];
#pragma unroll
	for (int k = 0; k < 6; ++k) c[k] = ci_oi[p * 6 + k];
	c[6] = (c[3] + c[4] + c[5]) / 3.0f;
	expose_store(fp, smp, c, chan, q8, fp.crop_x0 + (int)(p % w), fp.crop_y0 + (int)(p / w));
}

__global__ void quantize_u8_kernel(FrameParams fp, SamplerDev smp, const float* __restrict__ chan,
                                   const int* __restrict__ chans, int nchan, uint8_t* __restrict__ out) {
	const long long npix = (long long)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= npix) return;
	const double s = smp.dither ? (double)__ldg(smp.dither + p) : 0.0;
	for (int c = 0; c < nchan; ++c) {
		double value = chan[p * 9 + chans[c]];
		if (fp.q_one != 0.0f) {
			value = lround_d(0.0 + value * (double)(fp.q_one - 0.0f) + ((double)fp.q_dither * s));
			value = value < (double)fp.q_min ? (double)fp.q_min : (value > (double)fp.q_max ? (double)fp.q_max : value);
		}
		out[p * nchan + c] = (uint8_t)(int)value;
	}
}

// FormatBucketForDisplay (ddmanager.cpp:1054-1114) for one display request:
// element type T, the request's own quantize settings and dither values.
template <class T>
__global__ void display_kernel(FrameParams fp, QuantizeParams q, const float* __restrict__ dither,
                               const float* __restrict__ chan, const float* __restrict__ aov, int naov,
                               const int* __restrict__ chans, int nchan, T* __restrict__ out) {
	const long long npix = (long long)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= npix) return;
	const double s = dither ? (double)__ldg(dither + p) : 0.0;
	for (int c = 0; c < nchan; ++c) {
		const int ch = chans[c];
		double value = ch < 9 ? chan[p * 9 + ch] : aov[p * naov + (ch - 9)];
		if (q.one != 0.0f) {
			value = lround_d((double)q.zero + value * (double)(q.one - q.zero) + ((double)q.dither * s));
			value = value < (double)q.min ? (double)q.min : (value > (double)q.max ? (double)q.max : value);
		}
		T v;
		if constexpr (std::is_floating_point<T>::value) {
			v = (T)value;                                   // PkDspyFloat32
		} else if constexpr (sizeof(T) == 4) {
			// 32-bit integers are clamped to their range first (ddmanager.cpp:1075-1095)
			const double lo = T(-1) < T(0) ? -2147483648.0 : 0.0;
			const double hi = T(-1) < T(0) ? 2147483647.0 : 4294967295.0;
			value = value < lo ? lo : (value > hi ? hi : value);
			v = T(value == value ? (long long)value : 0);
		} else {
			// narrower types: the value is inside the quantize range; outside the
			// type's range the conversion wraps (through a 64-bit integer)
			value = value < -9.0e18 ? -9.0e18 : (value > 9.0e18 ? 9.0e18 : value);
			v = T(value == value ? (long long)value : 0);
		}
		out[p * nchan + c] = v;
	}
}

__global__ void test_invbilinear_kernel(const float* q, const float2* P, int n, float2* uv) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	V3f v[4] = {V3f{q[0], q[1], 0.0f}, V3f{q[2], q[3], 0.0f}, V3f{q[4], q[5], 0.0f}, V3f{q[6], q[7], 0.0f}};
	HitCoeffs h;
	hit_setup(v, 0, h);
	float u, w;
	inv_bilinear(h.ax, h.ay, h.e_x, h.e_y, h.f_x, h.f_y, h.g_x, h.g_y, h.linear, P[i].x, P[i].y, u, w);
	uv[i] = make_float2(u, w);
}

}  // namespace

void launch_filter(const FrameParams& fp, const SamplerDev& sm, const SampleStore& st, const float* ftab,
                   float* channels, uint8_t* q8, cudaStream_t s) {
	const int w = fp.crop_x1 - fp.crop_x0, h = fp.crop_y1 - fp.crop_y0;
	if (w <= 0 || h <= 0) return;
	const int ntiles = ((w + 15) / 16) * ((h + 15) / 16);
	int dev = 0, nsm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
	// tiles in flight per SM: by default as many as can be resident (the
	// filter is latency-bound: fewer tiles in flight, whose samples would stay
	// in L2 between the passes, measured slower)
	if (fp.shiftX == 1 && fp.shiftY == 1 && fp.spp <= AQH_MAX_SPP_DEV && !st.wmask) {
		// 3x3 windows: the rolling window reads each sample three times, not
		// nine (frames with window masks -- at most 16 samples per pixel --
		// read a word per sample and keep the tile kernel, measured faster)
		const dim3 rg((w + kRollThreads - 1) / kRollThreads, (h + kRollRows - 1) / kRollRows);
		switch (fp.spp) {
		case 4: filter_roll_kernel<4><<<rg, kRollThreads, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
		case 16: filter_roll_kernel<16><<<rg, kRollThreads, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
		case 36: filter_roll_kernel<36><<<rg, kRollThreads, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
		case 64: filter_roll_kernel<64><<<rg, kRollThreads, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
		default: filter_roll_kernel<0><<<rg, kRollThreads, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
		}
		return;
	}
	const int per_sm = fp.filter_ctas > 0 ? std::min(fp.filter_ctas, 8) : 8;
	const int grid = std::max(1, std::min(ntiles, nsm * per_sm));
	switch (fp.spp) {
	case 4: filter_kernel<4><<<grid, 256, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
	case 16: filter_kernel<16><<<grid, 256, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
	case 36: filter_kernel<36><<<grid, 256, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
	case 64: filter_kernel<64><<<grid, 256, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
	default: filter_kernel<0><<<grid, 256, 0, s>>>(fp, sm, st, ftab, channels, q8); break;
	}
}

void launch_imager(const FrameParams& fp, const SamplerDev& sm, const float* ci_oi, float* channels, uint8_t* q8,
                   cudaStream_t s) {
	const long long npix = (long long)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	if (npix <= 0) return;
	imager_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, s>>>(fp, sm, ci_oi, channels, q8);
}

void launch_filter_aov(const FrameParams& fp, const SamplerDev& sm, const SampleStore& st, const GridsDev& g,
                       const float* ftab, float* aov_channels, cudaStream_t s) {
	const int w = fp.crop_x1 - fp.crop_x0, h = fp.crop_y1 - fp.crop_y0;
	if (w <= 0 || h <= 0 || g.naov <= 0 || !st.aovsrc) return;
	const int ntiles = ((w + 15) / 16) * ((h + 15) / 16);
	int dev = 0, nsm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
	const int grid = std::max(1, std::min(ntiles, nsm * 8));
	switch (fp.spp) {
	case 16: filter_aov_kernel<16><<<grid, 256, 0, s>>>(fp, sm, st, g, ftab, aov_channels); break;
	default: filter_aov_kernel<0><<<grid, 256, 0, s>>>(fp, sm, st, g, ftab, aov_channels); break;
	}
}

void launch_quantize_u8(const FrameParams& fp, const SamplerDev& sm, const float* channels, const int* chans,
                        int nchan, uint8_t* out, cudaStream_t s) {
	const long long npix = (long long)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	if (npix <= 0) return;
	quantize_u8_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, s>>>(fp, sm, channels, chans, nchan, out);
}

void launch_display(const FrameParams& fp, const QuantizeParams& q, const float* dither, const float* channels,
                    const float* aov_channels, int naov, const int* chans, int nchan, int format, void* out,
                    cudaStream_t s) {
	const long long npix = (long long)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	if (npix <= 0) return;
	const unsigned nb = (unsigned)((npix + 255) / 256);
	switch (format) {
	case AQH_DSPY_FLOAT32: display_kernel<float><<<nb, 256, 0, s>>>(fp, q, dither, channels, aov_channels, naov, chans, nchan, (float*)out); break;
	case AQH_DSPY_UNSIGNED32: display_kernel<uint32_t><<<nb, 256, 0, s>>>(fp, q, dither, channels, aov_channels, naov, chans, nchan, (uint32_t*)out); break;
	case AQH_DSPY_SIGNED32: display_kernel<int32_t><<<nb, 256, 0, s>>>(fp, q, dither, channels, aov_channels, naov, chans, nchan, (int32_t*)out); break;
	case AQH_DSPY_UNSIGNED16: display_kernel<uint16_t><<<nb, 256, 0, s>>>(fp, q, dither, channels, aov_channels, naov, chans, nchan, (uint16_t*)out); break;
	case AQH_DSPY_SIGNED16: display_kernel<int16_t><<<nb, 256, 0, s>>>(fp, q, dither, channels, aov_channels, naov, chans, nchan, (int16_t*)out); break;
	case AQH_DSPY_UNSIGNED8: display_kernel<uint8_t><<<nb, 256, 0, s>>>(fp, q, dither, channels, aov_channels, naov, chans, nchan, (uint8_t*)out); break;
	default: display_kernel<int8_t><<<nb, 256, 0, s>>>(fp, q, dither, channels, aov_channels, naov, chans, nchan, (int8_t*)out); break;
	}
}

void launch_test_invbilinear(const float* quad8, const float2* P, int n, float2* uv, cudaStream_t s) {
	if (n <= 0) return;
	test_invbilinear_kernel<<<(n + 127) / 128, 128, 0, s>>>(quad8, P, n, uv);
}

}  // namespace aqh
