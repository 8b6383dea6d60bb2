// noalloc.cu -- aqh_render_noalloc: render a small opaque frame without
// allocating memory.
//
// For callers that cannot allocate device memory themselves or through this
// library: a host whose device memory is owned by another allocator, code
// that must not grow the process's footprint, or a driver-style plugin that
// runs inside someone else's CUDA context.  The caller passes the grids and
// the output buffer; everything in between (per-grid tables, bin lists, the
// sample store, the filter table) lives in file-scope device arrays of fixed
// size that every GPU loading this library holds until the process exits.
//
// Set-up: the first call on a device looks up those arrays' device
// addresses (cudaGetSymbolAddress) with that device current, so that first
// call should come before any stream capture.  All calls share the arrays and
// each call overwrites what it uses; calls whose work overlaps on the GPU
// (different streams, or different host threads) race on them.
//
// Every call copies its small host tables into the arrays and then waits for
// `stream` (cudaStreamSynchronize) before it returns, because those copies
// read host memory that the call owns only until it returns.
//
// All checks run on the host before anything is queued: pattern choices must
// name existing patterns, each grid's vertices must lie inside the caller's
// P (nP vertices) and Ci/Oi (nC vertices) arrays, and flags this form does not
// carry out (camera space, culling, trim curves) are refused, not ignored.
// Null Ci or Oi is allowed and means what it means on the context path:
// white colour, full opacity.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/aqh.h"
#include "aqh_internal.h"

namespace aqh {
namespace {

constexpr int kNaMaxGrids = AQH_NOALLOC_MAX_GRIDS;
constexpr int kNaMaxSamples = AQH_NOALLOC_MAX_SAMPLES;
constexpr int kNaMaxRegionPixels = AQH_NOALLOC_MAX_REGION_PIXELS;
constexpr int kNaMaxPatternEntries = AQH_NOALLOC_MAX_PATTERN_SAMPLES;
constexpr int kNaMaxFilterTable = 96 * 1024;
constexpr int kNaMaxSuperTiles = 16;
constexpr int kNaMaxRanges = (kNaMaxGrids + 4095) / 4096;
constexpr int kNaMaxList = kNaMaxSuperTiles * kNaMaxGrids;

// Scratch of aqh_render_noalloc (about 19 MB per device).
__device__ __align__(256) int32_t na_cu[kNaMaxGrids];
__device__ __align__(256) int32_t na_cv[kNaMaxGrids];
__device__ __align__(256) int32_t na_nkeys[kNaMaxGrids];
__device__ __align__(256) int32_t na_flags[kNaMaxGrids];
__device__ __align__(256) int32_t na_tbase[kNaMaxGrids];
__device__ __align__(256) int64_t na_pbase[kNaMaxGrids];
__device__ __align__(256) int64_t na_cbase[kNaMaxGrids];
__device__ __align__(256) int64_t na_mpbase[kNaMaxGrids];
__device__ __align__(256) int4 na_rect[kNaMaxGrids];
__device__ __align__(256) float na_minz[kNaMaxGrids];
__device__ __align__(256) int32_t na_stcount[kNaMaxSuperTiles * kNaMaxRanges + 1];
__device__ __align__(256) int32_t na_stoffset[kNaMaxSuperTiles * kNaMaxRanges + 1];
__device__ __align__(256) int32_t na_stlist[kNaMaxList];
__device__ __align__(256) float4 na_sa[kNaMaxSamples];
__device__ __align__(256) float4 na_sb[kNaMaxSamples];
__device__ __align__(256) float2 na_pos[kNaMaxPatternEntries];
__device__ __align__(256) uint32_t na_posidx[kNaMaxRegionPixels];
__device__ __align__(256) float na_ftab[kNaMaxFilterTable];

struct NaAddrs {
	int32_t *cu, *cv, *nkeys, *flags, *tbase;
	int64_t *pbase, *cbase, *mpbase;
	int4* rect;
	float* minz;
	int32_t *stcount, *stoffset, *stlist;
	float4 *sa, *sb;
	float2* pos;
	uint32_t* posidx;
	float* ftab;
};

std::mutex g_na_mutex;
NaAddrs g_na[64];
bool g_na_ready[64] = {};

// Device addresses of the scratch arrays for the current device, looked up
// once per device.  In host code the arrays' names are only host-side stand-ins.
cudaError_t na_addresses(int dev, NaAddrs& a) {
	std::lock_guard<std::mutex> lock(g_na_mutex);
	if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
	if (!g_na_ready[dev]) {
		NaAddrs t{};
		cudaError_t e = cudaSuccess;
		void* p = nullptr;
#define NA_SYM(field, name)                                   \
	if (e == cudaSuccess) {                                   \
		e = cudaGetSymbolAddress(&p, name);                   \
		t.field = reinterpret_cast<decltype(t.field)>(p);     \
	}
		NA_SYM(cu, na_cu) NA_SYM(cv, na_cv) NA_SYM(nkeys, na_nkeys) NA_SYM(flags, na_flags)
		NA_SYM(tbase, na_tbase) NA_SYM(pbase, na_pbase) NA_SYM(cbase, na_cbase) NA_SYM(mpbase, na_mpbase)
		NA_SYM(rect, na_rect) NA_SYM(minz, na_minz) NA_SYM(stcount, na_stcount) NA_SYM(stoffset, na_stoffset)
		NA_SYM(stlist, na_stlist) NA_SYM(sa, na_sa) NA_SYM(sb, na_sb) NA_SYM(pos, na_pos)
		NA_SYM(posidx, na_posidx) NA_SYM(ftab, na_ftab)
#undef NA_SYM
		if (e != cudaSuccess) return e;
		g_na[dev] = t;
		g_na_ready[dev] = true;
	}
	a = g_na[dev];
	return cudaSuccess;
}

aqh_status na_fail(char* err, size_t len, aqh_status s, const char* msg) {
	if (err && len) {
		std::strncpy(err, msg, len - 1);
		err[len - 1] = 0;
	}
	return s;
}

}  // namespace
}  // namespace aqh

using namespace aqh;

extern "C" aqh_status aqh_render_noalloc(const aqh_frame_desc* desc, const float* pos, int npatterns,
                                         const uint32_t* pos_index, int ngrids, const int32_t* cu,
                                         const int32_t* cv, const int32_t* flags, const int64_t* pbase,
                                         const int64_t* cbase, const float* d_P, size_t nP, const float* d_Ci,
                                         const float* d_Oi, size_t nC, float* d_channels,
                                         size_t channels_floats, void* stream, char* err, size_t err_len) {
	if (!desc || !pos || npatterns <= 0 || ngrids < 0 || (ngrids > 0 && (!cu || !cv || !flags || !pbase || !cbase)) ||
	    !d_P || !d_channels)
		return na_fail(err, err_len, AQH_EINVAL, "aqh_render_noalloc: null argument");
	if ((d_Ci || d_Oi) && nC == 0)
		return na_fail(err, err_len, AQH_EINVAL, "aqh_render_noalloc: colours given with nC == 0");
	FrameParams fp{};
	std::vector<float> ftab;
	std::string msg;
	aqh_status st = resolve_frame(*desc, fp, ftab, msg);
	if (st != AQH_OK) return na_fail(err, err_len, st, msg.c_str());
	char buf[256];
	const long long npix_disp = (long long)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	if ((unsigned long long)npix_disp * AQH_NCHANNELS > channels_floats) {
		snprintf(buf, sizeof buf, "aqh_render_noalloc: the output holds %zu floats; %lld needed", channels_floats,
		         npix_disp * AQH_NCHANNELS);
		return na_fail(err, err_len, AQH_EINVAL, buf);
	}
	const long long npix = (long long)fp.sw * fp.sh;
	const long long nsamp = npix * fp.spp;
	if (fp.use_dof) return na_fail(err, err_len, AQH_ELIMIT, "aqh_render_noalloc: depth of field is not supported");
	if (!fp.cullable || fp.midpoint_store)
		return na_fail(err, err_len, AQH_ELIMIT,
		               "aqh_render_noalloc: a z display with the midpoint, max or average depth filter is not supported");
	if (npix > kNaMaxRegionPixels || nsamp > kNaMaxSamples || (long long)store_size(npix, fp.spp) > kNaMaxSamples) {
		snprintf(buf, sizeof buf,
		         "aqh_render_noalloc: sample region %dx%d x %d samples exceeds the limit of %d pixels / %d samples",
		         fp.sw, fp.sh, fp.spp, kNaMaxRegionPixels, kNaMaxSamples);
		return na_fail(err, err_len, AQH_ELIMIT, buf);
	}
	if ((long long)npatterns * fp.spp > kNaMaxPatternEntries) {
		snprintf(buf, sizeof buf, "aqh_render_noalloc: %d patterns x %d samples exceeds %d pattern samples", npatterns,
		         fp.spp, kNaMaxPatternEntries);
		return na_fail(err, err_len, AQH_ELIMIT, buf);
	}
	if (!pos_index && npatterns < npix)
		return na_fail(err, err_len, AQH_EINVAL, "aqh_render_noalloc: explicit samples need one pattern per pixel");
	// every choice must name an existing pattern: the samplers index the
	// pattern array with it and do not check it again
	if (pos_index) {
		for (long long i = 0; i < npix; ++i)
			if (pos_index[i] >= (uint32_t)npatterns) {
				snprintf(buf, sizeof buf, "aqh_render_noalloc: pattern choice %u at pixel %lld; %d patterns",
				         pos_index[i], i, npatterns);
				return na_fail(err, err_len, AQH_EINVAL, buf);
			}
	}
	if (ngrids > kNaMaxGrids) {
		snprintf(buf, sizeof buf, "aqh_render_noalloc: %d grids exceeds the limit of %d", ngrids, kNaMaxGrids);
		return na_fail(err, err_len, AQH_ELIMIT, buf);
	}
	if ((int)ftab.size() > kNaMaxFilterTable)
		return na_fail(err, err_len, AQH_ELIMIT, "aqh_render_noalloc: filter table too large (filter too wide)");
	// host-side grid validation and first micropolygon ids
	std::vector<int32_t> nk(ngrids, 1), tb(ngrids, 0);
	std::vector<int64_t> mpb(ngrids);
	int64_t acc = 0;
	for (int i = 0; i < ngrids; ++i) {
		if (cu[i] <= 0 || cv[i] <= 0 || cu[i] > 65535 || cv[i] > 65535)
			return na_fail(err, err_len, AQH_EINVAL, "aqh_render_noalloc: empty or oversized grid");
		if (!(flags[i] & AQH_GRID_OPAQUE))
			return na_fail(err, err_len, AQH_ELIMIT,
			               "aqh_render_noalloc: every grid must be opaque (AQH_GRID_OPAQUE); transparency needs "
			               "the fragment pool of the context path");
		if (flags[i] & AQH_GRID_TRIANGULAR)
			return na_fail(err, err_len, AQH_ELIMIT, "aqh_render_noalloc: triangular grids are not supported");
		if (flags[i] & ~(AQH_GRID_SMOOTH | AQH_GRID_MATTE | AQH_GRID_MATTEALPHA | AQH_GRID_OPAQUE)) {
			snprintf(buf, sizeof buf,
			         "aqh_render_noalloc: grid %d has flags 0x%x; camera-space grids, culling and trim curves "
			         "are not supported (raster-space grids with AQH_GRID_SMOOTH, _MATTE, _MATTEALPHA, _OPAQUE only)",
			         i, (unsigned)flags[i]);
			return na_fail(err, err_len, AQH_ELIMIT, buf);
		}
		const int64_t nv = (int64_t)(cu[i] + 1) * (cv[i] + 1);
		if (pbase[i] < 0 || (uint64_t)(pbase[i] + nv) > (uint64_t)nP ||
		    ((d_Ci || d_Oi) && (cbase[i] < 0 || (uint64_t)(cbase[i] + nv) > (uint64_t)nC))) {
			snprintf(buf, sizeof buf, "aqh_render_noalloc: grid %d: vertices out of range (nP %zu, nC %zu)", i, nP, nC);
			return na_fail(err, err_len, AQH_EINVAL, buf);
		}
		mpb[i] = acc;
		acc += (int64_t)cu[i] * cv[i];
	}
	if (acc > INT32_MAX) return na_fail(err, err_len, AQH_ELIMIT, "aqh_render_noalloc: too many micropolygons");
	// tiling and super-tiles must fit the fixed bin arrays
	set_tiling(fp, 0);
	const int nst = fp.nstx * fp.nsty;
	BinBuffers bb{};
	bb.range_size = 4096;
	bb.nranges = std::max(1, (ngrids + bb.range_size - 1) / bb.range_size);
	if (nst > kNaMaxSuperTiles || (long long)nst * bb.nranges + 1 > kNaMaxSuperTiles * kNaMaxRanges + 1)
		return na_fail(err, err_len, AQH_ELIMIT, "aqh_render_noalloc: too many super-tiles");

	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	NaAddrs a{};
	if (e == cudaSuccess) e = na_addresses(dev, a);
	if (e != cudaSuccess) return na_fail(err, err_len, AQH_EDEVICE, cudaGetErrorString(e));
	cudaStream_t s = static_cast<cudaStream_t>(stream);

	// inputs into the fixed arrays (copies, not allocations)
	auto cp = [&](void* dst, const void* src, size_t bytes) {
		if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
	};
	cp(a.cu, cu, (size_t)ngrids * 4);
	cp(a.cv, cv, (size_t)ngrids * 4);
	cp(a.nkeys, nk.data(), (size_t)ngrids * 4);
	cp(a.flags, flags, (size_t)ngrids * 4);
	cp(a.tbase, tb.data(), (size_t)ngrids * 4);
	cp(a.pbase, pbase, (size_t)ngrids * 8);
	cp(a.cbase, cbase, (size_t)ngrids * 8);
	cp(a.mpbase, mpb.data(), (size_t)ngrids * 8);
	cp(a.pos, pos, (size_t)npatterns * fp.spp * sizeof(float2));
	if (pos_index) cp(a.posidx, pos_index, (size_t)npix * 4);
	cp(a.ftab, ftab.data(), ftab.size() * 4);
	// the host vectors above must outlive the copies
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) return na_fail(err, err_len, AQH_EDEVICE, cudaGetErrorString(e));

	GridsDev g{};
	g.ngrids = ngrids;
	g.cu = a.cu; g.cv = a.cv; g.nkeys = a.nkeys; g.flags = a.flags; g.tbase = a.tbase;
	g.pbase = a.pbase; g.cbase = a.cbase; g.mpbase = a.mpbase;
	g.times = nullptr;
	g.P = reinterpret_cast<const float4*>(d_P);
	g.Ci = reinterpret_cast<const float4*>(d_Ci);
	g.Oi = reinterpret_cast<const float4*>(d_Oi);
	g.culled = nullptr;
	SamplerDev smp{};
	smp.npatterns = npatterns;
	smp.pos = a.pos;
	smp.pos_index = pos_index ? a.posidx : nullptr;
	bb.grid_rect = a.rect;
	bb.grid_minz = a.minz;
	bb.st_count = a.stcount;
	bb.st_offset = a.stoffset;
	bb.st_list = a.stlist;
	bb.list_capacity = kNaMaxList;
	SampleStore store{};
	store.a = a.sa;
	store.b = a.sb;
	FragPool pool{};
	if (ngrids > 0) {
		launch_grid_rects(fp, g, bb, s);
		launch_st_count(fp, g, bb, s);
		launch_scan_i32(bb.st_count, bb.st_offset, nst * bb.nranges, nullptr, s);
		launch_st_write(fp, g, bb, s);
	} else {
		// no grids: an empty list for every super-tile
		e = cudaMemsetAsync(bb.st_offset, 0, sizeof(int32_t) * ((size_t)nst * bb.nranges + 1), s);
	}
	launch_sample_tiles(fp, g, smp, bb, store, pool, nullptr, s);
	launch_filter(fp, smp, store, a.ftab, d_channels, nullptr, s);
	if (e == cudaSuccess) e = cudaGetLastError();
	if (e != cudaSuccess) return na_fail(err, err_len, AQH_EDEVICE, cudaGetErrorString(e));
	return AQH_OK;
}
