// dspy_host.cpp -- sending a rendered frame to a RenderMan display driver, as
// the reference's CqDDManager / CqDisplayRequest do (libs/core/ddmanager/
// ddmanager.cpp): the driver library is loaded, DspyImageOpen receives the
// crop window's size, the request's channel formats and the "origin" and
// "OriginalSize" parameters (ddmanager.cpp:930-952); the driver may reorder
// the formats, which the host follows by channel name; the data goes out
// bucket by bucket, or one scanline at a time when the driver asks for
// scanline order (DisplayBucket / CollapseBucketsToScanlines /
// SendToDisplay, ddmanager.cpp:984-1176); DspyImageClose ends the image.
#include <dlfcn.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/aqh.h"
#include "dspy_abi.h"

namespace {

thread_local std::string g_err;

aqh_status fail(aqh_status s, const std::string& msg) {
	g_err = msg;
	return s;
}

size_t element_size(int fmt) {
	switch (fmt) {
	case kDspyFloat32: case kDspyUnsigned32: case kDspySigned32: return 4;
	case kDspyUnsigned16: case kDspySigned16: return 2;
	case kDspyUnsigned8: case kDspySigned8: return 1;
	}
	return 0;
}

}  // namespace

struct aqh_dspy {
	void* lib = nullptr;
	DspyImageOpenFn open = nullptr;
	DspyImageDataFn data = nullptr;
	DspyImageCloseFn close = nullptr;
	DspyImageHandle handle = nullptr;
	aqh_dspy_geometry geom{};
	aqh_display d{};
	int format = 0;
	size_t esize = 0;
	int flags = 0;
	std::vector<int> perm;  // driver element i takes the request's channel perm[i]
	// the format list handed to the driver (kept: a driver may hold on to it)
	std::vector<std::string> names;
	std::vector<DspyDevFormat> fm;
};

extern "C" {

const char* aqh_dspy_last_error(void) { return g_err.c_str(); }

aqh_status aqh_dspy_open(const char* driver_path, const char* filename, const aqh_dspy_geometry* g,
                         const aqh_display* d, const char* const* channel_names, aqh_dspy** out) {
	if (!driver_path || !g || !d || !channel_names || !out) return fail(AQH_EINVAL, "bad arguments");
	if (d->nchan <= 0 || d->nchan > 16) return fail(AQH_EINVAL, "1..16 channels per display");
	if (g->width <= 0 || g->height <= 0) return fail(AQH_EINVAL, "empty image");
	const int fmt = d->format ? d->format : aqh_display_format(d->q_one, d->q_min, d->q_max);
	if (element_size(fmt) == 0) return fail(AQH_EINVAL, "bad element type " + std::to_string(fmt));
	void* lib = dlopen(driver_path, RTLD_NOW | RTLD_LOCAL);
	if (!lib) return fail(AQH_EINVAL, std::string("cannot load display driver: ") + dlerror());
	auto* dd = new aqh_dspy;
	dd->lib = lib;
	dd->open = reinterpret_cast<DspyImageOpenFn>(dlsym(lib, "DspyImageOpen"));
	dd->data = reinterpret_cast<DspyImageDataFn>(dlsym(lib, "DspyImageData"));
	dd->close = reinterpret_cast<DspyImageCloseFn>(dlsym(lib, "DspyImageClose"));
	if (!dd->open || !dd->data) {
		dlclose(lib);
		delete dd;
		return fail(AQH_EINVAL, "display driver lacks DspyImageOpen / DspyImageData");
	}
	dd->geom = *g;
	dd->d = *d;
	dd->format = fmt;
	dd->esize = element_size(fmt);
	// formats in the request's order; the driver may reorder them
	std::vector<DspyDevFormat>& fm = dd->fm;
	std::vector<std::string>& names = dd->names;
	fm.resize(d->nchan);
	names.resize(d->nchan);
	for (int c = 0; c < d->nchan; ++c) {
		names[c] = channel_names[c] ? channel_names[c] : "";
		fm[c].name = const_cast<char*>(names[c].c_str());
		fm[c].type = (unsigned)fmt;
	}
	int origin[2] = {g->origin_x, g->origin_y};
	int original[2] = {g->full_width > 0 ? g->full_width : g->width, g->full_height > 0 ? g->full_height : g->height};
	DspyUserParameter params[2] = {{"origin", 'i', 2, origin, (int)sizeof origin},
	                               {"OriginalSize", 'i', 2, original, (int)sizeof original}};
	DspyFlagStuff flags{0};
	const DspyError e = dd->open(&dd->handle, driver_path, filename ? filename : "", g->width, g->height, 2, params,
	                             d->nchan, fm.data(), &flags);
	if (e != kDspyErrorNone) {
		dlclose(lib);
		delete dd;
		return fail(AQH_EINVAL, "DspyImageOpen failed: error " + std::to_string((int)e));
	}
	dd->flags = flags.flags;
	dd->perm.resize(d->nchan);
	for (int i = 0; i < d->nchan; ++i) {
		int j = -1;
		for (int c = 0; c < d->nchan && j < 0; ++c)
			if (fm[i].name && names[c] == fm[i].name) j = c;
		if (j < 0 || (fm[i].type & kDspyMaskType) != (unsigned)fmt) {
			if (dd->close) dd->close(dd->handle);
			dlclose(lib);
			delete dd;
			return fail(AQH_EINVAL, "display driver changed the formats to ones this host cannot supply");
		}
		dd->perm[i] = j;
	}
	*out = dd;
	return AQH_OK;
}

aqh_status aqh_dspy_send_image(aqh_dspy* dd, const void* image, size_t bytes) {
	if (!dd || !image) return fail(AQH_EINVAL, "bad arguments");
	const int w = dd->geom.width, h = dd->geom.height, n = dd->d.nchan;
	const size_t es = dd->esize, px = es * n;
	if (bytes < (size_t)w * h * px) return fail(AQH_EINVAL, "image smaller than the display");
	const unsigned char* src = static_cast<const unsigned char*>(image);
	// one pixel in the driver's element order
	auto put = [&](unsigned char* dst, int x, int y) {
		const unsigned char* s = src + ((size_t)y * w + x) * px;
		for (int i = 0; i < n; ++i) std::memcpy(dst + i * es, s + dd->perm[i] * es, es);
	};
	if (dd->flags & kDspyFlagsWantsScanLineOrder) {
		std::vector<unsigned char> row((size_t)w * px);
		for (int y = 0; y < h; ++y) {
			for (int x = 0; x < w; ++x) put(row.data() + (size_t)x * px, x, y);
			const DspyError e = dd->data(dd->handle, 0, w, y, y + 1, (int)px, row.data());
			if (e != kDspyErrorNone) return fail(AQH_EINVAL, "DspyImageData failed: error " + std::to_string((int)e));
		}
		return AQH_OK;
	}
	const int bx = dd->geom.bucket_x > 0 ? dd->geom.bucket_x : 16, by = dd->geom.bucket_y > 0 ? dd->geom.bucket_y : 16;
	std::vector<unsigned char> bucket((size_t)bx * by * px);
	for (int y0 = 0; y0 < h; y0 += by)
		for (int x0 = 0; x0 < w; x0 += bx) {
			const int x1 = std::min(w, x0 + bx), y1 = std::min(h, y0 + by);
			unsigned char* p = bucket.data();
			for (int y = y0; y < y1; ++y)
				for (int x = x0; x < x1; ++x, p += px) put(p, x, y);
			const DspyError e = dd->data(dd->handle, x0, x1, y0, y1, (int)px, bucket.data());
			if (e != kDspyErrorNone) return fail(AQH_EINVAL, "DspyImageData failed: error " + std::to_string((int)e));
		}
	return AQH_OK;
}

aqh_status aqh_dspy_send(aqh_dspy* dd, aqh_ctx* ctx) {
	if (!dd || !ctx) return fail(AQH_EINVAL, "bad arguments");
	const size_t bytes = (size_t)dd->geom.width * dd->geom.height * dd->d.nchan * dd->esize;
	std::vector<unsigned char> img(bytes);
	aqh_display d = dd->d;
	d.format = dd->format;
	int used = 0;
	const aqh_status st = aqh_read_display(ctx, &d, img.data(), img.size(), &used);
	if (st != AQH_OK) return fail(st, std::string("aqh_read_display: ") + aqh_last_error(ctx));
	return aqh_dspy_send_image(dd, img.data(), img.size());
}

aqh_status aqh_dspy_close(aqh_dspy* dd) {
	if (!dd) return AQH_EINVAL;
	DspyError e = kDspyErrorNone;
	if (dd->close) e = dd->close(dd->handle);
	dlclose(dd->lib);
	delete dd;
	return e == kDspyErrorNone ? AQH_OK : fail(AQH_EINVAL, "DspyImageClose failed: error " + std::to_string((int)e));
}

}  // extern "C"
