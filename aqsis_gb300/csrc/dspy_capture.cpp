// dspy_capture.cpp -- a headless RenderMan display driver (built as
// libaqh_dspy_capture.so).  It takes any channel list of one element type,
// reorders r, g, b, a to the front as file drivers do (so the host must
// follow the driver's order), keeps the image in memory, and at
// DspyImageClose writes a binary PPM (P6) of the first three 8-bit
// channels, or for other layouts a raw file: the line
// "AQHRAW <width> <height> <channels> <type>\n" and then the elements.  A
// file name that ends in "#scanline" (the suffix is dropped) asks for
// scanline order.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dspy_abi.h"

namespace {

struct Capture {
	int w = 0, h = 0, n = 0;
	size_t es = 0;
	unsigned type = 0;
	std::string file;
	std::vector<unsigned char> pix;
};

size_t element_size(unsigned t) {
	switch (t) {
	case kDspyFloat32: case kDspyUnsigned32: case kDspySigned32: return 4;
	case kDspyUnsigned16: case kDspySigned16: return 2;
	case kDspyUnsigned8: case kDspySigned8: return 1;
	}
	return 0;
}

int rank(const char* name) {
	static const char* order[4] = {"r", "g", "b", "a"};
	for (int i = 0; i < 4; ++i)
		if (name && std::strcmp(name, order[i]) == 0) return i;
	return 4;
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) DspyError DspyImageOpen(DspyImageHandle* image, const char*,
                                                               const char* filename, int width, int height, int,
                                                               const DspyUserParameter*, int nformat,
                                                               DspyDevFormat* format, DspyFlagStuff* flags) {
	if (!image || !format || nformat <= 0 || width <= 0 || height <= 0) return kDspyErrorBadParams;
	const unsigned t = format[0].type & kDspyMaskType;
	for (int i = 0; i < nformat; ++i)
		if ((format[i].type & kDspyMaskType) != t) return kDspyErrorUnsupported;
	if (element_size(t) == 0) return kDspyErrorUnsupported;
	// stable reorder: r, g, b, a first
	for (int i = 1; i < nformat; ++i)
		for (int j = i; j > 0 && rank(format[j].name) < rank(format[j - 1].name); --j) std::swap(format[j], format[j - 1]);
	auto* c = new Capture;
	c->w = width;
	c->h = height;
	c->n = nformat;
	c->type = t;
	c->es = element_size(t);
	c->file = filename ? filename : "";
	const std::string tag = "#scanline";
	if (flags) flags->flags = 0;
	if (c->file.size() >= tag.size() && c->file.compare(c->file.size() - tag.size(), tag.size(), tag) == 0) {
		c->file.resize(c->file.size() - tag.size());
		if (flags) flags->flags |= kDspyFlagsWantsScanLineOrder;
	}
	c->pix.assign((size_t)width * height * nformat * c->es, 0);
	*image = c;
	return kDspyErrorNone;
}

__attribute__((visibility("default"))) DspyError DspyImageQuery(DspyImageHandle image, DspyQuery q, size_t len,
                                                                void* data) {
	auto* c = static_cast<Capture*>(image);
	if (!c || !data) return kDspyErrorBadParams;
	if (q == kDspySizeQuery && len >= sizeof(DspySizeInfo)) {
		DspySizeInfo* s = static_cast<DspySizeInfo*>(data);
		s->width = (unsigned)c->w;
		s->height = (unsigned)c->h;
		s->aspectRatio = 1.0f;
		return kDspyErrorNone;
	}
	return kDspyErrorUnsupported;
}

__attribute__((visibility("default"))) DspyError DspyImageData(DspyImageHandle image, int xmin, int xmaxplus1,
                                                               int ymin, int ymaxplus1, int entrysize,
                                                               const unsigned char* data) {
	auto* c = static_cast<Capture*>(image);
	if (!c || !data) return kDspyErrorBadParams;
	const size_t px = c->es * c->n;
	if ((size_t)entrysize != px || xmin < 0 || ymin < 0 || xmaxplus1 > c->w || ymaxplus1 > c->h || xmin >= xmaxplus1 ||
	    ymin >= ymaxplus1)
		return kDspyErrorBadParams;
	const size_t rowb = (size_t)(xmaxplus1 - xmin) * px;
	for (int y = ymin; y < ymaxplus1; ++y) {
		std::memcpy(c->pix.data() + ((size_t)y * c->w + xmin) * px, data, rowb);
		data += rowb;
	}
	return kDspyErrorNone;
}

__attribute__((visibility("default"))) DspyError DspyImageClose(DspyImageHandle image) {
	auto* c = static_cast<Capture*>(image);
	if (!c) return kDspyErrorBadParams;
	DspyError e = kDspyErrorNone;
	if (!c->file.empty()) {
		FILE* f = std::fopen(c->file.c_str(), "wb");
		if (!f) {
			e = kDspyErrorNoResource;
		} else if (c->type == kDspyUnsigned8 && c->n >= 3) {
			std::fprintf(f, "P6\n%d %d\n255\n", c->w, c->h);
			for (size_t p = 0; p < (size_t)c->w * c->h; ++p) std::fwrite(c->pix.data() + p * c->n, 1, 3, f);
			std::fclose(f);
		} else {
			std::fprintf(f, "AQHRAW %d %d %d %u\n", c->w, c->h, c->n, c->type);
			std::fwrite(c->pix.data(), 1, c->pix.size(), f);
			std::fclose(f);
		}
	}
	delete c;
	return e;
}

}  // extern "C"
