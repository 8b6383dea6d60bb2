// dspy_abi.h -- the display-driver plugin ABI that RenderMan display drivers
// export (the reference declares it in include/aqsis/ri/ndspy.h): element
// type codes, error codes, the format / parameter / flag structures and the
// four entry points a driver library provides.  Declared here so the display
// host and the capture driver share one definition; layouts and values are
// the ABI's, so drivers built against the reference's header load unchanged.
#pragma once

#include <cstddef>

extern "C" {

enum {
	kDspyFloat32 = 1, kDspyUnsigned32 = 2, kDspySigned32 = 3, kDspyUnsigned16 = 4,
	kDspySigned16 = 5, kDspyUnsigned8 = 6, kDspySigned8 = 7
};
constexpr unsigned kDspyMaskType = 8191;

enum DspyError {
	kDspyErrorNone = 0,
	kDspyErrorNoMemory,
	kDspyErrorUnsupported,
	kDspyErrorBadParams,
	kDspyErrorNoResource,
	kDspyErrorUndefined
};

enum DspyQuery { kDspySizeQuery, kDspyOverwriteQuery };

constexpr int kDspyFlagsWantsScanLineOrder = 1;

struct DspyDevFormat {
	char* name;
	unsigned type;
};

struct DspyFlagStuff {
	int flags;
};

struct DspySizeInfo {
	unsigned width, height;
	float aspectRatio;
};

// RtToken name; char vtype ('i' int, 'f' float, 's' string), vcount;
// RtPointer value; int nbytes.
struct DspyUserParameter {
	const char* name;
	char vtype, vcount;
	void* value;
	int nbytes;
};

typedef void* DspyImageHandle;

typedef DspyError (*DspyImageOpenFn)(DspyImageHandle*, const char*, const char*, int, int, int,
                                     const DspyUserParameter*, int, DspyDevFormat*, DspyFlagStuff*);
typedef DspyError (*DspyImageQueryFn)(DspyImageHandle, DspyQuery, size_t, void*);
typedef DspyError (*DspyImageDataFn)(DspyImageHandle, int, int, int, int, int, const unsigned char*);
typedef DspyError (*DspyImageCloseFn)(DspyImageHandle);

}  // extern "C"
