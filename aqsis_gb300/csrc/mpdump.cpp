// mpdump.cpp -- micropolygon dump files as CqMPDump writes them
// (libs/core/mpdump.cpp:40-210): a native-endian int holding sizeof(TqFloat),
// then records that each start with a short id:
//   1  micropolygon: four vertices x y z in circular order (GetVertices P[0],
//      P[1], P[3], P[2]), then the colour and the opacity of vertex A (9 + 6
//      floats; (0.9, 0.9, 1) when the grid has no Ci / Oi)
//   2  pixel sample: pixel x, y and sample index (ints), position x, y (floats)
//   3  image information: x and y resolution (ints)
// Only dumps of float builds (sizeof(TqFloat) == 4) are read.  The reader
// hands the micropolygons back in the vertex order of a one-micropolygon grid
// (index, index+1, index+cu+1, index+cu+2), so they can be submitted as 1x1
// grids in insertion order.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/aqh.h"

namespace {

thread_local std::string g_err;

aqh_status fail(aqh_status s, const std::string& msg) {
	g_err = msg;
	return s;
}

struct File {
	FILE* f = nullptr;
	explicit File(const char* path, const char* mode) : f(std::fopen(path, mode)) {
		if (f) std::setvbuf(f, nullptr, _IOFBF, 1 << 20);
	}
	~File() {
		if (f) std::fclose(f);
	}
	template <class T>
	bool get(T* v, size_t n = 1) { return std::fread(v, sizeof(T), n, f) == n; }
	template <class T>
	bool put(const T* v, size_t n = 1) { return std::fwrite(v, sizeof(T), n, f) == n; }
};

constexpr size_t kMpBytes = 18 * sizeof(float);                   // 4 vertices + colour + opacity
constexpr size_t kSampleBytes = 3 * sizeof(int) + 2 * sizeof(float);
constexpr size_t kImageBytes = 2 * sizeof(int);

// One pass over the records; `mp` / `sample` / `image` see each record's payload.
template <class Mp, class Sample, class Image>
aqh_status walk(const char* path, Mp mp, Sample sample, Image image) {
	if (!path) return fail(AQH_EINVAL, "no path");
	File in(path, "rb");
	if (!in.f) return fail(AQH_EINVAL, std::string("cannot open ") + path);
	int sf = 0;
	if (!in.get(&sf)) return fail(AQH_EINVAL, "truncated header");
	if (sf != (int)sizeof(float)) return fail(AQH_EINVAL, "dump written with sizeof(TqFloat) = " + std::to_string(sf));
	unsigned char buf[kMpBytes];
	for (long long rec = 0;; ++rec) {
		short id = 0;
		if (!in.get(&id)) break;  // end of file
		size_t n = id == 1 ? kMpBytes : id == 2 ? kSampleBytes : id == 3 ? kImageBytes : 0;
		if (n == 0) return fail(AQH_EINVAL, "record " + std::to_string(rec) + ": unknown id " + std::to_string(id));
		if (!in.get(buf, n)) return fail(AQH_EINVAL, "record " + std::to_string(rec) + ": truncated");
		if (id == 1) mp(buf);
		else if (id == 2) sample(buf);
		else image(buf);
	}
	return AQH_OK;
}

}  // namespace

extern "C" {

const char* aqh_mpdump_last_error(void) { return g_err.c_str(); }

aqh_status aqh_mpdump_scan(const char* path, aqh_mpdump_info* info) {
	if (!info) return fail(AQH_EINVAL, "no info");
	aqh_mpdump_info r{};
	r.width = r.height = -1;
	aqh_status st = walk(
	    path, [&](const unsigned char*) { ++r.micropolygons; }, [&](const unsigned char*) { ++r.samples; },
	    [&](const unsigned char* b) {
		    std::memcpy(&r.width, b, sizeof(int));
		    std::memcpy(&r.height, b + sizeof(int), sizeof(int));
	    });
	if (st == AQH_OK) *info = r;
	return st;
}

aqh_status aqh_mpdump_read(const char* path, const aqh_mpdump_info* info, float* P, float* Ci, float* Oi,
                           int32_t* sample_pix, float* sample_pos) {
	if (!info) return fail(AQH_EINVAL, "no info");
	int64_t im = 0, is = 0;
	bool over = false;
	aqh_status st = walk(
	    path,
	    [&](const unsigned char* b) {
		    if (im >= info->micropolygons) { over = true; return; }
		    float v[18];
		    std::memcpy(v, b, sizeof v);
		    if (P) {
			    // file order A B D C (P[0] P[1] P[3] P[2]) -> grid order A B C D
			    static const int from[4] = {0, 1, 3, 2};
			    float* o = P + im * 16;
			    for (int k = 0; k < 4; ++k) {
				    o[4 * k] = v[3 * from[k]];
				    o[4 * k + 1] = v[3 * from[k] + 1];
				    o[4 * k + 2] = v[3 * from[k] + 2];
				    o[4 * k + 3] = 0.0f;
			    }
		    }
		    if (Ci) { float* o = Ci + im * 4; o[0] = v[12]; o[1] = v[13]; o[2] = v[14]; o[3] = 0.0f; }
		    if (Oi) { float* o = Oi + im * 4; o[0] = v[15]; o[1] = v[16]; o[2] = v[17]; o[3] = 0.0f; }
		    ++im;
	    },
	    [&](const unsigned char* b) {
		    if (is >= info->samples) { over = true; return; }
		    if (sample_pix) std::memcpy(sample_pix + is * 3, b, 3 * sizeof(int));
		    if (sample_pos) std::memcpy(sample_pos + is * 2, b + 3 * sizeof(int), 2 * sizeof(float));
		    ++is;
	    },
	    [&](const unsigned char*) {});
	if (st != AQH_OK) return st;
	if (over || im != info->micropolygons || is != info->samples)
		return fail(AQH_EINVAL, "file changed since aqh_mpdump_scan");
	return AQH_OK;
}

aqh_status aqh_mpdump_write(const char* path, int width, int height, int64_t nmp, const float* P, const float* Ci,
                            const float* Oi, int64_t nsamples, const int32_t* sample_pix, const float* sample_pos) {
	if (!path || nmp < 0 || nsamples < 0 || (nmp > 0 && !P) || (nsamples > 0 && (!sample_pix || !sample_pos)))
		return fail(AQH_EINVAL, "bad arguments");
	File out(path, "wb");
	if (!out.f) return fail(AQH_EINVAL, std::string("cannot create ") + path);
	bool ok = true;
	const int sf = sizeof(float);
	ok = ok && out.put(&sf);
	short id = 3;
	ok = ok && out.put(&id) && out.put(&width) && out.put(&height);
	static const float kNoColour[3] = {0.9f, 0.9f, 1.0f};  // CqMPDump::dump without Ci / Oi
	for (int64_t i = 0; ok && i < nmp; ++i) {
		id = 1;
		float v[18];
		static const int to[4] = {0, 1, 3, 2};  // grid order A B C D -> file order A B D C
		for (int k = 0; k < 4; ++k)
			for (int c = 0; c < 3; ++c) v[3 * k + c] = P[i * 16 + 4 * to[k] + c];
		for (int c = 0; c < 3; ++c) {
			v[12 + c] = Ci ? Ci[i * 4 + c] : kNoColour[c];
			v[15 + c] = Oi ? Oi[i * 4 + c] : kNoColour[c];
		}
		ok = out.put(&id) && out.put(v, 18);
	}
	for (int64_t i = 0; ok && i < nsamples; ++i) {
		id = 2;
		ok = out.put(&id) && out.put(sample_pix + i * 3, 3) && out.put(sample_pos + i * 2, 2);
	}
	if (!ok) return fail(AQH_EINVAL, std::string("error writing ") + path);
	return AQH_OK;
}

}  // extern "C"
