// server.cu -- serving: render jobs of different resolutions, sample counts
// and blur settings as they arrive, several in flight at once.
//
// No counterpart in the reference, which renders one frame per process.  A
// server owns `slots` hider contexts on one GPU; each slot has its own CUDA
// stream and keeps its device buffers (grids, sample store, bin lists,
// fragment pool) resident from job to job.  Jobs are admitted in arrival
// order when a slot is free and their estimated HBM footprint fits in what
// the admitted jobs leave of the budget; an admitted job runs on its slot's
// stream while other slots' jobs run on theirs, so work from different
// requests overlaps on the device.  With AQH_ADMIT_SMALLEST the smallest
// fitting job is admitted first (a job that has waited more than
// AQH_ADMIT_MAX_WAIT_MS goes first in arrival order).  A job that could never fit is rejected
// at submission.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/aqh.h"
#include "aqh_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
	int64_t id = 0;
	aqh_job j{};
	size_t footprint = 0;
	int state = 0;  // 0 pending, 1 running, 2 done, 3 failed, 4 cancelled
	aqh_status status = AQH_ENOTREADY;
	std::string error;
	double t_submit = 0, t_admit = 0, t_done = 0;
	float ms_device = 0;
	float ms_prepare = 0, ms_render = 0, ms_read = 0;
	int slot = -1;
};

}  // namespace

struct aqh_server {
	aqh_server_opts opts{};
	std::mutex mu;
	std::condition_variable cv_work, cv_done;
	std::deque<Job*> pending;
	std::map<int64_t, std::unique_ptr<Job>> jobs;
	int64_t next_id = 1;
	size_t in_use = 0;
	bool stop = false;
	std::vector<aqh_ctx*> ctx;
	std::vector<std::thread> workers;
	Clock::time_point t0 = Clock::now();
	int64_t completed = 0;
	size_t peak_in_use = 0;
	int running = 0, peak_running = 0;

	double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

extern "C" size_t aqh_job_footprint(const aqh_job* j) {
	if (!j) return 0;
	aqh::FrameParams fp{};
	std::vector<float> ftab;
	std::string err;
	if (aqh::resolve_frame(j->frame, fp, ftab, err) != AQH_OK) return 0;
	const size_t npix = (size_t)fp.sw * fp.sh;
	const size_t nsamp = npix * fp.spp;
	const size_t ndisp = (size_t)(fp.crop_x1 - fp.crop_x0) * (fp.crop_y1 - fp.crop_y0);
	size_t b = 0;
	b += j->nP * 16 + j->nC * 32 + (size_t)j->ngrids * (5 * 4 + 3 * 8) + j->ntimes * 4;  // grids
	b += (size_t)j->ngrids * (16 + 4 + 4 * 4) + 65536;                                  // bin
	if (j->culled) b += (size_t)j->micropolygons;                                        // culled flags
	bool moving = fp.use_dof != 0;
	for (int i = 0; i < j->ngrids && !moving; ++i) moving = j->nkeys[i] > 1;
	if (moving) b += (size_t)j->micropolygons * 16;                                      // staging bounds
	b += nsamp * (32 + 12);                                                              // sample store (+debug)
	bool transparent = false;
	for (int i = 0; i < j->ngrids && !transparent; ++i) transparent = !(j->flags[i] & AQH_GRID_OPAQUE);
	if (transparent) b += std::max<size_t>(1u << 20, nsamp * 2) * 20;                    // fragment pool
	if (transparent && !moving) b += nsamp * 4;                                          // list heads (Combine kernel)
	b += ndisp * (36 + 4);                                                                // channels + rgba
	const size_t np = (size_t)j->samples.npatterns * fp.spp;
	b += np * 28 + npix * 4 * 5;                                                          // patterns + choices
	b += ftab.size() * 4 + (1u << 20);
	return b + b / 10;
}

static void run_job(aqh_server* sv, int slot, Job* job) {
	aqh_ctx* c = sv->ctx[slot];
	const aqh_job& j = job->j;
	const double t0 = sv->now();
	aqh_status st = aqh_frame_begin(c, &j.frame);
	if (st == AQH_OK) st = aqh_set_samples(c, &j.samples);
	if (st == AQH_OK)
		st = aqh_submit_grids_host(c, j.ngrids, j.cu, j.cv, j.nkeys, j.flags, j.pbase, j.cbase, j.tbase, j.times,
		                           j.ntimes, j.P, j.nP, j.Ci, j.Oi, j.nC, j.culled, j.micropolygons);
	const double t1 = sv->now();
	if (st == AQH_OK) st = aqh_render(c, 1);
	const double t2 = sv->now();
	if (st == AQH_OK && j.rgba) {
		const int ch[4] = {0, 1, 2, 6};
		const size_t n = (size_t)(j.frame.crop_xmax - j.frame.crop_xmin) * (j.frame.crop_ymax - j.frame.crop_ymin);
		const size_t ndisp = n ? n : (size_t)j.frame.width * j.frame.height;
		st = aqh_read_quantized_u8(c, ch, 4, j.rgba, ndisp * 4);
	}
	if (st == AQH_OK && j.channels) {
		const size_t n = (size_t)(j.frame.crop_xmax - j.frame.crop_xmin) * (j.frame.crop_ymax - j.frame.crop_ymin);
		const size_t ndisp = n ? n : (size_t)j.frame.width * j.frame.height;
		st = aqh_read_channels(c, j.channels, ndisp * AQH_NCHANNELS);
	}
	aqh_frame_stats fs{};
	aqh_get_stats(c, &fs);
	const double t3 = sv->now();
	std::lock_guard<std::mutex> lock(sv->mu);
	job->ms_prepare = (float)(1e3 * (t1 - t0));
	job->ms_render = (float)(1e3 * (t2 - t1));
	job->ms_read = (float)(1e3 * (t3 - t2));
	job->status = st;
	job->error = st == AQH_OK ? "" : aqh_last_error(c);
	job->state = st == AQH_OK ? 2 : 3;
	job->ms_device = fs.ms_total;
	job->t_done = sv->now();
	sv->in_use -= job->footprint;
	sv->running--;
	sv->completed++;
}

static void worker_main(aqh_server* sv, int slot) {
	cudaSetDevice(sv->opts.device);
	for (;;) {
		Job* job = nullptr;
		{
			std::unique_lock<std::mutex> lock(sv->mu);
			for (;;) {
				if (sv->stop) return;
				// admission: the oldest pending job if its footprint fits now; with
				// AQH_ADMIT_SMALLEST the smallest fitting one, unless the oldest has
				// waited past the limit
				if (!sv->pending.empty()) {
					auto pick = sv->pending.begin();
					const bool aged =
						(sv->now() - (*pick)->t_submit) * 1e3 > AQH_ADMIT_MAX_WAIT_MS;
					if (sv->opts.admission == AQH_ADMIT_SMALLEST && !aged) {
						auto best = sv->pending.end();
						for (auto it = sv->pending.begin(); it != sv->pending.end(); ++it)
							if ((*it)->footprint + sv->in_use <= sv->opts.hbm_budget &&
							    (best == sv->pending.end() || (*it)->footprint < (*best)->footprint))
								best = it;
						if (best != sv->pending.end()) pick = best;
					}
					Job* head = *pick;
					if (head->footprint + sv->in_use <= sv->opts.hbm_budget) {
						sv->pending.erase(pick);
						job = head;
						job->state = 1;
						job->slot = slot;
						job->t_admit = sv->now();
						sv->in_use += job->footprint;
						sv->peak_in_use = std::max(sv->peak_in_use, sv->in_use);
						sv->running++;
						sv->peak_running = std::max(sv->peak_running, sv->running);
						break;
					}
				}
				sv->cv_work.wait(lock);
			}
		}
		run_job(sv, slot, job);
		sv->cv_done.notify_all();
		sv->cv_work.notify_all();  // memory freed: a waiting job may fit now
	}
}

extern "C" {

aqh_status aqh_server_create(const aqh_server_opts* o, aqh_server** out) {
	if (!o || !out || o->slots <= 0 || o->slots > 64) return AQH_EINVAL;
	if (o->admission != AQH_ADMIT_ARRIVAL && o->admission != AQH_ADMIT_SMALLEST) return AQH_EINVAL;
	*out = nullptr;
	std::unique_ptr<aqh_server> sv(new aqh_server());
	sv->opts = *o;
	if (cudaSetDevice(o->device) != cudaSuccess) return AQH_EDEVICE;
	if (sv->opts.hbm_budget == 0) {
		size_t fr = 0, tot = 0;
		if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return AQH_EDEVICE;
		sv->opts.hbm_budget = fr / 10 * 8;
	}
	for (int i = 0; i < o->slots; ++i) {
		aqh_device_opts d{o->device, 0, 0};
		aqh_ctx* c = nullptr;
		aqh_status st = aqh_create(&d, &c);
		if (st != AQH_OK) {
			for (aqh_ctx* x : sv->ctx) aqh_destroy(x);
			return st;
		}
		aqh_set_mode(c, o->mode);
		// several jobs are in flight: host arrays move on the copy engines,
		// colours beside P, while another slot's frame holds the SMs
		aqh_set_host_copy(c, AQH_HOST_COPY_ENGINES);
		sv->ctx.push_back(c);
	}
	aqh_server* raw = sv.release();
	for (int i = 0; i < o->slots; ++i) raw->workers.emplace_back(worker_main, raw, i);
	*out = raw;
	return AQH_OK;
}

void aqh_server_destroy(aqh_server* sv) {
	if (!sv) return;
	{
		std::lock_guard<std::mutex> lock(sv->mu);
		sv->stop = true;
	}
	sv->cv_work.notify_all();
	for (auto& t : sv->workers) t.join();
	for (aqh_ctx* c : sv->ctx) aqh_destroy(c);
	delete sv;
}

aqh_status aqh_server_submit(aqh_server* sv, const aqh_job* j, int64_t* id) {
	if (!sv || !j || !id) return AQH_EINVAL;
	const size_t fp = aqh_job_footprint(j);
	if (fp == 0) return AQH_EINVAL;
	if (fp > sv->opts.hbm_budget) return AQH_EREJECTED;
	std::unique_ptr<Job> job(new Job());
	job->j = *j;
	job->footprint = fp;
	{
		std::lock_guard<std::mutex> lock(sv->mu);
		job->id = sv->next_id++;
		job->t_submit = sv->now();
		*id = job->id;
		sv->pending.push_back(job.get());
		sv->jobs[job->id] = std::move(job);
	}
	sv->cv_work.notify_all();
	return AQH_OK;
}

static void fill_info(const Job* job, aqh_job_info* info) {
	if (!info) return;
	info->id = job->id;
	info->status = job->status;
	info->state = job->state;
	info->t_submit = job->t_submit;
	info->t_admit = job->t_admit;
	info->t_done = job->t_done;
	info->footprint = job->footprint;
	info->ms_device = job->ms_device;
	info->slot = job->slot;
	info->ms_prepare = job->ms_prepare;
	info->ms_render = job->ms_render;
	info->ms_read = job->ms_read;
}

aqh_status aqh_server_poll(aqh_server* sv, int64_t id, aqh_job_info* info) {
	if (!sv) return AQH_EINVAL;
	std::lock_guard<std::mutex> lock(sv->mu);
	auto it = sv->jobs.find(id);
	if (it == sv->jobs.end()) return AQH_EINVAL;
	fill_info(it->second.get(), info);
	return it->second->state >= 2 ? it->second->status : AQH_ENOTREADY;
}

aqh_status aqh_server_wait(aqh_server* sv, int64_t id, int timeout_ms, aqh_job_info* info) {
	if (!sv) return AQH_EINVAL;
	std::unique_lock<std::mutex> lock(sv->mu);
	auto it = sv->jobs.find(id);
	if (it == sv->jobs.end()) return AQH_EINVAL;
	Job* job = it->second.get();
	const bool done = sv->cv_done.wait_for(lock, std::chrono::milliseconds(std::max(0, timeout_ms)),
	                                       [&] { return job->state >= 2; });
	fill_info(job, info);
	if (!done) return AQH_ETIMEDOUT;
	return job->status;
}

aqh_status aqh_server_cancel(aqh_server* sv, int64_t id) {
	if (!sv) return AQH_EINVAL;
	std::lock_guard<std::mutex> lock(sv->mu);
	auto it = sv->jobs.find(id);
	if (it == sv->jobs.end()) return AQH_EINVAL;
	Job* job = it->second.get();
	if (job->state != 0) return AQH_ENOTREADY;  // already admitted: runs to completion
	sv->pending.erase(std::find(sv->pending.begin(), sv->pending.end(), job));
	job->state = 4;
	job->status = AQH_EREJECTED;
	job->t_done = sv->now();
	sv->cv_done.notify_all();
	return AQH_OK;
}

const char* aqh_server_job_error(aqh_server* sv, int64_t id) {
	if (!sv) return "null server";
	std::lock_guard<std::mutex> lock(sv->mu);
	auto it = sv->jobs.find(id);
	return it == sv->jobs.end() ? "unknown job" : it->second->error.c_str();
}

aqh_status aqh_server_stats(aqh_server* sv, aqh_server_info* info) {
	if (!sv || !info) return AQH_EINVAL;
	std::lock_guard<std::mutex> lock(sv->mu);
	info->budget = sv->opts.hbm_budget;
	info->in_use = sv->in_use;
	info->peak_in_use = sv->peak_in_use;
	info->pending = (int64_t)sv->pending.size();
	info->running = sv->running;
	info->peak_running = sv->peak_running;
	info->graphs_built = info->rerenders = 0;
	for (aqh_ctx* c : sv->ctx) {
		aqh_frame_stats fs{};
		aqh_get_stats(c, &fs);
		info->graphs_built += fs.graphs_built;
		info->rerenders += fs.rerenders;
	}
	info->completed = sv->completed;
	return AQH_OK;
}

}  // extern "C"
