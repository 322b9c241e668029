// The serving loop behind kdn_serve_*: resident scenes, a queue of requests
// admitted against free slots and a device-memory budget, worker threads
// that draw each request on a context sharing its scene's world (so frames
// of any scenes run side by side on the device, each on its own streams),
// progressive sessions whose accumulation and denoiser history stay
// resident on their own context, and the latency of every request.
//
// The reference's counterpart is the render host's request loop
// (core/plugin.h:241 hostRenderer with the viewer's progressive frames);
// it draws one frame at a time, this one as many as there are slots.
#include "kdn.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

// Device bytes a path takes in a frame's buffers (render.cpp kPathBytes),
// and a pixel's (sums, record, G-buffer, temporal state, image: 128; the
// surfaces pass's own queue, states and hits: 116).
constexpr uint64_t kPathBytes  = 420;
constexpr uint64_t kPixelBytes = 128 + 116;
// Stream priority of interactive requests (lower is more urgent; clamped
// to the device's range by kdn_open_sharing).
constexpr int kInteractivePriority = -8;
// March steps a ray takes in one trace launch (kdn_set_march_budget) of an
// interactive and of a batch request's frames
constexpr uint32_t kInteractiveMarchBudget = 64;
constexpr uint32_t kBatchMarchBudget       = 1024;

struct Job {
	uint64_t ticket = 0;
	kdn_request request {};
	float* out = nullptr;
	Clock::time_point submitted, started, finished;
	uint64_t need     = 0;
	uint32_t frame    = 0;
	kdn_status status = KDN_OK;
	bool done         = false;
};

struct Session {
	uint32_t scene   = 0;
	kdn_ctx* ctx     = nullptr;
	bool interactive = false; // the priority its context was opened at
	uint32_t frames  = 0;     // frames admitted so far
	uint32_t pending = 0;     // frames submitted and not yet done
	bool busy        = false;
	bool ended       = false;
};

struct Scene {
	kdn_ctx* ctx = nullptr;
	std::vector<kdn_ctx*> idle[2]; // contexts sharing its world: [0] normal, [1] interactive priority
};

} // namespace

struct kdn_server {
	int device        = 0;
	uint32_t slots    = 1;
	uint64_t budget   = 0;
	uint64_t slotCap  = 0; // the most path-buffer bytes one interactive request takes
	uint32_t batchSlots   = 1;
	uint32_t batchSms     = 0; // SMs a batch request's grids are sized for
	uint64_t batchCap     = 0; // the most path-buffer bytes one batch request takes
	int sms           = 0; // the device's SMs
	std::mutex m;
	std::condition_variable work, finished;
	std::vector<Scene> scenes;
	std::map<uint64_t, Session> sessions;
	std::deque<Job*> queue;
	std::map<uint64_t, std::unique_ptr<Job>> jobs;
	uint64_t nextTicket = 1;
	uint64_t inUse      = 0;
	uint32_t running      = 0;
	uint32_t runningBatch = 0; // of them not interactive
	uint32_t alive        = 0; // contexts opened and not closed
	bool closing        = false;
	std::vector<double> latencies, interactiveLatencies;
	std::string error;
	std::vector<std::thread> workers;

	kdn_status fail(kdn_status s, const std::string& message) {
		error = message;
		return s;
	}
};

namespace {

bool interactiveOf(const Job* j) { return (j->request.flags & KDN_REQUEST_INTERACTIVE) != 0; }

// The request that may start now: interactive requests first, then the
// rest, each oldest first; a slot is free (with more than one slot, one is
// kept for interactive requests), its session (if any) has no frame on the
// device, and its buffers fit in what the running requests leave of the
// budget (one request is always let in).
Job* admitted(kdn_server* S) {
	if (S->running >= S->slots) return nullptr;
	const bool batchRoom = S->runningBatch < S->batchSlots;
	for (int pass = 0; pass < 2; ++pass) {
		const bool wantInteractive = pass == 0;
		if (!wantInteractive && !batchRoom) break;
		for (auto it = S->queue.begin(); it != S->queue.end(); ++it) {
			Job* j = *it;
			if (interactiveOf(j) != wantInteractive) continue;
			Session* session = j->request.session ? &S->sessions[j->request.session] : nullptr;
			if (session != nullptr && session->busy) continue;
			if (S->running > 0 && S->inUse + j->need > S->budget) continue;
			S->queue.erase(it);
			S->inUse += j->need;
			S->running += 1;
			if (!wantInteractive) S->runningBatch += 1;
			if (session != nullptr) {
				session->busy = true;
				j->frame      = session->frames++;
			}
			return j;
		}
	}
	return nullptr;
}

// Close one idle context of the pools (to make room for another scene's).
bool closeOneIdle(kdn_server* S) {
	for (Scene& scene : S->scenes) {
		for (auto& pool : scene.idle) {
			if (pool.empty()) continue;
			kdn_close(pool.back());
			pool.pop_back();
			S->alive -= 1;
			return true;
		}
	}
	return false;
}

// A finished or ended session's context goes back to its scene's pool.
void retireSession(kdn_server* S, uint64_t id) {
	auto it = S->sessions.find(id);
	if (it == S->sessions.end()) return;
	Session& s = it->second;
	if (!s.ended || s.busy || s.pending > 0) return;
	if (s.ctx != nullptr) S->scenes[s.scene].idle[s.interactive ? 1 : 0].push_back(s.ctx);
	S->sessions.erase(it);
}

void serveLoop(kdn_server* S) {
	std::unique_lock<std::mutex> lock(S->m);
	for (;;) {
		Job* job = nullptr;
		while (!S->closing && (job = admitted(S)) == nullptr) S->work.wait(lock);
		if (job == nullptr) return;
		const bool interactive = interactiveOf(job);
		const uint64_t sessionId = job->request.session;
		const uint32_t sceneId = job->request.scene; // (scenes may grow meanwhile: index it under the lock)
		std::vector<kdn_ctx*>& pool = S->scenes[sceneId].idle[interactive ? 1 : 0];
		kdn_ctx* ctx = nullptr;
		bool fresh   = false;
		if (sessionId != 0) {
			ctx = S->sessions[sessionId].ctx;
		} else if (!pool.empty()) {
			ctx = pool.back();
			pool.pop_back();
		}
		if (ctx == nullptr) {
			// room for one more context: at most one a slot beside the sessions'
			while (S->alive >= S->slots + S->sessions.size() && closeOneIdle(S)) {
			}
			S->alive += 1;
			fresh = true;
		}
		kdn_ctx* sceneCtx = S->scenes[sceneId].ctx;
		job->started      = Clock::now();
		lock.unlock();

		kdn_status status = KDN_OK;
		std::string why;
		if (fresh) {
			status = kdn_open_sharing(sceneCtx, interactive ? kInteractivePriority : 0, &ctx);
			if (status == KDN_OK) status = kdn_set_frame_budget(ctx, S->slotCap);
			// batch frames: short chunks on their share of the SMs
			if (status == KDN_OK && !interactive) status = kdn_set_frame_budget(ctx, S->batchCap);
			if (status == KDN_OK && !interactive && S->slots > 1 && S->batchSms > 0) status = kdn_set_sm_limit(ctx, int(S->batchSms));
			// short trace launches: an interactive frame waits on no ray that
			// skims a surface, and a batch frame hands its SMs back often
			// (frames are the same to the bit with any budget)
			if (status == KDN_OK) status = kdn_set_march_budget(ctx, interactive ? kInteractiveMarchBudget : kBatchMarchBudget);
			if (status != KDN_OK) why = kdn_last_error(sceneCtx);
		}
		if (status == KDN_OK) {
			kdn_frame frame {};
			frame.width      = job->request.width;
			frame.height     = job->request.height;
			frame.samples    = job->request.samples;
			frame.surfaces   = job->request.surfaces;
			frame.seed       = job->request.seed;
			frame.first      = sessionId != 0 ? job->frame * uint32_t(std::max(job->request.samples, 0)) : 0;
			frame.accumulate = sessionId != 0 && job->frame > 0 ? 1 : 0;
			// a single frame, or a session's first, starts without history
			frame.flags = (job->request.flags & KDN_FRAME_DENOISE) | (frame.accumulate ? 0u : KDN_FRAME_RESTART);
			status      = kdn_render(ctx, &frame, job->out);
			if (status != KDN_OK) why = kdn_last_error(ctx);
		}
		job->finished = Clock::now();

		lock.lock();
		if (fresh && status != KDN_OK && ctx == nullptr) S->alive -= 1;
		if (sessionId != 0) {
			Session& s = S->sessions[sessionId];
			if (s.ctx == nullptr && ctx != nullptr) {
				s.ctx         = ctx;
				s.interactive = interactive;
			}
			s.busy = false;
			s.pending -= 1;
			retireSession(S, sessionId);
		} else if (ctx != nullptr) {
			S->scenes[sceneId].idle[interactive ? 1 : 0].push_back(ctx);
		}
		S->inUse -= job->need;
		S->running -= 1;
		if (!interactive) S->runningBatch -= 1;
		job->status = status;
		job->done   = true;
		if (status != KDN_OK) S->error = "request " + std::to_string(job->ticket) + ": " + why;
		S->finished.notify_all();
		S->work.notify_all();
	}
}

double percentile(std::vector<double> v, double p) {
	if (v.empty()) return 0;
	std::sort(v.begin(), v.end());
	const size_t rank = size_t(std::ceil(p * double(v.size())));
	return v[std::min(v.size() - 1, rank == 0 ? 0 : rank - 1)];
}

} // namespace

extern "C" {

kdn_status kdn_serve_open(const kdn_serve_options* options, kdn_server** out) {
	if (options == nullptr || out == nullptr) return KDN_BAD_ARG;
	*out = nullptr;
	if (options->slots == 0 || options->slots > 64) return KDN_BAD_ARG;
	kdn_server* S = new (std::nothrow) kdn_server();
	if (S == nullptr) return KDN_OOM;
	S->device  = options->device;
	S->slots   = options->slots;
	S->budget  = options->budget_bytes ? options->budget_bytes : uint64_t(120) << 30;
	S->slotCap = std::max<uint64_t>(S->budget / S->slots, uint64_t(64) << 20);
	S->batchSlots = options->batch_slots ? std::min(options->batch_slots, S->slots) : std::max<uint32_t>(1, S->slots / 4);
	S->batchCap   = std::min<uint64_t>(S->slotCap, options->batch_frame_bytes ? options->batch_frame_bytes : uint64_t(1) << 30);
	if (S->device >= 0 && cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, S->device) != cudaSuccess) {
		cudaGetLastError();
		S->sms = 0;
	}
	const uint32_t percent = options->batch_sm_percent ? std::min<uint32_t>(options->batch_sm_percent, 100) : 50;
	S->batchSms = std::max<uint32_t>(1, uint32_t(S->sms) * percent / 100 / S->batchSlots);
	for (uint32_t k = 0; k < S->slots; ++k) S->workers.emplace_back(serveLoop, S);
	*out = S;
	return KDN_OK;
}

kdn_status kdn_serve_add_scene(kdn_server* S, kdn_ctx* scene, uint32_t* id) {
	if (S == nullptr || scene == nullptr || id == nullptr) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(S->m);
	Scene entry;
	entry.ctx = scene;
	S->scenes.push_back(entry);
	*id = uint32_t(S->scenes.size() - 1);
	return KDN_OK;
}

kdn_status kdn_serve_submit(kdn_server* S, const kdn_request* request, float* out_rgb, uint64_t* ticket) {
	if (S == nullptr || request == nullptr || out_rgb == nullptr || ticket == nullptr) return KDN_BAD_ARG;
	if (request->width <= 0 || request->height <= 0 || request->samples <= 0 || request->surfaces <= 0) return S->fail(KDN_BAD_ARG, "kdn_serve_submit: a request needs a size, samples and surfaces");
	std::unique_ptr<Job> job(new (std::nothrow) Job());
	if (!job) return KDN_OOM;
	job->request   = *request;
	job->out       = out_rgb;
	job->submitted = Clock::now();
	const uint64_t pixels = uint64_t(request->width) * uint64_t(request->height);
	const uint64_t cap = (request->flags & KDN_REQUEST_INTERACTIVE) ? S->slotCap : S->batchCap;
	job->need = std::min<uint64_t>(pixels * uint64_t(request->samples) * kPathBytes, cap) + pixels * kPixelBytes;
	std::lock_guard<std::mutex> guard(S->m);
	if (S->closing) return S->fail(KDN_BAD_ARG, "kdn_serve_submit: the server is closing");
	if (request->scene >= S->scenes.size()) return S->fail(KDN_BAD_ARG, "kdn_serve_submit: no scene " + std::to_string(request->scene));
	if (request->session != 0) {
		auto it = S->sessions.find(request->session);
		if (it == S->sessions.end()) {
			Session s;
			s.scene = request->scene;
			it      = S->sessions.emplace(request->session, s).first;
		}
		if (it->second.scene != request->scene) return S->fail(KDN_BAD_ARG, "kdn_serve_submit: a session draws one scene");
		if (it->second.ended) return S->fail(KDN_BAD_ARG, "kdn_serve_submit: the session has ended");
		it->second.pending += 1;
	}
	job->ticket = S->nextTicket++;
	*ticket     = job->ticket;
	S->queue.push_back(job.get());
	S->jobs.emplace(job->ticket, std::move(job));
	S->work.notify_one();
	return KDN_OK;
}

kdn_status kdn_serve_wait(kdn_server* S, uint64_t ticket, kdn_served* out) {
	if (S == nullptr || out == nullptr) return KDN_BAD_ARG;
	std::unique_lock<std::mutex> lock(S->m);
	auto it = S->jobs.find(ticket);
	if (it == S->jobs.end()) return S->fail(KDN_BAD_ARG, "kdn_serve_wait: no request " + std::to_string(ticket) + " is waiting");
	Job* job = it->second.get();
	S->finished.wait(lock, [&] { return job->done; });
	const auto ms = [](Clock::duration d) { return std::chrono::duration<double, std::milli>(d).count(); };
	out->status     = job->status;
	out->frame      = job->frame;
	out->queued_ms  = ms(job->started - job->submitted);
	out->render_ms  = ms(job->finished - job->started);
	out->latency_ms = ms(job->finished - job->submitted);
	if (job->status == KDN_OK) {
		S->latencies.push_back(out->latency_ms);
		if (interactiveOf(job)) S->interactiveLatencies.push_back(out->latency_ms);
	}
	const kdn_status status = job->status;
	S->jobs.erase(it);
	return status;
}

kdn_status kdn_serve_cancel_queued(kdn_server* S, uint64_t* cancelled) {
	if (S == nullptr) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(S->m);
	uint64_t n = 0;
	for (Job* j : S->queue) {
		j->status  = KDN_NOT_READY;
		j->done    = true;
		j->started = j->finished = Clock::now();
		if (j->request.session != 0) {
			auto it = S->sessions.find(j->request.session);
			if (it != S->sessions.end()) {
				it->second.pending -= 1;
				retireSession(S, j->request.session);
			}
		}
		n += 1;
	}
	S->queue.clear();
	if (cancelled) *cancelled = n;
	S->finished.notify_all();
	return KDN_OK;
}

kdn_status kdn_serve_end_session(kdn_server* S, uint64_t session) {
	if (S == nullptr || session == 0) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(S->m);
	auto it = S->sessions.find(session);
	if (it == S->sessions.end()) return S->fail(KDN_BAD_ARG, "kdn_serve_end_session: no session " + std::to_string(session));
	it->second.ended = true;
	retireSession(S, session);
	return KDN_OK;
}

kdn_status kdn_serve_latency(kdn_server* S, int interactive_only, double* p50_ms, double* p99_ms, uint64_t* count) {
	if (S == nullptr || p50_ms == nullptr || p99_ms == nullptr || count == nullptr) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(S->m);
	const std::vector<double>& v = interactive_only ? S->interactiveLatencies : S->latencies;
	*p50_ms = percentile(v, 0.50);
	*p99_ms = percentile(v, 0.99);
	*count  = v.size();
	return KDN_OK;
}

kdn_status kdn_serve_reset_latency(kdn_server* S) {
	if (S == nullptr) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(S->m);
	S->latencies.clear();
	S->interactiveLatencies.clear();
	return KDN_OK;
}

const char* kdn_serve_last_error(const kdn_server* S) { return S ? S->error.c_str() : "no server"; }

kdn_status kdn_serve_close(kdn_server* S) {
	if (S == nullptr) return KDN_BAD_ARG;
	{
		std::lock_guard<std::mutex> guard(S->m);
		S->closing = true;
	}
	S->work.notify_all();
	for (std::thread& t : S->workers) t.join();
	// requests still queued are dropped (close after waiting for every ticket)
	S->queue.clear();
	for (auto& [id, s] : S->sessions) {
		if (s.ctx) kdn_close(s.ctx);
	}
	for (Scene& scene : S->scenes) {
		for (auto& pool : scene.idle) {
			for (kdn_ctx* ctx : pool) kdn_close(ctx);
		}
	}
	delete S;
	return KDN_OK;
}

} // extern "C"
