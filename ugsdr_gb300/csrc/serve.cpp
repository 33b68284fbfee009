// Continuous-batching acquisition and tracking server (ugsdr_server_*).
//
// `max_inflight` slots, each with two CUDA streams (normal and highest
// priority), its own scratch workspace and pinned host staging.  Requests
// queue on submit.  The admission thread picks a pending request (the oldest,
// or under the response-ratio policy the one with the largest
// (wait + service) / service), reserves a free slot if the request's
// device-memory estimate fits the budget (releasing idle slots' scratch first
// if needed), and launches it on the slot's stream — short searches on the
// high-priority one — with the server lock released.  The retirement thread
// polls the slots' completion events and turns finished cells into results.
// Admitted searches therefore overlap on the device while new requests keep
// arriving, and completions are seen while long searches are still being
// launched.  Code spectra are the context's resident cache, shared by every
// request.  Tracking requests advance a bank (its channels' loop and NCO
// state stay on the device between requests); a bank's requests are admitted
// one at a time, in submission order.
#include "internal.hpp"

#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <list>
#include <set>
#include <thread>

using namespace ugsdr_gpu;

namespace {
	// estimated service below which a search is short: it runs on a slot's
	// high-priority stream and may take the slot kept for short requests —
	// the served stream's latency target (p99 below 20 ms), so a request that
	// can meet it is never queued behind longer ones
	constexpr double kUrgentSeconds = 0.02;

	// Pinned host staging that grows without freeing while the server runs
	// (cudaFreeHost waits for the device); outgrown buffers are freed at exit.
	struct PinnedBuf {
		void* ptr = nullptr;
		size_t bytes = 0;
		std::vector<void*> outgrown;
		void reserve(size_t n) {
			if (n <= bytes)
				return;
			if (ptr)
				outgrown.push_back(ptr);
			ptr = nullptr;
			bytes = 0;
			if (cudaHostAlloc(&ptr, n, cudaHostAllocDefault) != cudaSuccess) {
				cudaGetLastError();
				ptr = nullptr;
				throw Error(UGSDR_E_NOMEM, "pinned host allocation failed");
			}
			bytes = n;
		}
		~PinnedBuf() {
			for (void* p : outgrown)
				cudaFreeHost(p);
			if (ptr)
				cudaFreeHost(ptr);
		}
	};

	// tracking work per second, in the acquisition estimate's units (cell-blocks):
	// channel-samples count a tenth of a cell-block each
	constexpr double kTrackWorkPerChannelSample = 0.1;

	struct Request {
		uint64_t ticket = 0;
		int kind = 0;               // 0 acquisition job, 1 tracking run of `bank`
		ugsdr_track_bank* bank = nullptr;
		int n_epochs = 0, track_type = 0;
		ugsdr_track_output* outputs = nullptr;  // caller's host array (tracking)
		size_t sample_bytes = 0, out_bytes = 0;
		ugsdr_acq_job job{};
		std::vector<int> codes;
		std::vector<char> samples;  // host copy (empty for device-resident samples)
		size_t estimate = 0;   // device bytes
		double work = 0;       // cell-blocks: codes x Doppler bins x N x K
		std::chrono::steady_clock::time_point queued;
		std::vector<ugsdr_acq_result> results;
		bool done = false;
		int status = UGSDR_OK;
		std::string error;
	};

	struct Slot {
		cudaStream_t stream = nullptr;   // normal priority
		cudaStream_t urgent = nullptr;   // highest priority (short searches under the response-ratio policy)
		cudaStream_t active = nullptr;   // the one the current job runs on
		cudaEvent_t event = nullptr;
		Workspace ws;
		PinnedBuf samples, cells;
		Request* req = nullptr;
		bool enqueuing = false;  // the worker is launching req's work (server lock released)
		EnqueuedBatch batch;
	};

	size_t sample_size(int type) {
		switch (type) {
		case UGSDR_SAMPLES_CF32: return 8;
		case UGSDR_SAMPLES_CI8: return 2;
		case UGSDR_SAMPLES_CI16: return 4;
		default: return 1;
		}
	}
}

struct ugsdr_server {
	ugsdr_ctx* ctx = nullptr;
	ugsdr_server_config cfg{};
	std::list<Slot> slots;  // stable addresses; slots own non-movable device buffers
	std::deque<Request*> pending;
	std::map<uint64_t, std::unique_ptr<Request>> requests;
	uint64_t next_ticket = 1;
	std::mutex mu;
	std::condition_variable cv_work, cv_done, cv_reap;
	std::thread worker, reaper;
	bool stop = false;
	size_t budget = 0;
	ugsdr_server_stats stats{};
	std::chrono::steady_clock::time_point busy_since;
	double done_work = 0;  // cell-blocks completed (throughput estimate with stats.busy_seconds)
	// UGSDR_SERVER_TRACE=1: one stderr line per admission and retirement (times in ms since creation)
	bool trace = std::getenv("UGSDR_SERVER_TRACE") != nullptr;
	std::chrono::steady_clock::time_point created = std::chrono::steady_clock::now();
	double since() const { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - created).count(); }
	std::set<ugsdr_track_bank*> busy_banks;  // banks with a request on the device

	// a tracking request may start only when its bank is idle and no earlier
	// request of the bank is still pending
	bool eligible(std::deque<Request*>::iterator it) {
		const Request* r = *it;
		if (r->kind == 0)
			return true;
		if (busy_banks.count(r->bank))
			return false;
		for (auto j = pending.begin(); j != it; ++j)
			if ((*j)->kind == 1 && (*j)->bank == r->bank)
				return false;
		return true;
	}

	// measured cell-blocks per second (a first guess until work has completed)
	double rate() const { return stats.busy_seconds > 0.05 && done_work > 0 ? done_work / stats.busy_seconds : 5e10; }

	// the pending request to admit next under cfg.policy (short_only: among
	// requests estimated below kUrgentSeconds of service)
	std::deque<Request*>::iterator pick(bool short_only) {
		const double rate = this->rate();
		auto admissible = [&](std::deque<Request*>::iterator it) {
			return eligible(it) && (!short_only || (*it)->work / rate < kUrgentSeconds);
		};
		if (cfg.policy != UGSDR_SERVE_RESPONSE_RATIO || pending.size() < 2) {
			for (auto it = pending.begin(); it != pending.end(); ++it)
				if (admissible(it))
					return it;
			return pending.end();
		}
		const auto now = std::chrono::steady_clock::now();
		auto best = pending.end();
		double best_ratio = -1;
		for (auto it = pending.begin(); it != pending.end(); ++it) {
			if (!admissible(it))
				continue;
			const double service = std::max((*it)->work / rate, 1e-4);
			const double wait = std::chrono::duration<double>(now - (*it)->queued).count();
			const double ratio = (wait + service) / service;
			if (ratio > best_ratio) {  // ties keep arrival order
				best_ratio = ratio;
				best = it;
			}
		}
		return best;
	}

	size_t held() const {
		size_t s = 0;
		for (const auto& sl : slots)
			s += sl.ws.reserved();
		return s;
	}

	void fail(Request* r, int status, const std::string& msg) {
		r->status = status;
		r->error = msg;
		r->done = true;
		++stats.failed;
		cv_done.notify_all();
	}

	// retire slots whose event fired; true if any did
	bool retire() {
		bool any = false;
		for (auto& sl : slots) {
			if (!sl.req || sl.enqueuing)
				continue;
			const cudaError_t q = cudaEventQuery(sl.event);
			if (q == cudaErrorNotReady)
				continue;
			Request* r = sl.req;
			sl.req = nullptr;
			any = true;
			--stats.inflight;
			if (stats.inflight == 0)
				stats.busy_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - busy_since).count();
			if (q != cudaSuccess) {
				cudaGetLastError();
				fail(r, UGSDR_E_CUDA, cudaGetErrorString(q));
				if (r->kind == 1)
					busy_banks.erase(r->bank);
				continue;
			}
			if (r->kind == 1) {
				std::memcpy(r->outputs, sl.cells.ptr, r->out_bytes);
				busy_banks.erase(r->bank);
				r->done = true;
				done_work += r->work;
				++stats.completed;
				cv_done.notify_all();
				continue;
			}
			r->results.resize(r->job.n_codes);
			ugsdr_acq_result* rp = r->results.data();
			finish_jobs(sl.batch, &r->job, 1, sl.cells.ptr, &rp, nullptr);
			r->done = true;
			done_work += r->work;
			if (trace)
				std::fprintf(stderr, "[serve] %.1f retire ticket %llu\n", since(), static_cast<unsigned long long>(r->ticket));
			++stats.completed;
			cv_done.notify_all();
		}
		return any;
	}

	// admit the oldest pending request if a slot and memory allow; true if admitted
	// Admits one request if a slot and memory allow; true if one was admitted
	// (or failed).  The launches run with the server lock released: polls,
	// submissions and retirement proceed while a long search is enqueued.
	bool admit(std::unique_lock<std::mutex>& lock) {
		if (pending.empty())
			return false;
		// under the response-ratio policy the last slot takes only short
		// requests (estimated service below kUrgentSeconds), so a queue of long
		// searches cannot hold every slot while short ones wait
		const bool reserve = cfg.policy == UGSDR_SERVE_RESPONSE_RATIO && slots.size() >= 2;
		Slot* free_general = nullptr;
		Slot* free_short = nullptr;
		for (auto& sl : slots) {
			if (sl.req)
				continue;
			if (reserve && &sl == &slots.back())
				free_short = &sl;
			else if (!free_general)
				free_general = &sl;
		}
		Slot* free_slot = free_general;
		auto pos = free_general ? pick(false) : pending.end();
		if (pos == pending.end() && free_short) {
			free_slot = free_short;
			pos = pick(true);
		}
		if (!free_slot)
			return false;
		if (pos == pending.end())
			return false;  // only tracking requests whose bank is busy
		Request* r = *pos;
		const size_t grow = r->estimate > free_slot->ws.reserved() ? r->estimate - free_slot->ws.reserved() : 0;
		if (held() + grow > budget) {
			// give back scratch of idle slots before waiting
			for (auto& sl : slots)
				if (!sl.req && &sl != free_slot)
					sl.ws.release();
			if (held() + grow > budget) {
				if (stats.inflight == 0) {
					pending.erase(pos);
					fail(r, UGSDR_E_NOMEM, "job needs " + std::to_string(r->estimate) + " device bytes, budget " + std::to_string(budget));
					return true;
				}
				return false;  // wait for running jobs to finish
			}
		}
		pending.erase(pos);
		const double t_admit = trace ? since() : 0.0;
		// reserve the slot, then launch without the server lock
		free_slot->req = r;
		free_slot->enqueuing = true;
		if (stats.inflight == 0)
			busy_since = std::chrono::steady_clock::now();
		++stats.inflight;
		stats.max_inflight_seen = std::max(stats.max_inflight_seen, stats.inflight);
		const bool urgent = cfg.policy == UGSDR_SERVE_RESPONSE_RATIO && r->work / rate() < kUrgentSeconds;
		if (r->kind == 1)
			busy_banks.insert(r->bank);
		lock.unlock();
		int fail_status = UGSDR_OK;
		std::string fail_msg;
		try {
			if (r->kind == 1) {
				// tracking: samples in through the slot's pinned and device
				// buffers, the bank's run, outputs back to pinned staging
				std::lock_guard<std::mutex> ctx_lock(ctx->mutex);
				free_slot->active = free_slot->stream;
				free_slot->ws.set_stream(free_slot->active);
				free_slot->samples.reserve(r->sample_bytes);
				std::memcpy(free_slot->samples.ptr, r->samples.data(), r->sample_bytes);
				free_slot->ws.samples.reserve(r->sample_bytes);
				free_slot->ws.cells.reserve(r->out_bytes);
				free_slot->cells.reserve(r->out_bytes);
				UG_CUDA(cudaMemcpyAsync(free_slot->ws.samples.ptr, free_slot->samples.ptr, r->sample_bytes, cudaMemcpyHostToDevice,
					free_slot->active));
				track_enqueue_on(r->bank, free_slot->ws.samples.ptr, r->track_type, r->n_epochs,
					free_slot->ws.cells.as<ugsdr_track_output>(), free_slot->active);
				UG_CUDA(cudaMemcpyAsync(free_slot->cells.ptr, free_slot->ws.cells.ptr, r->out_bytes, cudaMemcpyDeviceToHost,
					free_slot->active));
				UG_CUDA(cudaEventRecord(free_slot->event, free_slot->active));
			}
			else {
			ugsdr_acq_job job = r->job;
			job.codes = r->codes.data();
			if (!job.samples_on_device) {
				free_slot->samples.reserve(r->samples.size());
				std::memcpy(free_slot->samples.ptr, r->samples.data(), r->samples.size());
				job.samples = free_slot->samples.ptr;
			}
			size_t n_cells = 0;
			{
				std::lock_guard<std::mutex> ctx_lock(ctx->mutex);
				// cells: one record per (code, Doppler bin)
				n_cells = static_cast<size_t>(job.n_codes) * doppler_grid(job.doppler_range, job.doppler_step).size();
				free_slot->cells.reserve(16 * std::max<size_t>(n_cells, 1));
				// short searches run on the high-priority stream: the device
				// dispatches their CTAs ahead of the long jobs' (kUrgentSeconds of
				// estimated service); the slot's scratch follows the stream
				free_slot->active = urgent ? free_slot->urgent : free_slot->stream;
				free_slot->ws.set_stream(free_slot->active);
				free_slot->batch = enqueue_jobs(ctx, free_slot->ws, free_slot->active, &job, 1, free_slot->cells.ptr);
				UG_CUDA(cudaEventRecord(free_slot->event, free_slot->active));
				if (trace)
					std::fprintf(stderr, "[serve] %.1f admit ticket %llu work %.3g urgent %d enqueue %.1f ms\n", t_admit,
						static_cast<unsigned long long>(r->ticket), r->work, urgent ? 1 : 0, since() - t_admit);
			}
			r->job.codes = r->codes.data();
			}
		}
		catch (const Error& e) {
			fail_status = e.status;
			fail_msg = e.what();
		}
		catch (const std::exception& e) {
			fail_status = UGSDR_E_INVALID;
			fail_msg = e.what();
		}
		lock.lock();
		free_slot->enqueuing = false;
		// the retirement thread sleeps 5 ms while nothing is in flight: wake it
		// to poll this slot (a short search completes in well under that)
		cv_reap.notify_one();
		if (fail_status != UGSDR_OK) {
			if (r->kind == 1)
				busy_banks.erase(r->bank);
			free_slot->req = nullptr;
			if (--stats.inflight == 0)
				stats.busy_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - busy_since).count();
			fail(r, fail_status, fail_msg);
		}
		return true;
	}

	// Admission thread: admits and launches while a slot and memory allow,
	// otherwise sleeps until a submission or a retirement.
	void run() {
		cudaSetDevice(ctx->device);
		std::unique_lock<std::mutex> lock(mu);
		while (!stop) {
			bool progress = false;
			while (!stop && admit(lock))
				progress = true;
			stats.device_bytes = held();
			if (!progress)
				cv_work.wait_for(lock, std::chrono::milliseconds(5));
		}
	}

	// Retirement thread: polls the slots' completion events (every 50 us while
	// work is in flight), so completions are seen while the admission thread
	// is still launching a long search.
	void reap() {
		cudaSetDevice(ctx->device);
		std::unique_lock<std::mutex> lock(mu);
		while (!stop) {
			if (retire())
				cv_work.notify_all();
			if (stats.inflight > 0)
				cv_reap.wait_for(lock, std::chrono::microseconds(50));
			else
				cv_reap.wait_for(lock, std::chrono::milliseconds(5));
		}
	}
};

extern "C" {

int ugsdr_server_create(ugsdr_ctx* ctx, const ugsdr_server_config* cfg, ugsdr_server** server) {
	if (!ctx || !server)
		return UGSDR_E_INVALID;
	*server = nullptr;
	return guarded(ctx, [&] {
		auto s = std::make_unique<ugsdr_server>();
		s->ctx = ctx;
		if (cfg)
			s->cfg = *cfg;
		if (s->cfg.max_inflight <= 0)
			s->cfg.max_inflight = 4;
		if (s->cfg.queue_capacity <= 0)
			s->cfg.queue_capacity = 1024;
		require(s->cfg.policy == UGSDR_SERVE_FIFO || s->cfg.policy == UGSDR_SERVE_RESPONSE_RATIO, "unknown serving policy");
		require(s->cfg.max_inflight <= 64, "max_inflight above 64");
		UG_CUDA(cudaSetDevice(ctx->device));
		if (s->cfg.memory_budget) {
			s->budget = s->cfg.memory_budget;
		}
		else {
			size_t free_b = 0, total = 0;
			UG_CUDA(cudaMemGetInfo(&free_b, &total));
			s->budget = free_b / 10 * 8;
		}
		for (int i = 0; i < s->cfg.max_inflight; ++i)
			s->slots.emplace_back();
		int least = 0, greatest = 0;
		UG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
		for (auto& sl : s->slots) {
			UG_CUDA(cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, least));
			UG_CUDA(cudaStreamCreateWithPriority(&sl.urgent, cudaStreamNonBlocking, greatest));
			UG_CUDA(cudaEventCreateWithFlags(&sl.event, cudaEventDisableTiming));
			sl.active = sl.stream;
			sl.ws.set_stream(sl.stream);  // scratch grows stream-ordered, without a device-wide wait
		}
		ugsdr_server* raw = s.get();
		s->worker = std::thread([raw] { raw->run(); });
		s->reaper = std::thread([raw] { raw->reap(); });
		*server = s.release();
	});
}

int ugsdr_server_submit(ugsdr_server* server, const ugsdr_acq_job* job, uint64_t* ticket) {
	if (!server || !job || !ticket)
		return UGSDR_E_INVALID;
	ugsdr_ctx* ctx = server->ctx;
	auto r = std::make_unique<Request>();
	const int st = guarded(ctx, [&] {
		require(job->codes && job->n_codes > 0 && job->samples, "job without codes or samples");
		r->job = *job;
		r->codes.assign(job->codes, job->codes + job->n_codes);
		r->job.codes = r->codes.data();
		if (!job->samples_on_device) {
			const size_t bytes = sample_size(job->sample_type) * job->n_samples;
			r->samples.assign(static_cast<const char*>(job->samples), static_cast<const char*>(job->samples) + bytes);
			r->job.samples = r->samples.data();
		}
		std::lock_guard<std::mutex> lock(ctx->mutex);
		r->estimate = jobs_device_bytes(ctx, &r->job, 1);  // validates the job too
		r->work = static_cast<double>(r->job.n_codes) * doppler_grid(r->job.doppler_range, r->job.doppler_step).size() *
			static_cast<double>(r->job.block_samples) * static_cast<double>(r->job.n_blocks);
	});
	if (st != UGSDR_OK)
		return st;
	std::lock_guard<std::mutex> lock(server->mu);
	if (static_cast<int>(server->pending.size()) >= server->cfg.queue_capacity) {
		ctx->last_error = "serving queue is full";
		return UGSDR_E_QUEUE_FULL;
	}
	r->ticket = server->next_ticket++;
	r->queued = std::chrono::steady_clock::now();
	*ticket = r->ticket;
	if (server->trace)
		std::fprintf(stderr, "[serve] %.1f submit ticket %llu work %.3g\n", server->since(),
			static_cast<unsigned long long>(r->ticket), r->work);
	server->pending.push_back(r.get());
	server->requests[r->ticket] = std::move(r);
	++server->stats.submitted;
	server->cv_work.notify_one();
	return UGSDR_OK;
}

int ugsdr_server_submit_track(ugsdr_server* server, ugsdr_track_bank* bank, const void* samples, int sample_type,
	size_t samples_per_epoch, int n_epochs, ugsdr_track_output* outputs, uint64_t* ticket) {
	if (!server || !bank || !ticket)
		return UGSDR_E_INVALID;
	ugsdr_ctx* ctx = server->ctx;
	auto r = std::make_unique<Request>();
	const int st = guarded(ctx, [&] {
		ugsdr_ctx* bank_ctx = nullptr;
		int n_ch = 0;
		size_t spm = 0;
		double fs = 0;
		track_bank_shape(bank, &bank_ctx, &n_ch, &spm, &fs);
		require(bank_ctx == ctx, "the bank belongs to another context");
		require(samples && outputs && n_epochs > 0, "null samples or outputs, or no epochs");
		require(samples_per_epoch == spm, "samples_per_epoch must be the bank's sampling_rate / 1000");
		require(sample_type >= UGSDR_SAMPLES_CF32 && sample_type <= UGSDR_SAMPLES_RI8,
			"served tracking takes CF32, CI8, CI16 or RI8 samples");
		r->kind = 1;
		r->bank = bank;
		r->n_epochs = n_epochs;
		r->track_type = sample_type;
		r->outputs = outputs;
		r->sample_bytes = sample_size(sample_type) * spm * static_cast<size_t>(n_epochs);
		r->out_bytes = sizeof(ugsdr_track_output) * static_cast<size_t>(n_ch) * n_epochs;
		r->samples.assign(static_cast<const char*>(samples), static_cast<const char*>(samples) + r->sample_bytes);
		r->estimate = (r->sample_bytes + 255) / 256 * 256 + (r->out_bytes + 255) / 256 * 256;
		r->work = kTrackWorkPerChannelSample * static_cast<double>(n_ch) * static_cast<double>(spm) * n_epochs;
	});
	if (st != UGSDR_OK)
		return st;
	std::lock_guard<std::mutex> lock(server->mu);
	if (static_cast<int>(server->pending.size()) >= server->cfg.queue_capacity) {
		ctx->last_error = "serving queue is full";
		return UGSDR_E_QUEUE_FULL;
	}
	r->ticket = server->next_ticket++;
	r->queued = std::chrono::steady_clock::now();
	*ticket = r->ticket;
	server->pending.push_back(r.get());
	server->requests[r->ticket] = std::move(r);
	++server->stats.submitted;
	server->cv_work.notify_one();
	return UGSDR_OK;
}

int ugsdr_server_poll(ugsdr_server* server, uint64_t ticket, ugsdr_acq_result* results, int* done) {
	if (!server || !done)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(server->mu);
	auto it = server->requests.find(ticket);
	if (it == server->requests.end()) {
		server->ctx->last_error = "unknown ticket";
		return UGSDR_E_NOT_FOUND;
	}
	Request* r = it->second.get();
	*done = r->done ? 1 : 0;
	if (!r->done)
		return UGSDR_OK;
	const int st = r->status;
	if (st == UGSDR_OK && results)
		std::memcpy(results, r->results.data(), sizeof(ugsdr_acq_result) * r->results.size());
	if (st != UGSDR_OK)
		server->ctx->last_error = r->error;
	server->requests.erase(it);
	return st;
}

int ugsdr_server_drain(ugsdr_server* server) {
	if (!server)
		return UGSDR_E_INVALID;
	std::unique_lock<std::mutex> lock(server->mu);
	server->cv_done.wait(lock, [&] {
		for (const auto& kv : server->requests)
			if (!kv.second->done)
				return false;
		return true;
	});
	return UGSDR_OK;
}

int ugsdr_server_get_stats(ugsdr_server* server, ugsdr_server_stats* stats) {
	if (!server || !stats)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(server->mu);
	*stats = server->stats;
	return UGSDR_OK;
}

int ugsdr_server_destroy(ugsdr_server* server) {
	if (!server)
		return UGSDR_E_INVALID;
	{
		std::lock_guard<std::mutex> lock(server->mu);
		server->stop = true;
		server->cv_work.notify_all();
	}
	server->cv_reap.notify_all();
	if (server->worker.joinable())
		server->worker.join();
	if (server->reaper.joinable())
		server->reaper.join();
	for (auto& sl : server->slots) {
		sl.ws.release();  // stream-ordered frees, before the streams go
		for (cudaStream_t st : {sl.stream, sl.urgent})
			if (st)
				cudaStreamSynchronize(st);
		sl.ws.set_stream(nullptr);
		if (sl.event)
			cudaEventDestroy(sl.event);
		for (cudaStream_t st : {sl.stream, sl.urgent})
			if (st)
				cudaStreamDestroy(st);
	}
	delete server;
	return UGSDR_OK;
}
}
