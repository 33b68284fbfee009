// Continuous-batching acquisition server (ugsdr_server_*).
//
// A worker thread owns `max_inflight` slots, each a CUDA stream with its own
// scratch workspace and pinned host staging.  Requests queue on submit; the
// worker admits the oldest pending request whenever a slot is free and the
// request's device-memory estimate fits the budget (releasing idle slots'
// scratch first if needed), enqueues it asynchronously on the slot's stream,
// and retires slots whose completion event fired.  Admitted jobs therefore
// overlap on the device while new requests keep arriving.  Code spectra are
// the context's resident cache, shared by every request.
#include "internal.hpp"

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <thread>

using namespace ugsdr_gpu;

namespace {
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

	struct Request {
		uint64_t ticket = 0;
		ugsdr_acq_job job{};
		std::vector<int> codes;
		std::vector<char> samples;  // host copy (empty for device-resident samples)
		size_t estimate = 0;
		std::vector<ugsdr_acq_result> results;
		bool done = false;
		int status = UGSDR_OK;
		std::string error;
	};

	struct Slot {
		cudaStream_t stream = nullptr;
		cudaEvent_t event = nullptr;
		Workspace ws;
		PinnedBuf samples, cells;
		Request* req = nullptr;
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
	std::condition_variable cv_work, cv_done;
	std::thread worker;
	bool stop = false;
	size_t budget = 0;
	ugsdr_server_stats stats{};
	std::chrono::steady_clock::time_point busy_since;

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
			if (!sl.req)
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
				continue;
			}
			r->results.resize(r->job.n_codes);
			ugsdr_acq_result* rp = r->results.data();
			finish_jobs(sl.batch, &r->job, 1, sl.cells.ptr, &rp, nullptr);
			r->done = true;
			++stats.completed;
			cv_done.notify_all();
		}
		return any;
	}

	// admit the oldest pending request if a slot and memory allow; true if admitted
	bool admit() {
		if (pending.empty())
			return false;
		Slot* free_slot = nullptr;
		for (auto& sl : slots)
			if (!sl.req) {
				free_slot = &sl;
				break;
			}
		if (!free_slot)
			return false;
		Request* r = pending.front();
		const size_t grow = r->estimate > free_slot->ws.reserved() ? r->estimate - free_slot->ws.reserved() : 0;
		if (held() + grow > budget) {
			// give back scratch of idle slots before waiting
			for (auto& sl : slots)
				if (!sl.req && &sl != free_slot)
					sl.ws.release();
			if (held() + grow > budget) {
				if (stats.inflight == 0) {
					pending.pop_front();
					fail(r, UGSDR_E_NOMEM, "job needs " + std::to_string(r->estimate) + " device bytes, budget " + std::to_string(budget));
					return true;
				}
				return false;  // wait for running jobs to finish
			}
		}
		pending.pop_front();
		try {
			ugsdr_acq_job job = r->job;
			job.codes = r->codes.data();
			if (!job.samples_on_device) {
				free_slot->samples.reserve(r->samples.size());
				std::memcpy(free_slot->samples.ptr, r->samples.data(), r->samples.size());
				job.samples = free_slot->samples.ptr;
			}
			size_t n_cells = 0;
			{
				std::lock_guard<std::mutex> lock(ctx->mutex);
				// cells: one record per (code, Doppler bin)
				n_cells = static_cast<size_t>(job.n_codes) * doppler_grid(job.doppler_range, job.doppler_step).size();
				free_slot->cells.reserve(16 * std::max<size_t>(n_cells, 1));
				free_slot->batch = enqueue_jobs(ctx, free_slot->ws, free_slot->stream, &job, 1, free_slot->cells.ptr);
				UG_CUDA(cudaEventRecord(free_slot->event, free_slot->stream));
			}
			r->job.codes = r->codes.data();
			free_slot->req = r;
			if (stats.inflight == 0)
				busy_since = std::chrono::steady_clock::now();
			++stats.inflight;
			stats.max_inflight_seen = std::max(stats.max_inflight_seen, stats.inflight);
		}
		catch (const Error& e) {
			fail(r, e.status, e.what());
		}
		catch (const std::exception& e) {
			fail(r, UGSDR_E_INVALID, e.what());
		}
		return true;
	}

	void run() {
		cudaSetDevice(ctx->device);
		std::unique_lock<std::mutex> lock(mu);
		while (!stop) {
			bool progress = retire();
			while (admit())
				progress = true;
			stats.device_bytes = held();
			if (!progress) {
				if (stats.inflight > 0)
					cv_work.wait_for(lock, std::chrono::microseconds(50));
				else
					cv_work.wait(lock, [&] { return stop || !pending.empty(); });
			}
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
		for (auto& sl : s->slots) {
			UG_CUDA(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking));
			UG_CUDA(cudaEventCreateWithFlags(&sl.event, cudaEventDisableTiming));
			sl.ws.set_stream(sl.stream);  // scratch grows stream-ordered, without a device-wide wait
		}
		ugsdr_server* raw = s.get();
		s->worker = std::thread([raw] { raw->run(); });
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
	});
	if (st != UGSDR_OK)
		return st;
	std::lock_guard<std::mutex> lock(server->mu);
	if (static_cast<int>(server->pending.size()) >= server->cfg.queue_capacity) {
		ctx->last_error = "serving queue is full";
		return UGSDR_E_QUEUE_FULL;
	}
	r->ticket = server->next_ticket++;
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
	if (server->worker.joinable())
		server->worker.join();
	for (auto& sl : server->slots) {
		sl.ws.release();  // stream-ordered frees, before the stream goes
		if (sl.stream)
			cudaStreamSynchronize(sl.stream);
		sl.ws.set_stream(nullptr);
		if (sl.event)
			cudaEventDestroy(sl.event);
		if (sl.stream)
			cudaStreamDestroy(sl.stream);
	}
	delete server;
	return UGSDR_OK;
}
}
