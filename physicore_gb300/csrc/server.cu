// server.cu -- a simulation server: requests (configured, not yet initialised
// contexts) arrive at any time, are admitted by free device memory, stay resident
// on the device, and are stepped together through one batch (continuous batching:
// the active set is regrouped between ticks as requests finish and arrive).  No
// counterpart in the reference, which runs one simulation per process.
//
// One worker thread owns the scheduler (server_policy.h) and all device work.
// Submissions and cancellations reach it through an inbox, finished requests leave
// through an outbox; both are guarded by one mutex, never held during device work.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>

#include "pcg_internal.cuh"
#include "server_policy.h"

namespace pcg {
namespace {

struct GpuBackend
{
	int device = 0;
	bool autotune = false;
	uint64_t memory_limit = 0;        // 0: the device's free memory
	const serve::Stats* stats = nullptr;
	pcg_batch* batch = nullptr;
	std::string err;

	uint64_t free_bytes()
	{
		if (memory_limit)
			return memory_limit > stats->active_bytes ? memory_limit - stats->active_bytes : 0;
		size_t f = 0, t = 0;
		if (cudaMemGetInfo(&f, &t) != cudaSuccess)
		{
			cudaGetLastError();
			return 0;
		}
		return f + pool_idle_bytes(device); // blocks kept by the library's pool are free to it
	}
	uint64_t total_bytes()
	{
		if (memory_limit)
			return memory_limit;
		size_t f = 0, t = 0;
		if (cudaMemGetInfo(&f, &t) != cudaSuccess)
		{
			cudaGetLastError();
			return 0;
		}
		return t;
	}
	int admit(void* ctx)
	{
		// without waiting for the field fill: the batch step that follows orders it
		Context* c = static_cast<pcg_context*>(ctx);
		DeviceGuard g(c->device);
		const int rc = initialize_context(c, false);
		if (rc)
			err = pcg_last_error();
		return rc;
	}
	void drop()
	{
		if (batch)
			pcg_batch_destroy(batch);
		batch = nullptr;
	}
	// A batch whose steps are done and whose set changed: destroyed once the next
	// tick's steps are queued, so that its teardown does not delay them.  It is
	// never stepped again (its contexts may be destroyed by their owners
	// meanwhile; destroying a batch does not touch its contexts).
	std::vector<pcg_batch*> retired;
	void retire()
	{
		if (batch)
			retired.push_back(batch);
		batch = nullptr;
	}
	void reap()
	{
		for (pcg_batch* r : retired)
			pcg_batch_destroy(r);
		retired.clear();
	}
	// The next tick's batch, built and captured while the current tick runs.
	pcg_batch* next = nullptr;
	std::vector<void*> next_ctxs;
	void drop_next()
	{
		if (next)
			pcg_batch_destroy(next);
		next = nullptr;
		next_ctxs.clear();
	}
	// 0 when a batch was prepared; -1 when none is (empty set, or the tuner, which
	// times launches on the real fields, is on: not beside running steps)
	int prebuild(const std::vector<void*>& ctxs)
	{
		drop_next();
		if (autotune || ctxs.empty())
			return -1;
		std::vector<pcg_context*> c(ctxs.size());
		for (size_t i = 0; i < ctxs.size(); i++)
			c[i] = static_cast<pcg_context*>(ctxs[i]);
		int rc = pcg_batch_create(&next, c.data(), c.size());
		if (!rc)
			rc = pcg_batch_prepare(next);
		if (rc)
		{
			err = pcg_last_error();
			drop_next();
			return rc;
		}
		next_ctxs = ctxs;
		return PCG_OK;
	}
	int rebuild(const std::vector<void*>& ctxs)
	{
		if (next && next_ctxs == ctxs)
		{
			drop();
			batch = next;
			next = nullptr;
			next_ctxs.clear();
			return PCG_OK;
		}
		drop_next();
		drop();
		std::vector<pcg_context*> c(ctxs.size());
		for (size_t i = 0; i < ctxs.size(); i++)
			c[i] = static_cast<pcg_context*>(ctxs[i]);
		int rc = pcg_batch_create(&batch, c.data(), c.size());
		if (!rc && autotune)
			rc = pcg_batch_autotune(batch);
		if (rc)
		{
			err = pcg_last_error();
			drop();
		}
		return rc;
	}
	// The tick's first step in a call of its own: requests admitted since the last
	// tick rebuild their ballots there (their agents do not move while served), and
	// the remaining steps replay the step without the ballot-rebuild kernels.
	std::vector<uint64_t> first_, rest_;
	int step_begin(uint64_t k, const std::vector<uint64_t>& budgets)
	{
		first_.resize(budgets.size());
		rest_.resize(budgets.size());
		for (size_t i = 0; i < budgets.size(); i++)
		{
			first_[i] = std::min<uint64_t>(budgets[i], 1);
			rest_[i] = budgets[i] - first_[i];
		}
		int rc = pcg_batch_solve_budgets(batch, 1, first_.data());
		if (!rc && k > 1)
			rc = pcg_batch_solve_budgets(batch, k - 1, rest_.data());
		if (rc)
			err = pcg_last_error();
		reap();
		return rc;
	}
	// The finished request left the batch, so its field no longer changes: the
	// conversion and the copy run on its own streams while the next steps run.
	int readback_begin(serve::Request& r)
	{
		const int rc =
			pcg_get_field_async(static_cast<pcg_context*>(r.ctx), r.out, r.out_layout, r.out_dtype, &r.out_ticket);
		if (rc)
			err = pcg_last_error();
		return rc;
	}
	int readback_poll(const serve::Request& r, bool* done)
	{
		const int rc = readback_ready(static_cast<pcg_context*>(r.ctx), r.out_ticket, done);
		if (rc)
			err = pcg_last_error();
		return rc;
	}
	bool busy()
	{
		void* s = nullptr;
		if (!batch || pcg_batch_get_stream(batch, &s) != PCG_OK)
			return false;
		return cudaStreamQuery(static_cast<cudaStream_t>(s)) == cudaErrorNotReady;
	}
	int step_end()
	{
		const int rc = pcg_batch_synchronize(batch);
		if (rc)
			err = pcg_last_error();
		return rc;
	}
	std::string last_error() const { return err; }
};

} // namespace
} // namespace pcg

struct pcg_server
{
	int precision = PCG_FP32;
	int device = 0;
	pcg::GpuBackend backend;
	pcg::serve::Options options;
	std::unique_ptr<pcg::serve::Scheduler<pcg::GpuBackend>> sched;
	std::chrono::steady_clock::time_point t0;

	std::mutex mu;
	std::condition_variable cv_in, cv_out;
	std::deque<pcg::serve::Request> inbox;
	std::vector<uint64_t> cancels;
	std::deque<pcg::serve::Request> outbox;
	pcg::serve::Stats stats_snapshot;
	size_t queued_snapshot = 0, active_snapshot = 0;
	uint64_t in_flight = 0; // submitted and not yet in the outbox
	bool stop = false;
	std::thread worker;

	double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }

	void run()
	{
		cudaSetDevice(device);
		for (;;)
		{
			std::deque<pcg::serve::Request> in;
			std::vector<uint64_t> cx;
			{
				std::unique_lock<std::mutex> lk(mu);
				if (stop)
					break;
				in.swap(inbox);
				cx.swap(cancels);
			}
			const double t = now();
			for (auto& r : in)
				sched->submit(std::move(r), t);
			for (uint64_t tag : cx)
				sched->cancel(tag, t);
			const bool worked = sched->tick(now());
			if (sched->dirty())
				backend.retire(); // the batch may refer to retired contexts: never step it again
			std::vector<pcg::serve::Request> done = sched->take_finished();
			for (const auto& r : done) // a request cancelled or failed out of the prepared batch
				if (std::find(backend.next_ctxs.begin(), backend.next_ctxs.end(), r.ctx) != backend.next_ctxs.end())
					backend.drop_next();
			{
				std::unique_lock<std::mutex> lk(mu);
				for (auto& r : done)
					outbox.push_back(std::move(r));
				in_flight -= done.size();
				stats_snapshot = sched->stats();
				queued_snapshot = sched->queued();
				active_snapshot = sched->active();
				if (!done.empty())
					cv_out.notify_all();
				if (!worked && inbox.empty() && cancels.empty() && !stop)
					cv_in.wait_for(lk, std::chrono::milliseconds(2));
			}
		}
		backend.reap();
		backend.drop_next();
		backend.drop();
	}
};

using pcg::fail;

extern "C" {

int pcg_server_create(pcg_server** out, int precision, int device, const pcg_server_options* opts)
{
	if (!out)
		return fail(PCG_ERR_INVALID, "null argument");
	*out = nullptr;
	if (precision != PCG_FP32 && precision != PCG_FP64)
		return fail(PCG_ERR_INVALID, "precision must be PCG_FP32 or PCG_FP64");
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
	{
		cudaGetLastError();
		return fail(PCG_ERR_CUDA, "no such CUDA device");
	}
	auto* s = new pcg_server();
	s->precision = precision;
	s->device = device;
	if (opts)
	{
		if (opts->max_active)
			s->options.max_active = opts->max_active;
		if (opts->steps_per_tick)
			s->options.steps_per_tick = opts->steps_per_tick;
		s->options.reserve_bytes = opts->reserve_bytes;
		if (opts->max_queue)
			s->options.max_queue = opts->max_queue;
		s->backend.memory_limit = opts->memory_limit_bytes;
		s->backend.autotune = opts->autotune != 0;
	}
	s->backend.device = device;
	s->sched = std::make_unique<pcg::serve::Scheduler<pcg::GpuBackend>>(s->backend, s->options);
	s->backend.stats = &s->sched->stats();
	s->t0 = std::chrono::steady_clock::now();
	s->worker = std::thread([s] { s->run(); });
	*out = s;
	return PCG_OK;
}

int pcg_server_destroy(pcg_server* s)
{
	if (!s)
		return PCG_OK;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
	}
	s->cv_in.notify_all();
	if (s->worker.joinable())
		s->worker.join();
	// contexts still held by the server (queued, active, or finished but not polled)
	std::vector<void*> held;
	for (auto& r : s->inbox)
		held.push_back(r.ctx);
	for (auto& r : s->outbox)
		held.push_back(r.ctx);
	if (s->sched)
		for (void* c : s->sched->release_all())
			held.push_back(c);
	s->backend.reap();
	s->backend.drop_next();
	s->backend.drop();
	for (void* c : held)
		pcg_destroy(static_cast<pcg_context*>(c));
	delete s;
	return PCG_OK;
}

int pcg_server_submit(pcg_server* s, pcg_context* ctx, uint64_t steps, uint64_t tag)
{
	return pcg_server_submit_readback(s, ctx, steps, tag, nullptr, PCG_LAYOUT_INTERLEAVED, PCG_DTYPE_F64);
}

int pcg_server_submit_readback(pcg_server* s, pcg_context* ctx, uint64_t steps, uint64_t tag, void* host, int layout,
							   int dtype)
{
	if (!s || !ctx)
		return fail(PCG_ERR_INVALID, "null argument");
	if (host && ((layout != PCG_LAYOUT_INTERLEAVED && layout != PCG_LAYOUT_PLANAR) ||
				 (dtype != PCG_DTYPE_F32 && dtype != PCG_DTYPE_F64)))
		return fail(PCG_ERR_INVALID, "bad layout or dtype");
	pcg::Context* c = ctx;
	if (c->precision != s->precision || c->device != s->device)
		return fail(PCG_ERR_INVALID, "the request's precision or device differs from the server's");
	if (c->initialized)
		return fail(PCG_ERR_INVALID, "submit contexts before initialize: the server admits and initialises them");
	if (!c->mesh_set || c->S == 0)
		return fail(PCG_ERR_INVALID, "the request has no mesh or substrates");
	pcg::serve::Request r;
	r.ctx = ctx;
	r.tag = tag;
	r.steps = steps;
	r.bytes = pcg::estimate_device_bytes(c);
	r.vss_per_step = c->V * c->S;
	r.out = host;
	r.out_layout = layout;
	r.out_dtype = dtype;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		r.t_submit = s->now();
		s->inbox.push_back(std::move(r));
		s->in_flight++;
	}
	s->cv_in.notify_all();
	return PCG_OK;
}

int pcg_server_cancel(pcg_server* s, uint64_t tag)
{
	if (!s)
		return fail(PCG_ERR_INVALID, "null server");
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->cancels.push_back(tag);
	}
	s->cv_in.notify_all();
	return PCG_OK;
}

int pcg_server_poll(pcg_server* s, pcg_server_result* out, uint64_t cap, uint64_t* count, int wait_ms)
{
	if (!s || (!out && cap) || !count)
		return fail(PCG_ERR_INVALID, "null argument");
	std::unique_lock<std::mutex> lk(s->mu);
	if (s->outbox.empty() && wait_ms > 0)
		s->cv_out.wait_for(lk, std::chrono::milliseconds(wait_ms), [s] { return !s->outbox.empty(); });
	uint64_t n = 0;
	while (n < cap && !s->outbox.empty())
	{
		pcg::serve::Request r = std::move(s->outbox.front());
		s->outbox.pop_front();
		pcg_server_result& o = out[n++];
		memset(&o, 0, sizeof(o));
		o.ctx = static_cast<pcg_context*>(r.ctx);
		o.tag = r.tag;
		o.steps = r.steps;
		o.status = (int)r.status;
		o.code = r.code;
		o.t_submit = r.t_submit;
		o.t_admit = r.t_admit;
		o.t_done = r.t_done;
		o.device_bytes = r.bytes;
		snprintf(o.error, sizeof(o.error), "%s", r.error.c_str());
	}
	*count = n;
	return PCG_OK;
}

int pcg_server_get_stats(pcg_server* s, pcg_server_stats* st)
{
	if (!s || !st)
		return fail(PCG_ERR_INVALID, "null argument");
	std::lock_guard<std::mutex> lk(s->mu);
	const pcg::serve::Stats& x = s->stats_snapshot;
	memset(st, 0, sizeof(*st));
	st->submitted = x.submitted;
	st->admitted = x.admitted;
	st->completed = x.completed;
	st->cancelled = x.cancelled;
	st->refused = x.refused;
	st->failed = x.failed;
	st->ticks = x.ticks;
	st->rebuilds = x.rebuilds;
	st->steps = x.steps;
	st->vss = x.vss;
	st->active_bytes = x.active_bytes;
	st->queued = s->queued_snapshot + s->inbox.size();
	st->active = s->active_snapshot;
	st->in_flight = s->in_flight;
	st->uptime_s = s->now();
	st->rebuild_s = x.rebuild_s;
	st->step_s = x.step_s;
	st->admit_s = x.admit_s;
	st->prebuilds = x.prebuilds;
	st->prebuild_s = x.prebuild_s;
	return PCG_OK;
}

} // extern "C"
