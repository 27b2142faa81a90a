// server_policy.h -- scheduling policy of the simulation server: admission by free
// device memory, continuous batching of the admitted requests, completion,
// cancellation and failure handling.  No counterpart in the reference, which runs
// one simulation per process.
//
// The policy is host-only C++ over a Backend that performs the device work:
//   uint64_t free_bytes();                 free device memory now
//   uint64_t total_bytes();                memory the server may ever use
//   int admit(void* ctx);                  allocate and upload (PCG_OK, PCG_ERR_NOMEM, other codes)
//   int rebuild(const std::vector<void*>&) regroup the active set into one batch
//   int step_begin(uint64_t k, const std::vector<uint64_t>& budgets)
//                                          start k steps, simulation i taking part in the first budgets[i]
//   int step_end();                        wait for them
//   bool busy();                           the started steps are still running
//   int readback_begin(Request&);          start copying a finished request's field to its buffer
//   int readback_poll(const Request&, bool* done)  whether that copy has completed (no wait)
//   std::string last_error();
// so the same code runs against the GPU (server.cu) and against a fake backend in
// the CPU tests (admission refusals, allocation failures, malformed requests,
// cancellations and step faults are all injected on the host).
//
// One tick: regroup the batch if the active set changed; start steps_per_tick steps
// in which each active simulation takes part in min(steps_per_tick, its remaining
// steps); while they run, admit queued requests in arrival order while the active
// set has room and the next request's device bytes plus a reserve fit in free
// memory (admission overlaps the device work; admitted requests join at the next
// regroup); then wait for the steps and retire the finished simulations.  While
// simulations are stepping, admission stops once the steps are done (after at
// least one admission), so the device is not left idle behind host-side uploads;
// with nothing active it admits everything that fits.  A request submitted with
// a host buffer has its field copy started right after the tick in which it
// finished (the copy overlaps the following ticks: the request left the batch),
// and it is reported done once the copy has completed; a failed copy reports it
// failed.
// A request that does not fit now waits (memory is freed as active requests
// finish and as callers destroy returned ones); it is refused only when it could
// never fit (its bytes plus the reserve exceed total_bytes) or when its allocation
// failed kMaxAttempts times with nothing active.  Admission is first come, first
// served: a waiting request is not overtaken.
#pragma once

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <deque>
#include <string>
#include <vector>

namespace pcg::serve {

enum class Status : int
{
	Done = 0,
	Cancelled = 1,
	Refused = 2, // could not be admitted (memory, queue full)
	Failed = 3,  // admission or stepping failed
};

struct Request
{
	void* ctx = nullptr;
	uint64_t tag = 0;
	uint64_t steps = 0, remaining = 0;
	uint64_t bytes = 0;      // device bytes once admitted
	uint64_t vss_per_step = 0;
	double t_submit = -1, t_admit = -1, t_done = -1; // t_submit < 0: stamped by submit()
	uint32_t attempts = 0;   // admissions that failed for lack of memory
	void* out = nullptr;     // host buffer for the field when done (null: the caller reads it)
	int out_layout = 0, out_dtype = 0;
	uint64_t out_ticket = 0; // the backend's handle of the copy in flight
	Status status = Status::Done;
	int code = 0;
	std::string error;
};

struct Options
{
	uint64_t max_active = 1024;     // simulations stepped together
	uint64_t steps_per_tick = 8;    // steps between admission points
	uint64_t reserve_bytes = 1ull << 30;
	uint64_t max_queue = 1ull << 20;
};

struct Stats
{
	uint64_t submitted = 0, admitted = 0, completed = 0, cancelled = 0, refused = 0, failed = 0;
	uint64_t ticks = 0, rebuilds = 0, steps = 0;
	uint64_t prebuilds = 0;         // next-tick batches built while a tick ran
	uint64_t vss = 0;               // voxel-substrate-steps performed
	uint64_t active_bytes = 0;      // device bytes of the active set
	double rebuild_s = 0;           // host time regrouping the active set
	double step_s = 0;              // host time starting and waiting for steps (admission excluded)
	double admit_s = 0;             // host time admitting requests
	double prebuild_s = 0;          // host time building next-tick batches (the device busy meanwhile)
};

constexpr uint32_t kMaxAttempts = 3;

template <typename Backend>
class Scheduler
{
public:
	Scheduler(Backend& backend, Options options) : be_(backend), opt_(options) {}

	// Queues a request (false when the queue is full: the request is finished as Refused).
	bool submit(Request r, double now)
	{
		if (r.t_submit < 0)
			r.t_submit = now;
		r.remaining = r.steps;
		stats_.submitted++;
		if (r.steps == 0)
		{
			finish(r, Status::Done, 0, "", now);
			return true;
		}
		if (queue_.size() >= opt_.max_queue)
		{
			finish(r, Status::Refused, 0, "the request queue is full", now);
			return false;
		}
		queue_.push_back(std::move(r));
		return true;
	}

	// Cancels a queued or active request; it is finished at once (queued) or at
	// the next tick boundary (active: it is only ever touched between ticks).
	bool cancel(uint64_t tag, double now)
	{
		for (auto it = queue_.begin(); it != queue_.end(); ++it)
			if (it->tag == tag)
			{
				Request r = std::move(*it);
				queue_.erase(it);
				finish(r, Status::Cancelled, 0, "cancelled", now);
				return true;
			}
		for (size_t i = 0; i < active_.size(); i++)
			if (active_[i].tag == tag)
			{
				Request r = std::move(active_[i]);
				active_.erase(active_.begin() + (long)i);
				stats_.active_bytes -= r.bytes;
				dirty_ = true;
				finish(r, Status::Cancelled, 0, "cancelled", now);
				return true;
			}
		return false;
	}

	// One scheduling step; returns false when there is nothing to do.
	bool tick(double now)
	{
		const bool copied = poll_readbacks(now);
		const size_t stepped = active_.size();
		std::vector<uint64_t> budgets;
		if (stepped)
		{
			stats_.ticks++;
			if (dirty_)
			{
				std::vector<void*> ctxs;
				for (const Request& r : active_)
					ctxs.push_back(r.ctx);
				const auto t0 = clock::now();
				const int rc = be_.rebuild(ctxs);
				stats_.rebuild_s += seconds_since(t0);
				stats_.rebuilds++;
				if (rc)
				{
					fail_active(rc, be_.last_error(), now);
					return true;
				}
				dirty_ = false;
			}
			const uint64_t k = opt_.steps_per_tick;
			for (const Request& r : active_)
				budgets.push_back(std::min(k, r.remaining));
			const auto t0 = clock::now();
			const int rc = be_.step_begin(k, budgets);
			stats_.step_s += seconds_since(t0);
			if (rc)
			{
				fail_active(rc, be_.last_error(), now);
				return true;
			}
		}
		auto t0 = clock::now();
		const size_t admitted = admit(now, stepped > 0); // overlaps the steps just started
		stats_.admit_s += seconds_since(t0);
		if (!stepped)
			return admitted > 0 || copied;
		if (be_.busy())
		{
			// the next tick's set is known now (requests finish when their budget
			// runs out): build its batch while these steps run
			std::vector<void*> next;
			for (size_t i = 0; i < active_.size(); i++)
				if (i >= stepped || active_[i].remaining > budgets[i])
					next.push_back(active_[i].ctx);
			t0 = clock::now();
			if (be_.prebuild(next) == 0)
				stats_.prebuilds++;
			stats_.prebuild_s += seconds_since(t0);
		}
		t0 = clock::now();
		const int rc = be_.step_end();
		stats_.step_s += seconds_since(t0);
		if (rc)
		{
			fail_active(rc, be_.last_error(), now);
			return true;
		}
		stats_.steps += opt_.steps_per_tick;
		std::vector<Request> still;
		for (size_t i = 0; i < active_.size(); i++)
		{
			Request& r = active_[i];
			if (i < stepped)
			{
				r.remaining -= budgets[i];
				stats_.vss += r.vss_per_step * budgets[i];
				if (r.remaining == 0)
				{
					stats_.active_bytes -= r.bytes;
					dirty_ = true;
					const int rb = r.out ? be_.readback_begin(r) : 0;
					if (rb)
						finish(r, Status::Failed, rb, be_.last_error(), now);
					else if (r.out)
						reading_.push_back(std::move(r));
					else
						finish(r, Status::Done, 0, "", now);
					continue;
				}
			}
			still.push_back(std::move(r));
		}
		active_.swap(still);
		return true;
	}

	// Removes every request still held (server shutdown) and returns their contexts.
	std::vector<void*> release_all()
	{
		std::vector<void*> out;
		for (auto& r : queue_)
			out.push_back(r.ctx);
		for (auto& r : active_)
			out.push_back(r.ctx);
		for (auto& r : finished_)
			out.push_back(r.ctx);
		for (auto& r : reading_)
			out.push_back(r.ctx);
		queue_.clear();
		active_.clear();
		finished_.clear();
		reading_.clear();
		stats_.active_bytes = 0;
		dirty_ = true;
		return out;
	}

	std::vector<Request> take_finished()
	{
		std::vector<Request> out;
		out.swap(finished_);
		return out;
	}

	// The active set changed since the last rebuild (the backend's batch refers to
	// retired contexts until it is rebuilt or dropped).
	bool dirty() const { return dirty_; }
	bool idle() const { return queue_.empty() && active_.empty() && reading_.empty(); }
	size_t queued() const { return queue_.size(); }
	size_t active() const { return active_.size(); }
	const Stats& stats() const { return stats_; }

private:
	// Requests whose field copy has completed (or failed) are finished.
	bool poll_readbacks(double now)
	{
		bool any = false;
		std::vector<Request> still;
		for (Request& r : reading_)
		{
			bool done = false;
			const int rc = be_.readback_poll(r, &done);
			if (rc)
				finish(r, Status::Failed, rc, be_.last_error(), now);
			else if (done)
				finish(r, Status::Done, 0, "", now);
			else
			{
				still.push_back(std::move(r));
				continue;
			}
			any = true;
		}
		reading_.swap(still);
		return any;
	}

	using clock = std::chrono::steady_clock;
	static double seconds_since(clock::time_point t0)
	{
		return std::chrono::duration<double>(clock::now() - t0).count();
	}

	size_t admit(double now, bool while_busy)
	{
		size_t admitted = 0;
		while (!queue_.empty() && active_.size() < opt_.max_active)
		{
			if (while_busy && admitted > 0 && !be_.busy())
				break; // the steps are done: start the next ones before admitting more
			Request& r = queue_.front();
			const uint64_t total = be_.total_bytes();
			if (r.bytes + opt_.reserve_bytes > total)
			{
				Request x = std::move(r);
				queue_.pop_front();
				finish(x, Status::Refused, 3,
					   "needs " + std::to_string(x.bytes) + " device bytes plus the reserve; the server may use " +
						   std::to_string(total),
					   now);
				continue;
			}
			if (r.bytes + opt_.reserve_bytes > be_.free_bytes())
				return admitted; // wait for memory to be freed
			const int rc = be_.admit(r.ctx);
			if (rc == 3 /* PCG_ERR_NOMEM */)
			{
				// memory went elsewhere meanwhile: retry later, unless nothing of ours holds any
				if (!active_.empty() || ++r.attempts < kMaxAttempts)
					return admitted;
			}
			Request x = std::move(r);
			queue_.pop_front();
			if (rc)
			{
				finish(x, rc == 3 ? Status::Refused : Status::Failed, rc, be_.last_error(), now);
				continue;
			}
			x.t_admit = now;
			stats_.admitted++;
			stats_.active_bytes += x.bytes;
			active_.push_back(std::move(x));
			dirty_ = true;
			admitted++;
		}
		return admitted;
	}

	void fail_active(int rc, const std::string& msg, double now)
	{
		for (Request& r : active_)
		{
			stats_.active_bytes -= r.bytes;
			finish(r, Status::Failed, rc, msg, now);
		}
		active_.clear();
		dirty_ = true;
	}

	void finish(Request& r, Status s, int code, const std::string& msg, double now)
	{
		r.status = s;
		r.code = code;
		r.error = msg;
		r.t_done = now;
		switch (s)
		{
		case Status::Done: stats_.completed++; break;
		case Status::Cancelled: stats_.cancelled++; break;
		case Status::Refused: stats_.refused++; break;
		case Status::Failed: stats_.failed++; break;
		}
		finished_.push_back(std::move(r));
	}

	Backend& be_;
	Options opt_;
	std::deque<Request> queue_;
	std::vector<Request> active_;
	std::vector<Request> finished_;
	std::vector<Request> reading_; // done stepping, field copy in flight
	Stats stats_;
	bool dirty_ = false;
};

} // namespace pcg::serve
