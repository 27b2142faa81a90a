// CPU tests of the serving policy (physicore_gb300/csrc/server_policy.h) against a
// fake backend: admission by free memory, waiting versus refusal, allocation
// failures, malformed requests, cancellations, step faults and continuous
// batching.  All failures are injected on the host; no GPU is used.
#include <cstdio>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "../../physicore_gb300/csrc/server_policy.h"

using namespace pcg::serve;

static int g_failures = 0;
#define EXPECT(cond)                                                                                         \
	do                                                                                                       \
	{                                                                                                        \
		if (!(cond))                                                                                         \
		{                                                                                                    \
			std::printf("  FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);                                 \
			g_failures++;                                                                                    \
		}                                                                                                    \
	} while (0)

namespace {

// Contexts are small integers cast to void*; the fake tracks memory and steps.
struct FakeBackend
{
	uint64_t capacity = 1000;             // device bytes
	uint64_t used = 0;
	std::map<void*, uint64_t> bytes;      // per context
	std::set<void*> resident, batch;
	std::map<void*, uint64_t> stepped;    // steps each context received
	std::set<void*> fail_admit_nomem, fail_admit_invalid;
	bool fail_next_step = false;
	int rebuilds = 0;
	std::string err;

	uint64_t free_bytes() { return capacity - used; }
	uint64_t total_bytes() { return capacity; }
	int admit(void* c)
	{
		if (fail_admit_invalid.count(c))
		{
			err = "malformed request";
			return 1;
		}
		if (fail_admit_nomem.count(c) || used + bytes[c] > capacity)
		{
			err = "cudaMalloc failed";
			return 3;
		}
		used += bytes[c];
		resident.insert(c);
		return 0;
	}
	int rebuild(const std::vector<void*>& ctxs)
	{
		rebuilds++;
		batch = std::set<void*>(ctxs.begin(), ctxs.end());
		order = ctxs;
		for (void* c : ctxs)
			if (!resident.count(c))
			{
				err = "batch over a context that is not resident";
				return 1;
			}
		return 0;
	}
	std::vector<void*> order; // batch members in rebuild order
	int step_begin(uint64_t, const std::vector<uint64_t>& budgets)
	{
		if (fail_next_step)
		{
			fail_next_step = false;
			err = "device fault";
			return 4;
		}
		for (size_t i = 0; i < order.size(); i++)
			stepped[order[i]] += budgets[i];
		return 0;
	}
	int step_end() { return 0; }
	std::vector<void*> read_back;    // contexts whose field copy started, in order
	bool fail_readback = false;      // the copy fails when polled
	int copy_polls = 1;              // polls before a copy has completed
	std::map<void*, int> polls_left;
	int readback_begin(Request& r)
	{
		read_back.push_back(r.ctx);
		polls_left[r.ctx] = copy_polls;
		r.out_ticket = read_back.size();
		return 0;
	}
	int readback_poll(const Request& r, bool* done)
	{
		if (fail_readback)
		{
			err = "readback failed";
			return 4;
		}
		*done = --polls_left[r.ctx] <= 0;
		return 0;
	}
	std::vector<std::vector<void*>> prebuilt; // sets passed to prebuild, in order
	int prebuild(const std::vector<void*>& c)
	{
		prebuilt.push_back(c);
		return 0;
	}
	int busy_polls = 0; // busy() answers true this many times
	bool busy() { return busy_polls > 0 && busy_polls--; }
	std::string last_error() const { return err; }
	void release(void* c) // the caller destroys a returned context
	{
		if (resident.erase(c))
			used -= bytes[c];
	}
};

void* ctx(int i) { return reinterpret_cast<void*>(static_cast<uintptr_t>(i)); }

Request req(FakeBackend& be, int i, uint64_t steps, uint64_t bytes)
{
	be.bytes[ctx(i)] = bytes;
	Request r;
	r.ctx = ctx(i);
	r.tag = (uint64_t)i;
	r.steps = steps;
	r.bytes = bytes;
	r.vss_per_step = 10;
	return r;
}

// Runs ticks until idle, releasing finished contexts like a prompt caller.
std::vector<Request> run(Scheduler<FakeBackend>& s, FakeBackend& be, int max_ticks = 1000)
{
	std::vector<Request> done;
	for (int t = 0; t < max_ticks && !s.idle(); t++)
	{
		s.tick(t);
		for (Request& r : s.take_finished())
		{
			be.release(r.ctx);
			done.push_back(r);
		}
	}
	for (Request& r : s.take_finished())
		done.push_back(r);
	return done;
}

const Request* find(const std::vector<Request>& v, uint64_t tag)
{
	for (const Request& r : v)
		if (r.tag == tag)
			return &r;
	return nullptr;
}

void continuous_batching()
{
	FakeBackend be;
	Options o;
	o.reserve_bytes = 0;
	o.steps_per_tick = 4;
	Scheduler<FakeBackend> s(be, o);
	s.submit(req(be, 1, 10, 100), 0);
	s.submit(req(be, 2, 3, 100), 0);
	s.tick(0); // both admitted (nothing was running yet)
	EXPECT(s.active() == 2 && s.take_finished().empty());
	s.tick(1); // 4 steps for 1, 3 for 2 (its budget): 2 is done inside the tick
	auto f = s.take_finished();
	EXPECT(f.size() == 1 && !f.empty() && f[0].tag == 2 && f[0].status == Status::Done);
	if (!f.empty())
		be.release(f[0].ctx);
	EXPECT(be.stepped[ctx(1)] == 4 && be.stepped[ctx(2)] == 3);
	s.submit(req(be, 3, 2, 100), 1); // arrives while 1 runs: admitted during the next tick
	auto done = run(s, be);
	EXPECT(be.stepped[ctx(1)] == 10 && be.stepped[ctx(2)] == 3 && be.stepped[ctx(3)] == 2);
	EXPECT(find(done, 1) && find(done, 1)->status == Status::Done);
	EXPECT(find(done, 3) && find(done, 3)->status == Status::Done && find(done, 3)->t_admit >= 0);
	EXPECT(s.stats().completed == 3 && s.stats().vss == 10 * (10 + 3 + 2));
	EXPECT(be.rebuilds >= 2);
}

void admission_waits_for_memory()
{
	FakeBackend be;
	be.capacity = 250;
	Options o;
	o.reserve_bytes = 0;
	o.steps_per_tick = 5;
	Scheduler<FakeBackend> s(be, o);
	s.submit(req(be, 1, 10, 200), 0);
	s.submit(req(be, 2, 5, 200), 0); // does not fit beside 1: waits, is not refused
	s.tick(0);
	EXPECT(s.active() == 1 && s.queued() == 1);
	s.tick(1); // 5 of 10 steps
	s.tick(2); // 1 finishes; its memory stays held until the caller releases it
	auto f = s.take_finished();
	EXPECT(f.size() == 1 && !f.empty() && f[0].tag == 1);
	s.tick(3);
	EXPECT(s.active() == 0 && s.queued() == 1 && s.stats().refused == 0); // still waiting
	if (!f.empty())
		be.release(f[0].ctx);
	auto done = run(s, be);
	EXPECT(find(done, 2) && find(done, 2)->status == Status::Done);
	EXPECT(find(done, 2)->t_admit >= 0);
}

void refusal_when_it_can_never_fit()
{
	FakeBackend be;
	be.capacity = 100;
	Options o;
	o.reserve_bytes = 10;
	Scheduler<FakeBackend> s(be, o);
	s.submit(req(be, 1, 5, 95), 0); // 95 + reserve 10 > 100 with nothing active
	auto done = run(s, be);
	EXPECT(done.size() == 1 && done[0].status == Status::Refused && done[0].t_admit < 0);
	EXPECT(s.stats().refused == 1 && be.used == 0);
}

void allocation_failure_and_malformed_request()
{
	FakeBackend be;
	Options o;
	o.reserve_bytes = 0;
	Scheduler<FakeBackend> s(be, o);
	be.fail_admit_nomem.insert(ctx(1));
	be.fail_admit_invalid.insert(ctx(2));
	s.submit(req(be, 1, 5, 10), 0);
	s.submit(req(be, 2, 5, 10), 0);
	s.submit(req(be, 3, 5, 10), 0);
	auto done = run(s, be);
	// always out of memory with nothing else active: refused after kMaxAttempts tries
	EXPECT(find(done, 1)->status == Status::Refused && find(done, 1)->code == 3);
	EXPECT(find(done, 2)->status == Status::Failed && find(done, 2)->error == "malformed request");
	EXPECT(find(done, 3)->status == Status::Done);
}

void cancellation()
{
	FakeBackend be;
	Options o;
	o.reserve_bytes = 0;
	o.steps_per_tick = 2;
	Scheduler<FakeBackend> s(be, o);
	s.submit(req(be, 1, 100, 10), 0);
	s.submit(req(be, 2, 100, 10), 0);
	s.tick(0); // admitted
	s.tick(1); // 2 steps each
	EXPECT(s.cancel(1, 1));  // active
	EXPECT(!s.cancel(7, 1)); // unknown
	s.submit(req(be, 3, 100, 10), 1);
	EXPECT(s.cancel(3, 1));  // still queued
	auto f = s.take_finished();
	EXPECT(f.size() == 2 && f[0].status == Status::Cancelled && f[1].status == Status::Cancelled);
	for (auto& r : f)
		be.release(r.ctx);
	auto done = run(s, be);
	EXPECT(be.stepped[ctx(1)] == 2 && be.stepped[ctx(3)] == 0 && be.stepped[ctx(2)] == 100);
	EXPECT(s.stats().cancelled == 2);
}

void step_fault_fails_the_active_set()
{
	FakeBackend be;
	Options o;
	o.reserve_bytes = 0;
	Scheduler<FakeBackend> s(be, o);
	s.submit(req(be, 1, 50, 10), 0);
	s.submit(req(be, 2, 50, 10), 0);
	be.fail_next_step = true;
	s.tick(0); // admitted
	s.tick(1); // the step fails
	auto f = s.take_finished();
	EXPECT(f.size() == 2 && !f.empty() && f[0].status == Status::Failed && f[0].code == 4 &&
		   f[0].error == "device fault");
	EXPECT(s.idle() && s.stats().active_bytes == 0);
}

void admission_stops_when_steps_finish()
{
	FakeBackend be;
	Options o;
	o.reserve_bytes = 0;
	o.steps_per_tick = 1;
	Scheduler<FakeBackend> s(be, o);
	s.submit(req(be, 1, 100, 10), 0);
	s.tick(0); // nothing active: admitted without waiting for anything
	EXPECT(s.active() == 1);
	for (int i = 2; i <= 6; i++)
		s.submit(req(be, i, 100, 10), 0);
	be.busy_polls = 0; // the steps finish at once: one admission, then the next tick
	s.tick(1);
	EXPECT(s.active() == 2 && s.queued() == 4);
	be.busy_polls = 2; // still running for two more admissions
	s.tick(2);
	EXPECT(s.active() == 5 && s.queued() == 1);
	EXPECT(s.stats().admit_s >= 0 && s.stats().step_s >= 0 && s.stats().rebuild_s >= 0);
}

// While a tick's steps run, the next tick's set (those not finishing in it, then
// those admitted meanwhile) is handed to the backend to prepare; not when the
// steps are already done.
void prebuilds_the_next_set()
{
	FakeBackend be;
	Options o;
	o.reserve_bytes = 0;
	o.steps_per_tick = 4;
	Scheduler<FakeBackend> s(be, o);
	s.submit(req(be, 1, 4, 10), 0);   // finishes in the next tick
	s.submit(req(be, 2, 100, 10), 0);
	s.tick(0);
	EXPECT(s.active() == 2 && be.prebuilt.empty());
	s.submit(req(be, 3, 50, 10), 0);
	be.busy_polls = 1; // the steps run on while request 3 is admitted
	s.tick(1);
	EXPECT(be.prebuilt.size() == 1 && s.stats().prebuilds == 1);
	EXPECT(be.prebuilt.back() == (std::vector<void*> { ctx(2), ctx(3) }));
	be.busy_polls = 0; // done before the backend could prepare anything
	s.tick(2);
	EXPECT(be.prebuilt.size() == 1 && s.stats().prebuilds == 1 && s.stats().prebuild_s >= 0);
}

void readback_before_done()
{
	FakeBackend be;
	Options o;
	o.reserve_bytes = 0;
	o.steps_per_tick = 4;
	Scheduler<FakeBackend> s(be, o);
	static float buf[4];
	Request a = req(be, 1, 4, 10);
	a.out = buf;
	Request b = req(be, 2, 8, 10); // no buffer: the caller reads the field itself
	Request c = req(be, 3, 4, 10);
	c.out = buf;
	be.copy_polls = 2;
	s.submit(a, 0);
	s.submit(b, 0);
	s.tick(0);
	s.tick(1); // 1 finishes stepping: its copy starts and overlaps the next ticks
	EXPECT(s.take_finished().empty() && be.read_back.size() == 1 && be.read_back[0] == ctx(1));
	EXPECT(!s.idle());
	s.tick(2); // first poll: 1 still copying; 2 (no buffer) finishes and is reported at once
	auto f = s.take_finished();
	EXPECT(f.size() == 1 && !f.empty() && f[0].tag == 2 && f[0].status == Status::Done);
	s.tick(3); // second poll: 1's copy is done, reported only now
	f = s.take_finished();
	EXPECT(f.size() == 1 && !f.empty() && f[0].tag == 1 && f[0].status == Status::Done);
	be.fail_readback = true;
	s.submit(c, 3);
	auto done = run(s, be);
	EXPECT(find(done, 3) && find(done, 3)->status == Status::Failed && find(done, 3)->error == "readback failed");
	EXPECT(be.read_back.size() == 2 && s.idle());
}

void queue_limit_and_zero_steps()
{
	FakeBackend be;
	Options o;
	o.max_queue = 1;
	Scheduler<FakeBackend> s(be, o);
	EXPECT(s.submit(req(be, 1, 5, 10), 0));
	EXPECT(!s.submit(req(be, 2, 5, 10), 0));
	EXPECT(s.submit(req(be, 3, 0, 10), 0)); // nothing to do: done at once
	auto f = s.take_finished();
	EXPECT(f.size() == 2 && f[0].status == Status::Refused && f[1].status == Status::Done);
}

} // namespace

int main()
{
	struct
	{
		const char* name;
		void (*fn)();
	} tests[] = {
		{ "ServerPolicy.ContinuousBatching", continuous_batching },
		{ "ServerPolicy.AdmissionWaitsForMemory", admission_waits_for_memory },
		{ "ServerPolicy.RefusalWhenItCanNeverFit", refusal_when_it_can_never_fit },
		{ "ServerPolicy.AllocationFailureAndMalformedRequest", allocation_failure_and_malformed_request },
		{ "ServerPolicy.Cancellation", cancellation },
		{ "ServerPolicy.StepFaultFailsTheActiveSet", step_fault_fails_the_active_set },
		{ "ServerPolicy.QueueLimitAndZeroSteps", queue_limit_and_zero_steps },
		{ "ServerPolicy.AdmissionStopsWhenStepsFinish", admission_stops_when_steps_finish },
		{ "ServerPolicy.ReadbackBeforeDone", readback_before_done },
		{ "ServerPolicy.PrebuildsTheNextSet", prebuilds_the_next_set },
	};
	int n = 0;
	for (auto& t : tests)
	{
		const int before = g_failures;
		t.fn();
		std::printf("[%s] %s\n", g_failures == before ? "  OK  " : "FAILED", t.name);
		n++;
	}
	std::printf("%d tests, %d failures\n", n, g_failures);
	return g_failures ? 1 : 0;
}
