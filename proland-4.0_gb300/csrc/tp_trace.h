// Tracing: NVTX ranges around the library's launches and host phases (seen by
// Nsight tools; no-ops without one), and optional per-phase host timers read
// through tp_trace_host_times.  Both are off until tp_trace_set turns them on
// (or the TP_TRACE environment variable holds the flag bits at load).
#pragma once
#include <chrono>

namespace tp {

enum TracePhase {
    kPhSamplerRelease = 0,  // tp_sampler_update: tiles of vanished quads released
    kPhSamplerAcquire,      // tp_sampler_update: new quads' tiles acquired (getTile, schedule)
    kPhResiduals,           // scheduler: residual tiles (decode / upload / synthetic launch)
    kPhElevJobs,            // scheduler: job records of an elevation launch
    kPhFrameSetup,          // scheduler: frame class set-up and job checks
    kPhFrameLaunch,         // scheduler: job upload and the persistent launch
    kPhFinish,              // scheduler: produced tiles marked, their inputs released
    kPhNormals,             // scheduler: normal launches not fused into an elevation launch
    kPhLayers,              // scheduler: layer passes
    kPhLearned,             // learned predictor launches
    kPhCount
};

extern int g_trace_flags;  // bit 0: NVTX ranges, bit 1: host phase timers

void trace_push(const char *name);
void trace_pop();
void trace_add(int phase, double seconds);

// A scoped range: an NVTX range when bit 0 is set, a host timer of `phase` when bit 1 is.
class TraceScope {
public:
    TraceScope(const char *name, int phase) : phase_(phase), flags_(g_trace_flags)
    {
        if (flags_ & 1) trace_push(name);
        if (flags_ & 2) t0_ = std::chrono::steady_clock::now();
    }
    ~TraceScope()
    {
        if (flags_ & 2)
            trace_add(phase_, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count());
        if (flags_ & 1) trace_pop();
    }
    TraceScope(const TraceScope &) = delete;
    TraceScope &operator=(const TraceScope &) = delete;

private:
    int phase_, flags_;
    std::chrono::steady_clock::time_point t0_;
};

}  // namespace tp
