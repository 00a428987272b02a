// Tracing state: NVTX ranges (header-only NVTX v3: the calls reach a tool only when
// one is attached) and the per-phase host timers.
#include "tp_trace.h"

#include <atomic>
#include <cstdlib>
#include <mutex>

#include <nvtx3/nvToolsExt.h>

#include "tp_internal.h"

namespace tp {

static int env_flags()
{
    const char *v = std::getenv("TP_TRACE");
    return v ? std::atoi(v) & 3 : 0;
}

int g_trace_flags = env_flags();

namespace {
std::mutex g_mu;
double g_seconds[kPhCount];
long long g_calls[kPhCount];
const char *const kNames[kPhCount] = {"sampler_release", "sampler_acquire", "residuals", "elevation_jobs",
                                      "frame_setup", "frame_launch", "finish", "normals", "layers", "learned"};
}  // namespace

void trace_push(const char *name) { nvtxRangePushA(name); }
void trace_pop() { nvtxRangePop(); }

void trace_add(int phase, double seconds)
{
    if (phase < 0 || phase >= kPhCount) return;
    std::lock_guard<std::mutex> lk(g_mu);
    g_seconds[phase] += seconds;
    g_calls[phase] += 1;
}

}  // namespace tp

extern "C" int tp_trace_set(int flags)
{
    if (flags < 0 || flags > 3) return tp::fail(TP_E_BAD_ARG, "tp_trace_set: flags are bits 0 (NVTX) and 1 (host timers)");
    const int old = tp::g_trace_flags;
    tp::g_trace_flags = flags;
    return old;
}

extern "C" int tp_trace_host_times(double *seconds, long long *calls, int n, int reset)
{
    if (n < 0 || (n > 0 && (!seconds || !calls))) return tp::fail(TP_E_BAD_ARG, "tp_trace_host_times: bad arguments");
    std::lock_guard<std::mutex> lk(tp::g_mu);
    for (int i = 0; i < n && i < tp::kPhCount; ++i) {
        seconds[i] = tp::g_seconds[i];
        calls[i] = tp::g_calls[i];
    }
    if (reset)
        for (int i = 0; i < tp::kPhCount; ++i) {
            tp::g_seconds[i] = 0.0;
            tp::g_calls[i] = 0;
        }
    return tp::kPhCount;
}

extern "C" const char *tp_trace_phase_name(int phase)
{
    return phase >= 0 && phase < tp::kPhCount ? tp::kNames[phase] : nullptr;
}
