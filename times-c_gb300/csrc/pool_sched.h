// Admission decision of the job pool (pool.cpp), as a pure function of the queue
// and the workers' memory so that it can be tested without a GPU.
//
// A worker may start the oldest queued job whose footprint fits the budget on top
// of what the workers hold and have reserved.  Two rules keep a large job from
// waiting forever behind a stream of small ones:
//  * once the head of the queue has waited longer than head_wait_s, only the head
//    may start: workers finishing other jobs do not take new ones until it fits;
//  * idle workers give their workspaces back only when that lets a job start now
//    (the head, while it has priority; else the smallest queued job).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace tc {

struct SchedJob {
    uint64_t footprint = 0;
    double waited_s = 0;  // seconds since submission
};

struct SchedWorkers {
    uint64_t budget = 0;
    std::vector<uint64_t> held;  // workspace bytes per worker
    std::vector<uint64_t> resv;  // growth reserved for the job a worker runs
    std::vector<bool> busy;

    uint64_t total() const {
        uint64_t t = 0;
        for (size_t w = 0; w < held.size(); ++w) t += held[w] + resv[w];
        return t;
    }
    uint64_t idle_bytes() const {
        uint64_t t = 0;
        for (size_t w = 0; w < held.size(); ++w)
            if (!busy[w]) t += held[w];
        return t;
    }
};

struct SchedChoice {
    int index = -1;             // queue position to start, -1: none
    bool release_idle = false;  // hand back the idle workspaces first, then decide again
};

inline SchedChoice sched_pick(const std::vector<SchedJob>& queue, const SchedWorkers& ws, double head_wait_s) {
    SchedChoice c;
    if (queue.empty()) return c;
    const bool head_only = queue[0].waited_s > head_wait_s;
    const uint64_t used = ws.total();
    uint64_t smallest = queue[0].footprint;
    for (size_t i = 0; i < queue.size(); ++i) {
        if (used + queue[i].footprint <= ws.budget) {
            c.index = (int)i;
            return c;
        }
        if (head_only) break;
        if (queue[i].footprint < smallest) smallest = queue[i].footprint;
    }
    const uint64_t need = head_only ? queue[0].footprint : smallest;
    const uint64_t idle = ws.idle_bytes();
    c.release_idle = idle > 0 && used - idle + need <= ws.budget;
    return c;
}

}  // namespace tc
