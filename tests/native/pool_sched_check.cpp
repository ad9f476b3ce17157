// CPU check of the job pool's admission rule (times-c_gb300/csrc/pool_sched.h)
// with made-up footprints: a large job at the head of the queue is not overtaken
// forever by a stream of small jobs, and idle workspaces are handed back only
// when that lets a job start.  Built and run by tests/test_pool_sched.py.
#include <cstdio>
#include <deque>

#include "pool_sched.h"

using namespace tc;

static int fails = 0;
#define EXPECT(c)                                             \
    do {                                                      \
        if (!(c)) {                                           \
            printf("FAIL line %d: %s\n", __LINE__, #c);       \
            ++fails;                                          \
        }                                                     \
    } while (0)

static SchedWorkers workers(uint64_t budget, std::vector<uint64_t> held, std::vector<uint64_t> resv,
                            std::vector<bool> busy) {
    SchedWorkers w;
    w.budget = budget;
    w.held = held;
    w.resv = resv;
    w.busy = busy;
    return w;
}

// Event simulation: 3 workers, budget 100, small jobs (footprint 30, 1 s each)
// arrive every 0.4 s behind one large job (footprint 60, submitted first, at a
// moment when two small jobs already run).  Returns the time the large job starts
// (or -1 if it has not started after 60 s).
static double simulate(double head_wait_s) {
    struct Run { double end; uint64_t fp; };
    std::vector<Run> running = {{0.7, 30}, {0.9, 30}};
    struct Q { uint64_t fp; double t_sub; bool large; };
    std::deque<Q> q = {{60, 0.0, true}};
    double next_small = 0.0;
    for (double t = 0.0; t < 60.0; t += 0.05) {
        while (next_small <= t) { q.push_back({30, next_small, false}); next_small += 0.4; }
        for (size_t i = 0; i < running.size();)
            if (running[i].end <= t) running.erase(running.begin() + i); else ++i;
        for (;;) {
            if (running.size() >= 3 || q.empty()) break;
            std::vector<SchedJob> sj;
            for (auto& e : q) sj.push_back(SchedJob{e.fp, t - e.t_sub});
            SchedWorkers w = workers(100, {0, 0, 0}, {0, 0, 0}, {false, false, false});
            for (size_t i = 0; i < running.size(); ++i) { w.resv[i] = running[i].fp; w.busy[i] = true; }
            SchedChoice c = sched_pick(sj, w, head_wait_s);
            if (c.index < 0) break;
            if (q[c.index].large) return t;
            running.push_back({t + 1.0, q[c.index].fp});
            q.erase(q.begin() + c.index);
        }
    }
    return -1.0;
}

int main() {
    // the head fits: it starts
    {
        std::vector<SchedJob> q = {{40, 0.1}, {10, 0.0}};
        SchedChoice c = sched_pick(q, workers(100, {0, 0}, {50, 0}, {true, false}), 2.0);
        EXPECT(c.index == 0);
    }
    // the head does not fit and has not waited long: a later job that fits starts
    {
        std::vector<SchedJob> q = {{60, 0.5}, {30, 0.1}};
        SchedChoice c = sched_pick(q, workers(100, {0, 0, 0}, {30, 30, 0}, {true, true, false}), 2.0);
        EXPECT(c.index == 1);
    }
    // the head has waited past the limit: nothing else may start
    {
        std::vector<SchedJob> q = {{60, 2.5}, {30, 0.1}};
        SchedChoice c = sched_pick(q, workers(100, {0, 0, 0}, {30, 30, 0}, {true, true, false}), 2.0);
        EXPECT(c.index == -1);
        EXPECT(!c.release_idle);  // nothing idle to give back
    }
    // ... and once the running jobs drain it starts
    {
        std::vector<SchedJob> q = {{60, 3.0}, {30, 0.6}};
        SchedChoice c = sched_pick(q, workers(100, {0, 0, 0}, {30, 0, 0}, {true, false, false}), 2.0);
        EXPECT(c.index == 0);
    }
    // idle workspaces block the head: hand them back
    {
        std::vector<SchedJob> q = {{60, 0.2}};
        SchedChoice c = sched_pick(q, workers(100, {20, 30, 0}, {0, 0, 0}, {false, false, false}), 2.0);
        EXPECT(c.index == -1 && c.release_idle);
    }
    // idle workspaces are small; a busy worker's reservation blocks the head: keep them
    {
        std::vector<SchedJob> q = {{60, 0.2}};
        SchedChoice c = sched_pick(q, workers(100, {5, 0, 0}, {0, 50, 0}, {false, true, false}), 2.0);
        EXPECT(c.index == -1 && !c.release_idle);
    }
    // not yet prioritised: freeing is for the smallest queued job
    {
        std::vector<SchedJob> q = {{90, 0.2}, {30, 0.1}};
        SchedChoice c = sched_pick(q, workers(100, {40, 0}, {0, 40}, {false, true}), 2.0);
        EXPECT(c.index == -1 && c.release_idle);  // 40 busy + 30 fits once the 40 idle bytes go
    }
    // empty queue
    {
        SchedChoice c = sched_pick({}, workers(100, {0}, {0}, {false}), 2.0);
        EXPECT(c.index == -1 && !c.release_idle);
    }
    // the stream: with the rule the large job starts soon after the limit; with
    // an unreachable limit small jobs overtake it for the whole minute
    const double t_rule = simulate(2.0), t_none = simulate(1e9);
    printf("large job starts at %.2f s with the rule, %.2f without\n", t_rule, t_none);
    EXPECT(t_rule >= 2.0 && t_rule <= 4.0);
    EXPECT(t_none < 0);
    if (fails == 0) printf("ALL OK\n");
    return fails ? 1 : 0;
}
