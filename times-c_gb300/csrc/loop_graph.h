// The whole k-Shape loop as one CUDA graph (kshape.cuh:235-311 / :383-455): a WHILE
// node runs the iterations, each one the extraction and assignment stages (child
// graphs of their captured stage graphs) followed by small control kernels that
// restate the host loop's decisions on device-resident state - the class-count stop,
// the convergence test with its inertia rule, the old-label copy (an IF node), and the
// bounded assignment's refresh / regroup rule, whose outcome a SWITCH node turns into
// the next iteration's assignment variant.  No host round trip between iterations.
//
// The host runs an iteration itself while a stage it needs has no captured graph yet
// (its first runs set up buffers, tables and launch plans); the graph then returns at
// that iteration's start (LOOP_HOST) and is rebuilt once the stage is captured.
// tc_kshape_run uses it with TIMESC_DEVICE_LOOP=1: measured on a GB300, the two host
// read-backs per iteration it removes cost about what its conditional nodes and
// control kernels add, so it is not the default.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace tc {

// Bounds modes of one assignment (api.cpp): none, a full pass, a bounded pass, a
// bounded pass after regrouping the series.
enum { BOUNDS_OFF = 0, BOUNDS_AUTO = -1, BOUNDS_REFRESH = 1, BOUNDS_USE = 2, BOUNDS_USE_REGROUP = 3 };
// a full pass again once the bounded passes since the last one cost, beyond the
// cheapest of them, one full pass (sum of evaluated fractions - passes x minimum)
constexpr double BOUNDS_REFRESH_COST = 1.0;
// regroup once more than 1/20 of the series changed best centroid since the last grouping
// (at n = 1e6, m = 512, k = 32: 6.15 ms per iteration against 6.21 at 1/200 and 6.16
// with no regrouping, whose first bounded passes evaluate up to 15% more pairs)
// (TIMESC_REGROUP_SHARE=s in the environment: 1/s)
constexpr int64_t BOUNDS_REGROUP_SHARE = 20;

// The assignment stage variants a loop graph holds: 0 full pass (or no bounds),
// 1 bounded pass, 2 bounded pass on a new grouping.
inline int assign_variant(int bounds_mode) {
    return bounds_mode == BOUNDS_USE ? 1 : bounds_mode == BOUNDS_USE_REGROUP ? 2 : 0;
}

enum { LOOP_RUN = 0, LOOP_DONE = 1, LOOP_ERROR = 2, LOOP_HOST = 3 };

// Device-resident loop state; the host writes it before a launch and reads it after.
struct LoopCtl {
    // fixed for the launch
    int64_t n;
    int64_t regroup_share;  // regroup once moved x regroup_share > n
    int k, cap, cal_select, bnd;
    int avail;           // bit v: assignment variant v is in the graph
    int kern_extract;    // kernels of one extraction stage
    int kern_assign[3];  // kernels of each assignment variant
    // the loop
    int i;           // the iteration being run (on LOOP_HOST: the one the host runs next)
    int count_iter;  // iterations since the inertia last improved (kshape.cuh:303-307)
    int sum_class;
    int iterations;  // set on LOOP_DONE
    int stop;        // LOOP_*
    int mode;        // bounds mode of iteration i's assignment
    int bodies;      // loop bodies run by this launch (a backstop against running past cap)
    int pad0;
    double old_inertia, inertia;
    unsigned long long launched;  // kernels this launch ran
    // the bounded assignment's state, as BoundsState
    int valid, refresh, regroup, passes;
    unsigned long long moved;
    double sum_f, min_f;
    unsigned long long screened, bounded, bounded_pairs, series_pairs;
};

// The stage graphs a loop graph is built from (captured, not instantiated by it).
struct LoopGraphSpec {
    cudaGraph_t extract = nullptr;
    cudaGraph_t assign[3] = {nullptr, nullptr, nullptr};
    int order_tsl = 0;  // 0: extraction then assignment (k_shape); 1: the reverse (k_shape_tsl)
    LoopCtl* ctl = nullptr;
    const void* aux = nullptr;  // the stages' result words (changed, dist sum, class count, counters, errors)
    const int32_t* labels = nullptr;
    int32_t* old_labels = nullptr;
    int64_t n = 0;
};

// Builds and instantiates the loop graph; nullptr if the runtime refuses any part of
// it (the caller then keeps running iterations from the host).
cudaGraphExec_t build_loop_graph(const LoopGraphSpec& spec);

}  // namespace tc
