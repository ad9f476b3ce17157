// The whole k-Shape loop as one CUDA graph: control kernels and the graph builder
// (the design is described in loop_graph.h).
#include "loop_graph.h"

#include <cmath>

namespace tc {

namespace {

// The stages' result words in aux (the layout run_loop reads back).
struct AuxWords {
    int32_t changed, pad;
    double dsum;
    int32_t sum_class, bad_label;
    unsigned long long evals, moved, spairs;
    int32_t err[2];
};
static_assert(sizeof(AuxWords) == 56, "aux layout");

__device__ int next_mode(const LoopCtl& c) {
    if (!c.bnd) return BOUNDS_OFF;
    int use = c.refresh ? BOUNDS_REFRESH : (c.regroup ? BOUNDS_USE_REGROUP : BOUNDS_USE);
    if ((use == BOUNDS_USE || use == BOUNDS_USE_REGROUP) && !c.valid) use = BOUNDS_REFRESH;
    return use;
}

__device__ int variant_of(int mode) {
    return mode == BOUNDS_USE ? 1 : mode == BOUNDS_USE_REGROUP ? 2 : 0;
}

// After an extraction (kshape.cuh:241-262): the class count, and the stop when too
// few clusters kept members.
__device__ void extraction_done(LoopCtl& c, const AuxWords& a) {
    if (a.err[0] || a.err[1] || a.bad_label) {
        c.stop = LOOP_ERROR;  // the host reports which
        return;
    }
    if (!c.cal_select) c.sum_class = a.sum_class;  // get_class_centers_a leaves sum_class alone
    if (c.sum_class == 1 || c.sum_class <= c.k / 2) {
        c.iterations = c.i + 1;
        c.stop = LOOP_DONE;
    }
}

// After a bounded assignment: the refresh / regroup rule (restates the host's
// bounds_feedback with the same double arithmetic, no contractions).
__device__ void bounds_feedback(LoopCtl& c, int used, unsigned long long evals, unsigned long long moved,
                                unsigned long long spairs) {
    if (used == BOUNDS_REFRESH) {
        ++c.screened;
        c.moved = 0;
        c.regroup = 0;
        c.sum_f = 0;
        c.min_f = 2;
        c.passes = 0;
    } else if (used == BOUNDS_USE || used == BOUNDS_USE_REGROUP) {
        evals *= 128;  // the pass counts (128-row tile, centroid) pairs
        ++c.bounded;
        c.bounded_pairs += evals;
        c.series_pairs += spairs;
        c.moved = (used == BOUNDS_USE_REGROUP ? 0ull : c.moved) + moved;
        c.regroup = (long long)c.moved * c.regroup_share > c.n;
        const double f = __ddiv_rn((double)evals, __dmul_rn((double)c.n, (double)c.k));
        c.sum_f = __dadd_rn(c.sum_f, f);
        c.min_f = f < c.min_f ? f : c.min_f;
        ++c.passes;
        c.refresh = __dsub_rn(c.sum_f, __dmul_rn((double)c.passes, c.min_f)) >= BOUNDS_REFRESH_COST;
    }
}

// Iteration i is over: the next starts in the graph if its assignment variant is there.
__device__ void advance(LoopCtl& c, cudaGraphConditionalHandle hw) {
    c.i += 1;
    unsigned go = 0;
    if (c.i >= c.cap) {
        c.iterations = c.cap;
        c.stop = LOOP_DONE;
    } else if (++c.bodies >= c.cap) {
        c.stop = LOOP_ERROR;  // cannot happen: every body advances i or stops
    } else {
        c.mode = next_mode(c);
        if ((c.avail >> variant_of(c.mode)) & 1) go = 1;
        else c.stop = LOOP_HOST;
    }
    cudaGraphSetConditional(hw, go);
}

}  // namespace

// Before the assignment: (order 0) the extraction's checks, then the variant to run.
__global__ void k_loop_select(LoopCtl* ctl, const AuxWords* aux, cudaGraphConditionalHandle hsw, int after_extract) {
    LoopCtl& c = *ctl;
    unsigned sel = 3;  // no body
    if (c.stop == LOOP_RUN && after_extract) {
        c.launched += c.kern_extract;
        extraction_done(c, *aux);
    }
    if (c.stop == LOOP_RUN) sel = variant_of(c.mode);
    c.launched += 1;
    cudaGraphSetConditional(hsw, sel);
}

// After the assignment (kshape.cuh:270-307): bounds rule, inertia, convergence, the
// old-label copy; then (order 0) the next iteration, or (order 1) the extraction.
__global__ void k_loop_assigned(LoopCtl* ctl, const AuxWords* aux, cudaGraphConditionalHandle hcopy,
                                cudaGraphConditionalHandle hnext, int order_tsl) {
    LoopCtl& c = *ctl;
    const AuxWords a = *aux;
    unsigned copy = 0, next = 0;
    c.launched += 1;
    if (c.stop == LOOP_RUN) {
        c.launched += c.kern_assign[variant_of(c.mode)];
        if (a.err[0] || a.err[1]) {
            c.stop = LOOP_ERROR;
        } else {
            if (c.bnd) {
                if (c.mode == BOUNDS_REFRESH) {
                    c.valid = 1;
                    c.refresh = 0;
                }
                bounds_feedback(c, c.mode, a.evals, a.moved, a.spairs);
            }
            c.inertia = a.dsum / (double)c.n;
            if (a.changed == 0 || c.count_iter > 20) {
                c.iterations = c.i + 1;
                c.stop = LOOP_DONE;
            } else {
                if (c.inertia < c.old_inertia || fabs(c.old_inertia - c.inertia) < 1e-6) {
                    copy = 1;
                    c.old_inertia = c.inertia;
                    c.count_iter = 0;
                } else {
                    ++c.count_iter;
                }
                next = 1;
            }
        }
    }
    cudaGraphSetConditional(hcopy, copy);
    if (order_tsl) cudaGraphSetConditional(hnext, next);
    else if (next) advance(c, hnext);
    else cudaGraphSetConditional(hnext, 0);
}

// Order 1, after the extraction: its checks, then the next iteration.
__global__ void k_loop_extracted(LoopCtl* ctl, const AuxWords* aux, cudaGraphConditionalHandle hw) {
    LoopCtl& c = *ctl;
    c.launched += 1;
    if (c.stop == LOOP_RUN) {
        c.launched += c.kern_extract;
        extraction_done(c, *aux);
    }
    if (c.stop == LOOP_RUN) advance(c, hw);
    else cudaGraphSetConditional(hw, 0);
}

namespace {

struct Builder {
    cudaGraph_t top = nullptr;
    bool ok = true;

    void check(cudaError_t e) {
        if (e != cudaSuccess) ok = false;
    }
    cudaGraphNode_t kernel(cudaGraph_t g, const cudaGraphNode_t* dep, void* func, void** args) {
        cudaGraphNode_t node = nullptr;
        if (!ok) return node;
        cudaKernelNodeParams p{};
        p.func = func;
        p.gridDim = dim3(1);
        p.blockDim = dim3(1);
        p.sharedMemBytes = 0;
        p.kernelParams = args;
        check(cudaGraphAddKernelNode(&node, g, dep, dep ? 1 : 0, &p));
        return node;
    }
    cudaGraphNode_t child(cudaGraph_t g, const cudaGraphNode_t* dep, cudaGraph_t sub) {
        cudaGraphNode_t node = nullptr;
        if (ok) check(cudaGraphAddChildGraphNode(&node, g, dep, dep ? 1 : 0, sub));
        return node;
    }
    // a conditional node; its bodies come back in body[]
    cudaGraphNode_t conditional(cudaGraph_t g, const cudaGraphNode_t* dep, cudaGraphConditionalHandle h,
                                cudaGraphConditionalNodeType type, unsigned size, cudaGraph_t* body) {
        cudaGraphNode_t node = nullptr;
        if (!ok) return node;
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = type;
        p.conditional.size = size;
        check(cudaGraphAddNode(&node, g, dep, nullptr, dep ? 1 : 0, &p));
        if (ok)
            for (unsigned i = 0; i < size; ++i) body[i] = p.conditional.phGraph_out[i];
        return node;
    }
    // the while handle starts every launch at 1; the others are set by a control
    // kernel before their node runs
    cudaGraphConditionalHandle handle(cudaGraph_t g, unsigned dflt, unsigned flags = 0) {
        cudaGraphConditionalHandle h = 0;
        if (ok) check(cudaGraphConditionalHandleCreate(&h, g, dflt, flags));
        return h;
    }
};

}  // namespace

cudaGraphExec_t build_loop_graph(const LoopGraphSpec& sp) {
    Builder b;
    if (!sp.extract || cudaGraphCreate(&b.top, 0) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    cudaGraph_t body = nullptr;
    const cudaGraphConditionalHandle hw = b.handle(b.top, 1, cudaGraphCondAssignDefault);
    b.conditional(b.top, nullptr, hw, cudaGraphCondTypeWhile, 1, &body);
    const cudaGraphConditionalHandle hsw = b.handle(body, 3);
    const cudaGraphConditionalHandle hcopy = b.handle(body, 0);

    LoopCtl* ctl = sp.ctl;
    const AuxWords* aux = static_cast<const AuxWords*>(sp.aux);
    int after_extract = sp.order_tsl ? 0 : 1;
    int order = sp.order_tsl;
    cudaGraphNode_t last = nullptr;
    if (!sp.order_tsl) last = b.child(body, nullptr, sp.extract);
    {
        void* args[] = {&ctl, &aux, const_cast<cudaGraphConditionalHandle*>(&hsw), &after_extract};
        last = b.kernel(body, last ? &last : nullptr, (void*)k_loop_select, args);
    }
    cudaGraph_t variants[3] = {nullptr, nullptr, nullptr};
    last = b.conditional(body, &last, hsw, cudaGraphCondTypeSwitch, 3, variants);
    for (int v = 0; v < 3 && b.ok; ++v) {
        cudaGraphNode_t node = nullptr;
        if (sp.assign[v]) b.child(variants[v], nullptr, sp.assign[v]);
        else b.check(cudaGraphAddEmptyNode(&node, variants[v], nullptr, 0));
    }
    // order 0: the while handle comes next; order 1: the extraction's IF handle
    const cudaGraphConditionalHandle hnext = sp.order_tsl ? b.handle(body, 0) : hw;
    {
        void* args[] = {&ctl, &aux, const_cast<cudaGraphConditionalHandle*>(&hcopy),
                        const_cast<cudaGraphConditionalHandle*>(&hnext), &order};
        last = b.kernel(body, &last, (void*)k_loop_assigned, args);
    }
    cudaGraph_t copy_body = nullptr;
    last = b.conditional(body, &last, hcopy, cudaGraphCondTypeIf, 1, &copy_body);
    if (b.ok) {
        cudaGraphNode_t node = nullptr;
        b.check(cudaGraphAddMemcpyNode1D(&node, copy_body, nullptr, 0, sp.old_labels, sp.labels,
                                         sizeof(int32_t) * (size_t)sp.n, cudaMemcpyDeviceToDevice));
    }
    if (sp.order_tsl) {
        cudaGraph_t ext_body = nullptr;
        last = b.conditional(body, &last, hnext, cudaGraphCondTypeIf, 1, &ext_body);
        b.child(ext_body, nullptr, sp.extract);
        void* args[] = {&ctl, &aux, const_cast<cudaGraphConditionalHandle*>(&hw)};
        last = b.kernel(body, &last, (void*)k_loop_extracted, args);
    }
    cudaGraphExec_t exec = nullptr;
    if (b.ok && cudaGraphInstantiate(&exec, b.top, 0) != cudaSuccess) exec = nullptr;
    cudaGraphDestroy(b.top);
    cudaGetLastError();
    return exec;
}

}  // namespace tc
