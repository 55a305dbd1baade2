// el_batch.cu -- batched scenes: every scene's sub-step captured as one branch of a single CUDA
// graph, launched once per batch step.  Nothing is decided on the host between launches: each
// scene computes its own dt on the device (Simulator::update's CFL sub-stepping,
// simulator.cpp:23-42), runs update_second_order's work (apps/eulerian_liquid_3d.cpp:106-120,
// reinitialize() excluded) and solves with the mixed solver whose loops are conditional nodes.
//
// The advection writes into the context's ping-pong buffers and swaps them on the host while
// being captured, so a graph captured from one buffer assignment leaves the scene in the other.
// The batch therefore captures two graphs, one per assignment, and launches them alternately;
// the contexts' host-side pointers are set to match after every call.
#include <algorithm>
#include <array>
#include <cstring>
#include <vector>

#include "el_internal.cuh"

using namespace el;

namespace el {
int enqueue_step_device(el_ctx* ctx, const el_step_params& p, double cfl, double dt_frame, const BatchRecord* rec,
                        int kernels[3], bool fork);
int ensure_solver(el_ctx* ctx, int solver);
int prepare_device_solve(el_ctx* ctx);
int prepare_device_step(el_ctx* ctx);
}  // namespace el

namespace {

// Field and ping-pong buffer pointers of a context: the two states the graphs alternate between.
struct Buffers {
    std::array<void*, kMaxFields> field;
    std::array<void*, 4> tmp;
    bool operator==(const Buffers& o) const { return field == o.field && tmp == o.tmp; }
};

Buffers snapshot(const el_ctx* c) {
    Buffers b;
    std::copy(std::begin(c->field), std::end(c->field), b.field.begin());
    std::copy(std::begin(c->tmp), std::end(c->tmp), b.tmp.begin());
    return b;
}

void restore(el_ctx* c, const Buffers& b) {
    std::copy(b.field.begin(), b.field.end(), c->field);
    std::copy(b.tmp.begin(), b.tmp.end(), c->tmp);
}

// Running totals after a sub-step, from the outer scalars the step left behind.
template <typename T>
__global__ void record_kernel(const Scalars* s, BatchRecord* r, double dt_frame) {
    const double dt = s->dt;
    r->steps += 1;
    r->time += dt;
    r->last_dt = dt;
    // frame clock in the field type, as Simulator::update's float dt_total
    const T t = (T)r->frame_t + (T)dt;
    if (dt_frame > 0.0 && !(t < (T)dt_frame)) {
        r->frame_t = 0.0;
        r->frames += 1;
    } else {
        r->frame_t = (double)t;
    }
    r->iterations += s->inner_total;
    r->outer += s->outer;
    r->passes += s->inner_passes;
    const double rel = s->bb > 0.0 ? sqrt(s->rr / s->bb) : 0.0;
    r->max_relres = fmax(r->max_relres, rel);
    if (s->count == 0) {
        r->no_fluid += 1;
    } else if (!s->done) {
        r->unconverged += 1;
    }
    if (s->bad) r->bad += 1;
}

}  // namespace

struct el_batch {
    int device = 0;
    std::vector<el_ctx*> scenes;
    el_step_params params{};
    double cfl = 1.0, dt_frame = 0.0;
    cudaStream_t stream = nullptr;             // launches
    std::vector<cudaStream_t> branch;          // capture only: one per scene
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    std::vector<Buffers> state[2];             // per scene, before graph 0 / graph 1
    BatchRecord* rec = nullptr;                // device, one per scene
    std::vector<std::array<int, 3>> kernels;   // per scene: outside loops, per sweep, per pass
    int64_t graph_kernels = 0;
    // a scene's independent pieces (extrapolations, advections) as parallel graph branches: pays
    // for one or two scenes; with more, the scenes' own branches already fill the GPU and the
    // extra branches cost more than they overlap (a 32-scene step ran 1.5x slower with them)
    bool fork_steps = false;
    std::string error;
};

static int batch_error(el_batch* b, int code, const std::string& msg) {
    if (b) b->error = msg;
    return code;
}

static void batch_free(el_batch* b) {
    if (!b) return;
    DeviceGuard guard(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto& e : b->exec)
        if (e) cudaGraphExecDestroy(e);
    for (cudaStream_t s : b->branch)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : b->join)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->rec) cudaFree(b->rec);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Captures one graph: fork from the batch stream into a branch per scene, each scene's step,
// a record kernel, join.  Every scene's host-side buffer pointers advance by one step.
static int capture(el_batch* b, cudaGraphExec_t* out, bool count_kernels) {
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return batch_error(b, EL_ERR_CUDA, "begin capture");
    cudaEventRecord(b->fork, b->stream);
    int rc = EL_OK;
    for (size_t q = 0; q < b->scenes.size() && rc == EL_OK; ++q) {
        el_ctx* c = b->scenes[q];
        cudaStreamWaitEvent(b->branch[q], b->fork, 0);
        cudaStream_t own = c->stream;
        c->stream = b->branch[q];
        int k[3] = {0, 0, 0};
        rc = enqueue_step_device(c, b->params, b->cfl, b->dt_frame, b->rec + q, k, b->fork_steps);
        if (rc == EL_OK) {
            if (c->dtype == EL_F64)
                record_kernel<double><<<1, 1, 0, c->stream>>>(c->dscal, b->rec + q, b->dt_frame);
            else
                record_kernel<float><<<1, 1, 0, c->stream>>>(c->dscal, b->rec + q, b->dt_frame);
            k[0] += 1;
            if (count_kernels) b->kernels[q] = {k[0], k[1], k[2]};
            cudaEventRecord(b->join[q], c->stream);
            cudaStreamWaitEvent(b->stream, b->join[q], 0);
        } else {
            b->error = std::string("scene ") + std::to_string(q) + ": " + c->last_error;
        }
        c->stream = own;
    }
    const cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
    if (rc != EL_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return batch_error(b, EL_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    const cudaError_t ei = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return batch_error(b, EL_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ei));
    if (cudaGraphUpload(*out, b->stream) != cudaSuccess) return batch_error(b, EL_ERR_CUDA, "graph upload");
    return EL_OK;
}

// the graphs' buffer assignment that every scene is in now (-1: none, or not all the same)
static int current_parity(const el_batch* b) {
    int parity = -1;
    for (size_t q = 0; q < b->scenes.size(); ++q) {
        const Buffers now = snapshot(b->scenes[q]);
        const int p = now == b->state[0][q] ? 0 : (now == b->state[1][q] ? 1 : -1);
        if (p < 0 || (parity >= 0 && p != parity)) return -1;
        parity = p;
    }
    return parity;
}

// orders the batch stream after (to_batch) or before (!to_batch) every scene's own stream
static int order_with_scenes(el_batch* b, bool to_batch) {
    for (size_t q = 0; q < b->scenes.size(); ++q) {
        el_ctx* c = b->scenes[q];
        cudaStream_t from = to_batch ? c->stream : b->stream;
        cudaStream_t to = to_batch ? b->stream : c->stream;
        if (cudaEventRecord(b->join[q], from) != cudaSuccess || cudaStreamWaitEvent(to, b->join[q], 0) != cudaSuccess)
            return batch_error(b, EL_ERR_CUDA, "stream ordering");
    }
    return EL_OK;
}

#define EL_API extern "C" __attribute__((visibility("default")))

EL_API int el_batch_create(el_ctx* const* scenes, int count, const el_step_params* p, double cfl, double dt_frame,
                           el_batch** out) {
    if (!out) return EL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!scenes || count < 1 || !p || !(cfl > 0) || !(dt_frame >= 0)) return EL_ERR_INVALID_ARGUMENT;
    if (p->solve.solver != EL_SOLVER_MIXED || !(p->solve.tol > 0) || p->solve.max_iter < 1 ||
        p->extrapolation_layers < 0 || (p->trace_phi != EL_TRACE_RK2 && p->trace_phi != EL_TRACE_RK3) ||
        (p->trace_vel != EL_TRACE_RK2 && p->trace_vel != EL_TRACE_RK3) ||
        (p->sample_phi != EL_SAMPLE_TRILINEAR && p->sample_phi != EL_SAMPLE_WENO6) ||
        (p->sample_vel != EL_SAMPLE_TRILINEAR && p->sample_vel != EL_SAMPLE_WENO6))
        return EL_ERR_INVALID_ARGUMENT;
    for (int q = 0; q < count; ++q) {
        if (!scenes[q] || scenes[q]->device != scenes[0]->device || scenes[q]->prof_mask != 0)
            return EL_ERR_INVALID_ARGUMENT;
        for (int r = 0; r < q; ++r)
            if (scenes[r] == scenes[q]) return EL_ERR_INVALID_ARGUMENT;
    }
    el_batch* b = new (std::nothrow) el_batch();
    if (!b) return EL_ERR_OUT_OF_MEMORY;
    b->device = scenes[0]->device;
    b->scenes.assign(scenes, scenes + count);
    b->params = *p;
    b->fork_steps = count <= 2;
    b->cfl = cfl;
    b->dt_frame = dt_frame;
    b->kernels.assign(count, {0, 0, 0});
    int rc = EL_OK;
    auto fail = [&](int code) {
        batch_free(b);
        return code;
    };
    DeviceGuard guard(b->device);
    if (guard.err != cudaSuccess) return fail(EL_ERR_CUDA);
    for (el_ctx* c : b->scenes) {
        rc = ensure_solver(c, EL_SOLVER_MIXED);
        if (rc == EL_OK) rc = prepare_device_solve(c);
        if (rc == EL_OK) rc = ensure_extrapolation(c, 4);  // scratch of the captured step (allocates)
        if (rc == EL_OK && b->fork_steps) rc = prepare_device_step(c);
        if (rc != EL_OK) return fail(rc);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(EL_ERR_CUDA);
    }
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(EL_ERR_CUDA);
    if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) return fail(EL_ERR_CUDA);
    b->branch.assign(count, nullptr);
    b->join.assign(count, nullptr);
    for (int q = 0; q < count; ++q) {
        if (cudaStreamCreateWithFlags(&b->branch[q], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->join[q], cudaEventDisableTiming) != cudaSuccess)
            return fail(EL_ERR_CUDA);
    }
    if (cudaMalloc(&b->rec, count * sizeof(BatchRecord)) != cudaSuccess) return fail(EL_ERR_OUT_OF_MEMORY);
    if (cudaMemset(b->rec, 0, count * sizeof(BatchRecord)) != cudaSuccess) return fail(EL_ERR_CUDA);
    for (int parity = 0; parity < 2; ++parity) {
        b->state[parity].clear();
        for (el_ctx* c : b->scenes) b->state[parity].push_back(snapshot(c));
        rc = capture(b, &b->exec[parity], parity == 0);
        if (rc != EL_OK) {
            // put every scene back to the assignment it came in with
            for (int q = 0; q < count; ++q) restore(b->scenes[q], b->state[0][q]);
            const std::string msg = b->error;
            batch_free(b);
            if (!msg.empty()) scenes[0]->last_error = msg;
            return rc;
        }
    }
    // both captures done: the scenes are back in the assignment of graph 0
    b->graph_kernels = 0;
    for (auto& k : b->kernels) b->graph_kernels += k[0];
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return fail(EL_ERR_CUDA);
    *out = b;
    return EL_OK;
}

EL_API int el_batch_destroy(el_batch* b) {
    if (!b) return EL_ERR_INVALID_ARGUMENT;
    batch_free(b);
    return EL_OK;
}

EL_API const char* el_batch_last_error(const el_batch* b) { return b ? b->error.c_str() : "null batch"; }

EL_API int el_batch_step(el_batch* b, int steps) {
    if (!b || steps < 0) return EL_ERR_INVALID_ARGUMENT;
    if (steps == 0) return EL_OK;
    DeviceGuard guard(b->device);
    if (guard.err != cudaSuccess) return batch_error(b, EL_ERR_CUDA, cudaGetErrorString(guard.err));
    int parity = current_parity(b);
    if (parity < 0) return batch_error(b, EL_ERR_INVALID_ARGUMENT, "a scene was stepped outside the batch");
    int rc = order_with_scenes(b, true);
    if (rc != EL_OK) return rc;
    NvtxRange range("el_batch_step");
    for (int s = 0; s < steps; ++s) {
        const cudaError_t e = cudaGraphLaunch(b->exec[parity], b->stream);
        if (e != cudaSuccess) return batch_error(b, EL_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
        parity ^= 1;
    }
    for (size_t q = 0; q < b->scenes.size(); ++q) restore(b->scenes[q], b->state[parity][q]);
    return order_with_scenes(b, false);
}

EL_API int el_batch_sync(el_batch* b) {
    if (!b) return EL_ERR_INVALID_ARGUMENT;
    const cudaError_t e = cudaStreamSynchronize(b->stream);
    return e == cudaSuccess ? EL_OK : batch_error(b, EL_ERR_CUDA, cudaGetErrorString(e));
}

EL_API int el_batch_stats_get(el_batch* b, el_batch_stats* out) {
    if (!b || !out) return EL_ERR_INVALID_ARGUMENT;
    std::vector<BatchRecord> h(b->scenes.size());
    if (cudaMemcpyAsync(h.data(), b->rec, h.size() * sizeof(BatchRecord), cudaMemcpyDeviceToHost, b->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
        return batch_error(b, EL_ERR_CUDA, "stats copy");
    for (size_t q = 0; q < h.size(); ++q) {
        const BatchRecord& r = h[q];
        el_batch_stats& o = out[q];
        o.steps = r.steps;
        o.frames = r.frames;
        o.iterations = r.iterations;
        o.outer_iterations = r.outer;
        // the record kernel is counted among the kernels outside the loops
        o.kernels = r.steps * b->kernels[q][0] + r.outer * b->kernels[q][1] + r.passes * b->kernels[q][2];
        o.unconverged_steps = r.unconverged;
        o.no_fluid_steps = r.no_fluid;
        o.bad_steps = r.bad;
        o.time = r.time;
        o.last_dt = r.last_dt;
        o.max_relres = r.max_relres;
        o.frame_time = r.frame_t;
    }
    return EL_OK;
}

EL_API int el_batch_stats_reset(el_batch* b) {
    if (!b) return EL_ERR_INVALID_ARGUMENT;
    // keeps the frame clock: only the totals restart
    std::vector<BatchRecord> h(b->scenes.size());
    if (cudaMemcpyAsync(h.data(), b->rec, h.size() * sizeof(BatchRecord), cudaMemcpyDeviceToHost, b->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
        return batch_error(b, EL_ERR_CUDA, "stats copy");
    for (auto& r : h) {
        const double t = r.frame_t;
        r = BatchRecord{};
        r.frame_t = t;
    }
    if (cudaMemcpyAsync(b->rec, h.data(), h.size() * sizeof(BatchRecord), cudaMemcpyHostToDevice, b->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
        return batch_error(b, EL_ERR_CUDA, "stats reset");
    return EL_OK;
}

EL_API void* el_batch_get_stream(el_batch* b) { return b ? (void*)b->stream : nullptr; }

EL_API int64_t el_batch_graph_kernels(const el_batch* b) { return b ? b->graph_kernels : -1; }
