// irr_batch.cu -- many independent instances in one persistent launch, and the
// autotuner that picks the owner-computes kernel's shape.
//
// The reference runs one edge set per runtime (paper Sec. II-C); a batch here
// is a table of instance descriptors (each partitioned handle's positions, row
// offsets, entries, results and law) plus one work-item list that
// concatenates every instance's node blocks.  One launch of tiled_kernel
// serves all of them: its CTAs claim (instance, block) items from one queue,
// which is the reference's per-part atomicAdd queue (gpu_kernel.cu:64-72)
// generalised across instances.  After irr_batch_capture a step is one CUDA
// graph replay (queue reset + launch).
//
// Autotuning: candidate shapes (lanes per node row x rows per work item) are
// timed on the actual data with CUDA events, a few launches each; the fastest
// is kept and remembered per (GPU, size class) for the life of the process.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "irr_handle.cuh"
#include "irr_trace.cuh"

using namespace irr;

struct irr_batch {
    int device = 0;
    int sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<irr_handle*> handles;
    TiledShape shape{};
    bool finalized = false;
    InstDesc* d_insts = nullptr;
    std::vector<InstDesc> host_insts;  // host copy of d_insts (the launch's parameter table)
    WorkItem* d_items = nullptr;
    int num_items = 0;
    int* d_queue = nullptr;
    int* d_status = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t nodes = 0;
    int64_t edges = 0;
};

namespace {

int bfail(irr_batch* b, int code, const std::string& what, cudaError_t e = cudaSuccess)
{
    if (b) {
        b->err = what;
        if (e != cudaSuccess) b->err += std::string(": ") + cudaGetErrorString(e);
    }
    cudaGetLastError();
    return code;
}

#define B_CUDA(b, expr, what)                                                              \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return bfail((b), e_ == cudaErrorMemoryAllocation ? IRR_ERR_NOMEM : IRR_ERR_CUDA, \
                         what, e_);                                                        \
    } while (0)

void drop_graph(irr_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// Rebuilds the instance table from the handles' current layouts.
int upload_insts(irr_batch* b)
{
    std::vector<InstDesc> insts;
    for (irr_handle* h : b->handles) {
        InstDesc d{};
        d.pos = h->d_pos;
        d.row_off = h->part.row_off;
        d.col = h->part.col;
        d.force = h->d_force;
        d.slice_off = h->shape.staged ? h->st.slice_off : (h->sl.lanes ? h->sl.slice_off : nullptr);
        d.scol = h->sl.lanes ? h->sl.col : nullptr;
        d.words = h->shape.staged ? h->st.words : nullptr;
        d.tab = h->shape.staged ? h->st.ids : nullptr;
        d.law = h->law;
        d.n = h->n;
        insts.push_back(d);
    }
    if (!b->d_insts)
        B_CUDA(b, cudaMalloc(&b->d_insts, sizeof(InstDesc) * insts.size()), "instance table");
    B_CUDA(b, cudaMemcpy(b->d_insts, insts.data(), sizeof(InstDesc) * insts.size(), cudaMemcpyHostToDevice),
           "instance table");
    b->host_insts = std::move(insts);
    return IRR_OK;
}

// Every instance's layout for G lanes per row, staged or not (each handle
// rebuilds its own descriptor and items with it), then the batch's instance
// table.  IRR_ERR_CAPACITY (no failure recorded) when the staged layout was
// asked for and some instance's graph does not fit it.
int set_lanes(irr_batch* b, int lanes, int staged)
{
    for (irr_handle* h : b->handles) {
        if (h->shape.lanes_per_row == lanes && h->shape.staged == staged) continue;  // already laid out
        const int rc = irr_ensure_layout(h, lanes, h->shape.block_nodes, staged);
        if (rc) return bfail(b, rc, std::string("instance layout: ") + irr_last_error(h));
        if (h->shape.staged != staged) return IRR_ERR_CAPACITY;
    }
    return upload_insts(b);
}

// Rebuilds the concatenated work-item list for `shape` and uploads it.
int upload_items(irr_batch* b, const TiledShape& shape)
{
    std::vector<WorkItem> items;
    for (size_t k = 0; k < b->handles.size(); k++) {
        const irr_handle* h = b->handles[k];
        if (shape.staged) {
            for (WorkItem w : h->st.items) {
                w.inst = (int32_t)k;
                items.push_back(w);
            }
        } else {
            make_instance_items(h->host_row_off.data(), h->sl, h->n, (int)k, shape, items);
        }
    }
    if (b->d_items) cudaFree(b->d_items);
    b->d_items = nullptr;
    B_CUDA(b, cudaMalloc(&b->d_items, sizeof(WorkItem) * (items.empty() ? 1 : items.size())), "work items");
    if (!items.empty())
        B_CUDA(b, cudaMemcpyAsync(b->d_items, items.data(), sizeof(WorkItem) * items.size(),
                                  cudaMemcpyHostToDevice, b->stream), "work items");
    B_CUDA(b, cudaStreamSynchronize(b->stream), "work items");
    b->num_items = (int)items.size();
    return IRR_OK;
}

int launch_step(irr_batch* b, const TiledShape& shape)
{
    B_CUDA(b, cudaMemsetAsync(b->d_queue, 0, sizeof(int), b->stream), "queue");
    B_CUDA(b, launch_tiled(shape, b->d_insts, b->d_items, b->num_items, b->d_queue,
                           b->sms * kCtasPerSm, b->d_status, b->stream, b->host_insts.data(),
                           (int)b->host_insts.size()), "batched kernel");
    return IRR_OK;
}

// ---------------------------------------------------------------- tuning
std::mutex g_tune_mutex;
std::map<std::string, TiledShape> g_tune_cache;

std::string tune_key(int device, int64_t instances, int64_t nodes, int64_t entries, int periodic)
{
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, device);
    const double per_inst = instances > 0 ? (double)nodes / instances : 0.0;
    const double per_row = nodes > 0 ? (double)entries / nodes : 0.0;
    char buf[512];
    snprintf(buf, sizeof(buf), "%s|sm%d|inst2^%d|nodes2^%d|deg2^%d|p%d", prop.name, prop.multiProcessorCount,
             (int)std::lround(std::log2((double)std::max<int64_t>(instances, 1))),
             (int)std::lround(std::log2(std::max(per_inst, 1.0))),
             (int)std::lround(std::log2(std::max(per_row, 1.0))), periodic);
    return buf;
}

// Times `shape` over `reps` launches; returns milliseconds per launch (< 0 on error).
double time_shape(irr_batch* b, const TiledShape& shape, int reps)
{
    if (upload_items(b, shape) != IRR_OK) return -1.0;
    if (launch_step(b, shape) != IRR_OK) return -1.0;  // warm-up
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, b->stream);
    for (int r = 0; r < reps; r++)
        if (launch_step(b, shape) != IRR_OK) return -1.0;
    cudaEventRecord(e1, b->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / reps;
}

int autotune(irr_batch* b)
{
    const std::string key = tune_key(b->device, (int64_t)b->handles.size(), b->nodes, 2 * b->edges,
                                     b->shape.periodic);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) b->shape = it->second;
        if (it != g_tune_cache.end()) {
            const int rc = set_lanes(b, b->shape.lanes_per_row, b->shape.staged);
            return rc ? rc : upload_items(b, b->shape);
        }
    }
    const int lanes[] = {4, 8, 16};
    const int rows[] = {64, 256, 1024};
    TiledShape best = b->shape;
    double best_ms = 1e30;
    // the staged layout first (4 lanes per row; items are its own), where every instance takes it
    {
        int rc = set_lanes(b, 4, 1);
        if (rc == IRR_OK) {
            TiledShape s = b->shape;
            s.lanes_per_row = 4;
            s.staged = 1;
            const double ms = time_shape(b, s, 3);
            if (ms < 0) return bfail(b, IRR_ERR_CUDA, "autotune launch");
            best_ms = ms;
            best = s;
        } else if (rc != IRR_ERR_CAPACITY) {
            return rc;
        }
    }
    for (int g : lanes) {
        const int rc = set_lanes(b, g, 0);
        if (rc) return rc;
        for (int r : rows) {
            TiledShape s = b->shape;
            s.lanes_per_row = g;
            s.block_nodes = r;
            s.staged = 0;
            const double ms = time_shape(b, s, 3);
            if (ms < 0) return bfail(b, IRR_ERR_CUDA, "autotune launch");
            if (ms < best_ms) {
                best_ms = ms;
                best = s;
            }
        }
    }
    b->shape = best;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[key] = best;
    }
    const int rc = set_lanes(b, b->shape.lanes_per_row, b->shape.staged);
    return rc ? rc : upload_items(b, b->shape);
}

}  // namespace

extern "C" {

int irr_batch_create(int device, irr_batch** out)
{
    if (!out) return IRR_ERR_ARG;
    *out = nullptr;
    irr_batch* b = new (std::nothrow) irr_batch();
    if (!b) return IRR_ERR_NOMEM;
    b->device = device;
    DeviceGuard dev_guard(device);
    if (!dev_guard.ok() ||
        cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&b->d_queue, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&b->d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(b->d_status, 0, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        irr_batch_destroy(b);
        return IRR_ERR_CUDA;
    }
    b->stream = b->own_stream;
    b->shape.lanes_per_row = 4;
    b->shape.block_nodes = 1024;
    b->shape.stage_smem = 1;
    b->shape.periodic = -1;
    *out = b;
    return IRR_OK;
}

int irr_batch_destroy(irr_batch* b)
{
    if (!b) return IRR_ERR_ARG;
    DeviceGuard dev_guard(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    if (b->d_insts) cudaFree(b->d_insts);
    if (b->d_items) cudaFree(b->d_items);
    if (b->d_queue) cudaFree(b->d_queue);
    if (b->d_status) cudaFree(b->d_status);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return IRR_OK;
}

const char* irr_batch_last_error(const irr_batch* b) { return b ? b->err.c_str() : "null batch"; }

int irr_batch_set_stream(irr_batch* b, void* stream)
{
    if (!b) return IRR_ERR_ARG;
    drop_graph(b);
    b->stream = (cudaStream_t)stream;
    return IRR_OK;
}

int irr_batch_add(irr_batch* b, irr_handle* h)
{
    if (!b || !h) return IRR_ERR_ARG;
    if (b->finalized) return bfail(b, IRR_ERR_STATE, "irr_batch_add after irr_batch_finalize");
    if (h->device != b->device) return bfail(b, IRR_ERR_ARG, "handle on another device");
    if (h->cfg.exec != IRR_EXEC_PARTITIONED) return bfail(b, IRR_ERR_ARG, "batched instances must be partitioned handles");
    if (!h->inited) {
        const int rc = irr_init(h);
        if (rc) return bfail(b, rc, std::string("instance init: ") + irr_last_error(h));
    }
    if (b->shape.periodic < 0) b->shape.periodic = h->law.periodic;
    if (b->shape.periodic != h->law.periodic)
        return bfail(b, IRR_ERR_ARG, "instances of one batch must share periodic or open boundaries");
    if (b->handles.size() >= 0x7fffffff) return bfail(b, IRR_ERR_CAPACITY, "too many instances");
    b->handles.push_back(h);
    return IRR_OK;
}

int irr_batch_finalize(irr_batch* b, int autotune_shape)
{
    irr::TraceRange trace_("irr_batch_finalize");
    if (!b) return IRR_ERR_ARG;
    if (b->finalized) return IRR_OK;
    if (b->handles.empty()) return bfail(b, IRR_ERR_STATE, "empty batch");
    DeviceGuard dev_guard(b->device);
    b->nodes = b->edges = 0;
    for (irr_handle* h : b->handles) {
        cudaStreamSynchronize(h->stream);
        b->nodes += h->n;
        b->edges += h->e;
    }
    int rc = IRR_OK;
    if (autotune_shape) {
        rc = autotune(b);
    } else {
        // the staged layout where every instance takes it (4 lanes per row), else sliced / CSR
        b->shape.staged = b->shape.lanes_per_row == 4 ? 1 : 0;
        rc = set_lanes(b, b->shape.lanes_per_row, b->shape.staged);
        if (rc == IRR_ERR_CAPACITY) {
            b->shape.staged = 0;
            rc = set_lanes(b, b->shape.lanes_per_row, 0);
        }
        if (!rc) rc = upload_items(b, b->shape);
    }
    if (rc) return rc;
    b->finalized = true;
    return IRR_OK;
}

int irr_batch_step(irr_batch* b)
{
    irr::TraceRange trace_("irr_batch_step");
    if (!b) return IRR_ERR_ARG;
    if (!b->finalized) return bfail(b, IRR_ERR_STATE, "irr_batch_step before irr_batch_finalize");
    DeviceGuard dev_guard(b->device);
    if (b->exec) {
        B_CUDA(b, cudaGraphLaunch(b->exec, b->stream), "graph replay");
        return IRR_OK;
    }
    return launch_step(b, b->shape);
}

int irr_batch_capture(irr_batch* b)
{
    if (!b) return IRR_ERR_ARG;
    if (!b->finalized) return bfail(b, IRR_ERR_STATE, "irr_batch_capture before irr_batch_finalize");
    if (b->stream == nullptr) return bfail(b, IRR_ERR_STATE, "capture needs a non-default stream");
    DeviceGuard dev_guard(b->device);
    drop_graph(b);
    int rc = launch_step(b, b->shape);  // sets the kernel's attributes outside the capture
    if (rc) return rc;
    B_CUDA(b, cudaStreamSynchronize(b->stream), "capture");
    B_CUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    rc = launch_step(b, b->shape);
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    B_CUDA(b, ee, "end capture");
    b->graph = g;
    B_CUDA(b, cudaGraphInstantiate(&b->exec, b->graph, 0), "instantiate graph");
    return IRR_OK;
}

int irr_batch_sync(irr_batch* b)
{
    if (!b) return IRR_ERR_ARG;
    DeviceGuard dev_guard(b->device);
    B_CUDA(b, cudaStreamSynchronize(b->stream), "synchronise");
    int st = 0;
    B_CUDA(b, cudaMemcpy(&st, b->d_status, sizeof(int), cudaMemcpyDeviceToHost), "status");
    if (st) {
        cudaMemset(b->d_status, 0, sizeof(int));
        return bfail(b, IRR_ERR_DEVICE, "device status set (a bounded wait gave up)");
    }
    return IRR_OK;
}

int irr_batch_get_info(const irr_batch* b, irr_batch_info* info)
{
    if (!b || !info) return IRR_ERR_ARG;
    memset(info, 0, sizeof(*info));
    info->num_instances = (int64_t)b->handles.size();
    info->num_nodes = b->nodes;
    info->num_edges = b->edges;
    info->num_items = b->num_items;
    info->lanes_per_row = b->shape.lanes_per_row;
    info->block_nodes = b->shape.block_nodes;
    info->graph = b->exec != nullptr;
    return IRR_OK;
}

int irr_autotune(irr_handle* h)
{
    irr::TraceRange trace_("irr_autotune");
    if (!h) return IRR_ERR_ARG;
    if (h->cfg.exec != IRR_EXEC_PARTITIONED) return IRR_OK;  // nothing to tune
    if (!h->inited) {
        const int rc = irr_init(h);
        if (rc) return rc;
    }
    irr_batch* b = nullptr;
    int rc = irr_batch_create(h->device, &b);
    if (rc) return rc;
    irr_batch_set_stream(b, h->stream);
    b->shape = h->shape;
    b->shape.periodic = -1;
    rc = irr_batch_add(b, h);
    if (!rc) rc = irr_batch_finalize(b, 1);
    if (!rc) {
        // the handle's own layout and work items for the chosen shape
        rc = irr_ensure_layout(h, b->shape.lanes_per_row, b->shape.block_nodes, b->shape.staged);
    } else {
        h->err = std::string("autotune: ") + b->err;
    }
    b->stream = nullptr;  // the handle's stream is not the batch's to destroy
    irr_batch_destroy(b);
    return rc;
}

}  // extern "C"
