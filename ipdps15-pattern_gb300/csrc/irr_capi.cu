// irr_capi.cu -- the C ABI (include/irregular_gb300.h) over the kernels.
//
// One handle = one IrregularRuntime (moldyn/irregular/irregular_runtime.h:
// 12-112) on one GPU.  The reference's MPI split, CPU/GPU work sharing and
// per-iteration re-split are not reproduced: node data and the partition stay
// resident on the device, and a step is one kernel launch.
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <string>
#include <vector>

#include "irr_handle.cuh"
#include "irr_trace.cuh"

using namespace irr;

namespace {

// IRR_LAYOUT_AUTO takes the staged layout where it applies (4 lanes per row,
// shared-memory stages, every 8 rows within the table limit) and pays: each
// staged position must serve at least kStagedMinReuse entries on average.
// Curve-ordered MD-like graphs reuse each ~9 times (4M-node workload: 0.39 ms
// per step staged vs 0.46 sliced); in the caller's random order the tables
// hold about one id per entry and the staged layout is slower (2.00 vs 1.41
// ms per step at 4M nodes).
constexpr bool kAutoStaged = true;
constexpr int64_t kStagedMinReuse = 3;

// User maps: largest parameter block and result record.
constexpr int kUserParamMax = 65536;
constexpr int kUserValueMax = 256;

int fail(irr_handle* h, int code, const char* fmt, ...)
{
    if (h) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        h->err = buf;
    }
    return code;
}

int cuda_fail(irr_handle* h, cudaError_t e, const char* what)
{
    cudaGetLastError();  // clear a non-sticky error
    const int code = (e == cudaErrorMemoryAllocation) ? IRR_ERR_NOMEM : IRR_ERR_CUDA;
    return fail(h, code, "%s: %s", what, cudaGetErrorString(e));
}

#define H_CUDA(h, expr, what)                                 \
    do {                                                      \
        cudaError_t e_ = (expr);                              \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, what); \
    } while (0)

template <class T>
void dfree(T*& p)
{
    if (p) cudaFree((void*)p);
    p = nullptr;
}

void free_layout(irr_handle* h)
{
    dfree(h->d_pos);
    dfree(h->d_force);
    dfree(h->part.perm);
    dfree(h->part.inv);
    dfree(h->part.row_off);
    dfree(h->part.col);
    free_sliced(&h->sl);
    free_staged(&h->st);
    h->shape.staged = 0;
    h->host_row_off.clear();
    dfree(h->d_inst);
    dfree(h->d_items);
    h->num_items = 0;
    dfree(h->d_rec);
    dfree(h->d_vals);
    dfree(h->d_iota);
    dfree(h->d_param);
    h->inited = false;
}

// Node records: positions (12/16/24 bytes) for the built-in laws; any
// multiple of 4 bytes up to 1024 for a user map.
bool valid_node_elm(const irr_handle* h, int elm)
{
    if (h->user_launch) return elm >= 4 && elm <= 1024 && (elm & 3) == 0;
    return elm == 12 || elm == 16 || elm == 24;
}

// Law parameters from the reference's parameter block for the selected map.
int make_law(irr_handle* h)
{
    const unsigned char* p = h->param.data();
    const size_t sz = h->param.size();
    double rc2d = 0, side = 0;
    int periodic = 0;
    switch (h->map_idx) {
    case IRR_MAP_LJ_MOLDYN: {  // struct para {double side; double cutoffRadius;}
        if (sz < 16) return fail(h, IRR_ERR_ARG, "moldyn map needs a 16-byte {side, cutoffRadius} block");
        double rc;
        memcpy(&side, p, 8);
        memcpy(&rc, p + 8, 8);
        rc2d = rc * rc;  // moldyn/irregular.h:40 cutoffSquare = cutoffRadius * cutoffRadius
        periodic = 1;
        break;
    }
    case IRR_MAP_LJ_MINIMD:  // double cutforcesq
        if (sz < 8) return fail(h, IRR_ERR_ARG, "miniMD map needs an 8-byte cutforcesq");
        memcpy(&rc2d, p, 8);
        break;
    case IRR_MAP_LJ_MINIMD_PBC:  // {double cutforcesq; double side;}
        if (sz < 16) return fail(h, IRR_ERR_ARG, "miniMD PBC map needs a 16-byte {cutforcesq, side} block");
        memcpy(&rc2d, p, 8);
        memcpy(&side, p + 8, 8);
        periodic = 1;
        break;
    default:
        return fail(h, IRR_ERR_ARG, "unknown map index %d", h->map_idx);
    }
    if (!(rc2d >= 0.0) || !std::isfinite(rc2d)) return fail(h, IRR_ERR_ARG, "cutoff^2 must be finite and >= 0");
    if (periodic && !(side > 0.0 && std::isfinite(side))) return fail(h, IRR_ERR_ARG, "box side must be finite and > 0");
    LawParams L{};
    L.rc2d = rc2d;
    L.rc2 = (float)rc2d;
    L.rc2_lo = (float)(rc2d * (1.0 - 1.0 / 262144.0));
    L.rc2_hi = (float)(rc2d * (1.0 + 1.0 / 262144.0));
    L.periodic = periodic;
    L.side = side;
    L.halfd = 0.5 * side;
    L.half = (float)(0.5 * side);
    L.side_hi = (float)side;
    L.side_lo = (float)(side - (double)L.side_hi);
    // rd from the unwrapped d exceeds (side/2)^2 whenever a component needs a
    // wrap; the margin covers rd's rounding.  Non-periodic: never wrap.
    L.half2 = periodic ? (float)(0.25 * side * side * (1.0 - 1.0 / 65536.0)) : INFINITY;
    // the FP64 decision band: rc2_lo < rd < rc2_hi, widened for the rounding of rd - rc2
    L.band = (float)(rc2d * (2.0 / 262144.0));
    h->law = L;
    h->have_law = true;
    return IRR_OK;
}

int upload_inst(irr_handle* h)
{
    if (!h->inited || h->cfg.exec != IRR_EXEC_PARTITIONED) return IRR_OK;
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
    h->inst = d;
    H_CUDA(h, cudaMemcpyAsync(h->d_inst, &d, sizeof(d), cudaMemcpyHostToDevice, h->stream),
           "upload instance descriptor");
    H_CUDA(h, cudaStreamSynchronize(h->stream), "upload instance descriptor");
    return IRR_OK;
}

int upload_items(irr_handle* h)
{
    std::vector<WorkItem> items;
    if (h->shape.staged)
        items = h->st.items;
    else
        make_instance_items(h->host_row_off.data(), h->sl, h->n, 0, h->shape, items);
    dfree(h->d_items);
    h->num_items = 0;
    H_CUDA(h, cudaMalloc(&h->d_items, sizeof(WorkItem) * (items.size() ? items.size() : 1)), "allocate work items");
    if (!items.empty())
        H_CUDA(h, cudaMemcpyAsync(h->d_items, items.data(), sizeof(WorkItem) * items.size(),
                                  cudaMemcpyHostToDevice, h->stream), "upload work items");
    H_CUDA(h, cudaStreamSynchronize(h->stream), "upload work items");
    h->num_items = (int)items.size();
    return IRR_OK;
}

int check_status(irr_handle* h)
{
    int st = 0;
    H_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream),
           "read status");
    H_CUDA(h, cudaStreamSynchronize(h->stream), "synchronise");
    if (st & kStatusBadIndex) {
        cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream);
        return fail(h, IRR_ERR_INDEX, "an edge endpoint is outside [0, %lld)", (long long)h->n);
    }
    if (st) {
        cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream);
        return fail(h, IRR_ERR_DEVICE, "device status 0x%x (a bounded wait gave up)", st);
    }
    return IRR_OK;
}

int ensure_raw(irr_handle* h, size_t bytes)
{
    if (bytes <= h->raw_cap) return IRR_OK;
    dfree(h->d_raw);
    h->raw_cap = 0;
    H_CUDA(h, cudaMalloc(&h->d_raw, bytes), "allocate node staging");
    h->raw_cap = bytes;
    return IRR_OK;
}

int set_nodes_common(irr_handle* h, const void* src, int elm, int64_t n, cudaMemcpyKind kind)
{
    if (!h || (!src && n > 0) || n < 0) return fail(h, IRR_ERR_ARG, "bad node data arguments");
    if (!valid_node_elm(h, elm))
        return fail(h, IRR_ERR_ARG,
                    h->user_launch ? "node elm_size %d: use a multiple of 4 up to 1024" : "node elm_size %d: use 12, 16 or 24",
                    elm);
    if (n > 0x7fffffffLL) return fail(h, IRR_ERR_CAPACITY, "more than 2^31-1 nodes");
    if (h->inited && n != h->n) return fail(h, IRR_ERR_STATE, "node count changed after init (%lld -> %lld)", (long long)h->n, (long long)n);
    if (h->inited && h->user_launch && elm != h->raw_elm)
        return fail(h, IRR_ERR_STATE, "node record size changed after init (%d -> %d)", h->raw_elm, elm);
    if (kind == cudaMemcpyHostToDevice && h->inited && n > 0 && !h->user_launch) {
        // reset_node_data from page-locked host memory: the kernel reads the
        // caller's records in order over the host link and scatters them into
        // execution order (no staging copy, no second pass)
        if (const void* mapped = host_device_view(src)) {
            H_CUDA(h, launch_load_nodes_scatter(mapped, elm, h->part.inv, n, h->d_pos, h->stream),
                   "load node data");
            h->raw_elm = elm;
            h->raw_pending = false;
            return IRR_OK;
        }
    }
    int rc = ensure_raw(h, (size_t)(n > 0 ? n : 1) * (size_t)elm);
    if (rc) return rc;
    if (n > 0)
        H_CUDA(h, cudaMemcpyAsync(h->d_raw, src, (size_t)n * elm, kind, h->stream), "copy node data");
    h->n = n;
    h->raw_elm = elm;
    h->raw_pending = true;
    if (h->inited) {
        // reset_node_data: convert (and gather into partition order) now
        if (h->user_launch)
            H_CUDA(h, launch_gather_records(h->d_raw, elm, h->part.perm, n, h->d_rec, h->stream),
                   "load node records");
        else
            H_CUDA(h, launch_load_nodes(h->d_raw, elm, h->part.perm, n, h->d_pos, h->stream),
                   "load node data");
        h->raw_pending = false;
    }
    return IRR_OK;
}

int set_edges_common(irr_handle* h, const int32_t* src, int64_t e, cudaMemcpyKind kind)
{
    if (!h || (!src && e > 0) || e < 0) return fail(h, IRR_ERR_ARG, "bad edge arguments");
    if (e > 0x7fffffffLL) return fail(h, IRR_ERR_CAPACITY, "more than 2^31-1 edges");
    const size_t bytes = (size_t)(e > 0 ? e : 1) * sizeof(int2);
    if (bytes > h->edges_cap) {
        dfree(h->d_edges);
        h->edges_cap = 0;
        H_CUDA(h, cudaMalloc(&h->d_edges, bytes), "allocate edges");
        h->edges_cap = bytes;
    }
    if (e > 0) H_CUDA(h, cudaMemcpyAsync(h->d_edges, src, (size_t)e * sizeof(int2), kind, h->stream), "copy edges");
    h->e = e;
    if (h->inited) {
        // new edge list: the layout is rebuilt at the next init
        const int64_t n = h->n;
        if (!h->raw_pending && h->user_launch) {
            // keep the current node records: back into the caller's order
            int rc = ensure_raw(h, (size_t)(n > 0 ? n : 1) * h->raw_elm);
            if (rc) return rc;
            H_CUDA(h, launch_gather_records(h->d_rec, h->raw_elm, h->part.inv, n, h->d_raw, h->stream),
                   "save node records");
            h->raw_pending = true;
        } else if (!h->raw_pending) {
            // keep the current node data: write it back in the caller's order
            int rc = ensure_raw(h, (size_t)(n > 0 ? n : 1) * 16);
            if (rc) return rc;
            H_CUDA(h, launch_store_result(h->d_pos, h->part.inv, n, 16, h->d_raw, h->stream), "save node data");
            h->raw_elm = 16;
            h->raw_pending = true;
        }
        free_layout(h);
    }
    return IRR_OK;
}

// irr_set_shard: rows outside [own_lo, own_hi) (caller ids) lose their
// entries; h->m = the entries left.
int apply_shard(irr_handle* h)
{
    if (h->own_hi < 0) {
        h->m = 2 * h->e;
        return IRR_OK;
    }
    if (h->own_lo < 0 || h->own_lo > h->own_hi || h->own_hi > h->n)
        return fail(h, IRR_ERR_STATE, "shard rows [%lld, %lld) outside the %lld nodes", (long long)h->own_lo,
                    (long long)h->own_hi, (long long)h->n);
    H_CUDA(h, keep_rows(&h->part, h->n, h->own_lo, h->own_hi, &h->m, h->stream), "shard rows");
    return IRR_OK;
}

// Rows whose results a read returns: [lo, lo + count) of the caller's ids.
void result_rows(const irr_handle* h, int64_t* lo, int64_t* count)
{
    *lo = h->own_hi >= 0 ? h->own_lo : 0;
    *count = h->own_hi >= 0 ? h->own_hi - h->own_lo : h->n;
}

// The reduction of one step over the positions in d_pos, on h->stream.
int launch_reduction(irr_handle* h)
{
    if (h->cfg.exec == IRR_EXEC_PLAIN) {
        H_CUDA(h, cudaMemsetAsync(h->d_force, 0, (size_t)(h->n > 0 ? h->n : 1) * sizeof(float4), h->stream), "clear results");
        H_CUDA(h, launch_plain(h->d_pos, h->d_edges, h->e, h->d_force, h->law, h->stream), "plain kernel");
        return IRR_OK;
    }
    H_CUDA(h, cudaMemsetAsync(h->d_queue, 0, sizeof(int), h->stream), "clear work queue");
    const WaitPolicy wp = h->wait;
    h->wait.withhold = 0;  // one step only
    H_CUDA(h, launch_tiled(h->shape, h->d_inst, h->d_items, h->num_items, h->d_queue,
                           h->sms * kCtasPerSm, h->d_status, h->stream, &h->inst, 1, wp),
           "tiled kernel");
    return IRR_OK;
}

// Streams, events and staging of the pipelined path (grown as needed).
int ensure_pipe(irr_handle* h, size_t in_bytes, size_t out_bytes)
{
    irr_handle::Pipe& P = h->pipe;
    // each object made once; after a failed call the next one makes what is missing
    if (!P.s_in) H_CUDA(h, cudaStreamCreateWithFlags(&P.s_in, cudaStreamNonBlocking), "pipeline stream");
    if (!P.s_out) H_CUDA(h, cudaStreamCreateWithFlags(&P.s_out, cudaStreamNonBlocking), "pipeline stream");
    for (int s = 0; s < 2; s++) {
        cudaEvent_t* evs[4] = {&P.in_done[s], &P.in_free[s], &P.out_ready[s], &P.out_free[s]};
        for (cudaEvent_t* ev : evs)
            if (!*ev) H_CUDA(h, cudaEventCreateWithFlags(ev, cudaEventDisableTiming), "pipeline event");
    }
    if (in_bytes > P.in_cap || out_bytes > P.out_cap) {
        // no step in flight may use the old staging
        H_CUDA(h, cudaStreamSynchronize(P.s_in), "pipeline");
        H_CUDA(h, cudaStreamSynchronize(h->stream), "pipeline");
        H_CUDA(h, cudaStreamSynchronize(P.s_out), "pipeline");
        if (in_bytes > P.in_cap) {
            for (int s = 0; s < 2; s++) dfree(P.in[s]);
            P.in_cap = 0;
            for (int s = 0; s < 2; s++) H_CUDA(h, cudaMalloc(&P.in[s], in_bytes), "pipeline staging");
            P.in_cap = in_bytes;
        }
        if (out_bytes > P.out_cap) {
            for (int s = 0; s < 2; s++) dfree(P.out[s]);
            P.out_cap = 0;
            for (int s = 0; s < 2; s++) H_CUDA(h, cudaMalloc(&P.out[s], out_bytes), "pipeline staging");
            P.out_cap = out_bytes;
        }
    }
    return IRR_OK;
}

void free_pipe(irr_handle* h)
{
    irr_handle::Pipe& P = h->pipe;
    if (P.s_in) cudaStreamSynchronize(P.s_in);
    if (P.s_out) cudaStreamSynchronize(P.s_out);
    for (int s = 0; s < 2; s++) {
        dfree(P.in[s]);
        dfree(P.out[s]);
        for (cudaEvent_t* e : {&P.in_done[s], &P.in_free[s], &P.out_ready[s], &P.out_free[s]})
            if (*e) {
                cudaEventDestroy(*e);
                *e = nullptr;
            }
    }
    if (P.s_in) cudaStreamDestroy(P.s_in);
    if (P.s_out) cudaStreamDestroy(P.s_out);
    P = irr_handle::Pipe{};
}

// User map: positions for the partitioner (coordinates, else position-like
// records, else none: the caller's order is kept), then the partition, the
// node records in execution order, and the view's other arrays.
int init_user(irr_handle* h)
{
    cudaStream_t s = h->stream;
    const int64_t n = h->n, e = h->e;
    const size_t nb = (size_t)(n > 0 ? n : 1);
    H_CUDA(h, cudaMalloc(&h->d_pos, nb * sizeof(float4)), "allocate positions");
    int reorder = h->cfg.reorder;
    if (h->coord_n >= 0) {
        if (h->coord_n != n)
            return fail(h, IRR_ERR_STATE, "%lld coordinates for %lld nodes", (long long)h->coord_n, (long long)n);
        H_CUDA(h, launch_coords_to_pos(h->d_coord, h->coord_size, h->coord_dims, n, h->d_pos, s), "coordinates");
    } else if (h->raw_elm == 12 || h->raw_elm == 16 || h->raw_elm == 24) {
        H_CUDA(h, launch_load_nodes(h->d_raw, h->raw_elm, nullptr, n, h->d_pos, s), "load node positions");
    } else {
        H_CUDA(h, cudaMemsetAsync(h->d_pos, 0, nb * sizeof(float4), s), "clear positions");
        reorder = 0;
    }
    PartitionOut p;
    cudaError_t pe = build_partition(h->d_pos, n, h->d_edges, e, reorder, &p, s, h->cfg.order);
    h->part = p;
    if (pe != cudaSuccess) {
        free_layout(h);
        return cuda_fail(h, pe, "build partition");
    }
    int rc = apply_shard(h);
    if (rc) {
        free_layout(h);
        return rc;
    }
    dfree(h->d_pos);  // the user kernel reads the records
    H_CUDA(h, cudaMalloc(&h->d_rec, nb * h->raw_elm), "allocate node records");
    H_CUDA(h, launch_gather_records(h->d_raw, h->raw_elm, h->part.perm, n, h->d_rec, s), "gather node records");
    h->raw_pending = false;
    H_CUDA(h, cudaMalloc(&h->d_vals, nb * h->value_size), "allocate results");
    H_CUDA(h, cudaMemsetAsync(h->d_vals, 0, nb * h->value_size, s), "clear results");
    H_CUDA(h, cudaMalloc(&h->d_iota, nb * sizeof(int32_t)), "allocate part index");
    H_CUDA(h, launch_iota(h->d_iota, n, s), "part index");
    H_CUDA(h, cudaMalloc(&h->d_param, h->param.size() > 0 ? h->param.size() : 16), "allocate parameters");
    if (!h->param.empty())
        H_CUDA(h, cudaMemcpyAsync(h->d_param, h->param.data(), h->param.size(), cudaMemcpyHostToDevice, s),
               "copy parameters");
    h->dev_bytes = (int64_t)nb * (h->raw_elm + h->value_size + 3 * 4) + (int64_t)h->raw_cap + 4 * (n + 1) +
                   4 * h->m + (int64_t)h->coord_cap;
    h->inited = true;
    dfree(h->d_edges);
    h->edges_cap = 0;
    H_CUDA(h, cudaStreamSynchronize(s), "init");
    return IRR_OK;
}

int step_user(irr_handle* h)
{
    if (h->raw_pending) {
        H_CUDA(h, launch_gather_records(h->d_raw, h->raw_elm, h->part.perm, h->n, h->d_rec, h->stream),
               "load node records");
        h->raw_pending = false;
    }
    irr_user_view v{};
    v.num_nodes = h->n;
    v.row_off = h->part.row_off;
    v.col = h->part.col;
    v.node_data = h->d_rec;
    v.node_elm_size = h->raw_elm;
    v.value_size = h->value_size;
    v.param = h->d_param;
    v.param_size = (int)h->param.size();
    v.map_idx = h->user_map_idx;
    v.reduce_idx = h->user_reduce_idx;
    v.part_index = h->d_iota;
    v.values = h->d_vals;
    v.status = h->d_status;
    v.num_sms = h->sms;
    const int rc = h->user_launch(&v, (void*)h->stream, h->user_ctx);
    if (rc != IRR_OK) {
        const cudaError_t ce = cudaGetLastError();
        return fail(h, rc, "user map launch (map %d, reduce %d): %s", h->user_map_idx, h->user_reduce_idx,
                    rc == IRR_ERR_ARG ? "table index out of range, or VALUE size differs"
                                      : cudaGetErrorString(ce));
    }
    return IRR_OK;
}

// User-map results into d_out (device or page-locked host memory the device
// addresses): value_size records, or widened doubles at 2 * value_size.
int store_user(irr_handle* h, void* d_out, int elm_size)
{
    int64_t lo, count;
    result_rows(h, &lo, &count);
    if (elm_size == h->value_size)
        H_CUDA(h, launch_gather_records(h->d_vals, elm_size, h->part.inv + lo, count, d_out, h->stream),
               "store results");
    else
        H_CUDA(h, launch_widen_records(h->d_vals, h->value_size, h->part.inv + lo, count, d_out, h->stream),
               "store results");
    return IRR_OK;
}

bool user_result_ok(const irr_handle* h, int elm_size)
{
    return elm_size == h->value_size || (h->value_kind == IRR_VALUE_F32 && elm_size == 2 * h->value_size);
}

}  // namespace

int irr_ensure_layout(irr_handle* h, int lanes_per_row, int block_nodes, int staged_ok)
{
    TraceRange trace_("irr_layout");
    if (!h || !h->inited || h->cfg.exec != IRR_EXEC_PARTITIONED) return IRR_ERR_STATE;
    if (h->user_launch) return fail(h, IRR_ERR_STATE, "a handle with a user map runs its own kernel");
    DeviceGuard dev_guard(h->device);
    H_CUDA(h, cudaStreamSynchronize(h->stream), "layout");  // no launch may use the old layout
    const int64_t n = h->n, e = h->e;
    h->shape.lanes_per_row = lanes_per_row;
    h->shape.block_nodes = block_nodes;
    const int want = h->cfg.layout;
    bool staged = false;
    if (want == IRR_LAYOUT_STAGED && !staged_ok)
        return fail(h, IRR_ERR_STATE, "the handle is configured for the staged layout");
    if (want == IRR_LAYOUT_STAGED || (want == IRR_LAYOUT_AUTO && kAutoStaged && staged_ok)) {
        if (lanes_per_row == 4 && h->shape.stage_smem) {
            if (!h->st.words) {
                const cudaError_t se = build_staged(h->part.row_off, h->part.col, h->host_row_off.data(),
                                                    n, &h->st, h->stream);
                if (se != cudaSuccess) {
                    cudaGetLastError();
                    free_staged(&h->st);
                    if (want == IRR_LAYOUT_STAGED)
                        return se == cudaErrorNotSupported
                                   ? fail(h, IRR_ERR_CAPACITY,
                                          "staged layout: 8 rows touch more than %d nodes, or a row is too long",
                                          kHaloTabMax)
                                   : cuda_fail(h, se, "build staged layout");
                }
            }
            if (want == IRR_LAYOUT_AUTO && h->st.words && h->m < kStagedMinReuse * h->st.nids)
                free_staged(&h->st);  // too little reuse to pay for staging
            staged = h->st.words != nullptr || (n == 0 && want == IRR_LAYOUT_STAGED);
        } else if (want == IRR_LAYOUT_STAGED) {
            return fail(h, IRR_ERR_ARG, "the staged layout needs 4 lanes per row and stage_smem");
        }
    }
    h->shape.staged = staged ? 1 : 0;
    if (staged) {
        free_sliced(&h->sl);
    } else {
        free_staged(&h->st);
        if (want == IRR_LAYOUT_CSR) {
            free_sliced(&h->sl);
        } else if (h->sl.lanes != lanes_per_row) {
            const cudaError_t se = build_sliced(h->part.row_off, h->part.col, n, lanes_per_row, &h->sl, h->stream);
            if (se != cudaSuccess) {
                cudaGetLastError();
                free_sliced(&h->sl);
                if (want == IRR_LAYOUT_SLICED)
                    return se == cudaErrorInvalidValue
                               ? fail(h, IRR_ERR_CAPACITY, "sliced layout above 2^32 words")
                               : cuda_fail(h, se, "build sliced layout");
            } else if (want != IRR_LAYOUT_SLICED && !sliced_pays(h->sl, h->m)) {
                free_sliced(&h->sl);
            }
        }
    }
    int rc = upload_inst(h);
    if (rc) return rc;
    rc = upload_items(h);
    if (rc) return rc;
    h->dev_bytes = 2 * (int64_t)(n > 0 ? n : 1) * (int64_t)sizeof(float4) + (int64_t)h->raw_cap +
                   (int64_t)(2 * n + n + 1) * 4 + h->m * 4 +
                   (h->sl.lanes ? 4 * (h->sl.words + h->sl.slices + 1) : 0) +
                   (h->shape.staged ? 4 * (h->st.nwords + h->st.nids + h->st.slices + 1) : 0);
    return IRR_OK;
}

namespace {

int set_nodes_range_common(irr_handle* h, const void* src, int elm, int64_t first, int64_t count,
                           cudaMemcpyKind kind)
{
    if (!h || (!src && count > 0) || first < 0 || count < 0) return fail(h, IRR_ERR_ARG, "bad node range arguments");
    if (h->n < 0) return fail(h, IRR_ERR_STATE, "irr_set_nodes_range before irr_set_nodes");
    if (first + count > h->n)
        return fail(h, IRR_ERR_ARG, "node range [%lld, %lld) outside %lld nodes", (long long)first,
                    (long long)(first + count), (long long)h->n);
    if (count == 0) return IRR_OK;
    if (!h->inited || h->raw_pending || h->user_launch) {
        // the records wait in d_raw, in the caller's order: patch them there
        if (elm != h->raw_elm)
            return fail(h, IRR_ERR_STATE, "record size %d differs from the node data's %d", elm, h->raw_elm);
        if (h->inited && !h->raw_pending) {
            // user map after init: d_raw is stale, so bring it up to date first
            H_CUDA(h, launch_gather_records(h->d_rec, h->raw_elm, h->part.inv, h->n, h->d_raw, h->stream),
                   "save node records");
        }
        H_CUDA(h, cudaMemcpyAsync(static_cast<char*>(h->d_raw) + (size_t)first * elm, src, (size_t)count * elm,
                                  kind, h->stream), "copy node range");
        h->raw_pending = true;
        return IRR_OK;
    }
    if (!valid_node_elm(h, elm)) return fail(h, IRR_ERR_ARG, "node elm_size %d: use 12, 16 or 24", elm);
    const void* rec = src;
    if (kind == cudaMemcpyHostToDevice) {
        rec = host_device_view(src);
        if (!rec) {
            int rc = ensure_raw(h, (size_t)h->n * elm);
            if (rc) return rc;
            H_CUDA(h, cudaMemcpyAsync(h->d_raw, src, (size_t)count * elm, kind, h->stream), "copy node range");
            rec = h->d_raw;
        }
    }
    // records [first, first + count) in the caller's order -> execution order
    H_CUDA(h, launch_load_nodes_scatter(rec, elm, h->part.inv + first, count, h->d_pos, h->stream),
           "load node range");
    return IRR_OK;
}

}  // namespace

extern "C" {

void irr_config_default(irr_config* cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->device = 0;
    cfg->exec = IRR_EXEC_PARTITIONED;
    cfg->map_idx = IRR_MAP_LJ_MOLDYN;
    cfg->reduce_idx = IRR_REDUCE_SUM;
    cfg->block_nodes = 0;
    cfg->lanes_per_row = 0;
    cfg->reorder = 1;
    cfg->stage_smem = -1;
}

const char* irr_status_string(int status)
{
    switch (status) {
    case IRR_OK: return "ok";
    case IRR_ERR_ARG: return "bad argument";
    case IRR_ERR_INDEX: return "edge endpoint out of range";
    case IRR_ERR_STATE: return "call out of order";
    case IRR_ERR_CUDA: return "CUDA error";
    case IRR_ERR_NOMEM: return "out of memory";
    case IRR_ERR_CAPACITY: return "size above limit";
    case IRR_ERR_DEVICE: return "device-side fault reported";
    case IRR_ERR_BUDGET: return "over admission budget";
    default: return "unknown status";
    }
}

int irr_create(const irr_config* cfg, irr_handle** out)
{
    if (!out) return IRR_ERR_ARG;
    *out = nullptr;
    irr_config c;
    if (cfg)
        c = *cfg;
    else
        irr_config_default(&c);
    if (c.exec != IRR_EXEC_PLAIN && c.exec != IRR_EXEC_PARTITIONED) return IRR_ERR_ARG;
    if (c.reduce_idx != IRR_REDUCE_SUM) return IRR_ERR_ARG;
    if (c.map_idx < IRR_MAP_LJ_MOLDYN || c.map_idx > IRR_MAP_LJ_MINIMD_PBC) return IRR_ERR_ARG;
    if (c.block_nodes != 0 && (c.block_nodes < 64 || c.block_nodes > 4096 || (c.block_nodes & (c.block_nodes - 1))))
        return IRR_ERR_ARG;
    if (c.layout < IRR_LAYOUT_AUTO || c.layout > IRR_LAYOUT_STAGED) return IRR_ERR_ARG;
    if (c.order != IRR_ORDER_HILBERT && c.order != IRR_ORDER_MORTON) return IRR_ERR_ARG;
    if (c.wait_limit_us < 0) return IRR_ERR_ARG;
    if (c.lanes_per_row != 0 && c.lanes_per_row != 1 && c.lanes_per_row != 2 && c.lanes_per_row != 4 &&
        c.lanes_per_row != 8 && c.lanes_per_row != 16 && c.lanes_per_row != 32)
        return IRR_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return IRR_ERR_CUDA;
    }
    if (c.device < 0 || c.device >= ndev) return IRR_ERR_ARG;
    irr_handle* h = new (std::nothrow) irr_handle();
    if (!h) return IRR_ERR_NOMEM;
    h->cfg = c;
    h->device = c.device;
    h->map_idx = c.map_idx;
    h->reduce_idx = c.reduce_idx;
    DeviceGuard dev_guard(h->device);
    if (!dev_guard.ok() ||
        cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&h->d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(h->d_status, 0, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        if (h->own_stream) cudaStreamDestroy(h->own_stream);
        if (h->d_status) cudaFree(h->d_status);
        delete h;
        return IRR_ERR_CUDA;
    }
    h->stream = h->own_stream;
    if (c.wait_limit_us > 0) h->wait.wait_ns = 1000ull * (uint64_t)c.wait_limit_us;
    h->shape.lanes_per_row = c.lanes_per_row ? c.lanes_per_row : 4;
    h->shape.block_nodes = c.block_nodes ? c.block_nodes : 1024;
    h->shape.stage_smem = c.stage_smem < 0 ? 1 : (c.stage_smem ? 1 : 0);
    if (cudaMalloc(&h->d_queue, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamDestroy(h->own_stream);
        cudaFree(h->d_status);
        delete h;
        return IRR_ERR_CUDA;
    }
    *out = h;
    return IRR_OK;
}

int irr_destroy(irr_handle* h)
{
    if (!h) return IRR_ERR_ARG;
    DeviceGuard dev_guard(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_layout(h);
    dfree(h->d_raw);
    dfree(h->d_edges);
    dfree(h->d_status);
    dfree(h->d_queue);
    dfree(h->d_out);
    dfree(h->d_coord);
    free_pipe(h);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return IRR_OK;
}

const char* irr_last_error(const irr_handle* h) { return h ? h->err.c_str() : "null handle"; }

int irr_set_stream(irr_handle* h, void* stream)
{
    if (!h) return IRR_ERR_ARG;
    h->stream = (cudaStream_t)stream;  // used as given: NULL is the default stream
    return IRR_OK;
}

int irr_set_map(irr_handle* h, int map_idx)
{
    if (!h) return IRR_ERR_ARG;
    if (h->user_launch) {
        // an entry of the user's map table (range checked at launch)
        if (map_idx < 0) return fail(h, IRR_ERR_ARG, "negative map index %d", map_idx);
        h->user_map_idx = map_idx;
        return IRR_OK;
    }
    if (map_idx < IRR_MAP_LJ_MOLDYN || map_idx > IRR_MAP_LJ_MINIMD_PBC)
        return fail(h, IRR_ERR_ARG, "unknown map index %d", map_idx);
    h->map_idx = map_idx;
    h->have_law = false;
    if (!h->param.empty()) {
        int rc = make_law(h);
        if (rc) return rc;
        return upload_inst(h);
    }
    return IRR_OK;
}

int irr_set_reduce(irr_handle* h, int reduce_idx)
{
    if (!h) return IRR_ERR_ARG;
    if (h->user_launch) {
        if (reduce_idx < 0) return fail(h, IRR_ERR_ARG, "negative reduce index %d", reduce_idx);
        h->user_reduce_idx = reduce_idx;
        return IRR_OK;
    }
    if (reduce_idx != IRR_REDUCE_SUM) return fail(h, IRR_ERR_ARG, "unknown reduce index %d", reduce_idx);
    h->reduce_idx = reduce_idx;
    return IRR_OK;
}

int irr_set_params(irr_handle* h, const void* param, int param_size)
{
    if (!h) return IRR_ERR_ARG;
    if (!param || param_size <= 0) return fail(h, IRR_ERR_ARG, "empty parameter block");
    DeviceGuard dev_guard(h->device);
    if (h->user_launch) {
        // kept as given; the user map reads it from device memory
        if (param_size > kUserParamMax) return fail(h, IRR_ERR_CAPACITY, "parameter block above %d bytes", kUserParamMax);
        const bool resize = h->inited && (size_t)param_size != h->param.size();
        h->param.assign((const unsigned char*)param, (const unsigned char*)param + param_size);
        h->have_law = true;
        if (h->inited) {
            if (resize) {
                H_CUDA(h, cudaStreamSynchronize(h->stream), "parameters");
                dfree(h->d_param);
                H_CUDA(h, cudaMalloc(&h->d_param, h->param.size()), "allocate parameters");
            }
            H_CUDA(h, cudaMemcpyAsync(h->d_param, h->param.data(), h->param.size(), cudaMemcpyHostToDevice,
                                      h->stream), "copy parameters");
        }
        return IRR_OK;
    }
    std::vector<unsigned char> keep = h->param;
    h->param.assign((const unsigned char*)param, (const unsigned char*)param + param_size);
    int rc = make_law(h);
    if (rc) {
        h->param = keep;
        return rc;
    }
    return upload_inst(h);
}

int irr_set_edges(irr_handle* h, const int32_t* edges, int64_t num_edges)
{
    if (!h) return IRR_ERR_ARG;
    DeviceGuard dev_guard(h->device);
    return set_edges_common(h, edges, num_edges, cudaMemcpyHostToDevice);
}

int irr_set_edges_device(irr_handle* h, const int32_t* d_edges, int64_t num_edges)
{
    if (!h) return IRR_ERR_ARG;
    DeviceGuard dev_guard(h->device);
    return set_edges_common(h, d_edges, num_edges, cudaMemcpyDeviceToDevice);
}

int irr_set_nodes(irr_handle* h, const void* node_data, int elm_size, int64_t num_nodes)
{
    TraceRange trace_("irr_set_nodes");
    if (!h) return IRR_ERR_ARG;
    DeviceGuard dev_guard(h->device);
    return set_nodes_common(h, node_data, elm_size, num_nodes, cudaMemcpyHostToDevice);
}

int irr_set_nodes_device(irr_handle* h, const void* d_node_data, int elm_size, int64_t num_nodes)
{
    if (!h) return IRR_ERR_ARG;
    DeviceGuard dev_guard(h->device);
    return set_nodes_common(h, d_node_data, elm_size, num_nodes, cudaMemcpyDeviceToDevice);
}

int irr_init(irr_handle* h)
{
    TraceRange trace_("irr_init");
    if (!h) return IRR_ERR_ARG;
    if (h->inited) return IRR_OK;
    if (h->n < 0) return fail(h, IRR_ERR_STATE, "irr_init before irr_set_nodes");
    if (h->e < 0) return fail(h, IRR_ERR_STATE, "irr_init before irr_set_edges");
    if (!h->have_law) return fail(h, IRR_ERR_STATE, "irr_init before irr_set_params");
    if (h->user_launch && h->cfg.exec != IRR_EXEC_PARTITIONED)
        return fail(h, IRR_ERR_STATE, "a user map needs the partitioned executor");
    if (h->own_hi >= 0 && h->cfg.exec != IRR_EXEC_PARTITIONED)
        return fail(h, IRR_ERR_STATE, "a shard needs the partitioned executor");
    DeviceGuard dev_guard(h->device);
    cudaStream_t s = h->stream;
    const int64_t n = h->n, e = h->e;
    H_CUDA(h, launch_validate_edges(h->d_edges, e, n, h->d_status, s), "validate edges");
    int rc = check_status(h);
    if (rc) return rc;
    if (h->user_launch) return init_user(h);
    const size_t nb = (size_t)(n > 0 ? n : 1) * sizeof(float4);
    H_CUDA(h, cudaMalloc(&h->d_pos, nb), "allocate positions");
    H_CUDA(h, cudaMalloc(&h->d_force, nb), "allocate results");
    H_CUDA(h, cudaMemsetAsync(h->d_force, 0, nb, s), "clear results");
    h->dev_bytes = 2 * (int64_t)nb + (int64_t)h->raw_cap;
    if (h->cfg.exec == IRR_EXEC_PLAIN) {
        H_CUDA(h, launch_load_nodes(h->d_raw, h->raw_elm, nullptr, n, h->d_pos, s), "load node data");
        h->raw_pending = false;
        h->dev_bytes += (int64_t)h->edges_cap;
        h->inited = true;
        H_CUDA(h, cudaStreamSynchronize(s), "init");
        return IRR_OK;
    }
    // partitioned: positions in the caller's order feed the partitioner
    H_CUDA(h, launch_load_nodes(h->d_raw, h->raw_elm, nullptr, n, h->d_pos, s), "load node data");
    PartitionOut p;
    cudaError_t pe = build_partition(h->d_pos, n, h->d_edges, e, h->cfg.reorder, &p, s, h->cfg.order);
    h->part = p;
    if (pe != cudaSuccess) {
        free_layout(h);
        return cuda_fail(h, pe, "build partition");
    }
    rc = apply_shard(h);
    if (rc) {
        free_layout(h);
        return rc;
    }
    H_CUDA(h, launch_load_nodes(h->d_raw, h->raw_elm, h->part.perm, n, h->d_pos, s), "gather node data");
    h->raw_pending = false;
    // node blocks -> work items (cut on the row offsets)
    h->host_row_off.resize((size_t)n + 1);
    H_CUDA(h, cudaMemcpyAsync(h->host_row_off.data(), h->part.row_off, sizeof(uint32_t) * (n + 1),
                              cudaMemcpyDeviceToHost, s), "copy row offsets");
    H_CUDA(h, cudaStreamSynchronize(s), "copy row offsets");
    H_CUDA(h, cudaMalloc(&h->d_inst, sizeof(InstDesc)), "allocate instance descriptor");
    h->shape.periodic = h->law.periodic;
    h->inited = true;
    rc = irr_ensure_layout(h, h->shape.lanes_per_row, h->shape.block_nodes);
    if (rc) return rc;
    // the half list is not needed by the partitioned kernel
    dfree(h->d_edges);
    h->edges_cap = 0;
    H_CUDA(h, cudaStreamSynchronize(s), "init");
    return IRR_OK;
}

int irr_step(irr_handle* h)
{
    TraceRange trace_("irr_step");
    if (!h) return IRR_ERR_ARG;
    if (!h->inited) {
        int rc = irr_init(h);
        if (rc) return rc;
    }
    DeviceGuard dev_guard(h->device);
    if (h->user_launch) return step_user(h);
    if (h->raw_pending) {
        H_CUDA(h, launch_load_nodes(h->d_raw, h->raw_elm, h->part.perm, h->n, h->d_pos, h->stream), "load node data");
        h->raw_pending = false;
    }
    return launch_reduction(h);
}

int irr_step_pipelined(irr_handle* h, const void* node_data, int node_elm, void* out, int out_elm)
{
    TraceRange trace_("irr_step_pipelined");
    if (!h) return IRR_ERR_ARG;
    if (!h->inited) return fail(h, IRR_ERR_STATE, "irr_step_pipelined before irr_init");
    if (h->user_launch) return fail(h, IRR_ERR_STATE, "a handle with a user map steps with irr_step");
    if (!valid_node_elm(h, node_elm)) return fail(h, IRR_ERR_ARG, "node elm_size %d: use 12, 16 or 24", node_elm);
    if (out_elm != 12 && out_elm != 16 && out_elm != 24)
        return fail(h, IRR_ERR_ARG, "result elm_size %d: use 12, 16 or 24", out_elm);
    int64_t lo, count;
    result_rows(h, &lo, &count);
    if ((!node_data && h->n > 0) || (!out && count > 0)) return fail(h, IRR_ERR_ARG, "null buffer");
    DeviceGuard dev_guard(h->device);
    const int64_t n = h->n;
    int rc = ensure_pipe(h, (size_t)(n > 0 ? n : 1) * node_elm, (size_t)(count > 0 ? count : 1) * out_elm);
    if (rc) return rc;
    irr_handle::Pipe& P = h->pipe;
    const int s = (int)(P.issued & 1);
    // upload, once the reduction two steps back has consumed this slot
    H_CUDA(h, cudaStreamWaitEvent(P.s_in, P.in_free[s], 0), "pipeline order");
    if (n > 0)
        H_CUDA(h, cudaMemcpyAsync(P.in[s], node_data, (size_t)n * node_elm, cudaMemcpyHostToDevice, P.s_in),
               "upload node data");
    H_CUDA(h, cudaEventRecord(P.in_done[s], P.s_in), "pipeline order");
    // reduce: records -> execution order, the reduction, results -> staging
    H_CUDA(h, cudaStreamWaitEvent(h->stream, P.in_done[s], 0), "pipeline order");
    H_CUDA(h, launch_load_nodes(P.in[s], node_elm, h->part.perm, n, h->d_pos, h->stream), "load node data");
    H_CUDA(h, cudaEventRecord(P.in_free[s], h->stream), "pipeline order");
    h->raw_pending = false;
    rc = launch_reduction(h);
    if (rc) return rc;
    H_CUDA(h, cudaStreamWaitEvent(h->stream, P.out_free[s], 0), "pipeline order");
    H_CUDA(h, launch_store_result(h->d_force, h->part.inv ? h->part.inv + lo : nullptr, count, out_elm, P.out[s],
                                  h->stream), "store result");
    H_CUDA(h, cudaEventRecord(P.out_ready[s], h->stream), "pipeline order");
    // read back, while the next step reduces
    H_CUDA(h, cudaStreamWaitEvent(P.s_out, P.out_ready[s], 0), "pipeline order");
    if (count > 0)
        H_CUDA(h, cudaMemcpyAsync(out, P.out[s], (size_t)count * out_elm, cudaMemcpyDeviceToHost, P.s_out),
               "read back results");
    H_CUDA(h, cudaEventRecord(P.out_free[s], P.s_out), "pipeline order");
    P.issued++;
    return IRR_OK;
}

int irr_pipeline_sync(irr_handle* h)
{
    if (!h) return IRR_ERR_ARG;
    DeviceGuard dev_guard(h->device);
    if (h->pipe.s_out) H_CUDA(h, cudaStreamSynchronize(h->pipe.s_out), "pipeline");
    return check_status(h);
}

int irr_get_result_device(irr_handle* h, void* d_out, int elm_size)
{
    if (!h || !d_out) return fail(h, IRR_ERR_ARG, "null output");
    if (h->user_launch) {
        if (!user_result_ok(h, elm_size))
            return fail(h, IRR_ERR_ARG, "result elm_size %d: the user map's records are %d bytes", elm_size, h->value_size);
        if (!h->inited) return fail(h, IRR_ERR_STATE, "no result before irr_step");
        if (reinterpret_cast<uintptr_t>(d_out) % (elm_size == h->value_size ? 4 : 8))
            return fail(h, IRR_ERR_ARG, "result buffer not aligned to %d bytes", elm_size == h->value_size ? 4 : 8);
        DeviceGuard dev_guard(h->device);
        return store_user(h, d_out, elm_size);
    }
    if (elm_size != 12 && elm_size != 16 && elm_size != 24) return fail(h, IRR_ERR_ARG, "result elm_size %d: use 12, 16 or 24", elm_size);
    if (!h->inited) return fail(h, IRR_ERR_STATE, "no result before irr_step");
    const uintptr_t align = elm_size == 12 ? 4 : (elm_size == 16 ? 16 : 8);
    if (reinterpret_cast<uintptr_t>(d_out) % align)
        return fail(h, IRR_ERR_ARG, "result buffer not aligned to %d bytes for %d-byte records",
                    (int)align, elm_size);
    DeviceGuard dev_guard(h->device);
    int64_t lo, count;
    result_rows(h, &lo, &count);
    H_CUDA(h, launch_store_result(h->d_force, h->part.inv ? h->part.inv + lo : nullptr, count, elm_size, d_out,
                                  h->stream), "store result");
    return IRR_OK;
}

int irr_get_result(irr_handle* h, void* out, int elm_size)
{
    TraceRange trace_("irr_get_result");
    if (!h || (!out && h->n > 0)) return fail(h, IRR_ERR_ARG, "null output");
    if (h->user_launch ? !user_result_ok(h, elm_size) : (elm_size != 12 && elm_size != 16 && elm_size != 24))
        return fail(h, IRR_ERR_ARG, "result elm_size %d: not a record size of this handle", elm_size);
    if (!h->inited) return fail(h, IRR_ERR_STATE, "no result before irr_step");
    DeviceGuard dev_guard(h->device);
    int64_t lo, count;
    result_rows(h, &lo, &count);
    if (count > 0 && !h->user_launch) {
        // into page-locked host memory directly: written in order over the
        // host link, gathered from execution order on the device
        if (void* mapped = host_device_view(out)) {
            H_CUDA(h, launch_store_result(h->d_force, h->part.inv ? h->part.inv + lo : nullptr, count, elm_size,
                                          mapped, h->stream),
                   "store result");
            return check_status(h);
        }
    }
    const size_t bytes = (size_t)(count > 0 ? count : 1) * elm_size;
    if (bytes > h->out_cap) {
        dfree(h->d_out);
        h->out_cap = 0;
        H_CUDA(h, cudaMalloc(&h->d_out, bytes), "allocate result staging");
        h->out_cap = bytes;
    }
    int rc = irr_get_result_device(h, h->d_out, elm_size);
    if (rc) return rc;
    if (count > 0)
        H_CUDA(h, cudaMemcpyAsync(out, h->d_out, (size_t)count * elm_size, cudaMemcpyDeviceToHost, h->stream), "copy result");
    return check_status(h);
}

int irr_sync(irr_handle* h)
{
    if (!h) return IRR_ERR_ARG;
    DeviceGuard dev_guard(h->device);
    return check_status(h);
}

int irr_set_wait_limit(irr_handle* h, int64_t limit_us, int withhold_once)
{
    if (!h) return IRR_ERR_ARG;
    if (limit_us > (int64_t)1 << 40) return fail(h, IRR_ERR_ARG, "wait limit above 2^40 us");
    h->wait.wait_ns = limit_us > 0 ? 1000ull * (uint64_t)limit_us : kDefaultWaitNs;
    h->wait.withhold = withhold_once ? 1 : 0;
    return IRR_OK;
}

int irr_get_info(const irr_handle* h, irr_info* info)
{
    if (!h || !info) return IRR_ERR_ARG;
    memset(info, 0, sizeof(*info));
    info->num_nodes = h->n;
    info->num_edges = h->e;
    info->num_entries = h->cfg.exec == IRR_EXEC_PARTITIONED ? (h->inited ? h->m : 2 * (h->e > 0 ? h->e : 0))
                                                            : (h->e > 0 ? h->e : 0);
    info->own_lo = h->own_hi >= 0 ? h->own_lo : 0;
    info->own_hi = h->own_hi >= 0 ? h->own_hi : h->n;
    info->num_blocks = h->num_items;
    info->device_bytes = h->dev_bytes;
    info->block_nodes = h->shape.block_nodes;
    info->lanes_per_row = h->shape.lanes_per_row;
    info->stage_smem = h->shape.stage_smem;
    info->exec = h->cfg.exec;
    info->layout = h->shape.staged ? IRR_LAYOUT_STAGED : (h->sl.lanes ? IRR_LAYOUT_SLICED : IRR_LAYOUT_CSR);
    if (h->user_launch) info->num_blocks = 0;
    info->order = h->cfg.order;
    info->num_slots = h->shape.staged ? 2 * (h->st.nwords - 32 * h->st.slices)
                                      : (h->sl.lanes ? h->sl.words : info->num_entries);
    return IRR_OK;
}

int irr_get_partition(irr_handle* h, int32_t* perm, int64_t* row_off, int32_t* col)
{
    if (!h) return IRR_ERR_ARG;
    if (h->cfg.exec != IRR_EXEC_PARTITIONED) return fail(h, IRR_ERR_STATE, "handle is not partitioned");
    if (!h->inited) return fail(h, IRR_ERR_STATE, "no partition before irr_init");
    DeviceGuard dev_guard(h->device);
    const int64_t n = h->n, m = h->m;
    if (perm && n > 0)
        H_CUDA(h, cudaMemcpyAsync(perm, h->part.perm, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->stream), "copy perm");
    std::vector<uint32_t> ro;
    if (row_off) {
        ro.resize((size_t)n + 1);
        H_CUDA(h, cudaMemcpyAsync(ro.data(), h->part.row_off, sizeof(uint32_t) * (n + 1), cudaMemcpyDeviceToHost, h->stream), "copy row offsets");
    }
    if (col && m > 0)
        H_CUDA(h, cudaMemcpyAsync(col, h->part.col, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, h->stream), "copy entries");
    H_CUDA(h, cudaStreamSynchronize(h->stream), "copy partition");
    if (row_off)
        for (int64_t i = 0; i <= n; i++) row_off[i] = ro[(size_t)i];
    return IRR_OK;
}

int irr_get_staged(irr_handle* h, int64_t* counts, int32_t* items, uint32_t* slice_off,
                   uint32_t* words, int32_t* ids)
{
    if (!h) return IRR_ERR_ARG;
    if (!h->inited || !h->shape.staged) return fail(h, IRR_ERR_STATE, "the handle does not use the staged layout");
    DeviceGuard dev_guard(h->device);
    const Staged& st = h->st;
    if (counts) {
        counts[0] = (int64_t)st.items.size();
        counts[1] = st.nwords;
        counts[2] = st.nids;
    }
    if (items)
        for (size_t k = 0; k < st.items.size(); k++) {
            const WorkItem& w = st.items[k];
            const int32_t v[6] = {w.row0, w.nrows, (int32_t)w.ent0, (int32_t)w.nent, (int32_t)w.tab0,
                                  (int32_t)w.ntab};
            memcpy(items + 6 * k, v, sizeof(v));
        }
    if (slice_off && !st.host_off.empty())
        memcpy(slice_off, st.host_off.data(), sizeof(uint32_t) * st.host_off.size());
    if (words && st.nwords > 0)
        H_CUDA(h, cudaMemcpyAsync(words, st.words, sizeof(uint32_t) * st.nwords, cudaMemcpyDeviceToHost, h->stream), "copy words");
    if (ids && st.nids > 0)
        H_CUDA(h, cudaMemcpyAsync(ids, st.ids, sizeof(int32_t) * st.nids, cudaMemcpyDeviceToHost, h->stream), "copy tables");
    H_CUDA(h, cudaStreamSynchronize(h->stream), "copy staged layout");
    return IRR_OK;
}

int irr_set_user_map(irr_handle* h, irr_user_launch_fn launch, void* ctx, int value_size, int value_kind)
{
    if (!h) return IRR_ERR_ARG;
    if (h->inited) return fail(h, IRR_ERR_STATE, "irr_set_user_map after irr_init");
    if (launch && (value_size < 4 || value_size > kUserValueMax || (value_size & 3)))
        return fail(h, IRR_ERR_ARG, "value_size %d: use a multiple of 4 in [4, %d]", value_size, kUserValueMax);
    if (value_kind != IRR_VALUE_BYTES && value_kind != IRR_VALUE_F32)
        return fail(h, IRR_ERR_ARG, "unknown value kind %d", value_kind);
    if (h->n >= 0 && !(launch ? (h->raw_elm >= 4 && h->raw_elm <= 1024 && (h->raw_elm & 3) == 0)
                              : (h->raw_elm == 12 || h->raw_elm == 16 || h->raw_elm == 24)))
        return fail(h, IRR_ERR_STATE, "the node records already given (%d bytes) do not suit this map", h->raw_elm);
    h->user_launch = launch;
    h->user_ctx = launch ? ctx : nullptr;
    h->value_size = launch ? value_size : 0;
    h->value_kind = launch ? value_kind : IRR_VALUE_BYTES;
    h->user_map_idx = h->user_reduce_idx = 0;
    if (launch) {
        if (h->param.size() > (size_t)kUserParamMax) return fail(h, IRR_ERR_CAPACITY, "parameter block above %d bytes", kUserParamMax);
        h->have_law = true;  // a user map may take no parameter block
        return IRR_OK;
    }
    h->have_law = false;
    return h->param.empty() ? IRR_OK : make_law(h);
}

int irr_set_shard(irr_handle* h, int64_t own_lo, int64_t own_hi)
{
    if (!h) return IRR_ERR_ARG;
    if (h->inited) return fail(h, IRR_ERR_STATE, "irr_set_shard after irr_init");
    if (own_lo < 0 || own_hi < own_lo || own_hi > 0x7fffffffLL)
        return fail(h, IRR_ERR_ARG, "shard rows [%lld, %lld)", (long long)own_lo, (long long)own_hi);
    h->own_lo = own_lo;
    h->own_hi = own_hi;
    return IRR_OK;
}

int irr_set_nodes_range(irr_handle* h, const void* node_data, int elm_size, int64_t first, int64_t count)
{
    if (!h) return IRR_ERR_ARG;
    DeviceGuard dev_guard(h->device);
    return set_nodes_range_common(h, node_data, elm_size, first, count, cudaMemcpyHostToDevice);
}

int irr_set_nodes_range_device(irr_handle* h, const void* d_node_data, int elm_size, int64_t first, int64_t count)
{
    if (!h) return IRR_ERR_ARG;
    DeviceGuard dev_guard(h->device);
    return set_nodes_range_common(h, d_node_data, elm_size, first, count, cudaMemcpyDeviceToDevice);
}

int irr_set_coordinates(irr_handle* h, const void* coords, int coord_size, int num_dims, int64_t num_nodes)
{
    if (!h) return IRR_ERR_ARG;
    if ((!coords && num_nodes > 0) || num_nodes < 0) return fail(h, IRR_ERR_ARG, "bad coordinate arguments");
    if (coord_size != 4 && coord_size != 8) return fail(h, IRR_ERR_ARG, "coord_size %d: use 4 or 8", coord_size);
    if (num_dims != 2 && num_dims != 3) return fail(h, IRR_ERR_ARG, "num_dims %d: use 2 or 3", num_dims);
    if (num_nodes > 0x7fffffffLL) return fail(h, IRR_ERR_CAPACITY, "more than 2^31-1 nodes");
    DeviceGuard dev_guard(h->device);
    const size_t bytes = (size_t)(num_nodes > 0 ? num_nodes : 1) * coord_size * num_dims;
    if (bytes > h->coord_cap) {
        H_CUDA(h, cudaStreamSynchronize(h->stream), "coordinates");
        dfree(h->d_coord);
        h->coord_cap = 0;
        H_CUDA(h, cudaMalloc(&h->d_coord, bytes), "allocate coordinates");
        h->coord_cap = bytes;
    }
    if (num_nodes > 0)
        H_CUDA(h, cudaMemcpyAsync(h->d_coord, coords, (size_t)num_nodes * coord_size * num_dims,
                                  cudaMemcpyHostToDevice, h->stream), "copy coordinates");
    h->coord_size = coord_size;
    h->coord_dims = num_dims;
    h->coord_n = num_nodes;
    return IRR_OK;
}

}  // extern "C"
