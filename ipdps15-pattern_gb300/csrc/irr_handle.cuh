// irr_handle.cuh -- the irr_handle object, shared by the C-ABI translation units.
#pragma once
#include <string>
#include <vector>

#include "irr_internal.cuh"
#include "../../include/irregular_gb300.h"

using irr::InstDesc;
using irr::LawParams;
using irr::PartitionOut;
using irr::TiledShape;
using irr::WorkItem;

struct irr_handle {
    irr_config cfg{};
    int device = 0;
    int sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;

    int map_idx = IRR_MAP_LJ_MOLDYN;
    int reduce_idx = IRR_REDUCE_SUM;
    std::vector<unsigned char> param;
    bool have_law = false;
    LawParams law{};

    int64_t n = -1;
    int64_t e = -1;
    int64_t m = 0;               // directed entries held (2e, fewer for a shard)
    int64_t own_lo = 0;          // irr_set_shard: rows reduced and results read,
    int64_t own_hi = -1;         // caller ids [own_lo, own_hi); -1 = all
    void* d_raw = nullptr;       // node records as the caller passed them
    size_t raw_cap = 0;
    int raw_elm = 0;
    bool raw_pending = false;    // d_raw holds records not yet converted
    int2* d_edges = nullptr;     // caller's half list
    size_t edges_cap = 0;

    bool inited = false;
    TiledShape shape{};
    float4* d_pos = nullptr;     // execution order
    float4* d_force = nullptr;
    PartitionOut part{};
    std::vector<uint32_t> host_row_off;  // host copy of part.row_off (cuts work items)
    irr::Sliced sl{};                    // sliced layout, when in use
    irr::Staged st{};                    // staged layout, when in use
    InstDesc* d_inst = nullptr;
    InstDesc inst{};             // host copy of *d_inst (the single-instance launch parameter)
    WorkItem* d_items = nullptr;
    int num_items = 0;
    int* d_status = nullptr;
    int* d_queue = nullptr;      // work-queue cursor, cleared before each launch
    irr::WaitPolicy wait{};      // device-side wait limit; withhold: the next step only
    void* d_out = nullptr;       // result staging for host reads
    size_t out_cap = 0;
    int64_t dev_bytes = 0;

    // irr_step_pipelined: two slots of staging for the host copies, a
    // copy-in and a copy-out stream, and the events that order slot reuse
    // against the reduction on `stream`
    struct Pipe {
        cudaStream_t s_in = nullptr;
        cudaStream_t s_out = nullptr;
        void* in[2] = {nullptr, nullptr};
        void* out[2] = {nullptr, nullptr};
        size_t in_cap = 0;
        size_t out_cap = 0;
        cudaEvent_t in_done[2] = {nullptr, nullptr};    // upload of the slot finished
        cudaEvent_t in_free[2] = {nullptr, nullptr};    // the slot's records consumed
        cudaEvent_t out_ready[2] = {nullptr, nullptr};  // results staged in the slot
        cudaEvent_t out_free[2] = {nullptr, nullptr};   // the slot's read-back finished
        int64_t issued = 0;
    } pipe;

    // user map (the irregular.h plugin): bound by irr_set_user_map
    irr_user_launch_fn user_launch = nullptr;
    void* user_ctx = nullptr;
    int value_size = 0;
    int value_kind = IRR_VALUE_BYTES;
    int user_map_idx = 0;        // table entries the launch function is given
    int user_reduce_idx = 0;
    void* d_rec = nullptr;       // node records, execution order
    void* d_vals = nullptr;      // result records, execution order
    int32_t* d_iota = nullptr;   // part_index[x] = x
    void* d_param = nullptr;     // device copy of param
    void* d_coord = nullptr;     // irr_set_coordinates, caller's order
    size_t coord_cap = 0;
    int coord_size = 0;
    int coord_dims = 0;
    int64_t coord_n = -1;
};

// (Re)builds the handle's entry layout for G lanes per row as its config asks
// (staged, sliced or CSR), then its instance descriptor and work items, so
// that the three always agree.  staged_ok = 0 keeps an AUTO handle off the
// staged layout (a handle configured IRR_LAYOUT_STAGED then fails with
// IRR_ERR_STATE).  Partitioned, initialised handles only.
int irr_ensure_layout(irr_handle* h, int lanes_per_row, int block_nodes, int staged_ok = 1);
