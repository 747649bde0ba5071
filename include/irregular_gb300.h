/*
 * irregular_gb300.h -- C ABI of the GB300 irregular-reduction library.
 *
 * The irregular-reduction pattern: a node array, an edge list, and a per-edge
 * user function whose contributions are scatter-added into a per-node
 * reduction array.  This header is the drop-in boundary for the reference's
 * IrregularRuntime (moldyn/irregular/irregular_runtime.h:12-112) and its
 * user-function plugin (moldyn/irregular.h, miniMD/irregular.h).  Every entry
 * point takes plain pointers and sizes, returns an int status (IRR_OK == 0)
 * and never calls exit(); the reference exit()s on any CUDA or MPI error
 * (lib/macro.h:9-16).
 *
 * Threading: a handle is used by one host thread at a time.  Work is issued
 * on the handle's CUDA stream (irr_set_stream); calls that return data to the
 * host synchronise that stream.
 */
#ifndef IRREGULAR_GB300_H_
#define IRREGULAR_GB300_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define IRR_API __attribute__((visibility("default")))
#else
#define IRR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum irr_status {
    IRR_OK = 0,
    IRR_ERR_ARG = 1,      /* null pointer, negative size, unknown id or format     */
    IRR_ERR_INDEX = 2,    /* an edge endpoint outside [0, num_nodes)                */
    IRR_ERR_STATE = 3,    /* call out of order (e.g. step before nodes and edges)   */
    IRR_ERR_CUDA = 4,     /* a CUDA runtime call failed (text in irr_last_error)    */
    IRR_ERR_NOMEM = 5,    /* device or host allocation failed                       */
    IRR_ERR_CAPACITY = 6, /* a size above a documented limit                        */
    IRR_ERR_DEVICE = 7,   /* a kernel reported a fault through its status word      */
    IRR_ERR_BUDGET = 8    /* a job does not fit the admission budget                */
};

/* --------------------------------------------------- built-in user functions
 * Per-edge functions compiled into the library, selected by index the way the
 * reference selects map_function_table[map_idx] (moldyn/irregular.h:116-118,
 * irregular_runtime.cu:493-501).  All three are the Lennard-Jones law in the
 * reference's form d * (r^-14 - r^-8 / 2) (LJ force / 48 at eps = sigma = 1),
 * +f to idx0 and -f to idx1, applied when r^2 < cutoff^2.
 */
enum irr_map {
    /* moldyn `map` (moldyn/irregular.h:26-107): minimum image in a cubic box.
     * Parameter block: struct { double side; double cutoffRadius; }
     * (struct para, moldyn/moldyn.h:39-43). */
    IRR_MAP_LJ_MOLDYN = 0,
    /* miniMD `map1` (miniMD/irregular.h:109-163): open boundaries.
     * Parameter block: double cutforcesq (miniMD/ljs.cu:123). */
    IRR_MAP_LJ_MINIMD = 1,
    /* map1 with moldyn's minimum image (no reference counterpart: miniMD
     * builds no ghosts).  Parameter block: struct { double cutforcesq;
     * double side; }. */
    IRR_MAP_LJ_MINIMD_PBC = 2
};

/* `reduce` (moldyn/irregular.h:109-114): float3 +=. */
enum irr_reduce { IRR_REDUCE_SUM = 0 };

/* Execution strategy. */
enum irr_exec {
    /* Caller's node order and edge list as given; one thread per edge,
     * contributions added with global float4 atomics.  The straightforward
     * GPU form of compute_gpu (moldyn/irregular/gpu_kernel.cu:21-103). */
    IRR_EXEC_PLAIN = 0,
    /* GPU partitioner (Hilbert or Morton order, shared-memory-sized node blocks, edges
     * binned by owning block) and the tiled owner-computes kernel.  Each node
     * sums its own contributions in registers with compensated (two-sum)
     * partials; no atomics; results are bitwise reproducible. */
    IRR_EXEC_PARTITIONED = 1
};

/* Partitioned: the curve that orders the nodes (both quantise each axis of
 * the bounding box to 10 bits; ties keep the caller's order). */
enum irr_order {
    /* Hilbert curve (default): consecutive nodes are always face-adjacent
     * cells, so a block's neighbourhood touches fewer cache lines. */
    IRR_ORDER_HILBERT = 0,
    /* Morton (Z-order) curve: the order irr_morton_order_static returns. */
    IRR_ORDER_MORTON = 1
};

/* Partitioned: how each node block's directed entries are laid out. */
enum irr_layout {
    /* Sliced when its padding is at most half the entry count, else CSR. */
    IRR_LAYOUT_AUTO = 0,
    /* Rows of entries (CSR), columns ascending within a row. */
    IRR_LAYOUT_CSR = 1,
    /* Slices of 32 / lanes_per_row consecutive rows, each row padded to the
     * slice's longest (rounded up to 2 * lanes_per_row entries) and the
     * slice's entries interleaved so that one warp's lanes read one
     * contiguous, bank-conflict-free 256-byte line per step.  Same sums, in
     * the same order, as CSR. */
    IRR_LAYOUT_SLICED = 2,
    /* Staged ("halo"): work items of up to 64 consecutive rows, each with a
     * table of the node ids its rows touch; the kernel gathers the table's
     * positions into shared memory once per item and reads every entry's
     * neighbour from there, by a 16-bit table offset.  Each row's entries are
     * summed in an order chosen to spread shared-memory banks (not the CSR
     * order), so results differ from CSR / sliced in the last bits; 4 lanes
     * per row.  Applies when every 8 consecutive rows touch at most 640
     * distinct nodes and no row exceeds ~440 entries; else IRR_ERR_CAPACITY
     * (AUTO falls back). */
    IRR_LAYOUT_STAGED = 3
};

/* Node-data formats: the node_data_elm_size the reference passes. */
enum irr_node_format {
    IRR_NODES_F32X3 = 12, /* float xyz                                              */
    IRR_NODES_F32X4 = 16, /* float xyzw (w ignored)                                 */
    IRR_NODES_F64X3 = 24  /* double xyz: moldyn point_data, miniMD nodes            */
};

/* Result formats: the reduction_elm_size of get_reduction_result. */
enum irr_result_format {
    IRR_RESULT_F32X3 = 12, /* VALUE = float3 (moldyn/irregular/parameters.h:21-28) */
    IRR_RESULT_F32X4 = 16, /* float xyz + 0                                        */
    IRR_RESULT_F64X3 = 24  /* double xyz (moldyn's f[][3] buffer)                  */
};

typedef struct irr_config {
    int device;        /* CUDA device ordinal                                        */
    int exec;          /* enum irr_exec                                              */
    int map_idx;       /* enum irr_map                                               */
    int reduce_idx;    /* enum irr_reduce                                            */
    int block_nodes;   /* partitioned: nodes per block (power of two, 64..4096);
                          0 = tuned default                                          */
    int lanes_per_row; /* partitioned: lanes summing one node's row (1, 2, 4, 8, 16,
                          32); 0 = tuned default                                     */
    int reorder;       /* partitioned: 1 = curve order (default, see order), 0 = keep the
                          caller's order (blocks are then cut from it)              */
    int stage_smem;    /* partitioned: 1 = copy each block's entries (neighbour ids)
                          into a shared-memory ring with a bulk (TMA) copy, 0 = read
                          them from global memory; -1 = tuned default               */
    int layout;        /* partitioned: enum irr_layout                               */
    int order;         /* partitioned with reorder: enum irr_order                   */
    int wait_limit_us; /* partitioned: a device-side wait (a work item's entries, a free
                          ring stage) gives up after this many microseconds and the
                          next synchronising call returns IRR_ERR_DEVICE; 0 = 2 s    */
    int reserved[5];
} irr_config;

typedef struct irr_handle irr_handle;

/* Counts and sizes of a prepared handle. */
typedef struct irr_info {
    int64_t num_nodes;
    int64_t num_edges;
    int64_t num_entries;     /* directed entries held (2 * edges when partitioned) */
    int64_t num_blocks;      /* node blocks (partitioned)                          */
    int64_t device_bytes;    /* device memory held by the handle                   */
    int32_t block_nodes;
    int32_t lanes_per_row;
    int32_t stage_smem;
    int32_t exec;
    int32_t layout;          /* enum irr_layout in use (CSR or SLICED)              */
    int32_t order;           /* enum irr_order of the node order                    */
    int64_t num_slots;       /* entry slots stored: num_entries plus padding        */
    int64_t own_lo;          /* rows reduced: caller ids [own_lo, own_hi)           */
    int64_t own_hi;          /* (irr_set_shard; else [0, num_nodes))               */
} irr_info;

IRR_API void irr_config_default(irr_config *cfg);
IRR_API const char *irr_status_string(int status);

/* IrregularRuntime::IrregularRuntime (irregular_runtime.cu:17-48).  Creates
 * the handle and its stream on cfg->device; holds no node or edge data yet. */
IRR_API int irr_create(const irr_config *cfg, irr_handle **out);
/* IrregularRuntime::~IrregularRuntime (irregular_runtime.cu:446-458). */
IRR_API int irr_destroy(irr_handle *h);
/* Text of the last failure on this handle ("" when none). */
IRR_API const char *irr_last_error(const irr_handle *h);

/* Issue work on `stream` (a cudaStream_t, used as given: NULL is the CUDA
 * default stream) instead of the handle's own non-blocking stream. */
IRR_API int irr_set_stream(irr_handle *h, void *stream);
/* set_map_idx / set_reduce_idx (irregular_runtime.cu:493-501). */
IRR_API int irr_set_map(irr_handle *h, int map_idx);
IRR_API int irr_set_reduce(irr_handle *h, int reduce_idx);
/* The `parameter` block of the constructor, interpreted per map (above). */
IRR_API int irr_set_params(irr_handle *h, const void *param, int param_size);

/* The constructor's edges (EDGE = {int idx0, idx1}, moldyn/irregular/
 * data_type.h:5-9), host memory, 2*num_edges int32.  Copied; the caller's
 * array is never modified (the reference renumbers it in place,
 * reorder.cpp:160-172).  Endpoints are validated (IRR_ERR_INDEX) once the
 * node count is known. */
IRR_API int irr_set_edges(irr_handle *h, const int32_t *edges, int64_t num_edges);
/* Same, from device memory. */
IRR_API int irr_set_edges_device(irr_handle *h, const int32_t *d_edges, int64_t num_edges);

/* The constructor's node data, and reset_node_data (irregular_runtime.cu:
 * 436-439) on later calls: num_nodes records of elm_size bytes (enum
 * irr_node_format), host memory, in the caller's node order.  Positions are
 * used in float; the first three components are the coordinates.  Changing
 * num_nodes after irr_init is IRR_ERR_STATE.  After irr_init, page-locked host
 * memory on a 16-byte boundary is read in place, asynchronously: leave it
 * unchanged until the next irr_get_result or irr_sync returns. */
IRR_API int irr_set_nodes(irr_handle *h, const void *node_data, int elm_size, int64_t num_nodes);
/* Same, from device memory. */
IRR_API int irr_set_nodes_device(irr_handle *h, const void *d_node_data, int elm_size,
                         int64_t num_nodes);

/* IrregularInit (irregular_runtime.cu:50-193) plus the first split()
 * (:195-272): validates edges, runs the GPU partitioner (partitioned mode)
 * and lays the data out for the kernel.  Called by irr_step when needed. */
IRR_API int irr_init(irr_handle *h);

/* IrregularStart (irregular_runtime.cu:311-391): one reduction over all
 * edges with the current node data.  Enqueued on the handle's stream; the
 * host does not wait. */
IRR_API int irr_step(irr_handle *h);

/* get_reduction_result (irregular_runtime.cu:393-411): the per-node result
 * in the caller's node order, elm_size bytes per node (enum
 * irr_result_format), into host memory.  Synchronises the stream and reports
 * any device-side fault.  Page-locked host memory starting on a 16-byte
 * boundary is written by the kernel in place (no staging copy); so is the
 * node data irr_set_nodes reads after irr_init. */
IRR_API int irr_get_result(irr_handle *h, void *out, int elm_size);
/* Same, into device memory (aligned to 4, 16 or 8 bytes for 12-, 16- or
 * 24-byte records, else IRR_ERR_ARG); enqueued, does not synchronise. */
IRR_API int irr_get_result_device(irr_handle *h, void *d_out, int elm_size);

/* One step on new node data, pipelined with the steps before and after it:
 * irr_set_nodes + irr_step + irr_get_result for a stream of independent
 * inputs (a served stream, a parameter sweep), returning at once.  The
 * records (num_nodes of node_elm bytes, caller's order, host memory) are
 * copied to the device on a copy stream, reordered and reduced on the
 * handle's stream, and the result (out_elm bytes per result row, as
 * irr_get_result writes it) copied back to `out` on a second copy stream;
 * two slots of device staging let the upload of step k+1 and the read-back
 * of step k-1 run while step k reduces.  node_data is read and out written
 * asynchronously (page-locked memory gives overlapped copies; pageable memory
 * is copied synchronously): keep node_data unchanged and out unread until
 * irr_pipeline_sync returns.  After irr_init; built-in maps only.  No
 * counterpart in the reference, whose IrregularStart and
 * get_reduction_result each wait (irregular_runtime.cu:311-411). */
IRR_API int irr_step_pipelined(irr_handle *h, const void *node_data, int node_elm, void *out,
                               int out_elm);
/* Waits for every pipelined step issued so far (results in their `out`
 * buffers) and reports any device-side fault. */
IRR_API int irr_pipeline_sync(irr_handle *h);

/* Waits for the handle's stream and reports any device-side fault. */
IRR_API int irr_sync(irr_handle *h);
/* The limit of the partitioned kernel's device-side waits (irr_config
 * wait_limit_us; limit_us <= 0 restores the 2 s default).  withhold_once != 0
 * tests the time-out path: in the next irr_step the kernel's producers publish
 * no work, so every consumer's wait runs out after the limit, the launch ends
 * with nothing in flight, and the next synchronising call returns
 * IRR_ERR_DEVICE; the step after that runs normally.  No counterpart in the
 * reference, whose bucket-lock spins have no limit (moldyn/irregular/ros.cu:
 * 10-68). */
IRR_API int irr_set_wait_limit(irr_handle *h, int64_t limit_us, int withhold_once);
IRR_API int irr_get_info(const irr_handle *h, irr_info *info);

/* Partition outputs (partitioned mode, after irr_init), copied to host:
 * perm[new] = old node id, row_off[num_nodes + 1] (int64) and col[num_entries]
 * (the neighbour's new id of every directed entry, rows in node order,
 * entries within a row in edge-list order, idx0 side first).  Any pointer may
 * be NULL. */
IRR_API int irr_get_partition(irr_handle *h, int32_t *perm, int64_t *row_off, int32_t *col);

/* The staged layout of a handle that uses it (IRR_ERR_STATE otherwise),
 * copied to host so that it can be checked as integer work: counts[3] =
 * {items, words, table ids}; items: 6 int32 per item (first row, rows, first
 * word, words, first table id, table ids); slice_off: one uint32 per slice of
 * 8 rows, plus one; words; ids.  Any array may be NULL (counts alone size
 * them).  No reference counterpart. */
IRR_API int irr_get_staged(irr_handle *h, int64_t *counts, int32_t *items, uint32_t *slice_off,
                           uint32_t *words, int32_t *ids);

/* ------------------------------------------------- user per-edge functions
 * The irregular.h plugin.  The reference compiles the application's
 * irregular.h -- `map`, `reduce` and their __constant__ function tables
 * (moldyn/irregular.h:9-118) -- into its executors and calls
 * map_function_table[map_idx] once per edge (moldyn/irregular/gpu_kernel.cu:
 * 44-58, irregular_runtime.cu:493-501).  Here the application compiles its
 * irregular.h together with irregular_plugin.cuh, which turns the tables (or
 * one map) into a kernel and a launch function of type irr_user_launch_fn;
 * irr_set_user_map hands that function to a partitioned handle, and every
 * irr_step calls it with the view below on the handle's stream.
 *
 * The kernel gives each node's row its own reduction object and presents
 * each of the row's entries to `map` as the edge (row, neighbour): row is
 * idx0, part_index[x] == part_id holds for x == row only, and the object
 * keeps inserts keyed by the row (first insert copied, later ones combined
 * by `reduce` in the row's entry order, as the reference's reduction objects
 * do: moldyn/irregular/ros.cu:10-68).  Every listed edge is thus evaluated
 * once from each end, and each end keeps the contribution the map gives its
 * idx0: right for pair laws, whose idx1 contribution is the idx0
 * contribution of the reversed edge (both reference maps).  Node ids are
 * execution-order ids, consistent across point_data, part_index and keys. */
typedef struct irr_user_view {
    int64_t num_nodes;
    const uint32_t *row_off;  /* [num_nodes + 1] device; rows in execution order  */
    const int32_t *col;       /* [row_off[num_nodes]] neighbour ids, ascending     */
    void *node_data;          /* [num_nodes] node records, execution order         */
    int node_elm_size;        /* bytes per node record                             */
    int value_size;           /* bytes per result record (sizeof(VALUE))           */
    void *param;              /* device copy of the parameter block                */
    int param_size;
    int map_idx;              /* table entries chosen by irr_set_map / _reduce     */
    int reduce_idx;
    int *part_index;          /* [num_nodes] device, part_index[x] = x             */
    void *values;             /* [num_nodes] result records, execution order       */
    int *status;              /* device status word: nonzero reports IRR_ERR_DEVICE */
    int num_sms;
} irr_user_view;

/* Launches the user kernel on `stream` (a cudaStream_t); returns an
 * irr_status (IRR_ERR_ARG for a table index out of range). */
typedef int (*irr_user_launch_fn)(const irr_user_view *view, void *stream, void *ctx);

/* Result records of a user map. */
enum irr_value_kind {
    IRR_VALUE_BYTES = 0, /* opaque: read back at value_size bytes only          */
    IRR_VALUE_F32 = 1    /* floats: also readable widened to doubles, at twice
                            value_size (moldyn reads its float3 VALUEs into
                            double f[][3], moldyn/moldyn.cu:391)                */
};

/* Binds a user map to a partitioned handle before irr_init (IRR_ERR_STATE
 * after it, or on a plain handle at irr_init).  value_size: a multiple of 4
 * in [4, 256].  While bound: irr_set_map / irr_set_reduce select table
 * entries (map_idx / reduce_idx of the view; the launch function checks the
 * range); irr_set_params keeps the block as given (any size up to 64 KiB);
 * irr_set_nodes takes records of any multiple of 4 bytes up to 1024, and the
 * node order comes from irr_set_coordinates when given, else from records of
 * 12, 16 or 24 bytes read as positions, else the caller's order is kept;
 * irr_get_result reads value_size-byte records (or, for IRR_VALUE_F32,
 * 2 * value_size-byte doubles).  launch == NULL unbinds (before irr_init). */
IRR_API int irr_set_user_map(irr_handle *h, irr_user_launch_fn launch, void *ctx, int value_size,
                             int value_kind);
/* ----------------------------------------------------------------- shards
 * A handle reduces one shard of a larger problem: the reference's per-rank
 * view (moldyn/irregular/partition_view.cpp:44-282), in which a rank owns a
 * range of nodes, keeps every edge that touches one of them and receives the
 * positions of the remote endpoints (its halo) before each step (:285-435).
 * Here the shard's nodes are given to the handle as one node array -- owned
 * and halo nodes, in any order -- with the edges that touch an owned node;
 * irr_set_shard (before irr_init) names the owned nodes as the caller-id range
 * [own_lo, own_hi).  Rows of other nodes get no entries, so the step reduces
 * owned rows only, each over all of its edges; irr_get_result and
 * irr_get_result_device return own_hi - own_lo records (ids own_lo ...).
 * With reorder = 0 and the shard's nodes in the order of the whole problem's
 * execution order, every owned row holds the same neighbours in the same
 * order as in a handle over the whole problem, and with the CSR or sliced
 * layout its result is the same bit for bit. */
IRR_API int irr_set_shard(irr_handle *h, int64_t own_lo, int64_t own_hi);
/* Replaces node records [first, first + count) (caller ids) -- a shard's
 * halo before each step, or any range -- from host memory (page-locked memory
 * on a 16-byte boundary is read in place, as irr_set_nodes reads it) or, with
 * _device, from device memory; elm_size as irr_set_nodes gave. */
IRR_API int irr_set_nodes_range(irr_handle *h, const void *node_data, int elm_size, int64_t first,
                                int64_t count);
IRR_API int irr_set_nodes_range_device(irr_handle *h, const void *d_node_data, int elm_size,
                                       int64_t first, int64_t count);

/* The constructor's node_coordinates (irregular_runtime.cu:17-48):
 * num_nodes points of num_dims (2 or 3) components of coord_size (4 = float,
 * 8 = double) bytes, host memory, caller's order; copied.  Used to order the
 * nodes of a handle with a user map (above); ignored otherwise. */
IRR_API int irr_set_coordinates(irr_handle *h, const void *coords, int coord_size, int num_dims,
                                int64_t num_nodes);

/* ---------------------------------------------------------- file formats
 * The drivers' input files (host code; no GPU needed).
 * irr_read_graph: moldyn's adjacency format (moldyn/misc.c:62-146): '%'
 * comment lines before a "<nodes> <edges>" header, then one line per node of
 * 1-based neighbour ids, read up to the first value <= 0; only neighbours
 * j >= i are kept, so each pair is listed once, and their count must equal
 * the header's (else IRR_ERR_STATE).  Pairs are written to `edges` (at most
 * `cap`; NULL to count), 0-based as moldyn's build of the reader returns them
 * (misc.c defines CSTYLE), or 1-based when one_based != 0.
 * irr_read_coords: num_nodes whitespace-separated "x y z" triples
 * (moldyn/misc.c:224-246); a different count is IRR_ERR_STATE.
 * irr_write_graph / irr_write_coords: the same formats from a 0-based half
 * list (each pair on both endpoints' lines) and FP64 coordinates (%.17g). */
IRR_API int irr_read_graph(const char *path, int64_t *num_nodes, int64_t *num_edges,
                           int32_t *edges, int64_t cap, int one_based);
IRR_API int irr_read_coords(const char *path, int64_t num_nodes, double *xyz);
IRR_API int irr_write_graph(const char *path, int64_t num_nodes, const int32_t *edges,
                            int64_t num_edges);
IRR_API int irr_write_coords(const char *path, int64_t num_nodes, const double *xyz);

/* ----------------------------------------------------- batched instances
 * Many independent instances reduced by ONE persistent launch per step: the
 * reference's per-part work queue (moldyn/irregular/gpu_kernel.cu:60-77)
 * widened to (instance, node block) work items.  No counterpart in the
 * reference's API, which runs one edge set per runtime (paper Sec. II-C).
 * Instances are partitioned handles, borrowed: they must outlive the batch,
 * and their node data may change between steps (irr_set_nodes on the handle,
 * on the batch's stream or synchronised with it); results are read from each
 * handle (irr_get_result).  All instances share periodic or open
 * boundaries. */
typedef struct irr_batch irr_batch;
typedef struct irr_batch_info {
    int64_t num_instances;
    int64_t num_nodes;
    int64_t num_edges;
    int64_t num_items;
    int32_t lanes_per_row;
    int32_t block_nodes;
    int32_t graph;      /* 1 once a step is captured as a CUDA graph */
    int32_t reserved;
} irr_batch_info;

IRR_API int irr_batch_create(int device, irr_batch **out);
IRR_API int irr_batch_destroy(irr_batch *b);
IRR_API const char *irr_batch_last_error(const irr_batch *b);
IRR_API int irr_batch_set_stream(irr_batch *b, void *stream);
IRR_API int irr_batch_add(irr_batch *b, irr_handle *h);
/* Builds the instance table and the work-item list.  autotune != 0 times
 * candidate shapes (lanes per node row x rows per work item) on this data and
 * keeps the fastest, remembered per GPU and size class for the process. */
IRR_API int irr_batch_finalize(irr_batch *b, int autotune);
/* One reduction of every instance: one queue reset + one launch, or one CUDA
 * graph replay once irr_batch_capture has run.  Enqueued; does not wait. */
IRR_API int irr_batch_step(irr_batch *b);
/* Captures one step (queue reset + launch) into a CUDA graph replayed by
 * later irr_batch_step calls; needs a non-default stream. */
IRR_API int irr_batch_capture(irr_batch *b);
IRR_API int irr_batch_sync(irr_batch *b);
IRR_API int irr_batch_get_info(const irr_batch *b, irr_batch_info *info);
/* Picks the kernel shape of one partitioned handle by timing candidates. */
IRR_API int irr_autotune(irr_handle *h);

/* ------------------------------------------------------ neighbour lists
 * The half neighbour list the drivers build before the reduction, on the GPU
 * as a counting-sort cell list: miniMD's binned build (miniMD/neighbor.cpp:
 * 76-397) and moldyn's all-pairs RebuildNeighbor (moldyn/moldyn.cu:552-594).
 * pos: n records of pos_elm bytes (12, 16 or 24; xyz first), in host memory
 * or, with pos_on_device != 0, device memory.  box > 0: periodic cube of side
 * box (minimum image); box == 0: open boundaries.  A pair i < j is listed when
 * r2 <= list_cut2 with r2 = ((dx*dx + dy*dy) + dz*dz) in float, each operation
 * rounded, d wrapped once by +-box when |d| > box/2.  On success *d_edges is a
 * device array of 2 * *num_edges int32, pairs (i, j) sorted by i then j (free
 * it with irr_device_free). */
IRR_API int irr_neighbor_build(int device, void *stream, const void *pos, int pos_elm,
                               int pos_on_device, int64_t n, float box, float list_cut2,
                               int32_t **d_edges, int64_t *num_edges);
/* Frees device memory this library allocated for the caller. */
IRR_API int irr_device_free(int device, void *d_ptr);

/* ------------------------------------------------- molecular dynamics
 * A Lennard-Jones MD loop around the reduction, all on the GPU: the drivers'
 * step loops (moldyn/moldyn.cu:331-407; miniMD/ljs.cu:171-176) with the
 * velocity-Verlet integrator the reference leaves commented out
 * (miniMD/ljs.cu:39).  Periodic cube of side `side`, mass 1, LJ at
 * eps = sigma = 1 (force = 48 x the reduction's d (r^-14 - r^-8/2)) cut at
 * `cutforce`; the neighbour list is rebuilt on the GPU at cutforce + skin
 * every `rebuild_every` steps, and the nodes are re-partitioned each time.
 * Positions, velocities, the integration and the energy/virial sums are
 * FP64; per-edge forces are FP32 (the reduction). */
typedef struct irr_md_config {
    int device;
    int rebuild_every; /* steps between neighbour-list rebuilds (miniMD: 20) */
    double dt;         /* time step (0.005)                                 */
    double cutforce;   /* force cutoff (2.5)                                */
    double skin;       /* neighbour skin (0.3)                              */
    double side;       /* periodic box side; > 2 (cutforce + skin)          */
    int reorder_every; /* boxes with fewer than 3 list-cutoff cells on an   */
                       /* axis, or more cells than atoms: every this many   */
                       /* rebuilds the atoms are re-sorted along the curve  */
                       /* (10; 0 or 1: every rebuild).  Other boxes re-sort */
                       /* by cell at every rebuild.                         */
    int exec_plain;    /* 1: forces by the plain edge-parallel kernel over  */
                       /* the half list (atomics: the reference's per-edge  */
                       /* semantics, run to run not bitwise); 0 (default):  */
                       /* the partitioned owner-computes kernel             */
    int row_slots;     /* per-atom slots of the one-pass neighbour search   */
                       /* (0: the last rebuild's longest row + 25 % + 8; a  */
                       /* longer row falls back to counting first), 0..4096 */
    int reserved[5];
} irr_md_config;

typedef struct irr_md_info {
    int64_t num_atoms;
    int64_t num_edges; /* pairs in the current list */
    int64_t steps;
    int64_t rebuilds;
} irr_md_info;

typedef struct irr_md irr_md;

IRR_API void irr_md_config_default(irr_md_config *cfg);
/* pos, vel: 3n doubles (host).  Builds the list and the first forces. */
IRR_API int irr_md_create(const irr_md_config *cfg, const double *pos, const double *vel,
                          int64_t n, irr_md **out);
IRR_API int irr_md_destroy(irr_md *m);
IRR_API const char *irr_md_last_error(const irr_md *m);
IRR_API int irr_md_set_stream(irr_md *m, void *stream);
/* Enqueues `steps` velocity-Verlet steps (rebuilds included). */
IRR_API int irr_md_run(irr_md *m, int steps);
/* Kinetic and potential energy (4(r^-12 - r^-6) over pairs inside the cutoff)
 * and the virial sum of r.F, as FP64 sums; synchronises. */
IRR_API int irr_md_energy(irr_md *m, double *kinetic, double *potential, double *virial);
/* Positions and velocities (3n doubles each, caller's atom order; either may
 * be NULL); synchronises. */
IRR_API int irr_md_get_state(irr_md *m, double *pos, double *vel);
/* Current forces (3n doubles, caller's atom order); synchronises. */
IRR_API int irr_md_get_forces(irr_md *m, double *f);
IRR_API int irr_md_get_info(const irr_md *m, irr_md_info *info);

/* ------------------------------------------------------------ serving
 * A request loop for MD jobs with continuous batching (no counterpart in the
 * reference, which serves one edge set per process).  Jobs arrive as a seeded
 * Poisson stream; each is a Lennard-Jones system (miniMD's FCC lattice with a
 * small jitter, Maxwell velocities) of log-uniform size asking for
 * steps_per_job velocity-Verlet steps.  Arrived jobs are admitted in order
 * while their estimated device memory fits budget_bytes; every tick advances
 * every resident job one step with ONE batched force launch over all of
 * them; finished jobs leave and free their memory.  IRR_SERVE_SERIAL runs the
 * same jobs one at a time; IRR_SERVE_SERIAL_PLAIN one at a time with every
 * force evaluation by the plain edge-parallel kernel (irr_md_config
 * exec_plain).  A job's trajectory is bitwise the same alone (only_job = its
 * index) and in the mix. */
enum irr_serve_mode { IRR_SERVE_CONTINUOUS = 0, IRR_SERVE_SERIAL = 1, IRR_SERVE_SERIAL_PLAIN = 2 };
/* Which waiting job a free slot admits: the earliest arrival, or the smallest
 * job (shortest-job-first: the lowest mean latency, the largest jobs last). */
enum irr_serve_policy { IRR_SERVE_FIFO = 0, IRR_SERVE_SJF = 1 };

typedef struct irr_serve_config {
    int device;
    int num_jobs;
    int steps_per_job;
    int rebuild_every;
    int mode;           /* enum irr_serve_mode                                 */
    int only_job;       /* >= 0: run that job alone (arriving at t = 0)        */
    int max_resident;   /* slot limit on resident jobs (default 64)            */
    int reserved0;
    double arrival_rate; /* jobs per second (Poisson)                         */
    double density;
    double cutforce;
    double skin;
    double dt;
    double temperature;
    int64_t min_atoms;  /* sizes log-uniform in [min_atoms, max_atoms]         */
    int64_t max_atoms;
    double budget_bytes; /* admission budget of device memory                 */
    uint64_t seed;
    int policy;         /* enum irr_serve_policy: admission order (FIFO)      */
    int reserved[7];
} irr_serve_config;

typedef struct irr_serve_stats {
    int64_t jobs_done;
    int64_t rejected;     /* jobs larger than the whole budget                 */
    int64_t max_resident;
    int64_t reserved0;
    double p50_ms;        /* job latency: completion - arrival                 */
    double p99_ms;
    double mean_ms;
    double max_ms;
    double makespan_s;
    double pair_evals;    /* sum over jobs and steps of listed pairs reduced   */
    double edges_per_s;   /* pair_evals / makespan                             */
    double peak_budget_bytes;
} irr_serve_stats;

typedef struct irr_serve_job {
    int64_t atoms;
    int64_t edges;        /* pairs in the job's last list                      */
    double arrival_s;
    double admit_s;
    double done_s;
    double energy;        /* final kinetic + potential energy                  */
    uint64_t state_hash;  /* digest of the final FP64 positions by atom id     */
    int32_t status;
    int32_t reserved;
} irr_serve_job;

IRR_API void irr_serve_config_default(irr_serve_config *cfg);
/* Job `job` of the stream that cfg describes, as irr_serve_run makes it (host
 * code; no GPU): its atom count, box side, and initial state -- 3n FP64
 * positions and 3n velocities, the job's own atom order; any output may be
 * NULL.  A job's result can be replayed alone (irr_md_* on this state with
 * cfg's dt, cutforce, skin and rebuild_every gives the same trajectory bit for
 * bit) and checked against another implementation.  No counterpart in the
 * reference. */
IRR_API int irr_serve_job_state(const irr_serve_config *cfg, int job, int64_t *atoms,
                                double *side, double *pos, double *vel);
/* Runs the stream to completion; jobs_out (optional) has num_jobs records. */
IRR_API int irr_serve_run(const irr_serve_config *cfg, irr_serve_stats *stats,
                          irr_serve_job *jobs_out);

/* ------------------------------------------------ allocation-free ordering
 * No counterpart in the reference.  The partitioner's Morton node ordering
 * (perm[new] = old node id, bit for bit the perm that irr_get_partition
 * returns for reorder = 1, order = IRR_ORDER_MORTON) for callers that cannot allocate device memory --
 * an application that has already reserved the GPU's memory for its own
 * pool, or a latency-bound loop where cudaMalloc/cudaFree (which may
 * synchronise the device) are not acceptable.  It calls no allocator: its
 * scratch is a fixed device array inside this library of
 * IRR_MORTON_STATIC_SCRATCH_BYTES (about 12.3 MiB), held by every GPU that
 * loads the library until the process exits.
 *   d_pos: n device records of pos_elm bytes (12: float xyz, 16: float xyzw),
 *   on a 4-byte boundary; d_perm: n int32 of device output, on a 4-byte
 *   boundary (else IRR_ERR_ARG);  n <= IRR_MORTON_STATIC_MAX_NODES, else
 *   IRR_ERR_CAPACITY.
 * Each call on a stream that is not capturing looks up the array's device
 * address (so a device reset is picked up); a call on a capturing stream uses
 * the last look-up on that device: make the first call on a device before any
 * stream capture.  Every call shares the one array: calls that overlap on the
 * GPU race, so order them (one stream, or events).  Enqueued on `stream`; the
 * host does not wait.  The caller's current device is restored on return. */
#define IRR_MORTON_STATIC_MAX_NODES 1048576
#define IRR_MORTON_STATIC_SCRATCH_BYTES 12886272
IRR_API int irr_morton_order_static(int device, void *stream, const void *d_pos, int pos_elm,
                                    int64_t n, int32_t *d_perm);

#ifdef __cplusplus
}
#endif
#endif
