// irr_internal.cuh -- declarations shared by the library's translation units.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "irr_law.cuh"

namespace irr {

// Device status word bits (set by kernels, read by the host at sync points).
enum : int {
    kStatusBadIndex = 1 << 0,   // an edge endpoint outside [0, n)
    kStatusWaitTimeout = 1 << 1, // a bounded device-side wait gave up
    kStatusBadAlign = 1 << 2,   // a bulk copy was asked for an unaligned range
};

// Makes `device` current for the guard's lifetime and then restores the
// calling thread's previous current device, so that no entry point leaves a
// multi-GPU host program on another GPU.  ok() is false when the device could
// not be made current (the CUDA error is cleared).
class DeviceGuard {
public:
    explicit DeviceGuard(int device)
    {
        if (cudaGetDevice(&prev_) != cudaSuccess) {
            cudaGetLastError();
            prev_ = -1;
        }
        ok_ = cudaSetDevice(device) == cudaSuccess;
        if (!ok_) cudaGetLastError();
    }
    ~DeviceGuard()
    {
        if (prev_ >= 0 && cudaSetDevice(prev_) != cudaSuccess) cudaGetLastError();
    }
    bool ok() const { return ok_; }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;

private:
    int prev_ = -1;
    bool ok_ = false;
};

// One system of the (possibly batched) owner-computes reduction.
struct InstDesc {
    const float4* pos;        // node positions, execution (partition) order
    const uint32_t* row_off;  // n + 1 entry offsets
    const int32_t* col;       // neighbour of each directed entry (instance-local id)
    float4* force;            // per-node result, execution order
    const uint32_t* slice_off;  // sliced or staged layout: word offset of each slice (or null)
    const int32_t* scol;        // sliced layout: interleaved, padded entries
    const uint32_t* words;      // staged layout: headers and 16-bit table offsets
    const int32_t* tab;         // staged layout: the items' tables (node ids), concatenated
    LawParams law;
    int64_t n;
};

// One node block: rows [row0, row0 + nrows) of instance `inst`, whose
// directed entries are [ent0, ent0 + nent) of the instance's col array (or,
// with kItemSliced, words [ent0, ent0 + nent) of its sliced array: whole
// slices, so row0 is a multiple of the slice height; with kItemStaged, words
// of its staged array, and its table is ids [tab0, tab0 + ntab) of tab).
struct WorkItem {
    int32_t inst;
    int32_t row0;
    int32_t nrows;
    int32_t flags;       // kItemDirect: read entries from global memory
    uint32_t ent0;
    uint32_t nent;
    uint32_t tab0;
    uint32_t ntab;
};

enum : int { kItemDirect = 1, kItemSliced = 2, kItemStaged = 4 };

// Sliced entry layout of one instance, for G lanes per row.  A slice is
// R = 32 / G consecutive rows; each row is padded to the slice's longest row
// rounded up to 2G entries, so a slice is T = ceil(maxlen / 2G) steps of 64
// words.  In step t, lane i*G + l of a warp handles entries (2Gt + l,
// 2Gt + G + l) of row i, read together as the int2 at word 64t + 2(iG + l):
// the warp reads one contiguous 256-byte line, the same entry pairs the CSR
// path gives that lane, in the same order.  Padding words hold the row's
// own id (0 past the last row).
struct Sliced {
    uint32_t* slice_off = nullptr;   // [slices + 1] word offsets (multiples of 64)
    int32_t* col = nullptr;          // [words]
    int64_t slices = 0;
    int64_t words = 0;
    int lanes = 0;                   // G it was built for; 0 = not built
    std::vector<uint32_t> host_off;  // host copy of slice_off (cuts work items)
};

struct TiledShape {
    int lanes_per_row;   // 4, 8, 16 or 32
    int stage_smem;      // 1: entry segments bulk-copied into a shared-memory ring
    int block_nodes;     // max rows per work item
    int periodic;
    int staged = 0;      // 1: staged layout (the halo kernel; 4 lanes per row)
};

// Staged ("halo") layout of one instance, for 4 lanes per row and slices of 8
// rows (irr_staged.cu): per work item a table of node ids whose positions the
// kernel gathers into shared memory, and per slice 32 header words and 32
// words per step of 16-bit byte offsets into that table.
// (each can be set at build time, -DIRR_HALO_SLICES=... etc., to build and
// time variants; the oracle's layout takes the same three limits)
#ifndef IRR_HALO_SLICES
#define IRR_HALO_SLICES 8
#endif
#ifndef IRR_HALO_TABMAX
#define IRR_HALO_TABMAX 640
#endif
#ifndef IRR_HALO_STREAMMAX
#define IRR_HALO_STREAMMAX 3584
#endif
#ifndef IRR_HALO_STAGES
#define IRR_HALO_STAGES 2
#endif
constexpr int kHaloSlicesPerItem = IRR_HALO_SLICES;  // 64 rows per item at most
constexpr int kHaloTabMax = IRR_HALO_TABMAX;         // table ids per item (~10 KB of positions)
constexpr int kHaloStreamMax = IRR_HALO_STREAMMAX;   // words per item (14 KB)
constexpr int kHaloStages = IRR_HALO_STAGES;         // shared-memory ring depth
struct Staged {
    uint32_t* slice_off = nullptr;   // [slices + 1] word offsets (multiples of 32)
    uint32_t* words = nullptr;       // [nwords]
    int32_t* ids = nullptr;          // [nids] the items' tables, concatenated
    int64_t slices = 0;
    int64_t nwords = 0;
    int64_t nids = 0;
    std::vector<uint32_t> host_off;  // host copy of slice_off
    std::vector<WorkItem> items;     // the items (instance 0), flags kItemStaged
};
// Builds st from a CSR (rows in execution order, columns ascending) on the
// device; host_row_off is the host copy of row_off.  Synchronises s.
// cudaErrorNotSupported (nothing allocated) when a slice alone exceeds the
// limits above -- a row of more than ~440 entries, or 8 rows touching more
// than kHaloTabMax distinct nodes.
cudaError_t build_staged(const uint32_t* row_off, const int32_t* col, const uint32_t* host_row_off,
                         int64_t n, Staged* st, cudaStream_t s);
void free_staged(Staged* st, cudaStream_t s = nullptr);

// Shape of the owner-computes kernel; each can be set at build time
// (-DIRR_STAGES=... etc.) to build and time variants.
#ifndef IRR_STAGES
#define IRR_STAGES 2
#endif
// 5104 entries: 2 stages of (5104 + kColPad) words, the barriers and the
// per-CTA reserve keep 4 CTAs inside the 164 KB shared-memory carveout, so
// the SM keeps ~92 KB of L1 for the position gathers (at 5120 the next
// carveout, 196 KB, leaves ~60 KB: measured 2 % slower).  8 slices of the MD
// workloads (~4800 words) still fit one stage.
#ifndef IRR_STAGE_ENTRIES
#define IRR_STAGE_ENTRIES 5104
#endif
#ifndef IRR_CTAS_PER_SM
#define IRR_CTAS_PER_SM 4
#endif
constexpr int kStages = IRR_STAGES;              // shared-memory ring depth
constexpr int kStageEntries = IRR_STAGE_ENTRIES; // entries per stage (~20 KB)
constexpr int kColPad = 4;                       // entries allocated past the end of col
constexpr int kCtasPerSm = IRR_CTAS_PER_SM;      // resident CTAs per SM (registers, ring)

// Cuts rows [0, n) into work items of at most max_rows rows and (unless a
// single row is longer) at most kStageEntries entries, at a multiple of
// `round_rows` rows (the consumer warps' row groups) where that fits.
// row_off: host copy.
void make_work_items(const uint32_t* row_off, int64_t n, int inst, int max_rows, int staged,
                     std::vector<WorkItem>& out, int round_rows = 1);
// The same for a sliced layout: whole slices, at most max_rows rows and
// kStageEntries words per item (a longer slice is read from global memory),
// cut at multiples of kConsumerSlices slices where that fits.
void make_sliced_items(const Sliced& sl, int64_t n, int inst, int max_rows, int staged,
                       std::vector<WorkItem>& out);
#ifndef IRR_CONSUMER_WARPS
#define IRR_CONSUMER_WARPS 8
#endif
constexpr int kConsumerSlices = IRR_CONSUMER_WARPS;  // consumer warps of the tiled kernel
// One instance's items for `shape`: sliced items if sl was built for
// shape.lanes_per_row, else CSR items from the host row offsets.
void make_instance_items(const uint32_t* host_row_off, const Sliced& sl, int64_t n, int inst,
                         const TiledShape& shape, std::vector<WorkItem>& out);

// -- sliced layout (irr_partition.cu) --
// Builds sl for G lanes per row from a CSR (row_off, col) of n rows on the
// device; synchronises s (the host keeps the slice offsets).  Fails with
// cudaErrorInvalidValue if the layout would exceed 2^32 - 1 words.
cudaError_t build_sliced(const uint32_t* row_off, const int32_t* col, int64_t n, int G,
                         Sliced* sl, cudaStream_t s);
// s != nullptr: stream-ordered frees on s (the arrays come from cudaMallocAsync).
void free_sliced(Sliced* sl, cudaStream_t s = nullptr);
// The automatic choice: sliced when padding adds at most half the entries.
inline bool sliced_pays(const Sliced& sl, int64_t entries)
{
    return sl.words <= entries + entries / 2 + 64;
}

// -- device memory --
// Stream-ordered allocation from the library's own memory pool on the current
// device.  Its release threshold is unlimited: blocks freed with
// cudaFreeAsync stay in the pool for the next allocation instead of going back
// to the driver at every synchronisation (the default pool's behaviour), so a
// rebuild that frees and re-allocates ~300 MB of layout does not re-map it.
// The pool keeps the library's peak footprint until the process exits.
cudaError_t irr_malloc_async(void** p, size_t bytes, cudaStream_t s);
template <class T>
inline cudaError_t irr_malloc_async(T** p, size_t bytes, cudaStream_t s)
{
    return irr_malloc_async(reinterpret_cast<void**>(p), bytes, s);
}

// How long a kernel's device-side waits may last before it gives up
// (kStatusWaitTimeout), and the one-shot test of that path: withhold != 0
// makes the producers publish nothing, so every consumer wait runs out.
constexpr uint64_t kDefaultWaitNs = 2000000000ull;  // 2 s: far above any work item's time
struct WaitPolicy {
    uint64_t wait_ns = kDefaultWaitNs;
    int withhold = 0;
};

// -- reduction kernels (irr_reduce.cu) --
cudaError_t launch_plain(const float4* pos, const int2* edges, int64_t e, float4* force,
                         const LawParams& law, cudaStream_t s);
// A persistent grid of `grid` CTAs draws items from *d_queue (which must be
// 0 at launch).  host_insts (a host copy of the num_insts descriptors of
// d_insts) may be given: for one instance (the whole descriptor), or up to
// 1024 (the fields the step loop reads), the kernel then takes them as a
// launch parameter instead of holding them in registers across items.
cudaError_t launch_tiled(const TiledShape& shape, const InstDesc* d_insts,
                         const WorkItem* d_items, int num_items, int* d_queue, int grid,
                         int* d_status, cudaStream_t s, const InstDesc* host_insts = nullptr,
                         int num_insts = 0, const WaitPolicy& wp = WaitPolicy{});

// -- data movement (irr_partition.cu) --
// Raw node records (12/16/24 bytes) -> float4, optionally gathered: dst[k] =
// rec[perm ? perm[k] : k].
cudaError_t launch_load_nodes(const void* raw, int elm_size, const int32_t* perm, int64_t n,
                              float4* dst, cudaStream_t s);
// Records in the caller's order, read in order (rec may be page-locked host
// memory the device addresses: see host_device_view) and scattered into
// execution order: dst[inv ? inv[i] : i] = record i.
cudaError_t launch_load_nodes_scatter(const void* rec, int elm_size, const int32_t* inv, int64_t n,
                                      float4* dst, cudaStream_t s);
// p itself when it is page-locked host memory that kernels can read and
// write at the same address and it starts on a 16-byte boundary, else
// nullptr (other host memory goes through staging copies).
void* host_device_view(const void* p);
// Results: out[i] = force[inv ? inv[i] : i] in the requested format, written
// in order (out may be device memory or page-locked host memory).
cudaError_t launch_store_result(const float4* force, const int32_t* inv, int64_t n,
                                int elm_size, void* out, cudaStream_t s);
cudaError_t launch_validate_edges(const int2* edges, int64_t e, int64_t n, int* d_status,
                                  cudaStream_t s);

// -- user-map records (irr_user.cu) --
// dst record k = src record idx[k] (idx nullptr: k); elm_size a multiple of 4.
cudaError_t launch_gather_records(const void* src, int elm_size, const int32_t* idx, int64_t n,
                                  void* dst, cudaStream_t s);
// Same, each float of a record widened to a double (dst records are
// 2 * elm_size bytes).
cudaError_t launch_widen_records(const void* src, int elm_size, const int32_t* idx, int64_t n,
                                 void* dst, cudaStream_t s);
// out[i] = i.
cudaError_t launch_iota(int32_t* out, int64_t n, cudaStream_t s);
// Points of dims (2 or 3) components of coord_size (4 or 8) bytes -> float4.
cudaError_t launch_coords_to_pos(const void* coords, int coord_size, int dims, int64_t n, float4* dst,
                                 cudaStream_t s);

// -- partitioner (irr_partition.cu) --
// Hilbert index of a cell on the 2^10-per-axis grid: Skilling's transform
// (J. Skilling, "Programming the Hilbert curve", AIP Conf. Proc. 707, 2004)
// from axes to the transposed index, whose bits are then interleaved, axis 0
// in the high bit of each 3-bit group.  The oracle restates it bit for bit.
__device__ __forceinline__ uint32_t hilbert10(uint32_t x0, uint32_t x1, uint32_t x2)
{
    uint32_t X[3] = {x0, x1, x2};
    for (uint32_t Q = 1u << 9; Q > 1; Q >>= 1) {
        const uint32_t P = Q - 1;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            if (X[i] & Q) {
                X[0] ^= P;  // invert
            } else {
                const uint32_t t = (X[0] ^ X[i]) & P;  // exchange
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];  // Gray encode
    X[2] ^= X[1];
    uint32_t t = 0;
    for (uint32_t Q = 1u << 9; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    uint32_t key = 0;
    for (int b = 9; b >= 0; b--)
        key = (key << 3) | (((X[0] >> b) & 1u) << 2) | (((X[1] >> b) & 1u) << 1) | ((X[2] >> b) & 1u);
    return key;
}

struct PartitionOut {
    int32_t* perm = nullptr;      // [n] new -> old
    int32_t* inv = nullptr;       // [n] old -> new
    uint32_t* row_off = nullptr;  // [n + 1]
    int32_t* col = nullptr;       // [2e]
};
// Per-axis min and max of pos (synchronises s).
cudaError_t bbox_minmax(const float4* pos, int64_t n, float lo[3], float hi[3], cudaStream_t s);
// Computes the curve frame (per-axis min and 1024 / extent) of pos: the
// 10-bit grid both node orders quantise on.
cudaError_t bbox_frame(const float4* pos, int64_t n, float lo[3], float scale[3],
                       cudaStream_t s);
// Full partition of n nodes and e half edges.  Allocates out's arrays with
// cudaMallocAsync on s (caller frees).  reorder == 0 keeps the identity order.
// curve: 0 = Hilbert (IRR_ORDER_HILBERT), 1 = Morton.
cudaError_t build_partition(const float4* pos_user, int64_t n, const int2* edges, int64_t e,
                            int reorder, PartitionOut* out, cudaStream_t s, int curve = 0);
// A shard's partition: rows whose caller id is outside [lo, hi) lose their
// entries (row_off and col rebuilt, order kept); *m_out = entries left.
cudaError_t keep_rows(PartitionOut* p, int64_t n, int64_t lo, int64_t hi, int64_t* m_out, cudaStream_t s);
// Half neighbour list (irr_neighbor.cu); *d_edges is cudaMalloc'd, or, with
// stream_ordered, cudaMallocAsync'd on s (free it with cudaFreeAsync).
// sort_rows == false returns the same pairs (i < j) in no particular order,
// for a caller that re-sorts them anyway, like the partitioner (found by a
// half-stencil search when the box has at least 3 cells per axis).
cudaError_t build_neighbor_list(const float4* pos, int64_t n, float box, float cut2,
                                int2** d_edges, int64_t* num_edges, cudaStream_t s,
                                bool stream_ordered = false, bool sort_rows = true);
// Full neighbour rows of a periodic box of at least 3 cells per axis (and no
// more cells than nodes), for the MD rebuild: out->perm (new -> old) orders
// the nodes by the Hilbert index of their cell, out->row_off / out->col hold
// each node's partners j != i (rule of build_neighbor_list) in that order,
// ascending; out->inv is not made.  *num_edges = pairs (entries / 2),
// *longest = the longest row.  cap_hint > 0 (e.g. from the previous build's
// longest row) lets one search pass write rows of up to cap_hint entries into
// per-node slots, packed afterwards; 0, or a longer row, takes a counting and
// a writing pass.  cudaErrorNotSupported, with nothing allocated, for other
// boxes.
cudaError_t build_rows_by_cell(const float4* pos, int64_t n, float box, float cut2, PartitionOut* out,
                               int64_t* num_edges, uint32_t* longest, uint32_t cap_hint, cudaStream_t s);
// Sorts each row of a CSR (row_off[n + 1], col) ascending; every row must
// hold at most kRowSortMax entries.
constexpr int kRowSortMax = 1024;
cudaError_t launch_row_sort(const uint32_t* row_off, int64_t n, int32_t* col, cudaStream_t s);
// The longest row of a CSR (synchronises s).
cudaError_t max_row_len(const uint32_t* row_off, int64_t n, uint32_t* result, cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs on key bits [0, key_bits).
// Sorted data ends in (keys, vals); tmp arrays have n entries each.
cudaError_t radix_sort_pairs(uint32_t* keys, int32_t* vals, uint32_t* keys_tmp,
                             int32_t* vals_tmp, int64_t n, int key_bits, cudaStream_t s);
// Exclusive prefix sum of n uint32 into out (out may alias in); *total, if
// non-null, receives the sum (device pointer).
cudaError_t scan_exclusive_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* d_total,
                               cudaStream_t s);

// Scan and radix-sort building blocks (irr_partition.cu).
constexpr int kScanThreads = 256;
constexpr int kScanBlock = kScanThreads * 4;
constexpr int kSortThreads = 256;
constexpr int kSortTile = kSortThreads * 16;
__global__ void scan_blocks_kernel(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* block_sums);
__global__ void add_offsets_kernel(uint32_t* out, int64_t n, const uint32_t* block_off);
__global__ void radix_hist_kernel(const uint32_t* keys, int64_t n, int shift, uint32_t* hist,
                                  int64_t ntiles);
__global__ void radix_scatter_kernel(const uint32_t* kin, const int32_t* vin, uint32_t* kout,
                                     int32_t* vout, int64_t n, int shift, const uint32_t* offs,
                                     int64_t ntiles);

// Morton key of one position in a frame (shared with the oracle bit for bit).
__host__ __device__ __forceinline__ uint32_t spread3(uint32_t v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

}  // namespace irr

#define IRR_CUDA_TRY(expr)                         \
    do {                                           \
        cudaError_t irr_e_ = (expr);               \
        if (irr_e_ != cudaSuccess) return irr_e_;  \
    } while (0)
