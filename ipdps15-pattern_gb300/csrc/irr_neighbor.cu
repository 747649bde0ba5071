// irr_neighbor.cu -- half neighbour list on the GPU by a counting-sort cell list.
//
// Replaces miniMD's serial binned build (miniMD/neighbor.cpp:76-205: linked-list
// bins filled by binatoms :209-239, a half stencil from setup :289-397) and
// moldyn's O(N^2) all-pairs RebuildNeighbor (moldyn/moldyn.cu:552-594):
//   1. each node gets a cell key (cells at least as wide as the list cutoff);
//   2. a stable radix sort by key orders nodes by cell; a count + scan gives
//      each cell's start;
//   3. positions are copied into cell order, so a cell's candidates are
//      contiguous and each is one load, not an id load and then a dependent
//      position load;
//   4. one thread per node (in cell order, so a warp shares cells) scans the
//      27 surrounding cells for partners j > i with r2 <= cut2, first counting,
//      then -- after a scan of the counts -- writing them; a warp per row then
//      sorts each row by j.  A caller that re-sorts the pairs anyway gets
//      them in no particular order, from a half stencil (pairs_half_kernel:
//      each pair found once, from one end), written straight as pairs.
// The pair rule is shared bit for bit with the CPU oracle: d = x_i - x_j in
// float, wrapped once by +-box when |d| > box/2 (periodic), r2 = ((dx*dx +
// dy*dy) + dz*dz) with every operation rounded.  Output: pairs (i, j), i < j,
// sorted by i then j -- moldyn's loop order; miniMD lists the same pairs.
// With at least 5 cells per axis and every position inside the periodic box,
// a neighbour cell decides the image of all its partners (list_pair_shifted).
//
// The MD rebuild takes another route (build_rows_by_cell): the nodes are
// re-sorted by the Hilbert index of their cell, and each node's full row is
// written by one search over its 27 cells visited in curve order -- ascending
// by construction, so the rows need neither the pair list, nor atomic row
// cursors, nor a sort.
#include <cmath>
#include <type_traits>
#include <vector>

#include "irr_internal.cuh"
#include "irr_trace.cuh"
#include "../../include/irregular_gb300.h"

namespace irr {
namespace {

struct Grid {
    int nc[3];
    int offs[3][3];   // neighbour cell offsets per axis (deduplicated)
    int noff[3];
    double org[3];
    double inv[3];    // 1 / cell size
    float box, hb, cut2;
    int periodic;
    int fast;         // periodic with >= 5 cells per axis: image decided by the cell
};

__device__ __forceinline__ bool list_pair(float4 a, float4 b, const Grid& g)
{
    float d[3] = {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
    if (g.periodic) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (d[c] > g.hb)
                d[c] = __fsub_rn(d[c], g.box);
            else if (d[c] < -g.hb)
                d[c] = __fadd_rn(d[c], g.box);
        }
    }
    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])),
                               __fmul_rn(d[2], d[2]));
    return r2 <= g.cut2;
}

// The same rule when the neighbour cell decides the image: with at least 5
// cells per axis and every position in [0, box), a partner in a cell that is
// adjacent without wrapping is less than 2/5 of the box away on that axis
// (the rule keeps d), and one in a cell reached across the boundary more
// than 3/5 (the rule adds or subtracts the box, always the same way), so the
// cell's shift s (0 or +-box) is added instead of compared for.  d + 0 is d
// except for d = -0, whose square is the same.
__device__ __forceinline__ bool list_pair_shifted(float4 a, float4 b, float sx, float sy, float sz,
                                                  float cut2)
{
    const float dx = __fadd_rn(__fsub_rn(a.x, b.x), sx);
    const float dy = __fadd_rn(__fsub_rn(a.y, b.y), sy);
    const float dz = __fadd_rn(__fsub_rn(a.z, b.z), sz);
    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    return r2 <= cut2;
}

// list_pair_shifted with no shift (a cell reached without crossing the box).
__device__ __forceinline__ bool list_pair_unshifted(float4 a, float4 b, float cut2)
{
    const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    return r2 <= cut2;
}

template <bool FAST>
__device__ __forceinline__ bool pair_hit(float4 a, float4 b, const Grid& g, float sx, float sy, float sz)
{
    return FAST ? list_pair_shifted(a, b, sx, sy, sz, g.cut2) : list_pair(a, b, g);
}

// Neighbour cell (x, y, z) of a periodic grid wrapped into range, with the
// image shift of each wrapped axis: a cell reached below 0 lies at the top of
// the box (its partners are pulled down by +box), one reached past the top
// at the bottom (-box).
__device__ __forceinline__ void wrap_cell(int& v, int nc, float box, float& s)
{
    s = 0.f;
    if (v < 0) {
        v += nc;
        s = box;
    } else if (v >= nc) {
        v -= nc;
        s = -box;
    }
}

__device__ __forceinline__ int cell_coord(float x, int axis, const Grid& g)
{
    long long k = (long long)floor(((double)x - g.org[axis]) * g.inv[axis]);
    if (g.periodic) k = ((k % g.nc[axis]) + g.nc[axis]) % g.nc[axis];
    if (k < 0) k = 0;
    if (k >= g.nc[axis]) k = g.nc[axis] - 1;
    return (int)k;
}

// Also raises *outside when a position of a periodic box lies outside
// [0, box) (or is NaN): the cell-decided image above then does not hold.
__global__ void cell_keys_kernel(const float4* pos, int64_t n, const __grid_constant__ Grid g, uint32_t* keys,
                                 int32_t* vals, uint32_t* cell_count, int* outside)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        if (g.periodic && !(p.x >= 0.f && p.x < g.box && p.y >= 0.f && p.y < g.box && p.z >= 0.f &&
                            p.z < g.box))
            *outside = 1;
        const uint32_t c = ((uint32_t)cell_coord(p.z, 2, g) * g.nc[1] + cell_coord(p.y, 1, g)) *
                               g.nc[0] +
                           cell_coord(p.x, 0, g);
        keys[i] = c;
        vals[i] = (int32_t)i;
        atomicAdd(cell_count + c, 1u);
    }
}

// pos_c[q] = pos[sorted[q]]: positions in cell order
__global__ void cell_order_kernel(const float4* __restrict__ pos, const int32_t* __restrict__ sorted,
                                  int64_t n, float4* __restrict__ pos_c)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x)
        pos_c[q] = pos[sorted[q]];
}

// WRITE == false: counts partners; WRITE == true: writes them from row_off[i],
// as neighbour ids into nbr (with sort_here, sorting the row by j in place:
// only for rows too long for the row sort that otherwise follows) or, when
// pairs != nullptr, as the pairs (i, j) themselves.  FAST: the image decided
// by the cell (list_pair_shifted).
template <bool WRITE, bool FAST>
__device__ __forceinline__ void pairs_rows(const float4* __restrict__ pos_c, const int32_t* __restrict__ sorted,
                                           const uint32_t* __restrict__ cell_start, int64_t n,
                                           const Grid& g, uint32_t* count,
                                           const uint32_t* __restrict__ row_off, int32_t* nbr,
                                           int2* pairs, int sort_here)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = sorted[t];
        const float4 a = pos_c[t];
        const int cx = cell_coord(a.x, 0, g), cy = cell_coord(a.y, 1, g), cz = cell_coord(a.z, 2, g);
        uint32_t m = 0;
        const uint32_t base = WRITE ? row_off[i] : 0;
        for (int oz = 0; oz < g.noff[2]; oz++) {
            int z = cz + g.offs[2][oz];
            float sz = 0.f;
            if (FAST) wrap_cell(z, g.nc[2], g.box, sz);
            else if (g.periodic) z = (z + g.nc[2]) % g.nc[2];
            else if (z < 0 || z >= g.nc[2]) continue;
            for (int oy = 0; oy < g.noff[1]; oy++) {
                int y = cy + g.offs[1][oy];
                float sy = 0.f;
                if (FAST) wrap_cell(y, g.nc[1], g.box, sy);
                else if (g.periodic) y = (y + g.nc[1]) % g.nc[1];
                else if (y < 0 || y >= g.nc[1]) continue;
                for (int ox = 0; ox < g.noff[0]; ox++) {
                    int x = cx + g.offs[0][ox];
                    float sx = 0.f;
                    if (FAST) wrap_cell(x, g.nc[0], g.box, sx);
                    else if (g.periodic) x = (x + g.nc[0]) % g.nc[0];
                    else if (x < 0 || x >= g.nc[0]) continue;
                    const uint32_t c = ((uint32_t)z * g.nc[1] + y) * g.nc[0] + x;
                    const uint32_t q1 = cell_start[c + 1];
#pragma unroll 2
                    for (uint32_t q = cell_start[c]; q < q1; q++) {
                        const int32_t j = sorted[q];
                        const float4 b = pos_c[q];
                        if (j <= i) continue;
                        if (pair_hit<FAST>(a, b, g, sx, sy, sz)) {
                            if (WRITE) {
                                if (pairs)
                                    pairs[base + m] = make_int2(i, j);
                                else
                                    nbr[base + m] = j;
                            }
                            m++;
                        }
                    }
                }
            }
        }
        if (!WRITE) {
            count[i] = m;
        } else if (sort_here && !pairs) {
            // insertion sort of the row in place
            for (uint32_t u = 1; u < m; u++) {
                const int32_t v = nbr[base + u];
                uint32_t w = u;
                while (w > 0 && nbr[base + w - 1] > v) {
                    nbr[base + w] = nbr[base + w - 1];
                    w--;
                }
                nbr[base + w] = v;
            }
        }
    }
}

template <bool WRITE>
__global__ void pairs_kernel(const float4* __restrict__ pos_c, const int32_t* __restrict__ sorted,
                             const uint32_t* __restrict__ cell_start, int64_t n,
                             const __grid_constant__ Grid g, const int* __restrict__ outside,
                             uint32_t* count, const uint32_t* __restrict__ row_off, int32_t* nbr,
                             int2* pairs, int sort_here)
{
    if (g.fast && *outside == 0)
        pairs_rows<WRITE, true>(pos_c, sorted, cell_start, n, g, count, row_off, nbr, pairs, sort_here);
    else
        pairs_rows<WRITE, false>(pos_c, sorted, cell_start, n, g, count, row_off, nbr, pairs, sort_here);
}

// The same pairs from a half stencil, for callers that take the pairs in any
// order (with at least 3 cells per axis, so no cell is its own neighbour):
// node t (in cell order) pairs with the later nodes of its own cell and with
// the nodes of the 13 neighbour cells whose offset (dz, dy, dx) comes after
// (0, 0, 0) in lexicographic order.  Each pair is found once and written as
// (min id, max id).
template <bool WRITE, bool FAST>
__device__ __forceinline__ void half_rows(const float4* __restrict__ pos_c, const int32_t* __restrict__ sorted,
                                          const uint32_t* __restrict__ cell_start, int64_t n,
                                          const Grid& g, uint32_t* count,
                                          const uint32_t* __restrict__ row_off, int2* pairs)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = sorted[t];
        const float4 a = pos_c[t];
        const int cx = cell_coord(a.x, 0, g), cy = cell_coord(a.y, 1, g), cz = cell_coord(a.z, 2, g);
        uint32_t m = 0;
        const uint32_t base = WRITE ? row_off[i] : 0;
        for (int o = 0; o < 14; o++) {
            // o = 0: the own cell (later nodes only); o = 1..13: forward offsets
            const int k = o == 0 ? 13 : 13 + o;  // (dz+1)*9 + (dy+1)*3 + (dx+1)
            int z = cz + k / 9 - 1, y = cy + (k / 3) % 3 - 1, x = cx + k % 3 - 1;
            float sx = 0.f, sy = 0.f, sz = 0.f;
            if (g.periodic) {
                wrap_cell(z, g.nc[2], g.box, sz);
                wrap_cell(y, g.nc[1], g.box, sy);
                wrap_cell(x, g.nc[0], g.box, sx);
            } else if (z < 0 || z >= g.nc[2] || y < 0 || y >= g.nc[1] || x < 0 || x >= g.nc[0]) {
                continue;
            }
            const uint32_t c = ((uint32_t)z * g.nc[1] + y) * g.nc[0] + x;
            const uint32_t q1 = cell_start[c + 1];
#pragma unroll 2
            for (uint32_t q = o == 0 ? (uint32_t)t + 1 : cell_start[c]; q < q1; q++) {
                const float4 b = pos_c[q];
                if (pair_hit<FAST>(a, b, g, sx, sy, sz)) {
                    if (WRITE) {
                        const int32_t j = sorted[q];
                        pairs[base + m] = i < j ? make_int2(i, j) : make_int2(j, i);
                    }
                    m++;
                }
            }
        }
        if (!WRITE) count[i] = m;
    }
}

template <bool WRITE>
__global__ void pairs_half_kernel(const float4* __restrict__ pos_c, const int32_t* __restrict__ sorted,
                                  const uint32_t* __restrict__ cell_start, int64_t n,
                                  const __grid_constant__ Grid g, const int* __restrict__ outside,
                                  uint32_t* count, const uint32_t* __restrict__ row_off, int2* pairs)
{
    if (g.fast && *outside == 0)
        half_rows<WRITE, true>(pos_c, sorted, cell_start, n, g, count, row_off, pairs);
    else
        half_rows<WRITE, false>(pos_c, sorted, cell_start, n, g, count, row_off, pairs);
}

// One warp per row: the lanes write consecutive pairs (coalesced stores).
__global__ void expand_pairs_kernel(const uint32_t* row_off, const int32_t* nbr, int64_t n,
                                    int2* edges)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const uint32_t k1 = row_off[i + 1];
        for (uint32_t k = row_off[i] + lane; k < k1; k += 32) edges[k] = make_int2((int)i, nbr[k]);
    }
}

// ---- full rows in cell order (the MD rebuild)
// Nodes sorted by the Hilbert index of their cell (cells of the 10-bit curve
// grid: at most 1024 per axis), so each cell's nodes are one contiguous run
// and runs follow the curve; a node's row visits its 27 neighbour cells in
// curve order, so the row comes out ascending with no sort and no atomics.

__device__ __forceinline__ uint32_t cell_of(float4 p, const Grid& g)
{
    return ((uint32_t)cell_coord(p.z, 2, g) * g.nc[1] + cell_coord(p.y, 1, g)) * g.nc[0] +
           cell_coord(p.x, 0, g);
}

// keys[i] = curve index of node i's cell, vals[i] = i; *outside as in cell_keys.
__global__ void cell_curve_keys_kernel(const float4* pos, int64_t n, const __grid_constant__ Grid g,
                                       uint32_t* keys, int32_t* vals, int* outside)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        if (g.periodic && !(p.x >= 0.f && p.x < g.box && p.y >= 0.f && p.y < g.box && p.z >= 0.f &&
                            p.z < g.box))
            *outside = 1;
        keys[i] = hilbert10(cell_coord(p.x, 0, g), cell_coord(p.y, 1, g), cell_coord(p.z, 2, g));
        vals[i] = (int32_t)i;
    }
}

// span[c] = [first, end) of cell c's run in the sorted order (0, 0 if empty).
__global__ void cell_spans_kernel(const float4* __restrict__ pos_c, const uint32_t* __restrict__ keys,
                                  int64_t n, const __grid_constant__ Grid g, uint2* span)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t k = keys[t];
        const bool first = t == 0 || keys[t - 1] != k;
        const bool last = t == n - 1 || keys[t + 1] != k;
        if (first || last) {
            const uint32_t c = cell_of(pos_c[t], g);
            if (first) span[c].x = (uint32_t)t;
            if (last) span[c].y = (uint32_t)(t + 1);
        }
    }
}

// Per cell, its 27 neighbour cells (periodic, at least 3 per axis, so all
// distinct) in curve order: {run first, run end, image code}, the code 2 bits
// per axis (1: +box, 2: -box; the shift list_pair_shifted adds) and kOwnCell
// on the cell itself (whose run holds the node: the only one that needs a
// self test).  One warp
// per cell: lane k < 27 takes neighbour k, and a bitonic network over the
// warp's 32 (key, lane) pairs (5 padding keys at the top) puts them in order.
constexpr int kOwnCell = 64;

__global__ void cell_stencil_kernel(const __grid_constant__ Grid g, const uint2* __restrict__ span,
                                    int64_t ncell, int4* table)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < ncell; c += warps) {
        const int cx = (int)(c % g.nc[0]), cy = (int)((c / g.nc[0]) % g.nc[1]),
                  cz = (int)(c / ((int64_t)g.nc[0] * g.nc[1]));
        uint32_t key = 0xffffffffu;
        int4 ent = make_int4(0, 0, 0, 0);
        if (lane < 27) {
            int z = cz + lane / 9 - 1, y = cy + (lane / 3) % 3 - 1, x = cx + lane % 3 - 1;
            float sx, sy, sz;
            wrap_cell(z, g.nc[2], g.box, sz);
            wrap_cell(y, g.nc[1], g.box, sy);
            wrap_cell(x, g.nc[0], g.box, sx);
            const int code = (sx > 0.f ? 1 : sx < 0.f ? 2 : 0) | (sy > 0.f ? 4 : sy < 0.f ? 8 : 0) |
                             (sz > 0.f ? 16 : sz < 0.f ? 32 : 0) | (lane == 13 ? kOwnCell : 0);
            const uint2 sp = span[((int64_t)z * g.nc[1] + y) * g.nc[0] + x];
            key = hilbert10((uint32_t)x, (uint32_t)y, (uint32_t)z);
            ent = make_int4((int)sp.x, (int)sp.y, code, 0);
        }
        int src = lane;  // whose entry this lane holds after the network
#pragma unroll
        for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                const uint32_t ok = __shfl_xor_sync(0xffffffffu, key, stride);
                const int os = __shfl_xor_sync(0xffffffffu, src, stride);
                const bool up = (lane & size) == 0;
                const bool lower = (lane & stride) == 0;
                // keep the smaller key in the lower lane of an ascending pair
                const bool take = (up == lower) ? (ok < key) : (ok > key);
                if (take) {
                    key = ok;
                    src = os;
                }
            }
        }
        const int4 got = make_int4(__shfl_sync(0xffffffffu, ent.x, src), __shfl_sync(0xffffffffu, ent.y, src),
                                   __shfl_sync(0xffffffffu, ent.z, src), 0);
        if (lane < 27) table[c * 27 + lane] = got;
    }
}

__device__ __forceinline__ float image_shift(int code, float box)
{
    return code == 1 ? box : (code == 2 ? -box : 0.f);
}

// MODE kCount: deg[t] = row length.  kWrite: the row's columns from
// row_off[t], ascending.  kScratch: both in one pass, the columns into a
// fixed-capacity slot scratch[t * cap, +cap) (the count goes on past cap, so
// an overflowing row is known and its entries are not stored).
enum RowsMode { kCount = 0, kWrite = 1, kScratch = 2 };

template <int MODE, bool FAST>
__device__ __forceinline__ void cell_rows_body(const float4* __restrict__ pos_c, int64_t n, const Grid& g,
                                               const int4* __restrict__ table, uint32_t* deg,
                                               const uint32_t* __restrict__ row_off, int32_t* col,
                                               uint32_t cap)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = pos_c[t];
        const int4* st = table + (int64_t)cell_of(a, g) * 27;
        uint32_t m = 0;
        int32_t* out = MODE == kWrite ? col + row_off[t] : (MODE == kScratch ? col + t * (int64_t)cap : nullptr);
        // one run of candidates; SELF: the node's own run (skip q == t),
        // SHIFT: a run across the box boundary (FAST only: elsewhere the cell
        // decides no shift, and the rule's own test runs when !FAST)
        auto run = [&](auto self, auto shift, uint32_t q0, uint32_t q1, float sx, float sy, float sz) {
            constexpr bool SELF = decltype(self)::value, SHIFT = decltype(shift)::value;
#pragma unroll 4
            for (uint32_t q = q0; q < q1; q++) {
                const float4 b = pos_c[q];
                bool hit;
                if (!FAST)
                    hit = list_pair(a, b, g);
                else if (SHIFT)
                    hit = list_pair_shifted(a, b, sx, sy, sz, g.cut2);
                else
                    hit = list_pair_unshifted(a, b, g.cut2);
                if (SELF) hit = hit && q != (uint32_t)t;
                if (hit) {
                    if (MODE == kWrite || (MODE == kScratch && m < cap)) out[m] = (int32_t)q;
                    m++;
                }
            }
        };
        using T = std::true_type;
        using F = std::false_type;
        for (int k = 0; k < 27; k++) {
            const int4 e = st[k];
            const uint32_t q0 = (uint32_t)e.x, q1 = (uint32_t)e.y;
            if (e.z & kOwnCell) {
                run(T{}, F{}, q0, q1, 0.f, 0.f, 0.f);
            } else if (FAST && e.z != 0) {
                run(F{}, T{}, q0, q1, image_shift(e.z & 3, g.box), image_shift((e.z >> 2) & 3, g.box),
                    image_shift((e.z >> 4) & 3, g.box));
            } else {
                run(F{}, F{}, q0, q1, 0.f, 0.f, 0.f);
            }
        }
        if (MODE != kWrite) deg[t] = m;
    }
}

// Scratch rows (cap apart) packed into col at row_off: one warp per row.
__global__ void compact_rows_kernel(const int32_t* __restrict__ scratch, uint32_t cap,
                                    const uint32_t* __restrict__ row_off, int64_t n, int32_t* __restrict__ col)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < n; t += warps) {
        const uint32_t b = row_off[t], len = row_off[t + 1] - b;
        const int32_t* src = scratch + t * (int64_t)cap;
        for (uint32_t k = lane; k < len; k += 32) col[b + k] = src[k];
    }
}

// total[0] += sum of deg[0, n) in 64 bits (the row offsets are 32-bit: the
// caller refuses a list whose entries do not fit), and total[1] = max(total[1], the longest row).
__global__ void sum_u32_kernel(const uint32_t* __restrict__ deg, int64_t n, unsigned long long* total)
{
    unsigned long long w = 0, mx = 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        w += deg[t];
        mx = deg[t] > mx ? deg[t] : mx;
    }
    for (int off = 16; off > 0; off >>= 1) {
        w += __shfl_down_sync(0xffffffffu, w, off);
        const unsigned long long o = __shfl_down_sync(0xffffffffu, mx, off);
        mx = o > mx ? o : mx;
    }
    if ((threadIdx.x & 31) == 0) {
        if (w) atomicAdd(total, w);
        if (mx) atomicMax(total + 1, mx);
    }
}

template <int MODE>
__global__ void cell_rows_kernel(const float4* __restrict__ pos_c, int64_t n, const __grid_constant__ Grid g,
                                 const int* __restrict__ outside, const int4* __restrict__ table,
                                 uint32_t* deg, const uint32_t* __restrict__ row_off, int32_t* col,
                                 uint32_t cap)
{
    if (g.fast && *outside == 0)
        cell_rows_body<MODE, true>(pos_c, n, g, table, deg, row_off, col, cap);
    else
        cell_rows_body<MODE, false>(pos_c, n, g, table, deg, row_off, col, cap);
}

int grid_of(int64_t n)
{
    int64_t g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 8192 ? 8192 : g));
}

}  // namespace

// Builds the list; *d_edges is cudaMalloc'd, or cudaMallocAsync'd on s when
// stream_ordered (2 * *num_edges int32).
namespace {

// The cell grid of a list cutoff: cells at least as wide as the cutoff (so a
// partner is in the same or an adjacent cell), at most 1024 per axis and a
// few per node; a periodic axis of fewer than 3 cells becomes one cell.
cudaError_t make_grid(const float4* pos, int64_t n, float box, float cut2, Grid* out, cudaStream_t s)
{
    Grid g{};
    g.periodic = box > 0.0f;
    g.box = box;
    g.hb = 0.5f * box;
    g.cut2 = cut2;
    const double cut = std::sqrt((double)cut2) * 1.0001 + 1e-12;
    double lo[3] = {0, 0, 0}, ext[3] = {box, box, box};
    if (!g.periodic) {
        float flo[3], fhi[3];
        IRR_CUDA_TRY(bbox_minmax(pos, n, flo, fhi, s));
        for (int c = 0; c < 3; c++) {
            lo[c] = flo[c];
            ext[c] = (double)fhi[c] - (double)flo[c];
        }
    }
    for (int c = 0; c < 3; c++) {
        int k = (int)std::floor(ext[c] / cut);
        if (g.periodic && k < 3) k = 1;
        if (k < 1) k = 1;
        if (k > 1024) k = 1024;
        g.nc[c] = k;
    }
    // keep the cell count within a few cells per node (coarser cells stay valid)
    while ((double)g.nc[0] * g.nc[1] * g.nc[2] > 8.0 * (double)n + 64.0) {
        int a = (g.nc[0] >= g.nc[1] && g.nc[0] >= g.nc[2]) ? 0 : (g.nc[1] >= g.nc[2] ? 1 : 2);
        g.nc[a] = g.nc[a] / 2;
        if (g.periodic && g.nc[a] < 3) g.nc[a] = 1;
        if (g.nc[a] < 1) g.nc[a] = 1;
    }
    for (int c = 0; c < 3; c++) {
        g.org[c] = g.periodic ? 0.0 : lo[c];
        // slightly wider cells than ext/nc so the max coordinate maps inside
        // (clamped anyway); the layout never decides a pair, the rule does
        const double csz = ext[c] > 0 ? ext[c] / g.nc[c] : 1.0;
        g.inv[c] = 1.0 / csz;
        if (g.nc[c] >= 3) {
            g.offs[c][0] = -1; g.offs[c][1] = 0; g.offs[c][2] = 1; g.noff[c] = 3;
        } else if (g.nc[c] == 2) {
            g.offs[c][0] = 0; g.offs[c][1] = 1; g.noff[c] = 2;
            if (!g.periodic) { g.offs[c][0] = -1; g.offs[c][1] = 0; g.offs[c][2] = 1; g.noff[c] = 3; }
        } else {
            g.offs[c][0] = 0; g.noff[c] = 1;
        }
    }
    g.fast = g.periodic && g.nc[0] >= 5 && g.nc[1] >= 5 && g.nc[2] >= 5;
    *out = g;
    return cudaSuccess;
}

}  // namespace

cudaError_t build_neighbor_list(const float4* pos, int64_t n, float box, float cut2,
                                int2** d_edges, int64_t* num_edges, cudaStream_t s,
                                bool stream_ordered, bool sort_rows)
{
    *d_edges = nullptr;
    *num_edges = 0;
    if (n <= 1) return cudaSuccess;
    Grid g{};
    IRR_CUDA_TRY(make_grid(pos, n, box, cut2, &g, s));
    const int64_t ncell = (int64_t)g.nc[0] * g.nc[1] * g.nc[2];
    uint32_t *keys = nullptr, *keys_tmp = nullptr, *cell_start = nullptr, *cnt = nullptr;
    int32_t *sorted = nullptr, *vals_tmp = nullptr, *nbr = nullptr;
    IRR_CUDA_TRY(irr_malloc_async((void**)&keys, sizeof(uint32_t) * n, s));
    IRR_CUDA_TRY(irr_malloc_async((void**)&keys_tmp, sizeof(uint32_t) * n, s));
    IRR_CUDA_TRY(irr_malloc_async((void**)&sorted, sizeof(int32_t) * n, s));
    IRR_CUDA_TRY(irr_malloc_async((void**)&vals_tmp, sizeof(int32_t) * n, s));
    IRR_CUDA_TRY(irr_malloc_async((void**)&cell_start, sizeof(uint32_t) * (ncell + 1), s));
    // cnt[n + 1]: the flag that some position lies outside the box
    IRR_CUDA_TRY(irr_malloc_async((void**)&cnt, sizeof(uint32_t) * (n + 2), s));
    int* outside = reinterpret_cast<int*>(cnt + n + 1);
    IRR_CUDA_TRY(cudaMemsetAsync(cell_start, 0, sizeof(uint32_t) * (ncell + 1), s));
    IRR_CUDA_TRY(cudaMemsetAsync(outside, 0, sizeof(int), s));
    cell_keys_kernel<<<grid_of(n), 256, 0, s>>>(pos, n, g, keys, sorted, cell_start, outside);
    IRR_CUDA_TRY(cudaGetLastError());
    int bits = 1;
    while (bits < 32 && ((int64_t)1 << bits) < ncell) bits++;
    IRR_CUDA_TRY(radix_sort_pairs(keys, sorted, keys_tmp, vals_tmp, n, bits, s));
    IRR_CUDA_TRY(scan_exclusive_u32(cell_start, cell_start, ncell + 1, nullptr, s));
    float4* pos_c = nullptr;
    IRR_CUDA_TRY(irr_malloc_async((void**)&pos_c, sizeof(float4) * n, s));
    cell_order_kernel<<<grid_of(n), 256, 0, s>>>(pos, sorted, n, pos_c);
    IRR_CUDA_TRY(cudaGetLastError());
    // rows in any order are asked for: the half stencil, where the box allows it
    const bool half = !sort_rows && g.nc[0] >= 3 && g.nc[1] >= 3 && g.nc[2] >= 3;
    if (half)
        pairs_half_kernel<false><<<grid_of(n), 256, 0, s>>>(pos_c, sorted, cell_start, n, g, outside,
                                                            cnt, nullptr, nullptr);
    else
        pairs_kernel<false><<<grid_of(n), 256, 0, s>>>(pos_c, sorted, cell_start, n, g, outside, cnt,
                                                       nullptr, nullptr, nullptr, 0);
    IRR_CUDA_TRY(cudaGetLastError());
    IRR_CUDA_TRY(cudaMemsetAsync(cnt + n, 0, sizeof(uint32_t), s));
    uint32_t* d_total = keys_tmp;  // reuse as the total's slot
    IRR_CUDA_TRY(scan_exclusive_u32(cnt, cnt, n + 1, d_total, s));
    uint32_t total = 0;
    IRR_CUDA_TRY(cudaMemcpyAsync(&total, d_total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    IRR_CUDA_TRY(cudaStreamSynchronize(s));
    if ((int64_t)total > 0x7fffffffLL) {
        void* tmp[] = {keys, keys_tmp, sorted, vals_tmp, cell_start, cnt, pos_c};
        for (void* q : tmp) cudaFreeAsync(q, s);
        return cudaErrorInvalidValue;
    }
    int2* edges = nullptr;
    if (total > 0) {
        if (stream_ordered)
            IRR_CUDA_TRY(irr_malloc_async((void**)&edges, sizeof(int2) * total, s));
        else
            IRR_CUDA_TRY(cudaMalloc((void**)&edges, sizeof(int2) * total));
        if (sort_rows) {
            uint32_t longest = 0;
            IRR_CUDA_TRY(max_row_len(cnt, n, &longest, s));
            const int sort_here = longest > (uint32_t)kRowSortMax;
            IRR_CUDA_TRY(irr_malloc_async((void**)&nbr, sizeof(int32_t) * total, s));
            pairs_kernel<true><<<grid_of(n), 256, 0, s>>>(pos_c, sorted, cell_start, n, g, outside,
                                                          nullptr, cnt, nbr, nullptr, sort_here);
            IRR_CUDA_TRY(cudaGetLastError());
            if (!sort_here) IRR_CUDA_TRY(launch_row_sort(cnt, n, nbr, s));
            expand_pairs_kernel<<<grid_of(32 * n), 256, 0, s>>>(cnt, nbr, n, edges);
            IRR_CUDA_TRY(cudaGetLastError());
            IRR_CUDA_TRY(cudaFreeAsync(nbr, s));
        } else if (half) {
            pairs_half_kernel<true><<<grid_of(n), 256, 0, s>>>(pos_c, sorted, cell_start, n, g,
                                                               outside, nullptr, cnt, edges);
            IRR_CUDA_TRY(cudaGetLastError());
        } else {
            pairs_kernel<true><<<grid_of(n), 256, 0, s>>>(pos_c, sorted, cell_start, n, g, outside,
                                                          nullptr, cnt, nullptr, edges, 0);
            IRR_CUDA_TRY(cudaGetLastError());
        }
    }
    IRR_CUDA_TRY(cudaFreeAsync(keys, s));
    IRR_CUDA_TRY(cudaFreeAsync(keys_tmp, s));
    IRR_CUDA_TRY(cudaFreeAsync(sorted, s));
    IRR_CUDA_TRY(cudaFreeAsync(vals_tmp, s));
    IRR_CUDA_TRY(cudaFreeAsync(cell_start, s));
    IRR_CUDA_TRY(cudaFreeAsync(cnt, s));
    IRR_CUDA_TRY(cudaFreeAsync(pos_c, s));
    IRR_CUDA_TRY(cudaStreamSynchronize(s));
    *d_edges = edges;
    *num_edges = total;
    return cudaSuccess;
}

namespace {

// Stream-ordered temporaries freed on every return.
struct Temps {
    cudaStream_t s;
    std::vector<void*> p;
    template <typename T>
    cudaError_t get(T** out, size_t count)
    {
        *out = nullptr;
        const cudaError_t e = irr_malloc_async((void**)out, sizeof(T) * (count ? count : 1), s);
        if (e == cudaSuccess) p.push_back(*out);
        return e;
    }
    ~Temps()
    {
        for (void* q : p) cudaFreeAsync(q, s);
    }
};

}  // namespace

cudaError_t build_rows_by_cell(const float4* pos, int64_t n, float box, float cut2, PartitionOut* out,
                               int64_t* num_edges, uint32_t* longest, uint32_t cap_hint, cudaStream_t s)
{
    *out = PartitionOut{};
    *num_edges = 0;
    *longest = 0;
    if (n <= 1 || !(box > 0.0f) || n > 0x7fffffffLL) return cudaErrorNotSupported;
    Grid g{};
    IRR_CUDA_TRY(make_grid(pos, n, box, cut2, &g, s));  // periodic: host arithmetic only
    const int64_t ncell = (int64_t)g.nc[0] * g.nc[1] * g.nc[2];
    if (g.nc[0] < 3 || g.nc[1] < 3 || g.nc[2] < 3 || ncell > n) return cudaErrorNotSupported;
    Temps tmp{s, {}};
    uint32_t *keys = nullptr, *keys_tmp = nullptr;
    int32_t *vals_tmp = nullptr, *scratch = nullptr;
    float4* pos_c = nullptr;
    uint2* span = nullptr;
    int4* table = nullptr;
    unsigned long long* aux = nullptr;  // [0] the entry count, [1] the longest row, [2] the outside flag
    PartitionOut p;
    auto run = [&]() -> cudaError_t {
        IRR_CUDA_TRY(irr_malloc_async((void**)&p.perm, sizeof(int32_t) * n, s));
        IRR_CUDA_TRY(irr_malloc_async((void**)&p.row_off, sizeof(uint32_t) * (n + 1), s));
        IRR_CUDA_TRY(tmp.get(&keys, n));
        IRR_CUDA_TRY(tmp.get(&keys_tmp, n));
        IRR_CUDA_TRY(tmp.get(&vals_tmp, n));
        IRR_CUDA_TRY(tmp.get(&pos_c, n));
        IRR_CUDA_TRY(tmp.get(&span, ncell));
        IRR_CUDA_TRY(tmp.get(&table, ncell * 27));
        IRR_CUDA_TRY(tmp.get(&aux, 3));
        // one search pass into cap_hint slots per node when they fit in memory;
        // otherwise (and at the first build) a counting pass, then the writing one
        bool one_pass = false;
        if (cap_hint > 0 && cap_hint <= 4096) {
            one_pass = tmp.get(&scratch, (size_t)n * cap_hint) == cudaSuccess;
            if (!one_pass) cudaGetLastError();
        }
        IRR_CUDA_TRY(cudaMemsetAsync(span, 0, sizeof(uint2) * ncell, s));
        IRR_CUDA_TRY(cudaMemsetAsync(aux, 0, 3 * sizeof(unsigned long long), s));
        int* outside = reinterpret_cast<int*>(aux + 2);
        const int gn = grid_of(n);
        cell_curve_keys_kernel<<<gn, 256, 0, s>>>(pos, n, g, keys, p.perm, outside);
        IRR_CUDA_TRY(cudaGetLastError());
        IRR_CUDA_TRY(radix_sort_pairs(keys, p.perm, keys_tmp, vals_tmp, n, 30, s));
        cell_order_kernel<<<gn, 256, 0, s>>>(pos, p.perm, n, pos_c);
        cell_spans_kernel<<<gn, 256, 0, s>>>(pos_c, keys, n, g, span);
        cell_stencil_kernel<<<grid_of(32 * ncell), 256, 0, s>>>(g, span, ncell, table);
        if (one_pass)
            cell_rows_kernel<kScratch><<<gn, 256, 0, s>>>(pos_c, n, g, outside, table, p.row_off, nullptr,
                                                          scratch, cap_hint);
        else
            cell_rows_kernel<kCount><<<gn, 256, 0, s>>>(pos_c, n, g, outside, table, p.row_off, nullptr,
                                                        nullptr, 0);
        sum_u32_kernel<<<gn < 256 ? gn : 256, 256, 0, s>>>(p.row_off, n, aux);  // few atomics
        IRR_CUDA_TRY(cudaGetLastError());
        unsigned long long host_aux[2] = {0, 0};
        IRR_CUDA_TRY(cudaMemcpyAsync(host_aux, aux, sizeof(host_aux), cudaMemcpyDeviceToHost, s));
        IRR_CUDA_TRY(cudaStreamSynchronize(s));
        const unsigned long long total = host_aux[0];
        if (total > 0x7fffffffull) return cudaErrorInvalidValue;
        IRR_CUDA_TRY(cudaMemsetAsync(p.row_off + n, 0, sizeof(uint32_t), s));
        IRR_CUDA_TRY(scan_exclusive_u32(p.row_off, p.row_off, n + 1, nullptr, s));
        // + kColPad: bulk copies of an entry segment may read past the last one
        IRR_CUDA_TRY(irr_malloc_async((void**)&p.col, sizeof(int32_t) * (total + kColPad), s));
        IRR_CUDA_TRY(cudaMemsetAsync(p.col + total, 0, sizeof(int32_t) * kColPad, s));
        if (one_pass && host_aux[1] <= cap_hint)
            compact_rows_kernel<<<grid_of(32 * n), 256, 0, s>>>(scratch, cap_hint, p.row_off, n, p.col);
        else  // a row longer than the slots (or no scratch): search again, writing in place
            cell_rows_kernel<kWrite><<<gn, 256, 0, s>>>(pos_c, n, g, outside, table, nullptr, p.row_off,
                                                        p.col, 0);
        IRR_CUDA_TRY(cudaGetLastError());
        *num_edges = (int64_t)(total / 2);
        *longest = (uint32_t)host_aux[1];
        return cudaSuccess;
    };
    const cudaError_t e = run();
    if (e != cudaSuccess) {
        if (p.perm) cudaFreeAsync(p.perm, s);
        if (p.row_off) cudaFreeAsync(p.row_off, s);
        if (p.col) cudaFreeAsync(p.col, s);
        *num_edges = 0;
        *longest = 0;
        return e;
    }
    *out = p;
    return cudaSuccess;
}

}  // namespace irr

extern "C" {

int irr_neighbor_build(int device, void* stream, const void* pos, int pos_elm, int pos_on_device,
                       int64_t n, float box, float list_cut2, int32_t** d_edges,
                       int64_t* num_edges)
{
    irr::TraceRange trace_("irr_neighbor_build");
    if (!d_edges || !num_edges || n < 0 || (n > 0 && !pos)) return IRR_ERR_ARG;
    if (pos_elm != 12 && pos_elm != 16 && pos_elm != 24) return IRR_ERR_ARG;
    if (!(box >= 0.0f) || !(list_cut2 >= 0.0f) || !std::isfinite(box) || !std::isfinite(list_cut2))
        return IRR_ERR_ARG;
    if (n > 0x7fffffffLL) return IRR_ERR_CAPACITY;
    *d_edges = nullptr;
    *num_edges = 0;
    irr::DeviceGuard dev_guard(device);
    if (!dev_guard.ok()) return IRR_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    void* raw = nullptr;
    float4* p4 = nullptr;
    int rc = IRR_OK;
    cudaError_t e = cudaSuccess;
    const void* src = pos;
    if (n > 0 && !pos_on_device) {
        e = cudaMalloc(&raw, (size_t)n * pos_elm);
        if (e == cudaSuccess) e = cudaMemcpyAsync(raw, pos, (size_t)n * pos_elm, cudaMemcpyHostToDevice, s);
        src = raw;
    }
    if (e == cudaSuccess && n > 0) e = cudaMalloc((void**)&p4, sizeof(float4) * (size_t)n);
    if (e == cudaSuccess && n > 0) e = irr::launch_load_nodes(src, pos_elm, nullptr, n, p4, s);
    int2* edges = nullptr;
    int64_t cnt = 0;
    if (e == cudaSuccess) e = irr::build_neighbor_list(p4, n, box, list_cut2, &edges, &cnt, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        rc = (e == cudaErrorMemoryAllocation) ? IRR_ERR_NOMEM : (e == cudaErrorInvalidValue ? IRR_ERR_CAPACITY : IRR_ERR_CUDA);
        if (edges) cudaFree(edges);
        edges = nullptr;
        cnt = 0;
    }
    if (raw) cudaFree(raw);
    if (p4) cudaFree(p4);
    *d_edges = (int32_t*)edges;
    *num_edges = cnt;
    return rc;
}

int irr_device_free(int device, void* d_ptr)
{
    if (!d_ptr) return IRR_OK;
    irr::DeviceGuard dev_guard(device);
    if (!dev_guard.ok() || cudaFree(d_ptr) != cudaSuccess) {
        cudaGetLastError();
        return IRR_ERR_CUDA;
    }
    return IRR_OK;
}

}  // extern "C"
