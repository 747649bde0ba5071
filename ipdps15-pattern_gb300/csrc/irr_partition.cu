// irr_partition.cu -- the GPU partitioner and the node/result data movers.
//
// The reference partitions on the host: a randomized quickselect recursive
// bisection of the coordinates into shared-memory-sized parts
// (moldyn/irregular/partitioner.cpp:348-437), then an O(E) pass that copies
// every edge into the part of each endpoint with std::vector push_back
// (partitioner.cpp:142-297), then part_index (:490-499).  Here the whole pass
// runs on the GPU and is deterministic:
//   1. a curve key per node: each axis quantised to 10 bits in the bounding
//      box frame (float ops, each rounded), then the cell's Hilbert index
//      (default) or Morton index (bits interleaved);
//   2. stable LSD radix sort of (key, node) -> perm[new] = old, inv[old] = new;
//   3. every half edge (i, j) at list position t becomes the directed entries
//      (inv[i] <- inv[j]) and (inv[j] <- inv[i]), laid out in (row, col)
//      order: a degree count + scan gives the row offsets, the entries are
//      filled at per-row cursors and each row is sorted by one warp, in
//      registers (rows up to 256 entries) or in shared memory (up to
//      kRowSortMax); a graph with a longer row is put in order by stable radix
//      sorts by column, then by row.
// Node blocks are then consecutive ranges of rows.  Every output is an
// integer function of the inputs, reproduced bit for bit by the CPU oracle.
// 4. Optionally the sliced layout (struct Sliced): the same entries regrouped
//    so that one warp reads one contiguous line per step.
#include <algorithm>
#include <mutex>

#include "irr_internal.cuh"

namespace irr {

static __device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ------------------------------------------------------------------ scan
constexpr int kScanItems = kScanBlock / kScanThreads;

__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(const uint32_t* in,
                                                                   uint32_t* out, int64_t n,
                                                                   uint32_t* block_sums)
{
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)tid * kScanItems;
    uint32_t v[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        sum += v[k];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < kScanThreads / 32 ? warp_tot[lane] : 0u;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, off);
            if (lane >= off) t += y;
        }
        if (lane < kScanThreads / 32) warp_tot[lane] = t;  // inclusive
    }
    __syncthreads();
    uint32_t run = incl - sum + (warp > 0 ? warp_tot[warp - 1] : 0u);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (tid == kScanThreads - 1) block_sums[blockIdx.x] = warp_tot[kScanThreads / 32 - 1];
}

__global__ void add_offsets_kernel(uint32_t* out, int64_t n, const uint32_t* block_off)
{
    const uint32_t add = block_off[blockIdx.x];
    const int64_t base = (int64_t)blockIdx.x * kScanBlock;
    for (int k = threadIdx.x; k < kScanBlock; k += blockDim.x)
        if (base + k < n) out[base + k] += add;
}

static __global__ void copy_u32_kernel(const uint32_t* src, uint32_t* dst) { *dst = *src; }

// ------------------------------------------------------------ radix sort
constexpr int kSortRounds = kSortTile / kSortThreads;  // a tile's items, in order
constexpr int kSortWarps = kSortThreads / 32;

__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const uint32_t* keys, int64_t n,
                                                                  int shift, uint32_t* hist,
                                                                  int64_t ntiles)
{
    __shared__ uint32_t cnt[256];
    const int tid = threadIdx.x;
    cnt[tid] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; r++) {
        const int64_t i = base + r * kSortThreads + tid;
        const bool v = i < n;
        const uint32_t d = v ? (keys[i] >> shift) & 255u : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (v && (peers & lanemask_lt()) == 0) atomicAdd(&cnt[d], (uint32_t)__popc(peers));
    }
    __syncthreads();
    hist[(int64_t)tid * ntiles + blockIdx.x] = cnt[tid];
}

// Stable scatter: items of a tile keep their index order within each digit.
// Round r covers tile items [r*256, r*256+256): item k goes to thread k.
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const uint32_t* kin, const int32_t* vin, uint32_t* kout, int32_t* vout, int64_t n, int shift,
    const uint32_t* offs, int64_t ntiles)
{
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[kSortWarps][256];
    const int tid = threadIdx.x, warp = tid >> 5;
    base[tid] = offs[(int64_t)tid * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kSortWarps; w++) wcnt[w][tid] = 0;
    __syncthreads();
    const int64_t tile0 = (int64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; r++) {
        const int64_t i = tile0 + r * kSortThreads + tid;
        const bool v = i < n;
        const uint32_t key = v ? kin[i] : 0u;
        const int32_t val = v ? vin[i] : 0;
        const uint32_t d = v ? (key >> shift) & 255u : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t below = peers & lanemask_lt();
        if (v && below == 0) wcnt[warp][d] = (uint32_t)__popc(peers);
        __syncthreads();
        // thread t owns digit t: exclusive prefix over warps, round total
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; w++) {
            const uint32_t c = wcnt[w][tid];
            wcnt[w][tid] = run;
            run += c;
        }
        __syncthreads();
        if (v) {
            const uint32_t dst = base[d] + wcnt[warp][d] + (uint32_t)__popc(below);
            kout[dst] = key;
            vout[dst] = val;
        }
        __syncthreads();
        base[tid] += run;
#pragma unroll
        for (int w = 0; w < kSortWarps; w++) wcnt[w][tid] = 0;
        __syncthreads();
    }
}

// ------------------------------------------------------------ row sort
// Each row of a CSR (row_off[n + 1], col) sorted ascending, one warp per row,
// by a bitonic network over the row padded to a power of two.  Rows of up to
// 256 entries stay in registers (entry k at lane k % 32, slot k / 32):
// exchanges across lanes are shuffles, within a lane min/max pairs.  Longer
// rows, up to kRowSortMax entries, go through a shared-memory buffer.
constexpr int kRowSortWarps = 8;

template <int E>
__device__ __forceinline__ void sort_row_in_registers(int32_t* col, uint32_t beg, uint32_t len,
                                                      int lane)
{
    int32_t v[E];
#pragma unroll
    for (int r = 0; r < E; r++) {
        const uint32_t k = (uint32_t)(r * 32 + lane);
        v[r] = k < len ? col[beg + k] : 0x7fffffff;
    }
#pragma unroll
    for (int size = 2; size <= 32 * E; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= 32) {  // partner in the same lane, slot r ^ (stride / 32)
#pragma unroll
                for (int r = 0; r < E; r++) {
                    const int r2 = r ^ (stride / 32);
                    if (r2 < r) continue;
                    const bool up = ((r * 32) & size) == 0;  // size >= 64: the lane bits do not reach it
                    const int32_t lo = min(v[r], v[r2]), hi = max(v[r], v[r2]);
                    v[r] = up ? lo : hi;
                    v[r2] = up ? hi : lo;
                }
            } else {
#pragma unroll
                for (int r = 0; r < E; r++) {
                    const int32_t o = __shfl_xor_sync(0xffffffffu, v[r], stride);
                    const bool up = ((r * 32 + lane) & size) == 0;
                    const bool lower = (lane & stride) == 0;
                    v[r] = up == lower ? min(v[r], o) : max(v[r], o);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < E; r++) {
        const uint32_t k = (uint32_t)(r * 32 + lane);
        if (k < len) col[beg + k] = v[r];
    }
}

__global__ void __launch_bounds__(kRowSortWarps * 32) row_sort_kernel(const uint32_t* __restrict__ row_off,
                                                                     int64_t n, int32_t* col)
{
    __shared__ int32_t buf[kRowSortWarps][kRowSortMax];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    int32_t* b = buf[warp];
    for (int64_t r = (int64_t)blockIdx.x * kRowSortWarps + warp; r < n;
         r += (int64_t)gridDim.x * kRowSortWarps) {
        const uint32_t beg = row_off[r];
        const uint32_t len = row_off[r + 1] - beg;
        if (len < 2) continue;
        if (len <= 32) {
            sort_row_in_registers<1>(col, beg, len, lane);
            continue;
        }
        if (len <= 64) {
            sort_row_in_registers<2>(col, beg, len, lane);
            continue;
        }
        if (len <= 128) {
            sort_row_in_registers<4>(col, beg, len, lane);
            continue;
        }
        if (len <= 256) {
            sort_row_in_registers<8>(col, beg, len, lane);
            continue;
        }
        uint32_t P = 2;
        while (P < len) P <<= 1;  // len <= kRowSortMax, so P <= kRowSortMax
        for (uint32_t k = lane; k < P; k += 32) b[k] = k < len ? col[beg + k] : 0x7fffffff;
        __syncwarp();
        for (uint32_t size = 2; size <= P; size <<= 1) {
            for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                for (uint32_t k = lane; k < P; k += 32) {
                    const uint32_t o = k ^ stride;
                    if (o > k) {
                        const int32_t x = b[k], y = b[o];
                        if ((x > y) == ((k & size) == 0)) {
                            b[k] = y;
                            b[o] = x;
                        }
                    }
                }
                __syncwarp();
            }
        }
        for (uint32_t k = lane; k < len; k += 32) col[beg + k] = b[k];
        __syncwarp();
    }
}

// *out = max over rows of row_off[r + 1] - row_off[r] (out must start at 0)
__global__ void max_row_len_kernel(const uint32_t* __restrict__ row_off, int64_t n, uint32_t* out)
{
    uint32_t m = 0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
         r += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t len = row_off[r + 1] - row_off[r];
        m = len > m ? len : m;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const uint32_t o = __shfl_xor_sync(0xffffffffu, m, off);
        m = o > m ? o : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// *out = max of deg[0, n) (out must start at 0)
__global__ void max_u32_kernel(const uint32_t* __restrict__ a, int64_t n, uint32_t* out)
{
    uint32_t m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        m = a[i] > m ? a[i] : m;
    for (int off = 16; off > 0; off >>= 1) {
        const uint32_t o = __shfl_xor_sync(0xffffffffu, m, off);
        m = o > m ? o : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

namespace {

// --------------------------------------------------------------- bbox
__global__ void bbox_partial_kernel(const float4* pos, int64_t n, float* part)
{
    __shared__ float red[6][256];
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        mn[0] = fminf(mn[0], p.x);
        mn[1] = fminf(mn[1], p.y);
        mn[2] = fminf(mn[2], p.z);
        mx[0] = fmaxf(mx[0], p.x);
        mx[1] = fmaxf(mx[1], p.y);
        mx[2] = fmaxf(mx[2], p.z);
    }
    for (int c = 0; c < 3; c++) {
        red[c][threadIdx.x] = mn[c];
        red[3 + c][threadIdx.x] = mx[c];
    }
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int c = 0; c < 3; c++) {
                red[c][threadIdx.x] = fminf(red[c][threadIdx.x], red[c][threadIdx.x + s]);
                red[3 + c][threadIdx.x] =
                    fmaxf(red[3 + c][threadIdx.x], red[3 + c][threadIdx.x + s]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = red[threadIdx.x][0];
}

// One warp: lanes take the blocks' partials in turn, then a shuffle reduction.
__global__ void bbox_final_kernel(const float* part, int nparts, float* out)
{
    const int lane = threadIdx.x & 31;
    float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int b = lane; b < nparts; b += 32)
        for (int c = 0; c < 3; c++) {
            v[c] = fminf(v[c], part[b * 6 + c]);
            v[3 + c] = fmaxf(v[3 + c], part[b * 6 + 3 + c]);
        }
    for (int off = 16; off > 0; off >>= 1)
        for (int c = 0; c < 3; c++) {
            v[c] = fminf(v[c], __shfl_xor_sync(0xffffffffu, v[c], off));
            v[3 + c] = fmaxf(v[3 + c], __shfl_xor_sync(0xffffffffu, v[3 + c], off));
        }
    if (lane == 0)
        for (int c = 0; c < 6; c++) out[c] = v[c];
}

// ------------------------------------------------------------- morton
__device__ __forceinline__ uint32_t quant10(float x, float lo, float scale)
{
    float t = __fsub_rn(x, lo);
    t = __fmul_rn(t, scale);
    if (!(t > 0.0f)) return 0u;
    if (t >= 1023.0f) return 1023u;
    return __float2uint_rz(t);
}

// Curve key of each node (curve 0: Hilbert, 1: Morton) on the 10-bit grid.
__global__ void curve_key_kernel(const float4* pos, int64_t n, float3 lo, float3 scale, int curve,
                                 uint32_t* keys, int32_t* vals)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        const uint32_t qx = quant10(p.x, lo.x, scale.x), qy = quant10(p.y, lo.y, scale.y),
                       qz = quant10(p.z, lo.z, scale.z);
        keys[i] = curve == 0 ? hilbert10(qx, qy, qz)
                             : (spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2));
        vals[i] = (int32_t)i;
    }
}

__global__ void iota_kernel(int32_t* a, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        a[i] = (int32_t)i;
}

__global__ void invert_kernel(const int32_t* perm, int64_t n, int32_t* inv)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        inv[perm[k]] = (int32_t)k;
}

__global__ void entries_kernel(const int2* edges, int64_t e, const int32_t* inv, uint32_t* rows,
                               int32_t* cols, uint32_t* deg)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < e;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int2 ed = edges[t];
        const int32_t a = inv[ed.x], b = inv[ed.y];
        rows[2 * t] = (uint32_t)a;
        cols[2 * t] = b;
        rows[2 * t + 1] = (uint32_t)b;
        cols[2 * t + 1] = a;
        atomicAdd(deg + a, 1u);
        atomicAdd(deg + b, 1u);
    }
}

// Degrees of the directed entries (both endpoints of every half edge).
// Adds 1 to ctr[key] for every lane of the warp with valid == true, one
// atomic per distinct key (lanes of a warp often share a row: the edges of a
// sorted list, or of one node's neighbour search); returns the lane's own
// slot, the counter's value before it plus its rank among the key's lanes.
// All 32 lanes must call it together.
__device__ __forceinline__ uint32_t add_grouped(uint32_t* ctr, int32_t key, bool valid)
{
    const uint32_t peers = __match_any_sync(0xffffffffu, valid ? key : -1);
    const uint32_t rank = (uint32_t)__popc(peers & lanemask_lt());
    uint32_t base = 0;
    if (valid && rank == 0) base = atomicAdd(ctr + key, (uint32_t)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, __ffs(peers) - 1);
    return base + rank;
}

// Whole warps walk the edges (t = warp start + lane), so every lane takes
// part in the grouped adds.
__global__ void degree_kernel(const int2* edges, int64_t e, const int32_t* inv, uint32_t* deg)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); t0 < e; t0 += stride) {
        const int64_t t = t0 + (threadIdx.x & 31);
        const bool v = t < e;
        const int2 ed = v ? edges[t] : make_int2(0, 0);
        const int32_t a = v ? inv[ed.x] : 0, b = v ? inv[ed.y] : 0;
        add_grouped(deg, a, v);
        add_grouped(deg, b, v);
    }
}

// Directed entries into their rows at per-row cursors (order within a row
// arbitrary until the row sort).
__global__ void fill_rows_kernel(const int2* edges, int64_t e, const int32_t* inv,
                                 uint32_t* cursor, int32_t* col)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); t0 < e; t0 += stride) {
        const int64_t t = t0 + (threadIdx.x & 31);
        const bool v = t < e;
        const int2 ed = v ? edges[t] : make_int2(0, 0);
        const int32_t a = v ? inv[ed.x] : 0, b = v ? inv[ed.y] : 0;
        const uint32_t sa = add_grouped(cursor, a, v);
        const uint32_t sb = add_grouped(cursor, b, v);
        if (v) {
            col[sa] = b;
            col[sb] = a;
        }
    }
}

// --------------------------------------------------------- data movers
__global__ void load_nodes_kernel(const char* raw, int elm, const int32_t* perm, int64_t n,
                                  float4* dst)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t src = perm ? perm[k] : k;
        float4 p;
        if (elm == 24) {
            const double* d = reinterpret_cast<const double*>(raw + src * 24);
            p = make_float4((float)d[0], (float)d[1], (float)d[2], 0.f);
        } else if (elm == 16) {
            p = reinterpret_cast<const float4*>(raw)[src];
            p.w = 0.f;
        } else {
            const float* f = reinterpret_cast<const float*>(raw + src * 12);
            p = make_float4(f[0], f[1], f[2], 0.f);
        }
        dst[k] = p;
    }
}

// Node records read in order -- from page-locked host memory the device
// addresses directly, where the link wants contiguous reads -- and scattered
// into execution order on the device: dst[inv ? inv[i] : i] = record i.
// vec12: 12-byte records at a 16-byte aligned base.  A block moves tiles of
// kMoveThreads * 4 records (3 * kMoveThreads 16-byte words): the words are
// loaded with consecutive threads on consecutive words (each warp instruction
// one contiguous 512-byte run: what the host link wants), then each thread
// takes its four records from shared memory.
constexpr int kMoveThreads = 256;

__global__ void __launch_bounds__(kMoveThreads) load_nodes_scatter_kernel(
    const char* __restrict__ rec, int elm, int vec12, const int32_t* __restrict__ inv, int64_t n,
    float4* __restrict__ dst)
{
    __shared__ float4 tile[3 * kMoveThreads];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t head = 0;  // records moved in whole tiles
    if (vec12) {
        constexpr int64_t kTile = 4 * kMoveThreads;
        head = n / kTile * kTile;
        const float4* w = reinterpret_cast<const float4*>(rec);
        for (int64_t t0 = (int64_t)blockIdx.x * kTile; t0 < head; t0 += (int64_t)gridDim.x * kTile) {
            const float4* src = w + t0 / 4 * 3;
#pragma unroll
            for (int k = 0; k < 3; k++) tile[k * kMoveThreads + threadIdx.x] = src[k * kMoveThreads + threadIdx.x];
            __syncthreads();
            const float4 a = tile[3 * threadIdx.x], b = tile[3 * threadIdx.x + 1], c = tile[3 * threadIdx.x + 2];
            __syncthreads();
            const int64_t i = t0 + 4 * threadIdx.x;
            dst[inv ? inv[i] : i] = make_float4(a.x, a.y, a.z, 0.f);
            dst[inv ? inv[i + 1] : i + 1] = make_float4(a.w, b.x, b.y, 0.f);
            dst[inv ? inv[i + 2] : i + 2] = make_float4(b.z, b.w, c.x, 0.f);
            dst[inv ? inv[i + 3] : i + 3] = make_float4(c.y, c.z, c.w, 0.f);
        }
    }
    for (int64_t i = head + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float4 p;
        if (elm == 24) {
            const double* d = reinterpret_cast<const double*>(rec + i * 24);
            p = make_float4((float)d[0], (float)d[1], (float)d[2], 0.f);
        } else if (elm == 16) {
            p = reinterpret_cast<const float4*>(rec)[i];
            p.w = 0.f;
        } else {
            const float* f = reinterpret_cast<const float*>(rec + i * 12);
            p = make_float4(f[0], f[1], f[2], 0.f);
        }
        dst[inv ? inv[i] : i] = p;
    }
}

// Results in the caller's order: out[i] = force[inv ? inv[i] : i], written in
// order (device staging or page-locked host memory).  vec12: 12-byte records
// at a 16-byte aligned base, packed four per thread into shared memory and
// stored in tiles with consecutive threads on consecutive 16-byte words.
__global__ void __launch_bounds__(kMoveThreads) store_result_kernel(
    const float4* force, const int32_t* inv, int64_t n, int elm, int vec12, char* out)
{
    __shared__ float4 tile[3 * kMoveThreads];
    int64_t head = 0;
    if (vec12) {
        constexpr int64_t kTile = 4 * kMoveThreads;
        head = n / kTile * kTile;
        float4* w = reinterpret_cast<float4*>(out);
        for (int64_t t0 = (int64_t)blockIdx.x * kTile; t0 < head; t0 += (int64_t)gridDim.x * kTile) {
            const int64_t i = t0 + 4 * threadIdx.x;
            const float4 f0 = force[inv ? inv[i] : i], f1 = force[inv ? inv[i + 1] : i + 1];
            const float4 f2 = force[inv ? inv[i + 2] : i + 2], f3 = force[inv ? inv[i + 3] : i + 3];
            tile[3 * threadIdx.x] = make_float4(f0.x, f0.y, f0.z, f1.x);
            tile[3 * threadIdx.x + 1] = make_float4(f1.y, f1.z, f2.x, f2.y);
            tile[3 * threadIdx.x + 2] = make_float4(f2.z, f3.x, f3.y, f3.z);
            __syncthreads();
            float4* dstw = w + t0 / 4 * 3;
#pragma unroll
            for (int k = 0; k < 3; k++) dstw[k * kMoveThreads + threadIdx.x] = tile[k * kMoveThreads + threadIdx.x];
            __syncthreads();
        }
    }
    for (int64_t i = head + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float4 f = force[inv ? inv[i] : i];
        if (elm == 24) {
            double* d = reinterpret_cast<double*>(out + i * 24);
            d[0] = f.x;
            d[1] = f.y;
            d[2] = f.z;
        } else if (elm == 16) {
            reinterpret_cast<float4*>(out)[i] = make_float4(f.x, f.y, f.z, 0.f);
        } else {
            float* o = reinterpret_cast<float*>(out + i * 12);
            o[0] = f.x;
            o[1] = f.y;
            o[2] = f.z;
        }
    }
}

__global__ void validate_edges_kernel(const int2* edges, int64_t e, int64_t n, int* status)
{
    bool bad = false;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < e;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int2 ed = edges[t];
        bad |= ed.x < 0 || ed.y < 0 || ed.x >= n || ed.y >= n;
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, kStatusBadIndex);
}

int grid_for(int64_t n, int threads = 256)
{
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > 8192) g = 8192;
    return (int)g;
}

template <class T>
cudaError_t alloc_async(T** p, int64_t count, cudaStream_t s)
{
    return irr_malloc_async(p, sizeof(T) * (size_t)(count > 0 ? count : 1), s);
}

// ------------------------------------------------------- sliced layout
// words[q] = 64 * ceil(longest row of slice q / 2G); *total += words[q] (64-bit,
// so an overflowing layout is seen by the host before the 32-bit scan is used).
// Whole warps walk the slices, so the total is summed over the warp first
// (one atomic per warp instead of one per slice on a single address).
__global__ void slice_words_kernel(const uint32_t* row_off, int64_t n, int G, int64_t slices,
                                   uint32_t* words, unsigned long long* total)
{
    const int R = 32 / G;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); q0 < slices; q0 += stride) {
        const int64_t q = q0 + (threadIdx.x & 31);
        unsigned long long w = 0;
        if (q < slices) {
            uint32_t longest = 0;
            const int64_t r0 = q * R;
            const int64_t r1 = r0 + R < n ? r0 + R : n;
            for (int64_t r = r0; r < r1; r++) {
                const uint32_t len = row_off[r + 1] - row_off[r];
                longest = len > longest ? len : longest;
            }
            w = 64ull * ((longest + 2ull * G - 1) / (2ull * G));
            words[q] = (uint32_t)w;
        }
        for (int off = 16; off > 0; off >>= 1) w += __shfl_xor_sync(0xffffffffu, w, off);
        if ((threadIdx.x & 31) == 0 && w) atomicAdd(total, w);
    }
}

// One warp per slice, lane i*G + l serving row i of the slice: per step t it
// writes the pair (entry 2Gt + l, entry 2Gt + G + l) of its row as the int2 at
// word 64t + 2*lane, so each step is one contiguous 256-byte store (G is a
// power of two: lg = log2 G).  A padding word holds the row's own id (0 for a
// row past n), so the kernel's gathers need no predicate: a padded slot reads
// its own position, d = 0, and is masked to 0.
__global__ void slice_fill_kernel(const uint32_t* row_off, const int32_t* col, int64_t n, int lg,
                                  int64_t slices, const uint32_t* slice_off, int32_t* out)
{
    const int G = 1 << lg;
    const int lane = threadIdx.x & 31;
    const int i = lane >> lg, l = lane & (G - 1);
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < slices; q += warps) {
        const int64_t r = (q << (5 - lg)) + i;
        const uint32_t o = slice_off[q];
        const uint32_t steps = (slice_off[q + 1] - o) >> 6;
        const uint32_t beg = r < n ? row_off[r] : 0u;
        const uint32_t len = r < n ? row_off[r + 1] - beg : 0u;
        const int32_t pad = r < n ? (int32_t)r : 0;
        int2* line = reinterpret_cast<int2*>(out + o) + lane;
        for (uint32_t t = 0; t < steps; t++) {
            const uint32_t k0 = (t << (lg + 1)) + l, k1 = k0 + G;
            line[32 * t] = make_int2(k0 < len ? col[beg + k0] : pad, k1 < len ? col[beg + k1] : pad);
        }
    }
}

}  // namespace

cudaError_t scan_exclusive_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* d_total,
                               cudaStream_t s)
{
    if (n <= 0) {
        if (d_total) IRR_CUDA_TRY(cudaMemsetAsync(d_total, 0, sizeof(uint32_t), s));
        return cudaSuccess;
    }
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    uint32_t* sums = nullptr;
    IRR_CUDA_TRY(alloc_async(&sums, nb, s));
    scan_blocks_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, sums);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) {
        if (nb == 1) {
            if (d_total) copy_u32_kernel<<<1, 1, 0, s>>>(sums, d_total);
        } else {
            err = scan_exclusive_u32(sums, sums, nb, d_total, s);
            if (err == cudaSuccess)
                add_offsets_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(out, n, sums);
        }
        if (err == cudaSuccess) err = cudaGetLastError();
    }
    cudaError_t ferr = cudaFreeAsync(sums, s);
    return err != cudaSuccess ? err : ferr;
}

cudaError_t radix_sort_pairs(uint32_t* keys, int32_t* vals, uint32_t* keys_tmp,
                             int32_t* vals_tmp, int64_t n, int key_bits, cudaStream_t s)
{
    if (n <= 1 || key_bits <= 0) return cudaSuccess;
    if (n > 0xffffffffLL) return cudaErrorInvalidValue;
    const int64_t ntiles = (n + kSortTile - 1) / kSortTile;
    uint32_t* hist = nullptr;
    IRR_CUDA_TRY(alloc_async(&hist, 256 * ntiles, s));
    uint32_t *ka = keys, *kb = keys_tmp;
    int32_t *va = vals, *vb = vals_tmp;
    cudaError_t err = cudaSuccess;
    int passes = 0;
    for (int shift = 0; shift < key_bits && err == cudaSuccess; shift += 8, passes++) {
        radix_hist_kernel<<<(unsigned)ntiles, kSortThreads, 0, s>>>(ka, n, shift, hist, ntiles);
        err = cudaGetLastError();
        if (err == cudaSuccess) err = scan_exclusive_u32(hist, hist, 256 * ntiles, nullptr, s);
        if (err == cudaSuccess) {
            radix_scatter_kernel<<<(unsigned)ntiles, kSortThreads, 0, s>>>(ka, va, kb, vb, n, shift,
                                                                          hist, ntiles);
            err = cudaGetLastError();
        }
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (err == cudaSuccess && (passes & 1)) {
        err = cudaMemcpyAsync(keys, ka, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(vals, va, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    }
    cudaError_t ferr = cudaFreeAsync(hist, s);
    return err != cudaSuccess ? err : ferr;
}

cudaError_t bbox_minmax(const float4* pos, int64_t n, float lo[3], float hi[3], cudaStream_t s)
{
    for (int c = 0; c < 3; c++) {
        lo[c] = 0.f;
        hi[c] = 0.f;
    }
    if (n <= 0) return cudaSuccess;
    const int nparts = (int)std::min<int64_t>((n + 255) / 256, 1024);
    float* part = nullptr;
    IRR_CUDA_TRY(alloc_async(&part, 6 * (int64_t)nparts + 6, s));
    bbox_partial_kernel<<<nparts, 256, 0, s>>>(pos, n, part);
    bbox_final_kernel<<<1, 32, 0, s>>>(part, nparts, part + 6 * nparts);
    float h[6];
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(h, part + 6 * nparts, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    cudaError_t ferr = cudaFreeAsync(part, s);
    if (err != cudaSuccess) return err;
    for (int c = 0; c < 3; c++) {
        lo[c] = h[c];
        hi[c] = h[3 + c];
    }
    return ferr;
}

cudaError_t bbox_frame(const float4* pos, int64_t n, float lo[3], float scale[3], cudaStream_t s)
{
    float hi[3];
    IRR_CUDA_TRY(bbox_minmax(pos, n, lo, hi, s));
    for (int c = 0; c < 3; c++) {
        const float ext = hi[c] - lo[c];
        scale[c] = ext > 0.0f ? 1024.0f / ext : 0.0f;
    }
    return cudaSuccess;
}

cudaError_t launch_row_sort(const uint32_t* row_off, int64_t n, int32_t* col, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + kRowSortWarps - 1) / kRowSortWarps;
    if (blocks > 65536) blocks = 65536;
    row_sort_kernel<<<(unsigned)blocks, kRowSortWarps * 32, 0, s>>>(row_off, n, col);
    return cudaGetLastError();
}

cudaError_t max_row_len(const uint32_t* row_off, int64_t n, uint32_t* result, cudaStream_t s)
{
    *result = 0;
    if (n <= 0) return cudaSuccess;
    uint32_t* d_max = nullptr;
    IRR_CUDA_TRY(alloc_async(&d_max, 1, s));
    IRR_CUDA_TRY(cudaMemsetAsync(d_max, 0, sizeof(uint32_t), s));
    max_row_len_kernel<<<grid_for(n), 256, 0, s>>>(row_off, n, d_max);
    IRR_CUDA_TRY(cudaGetLastError());
    IRR_CUDA_TRY(cudaMemcpyAsync(result, d_max, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    IRR_CUDA_TRY(cudaFreeAsync(d_max, s));
    return cudaStreamSynchronize(s);
}

cudaError_t build_partition(const float4* pos_user, int64_t n, const int2* edges, int64_t e,
                            int reorder, PartitionOut* out, cudaStream_t s, int curve)
{
    if (n < 0 || e < 0 || n > 0x7fffffffLL || 2 * e > 0xffffffffLL) return cudaErrorInvalidValue;
    *out = PartitionOut{};
    IRR_CUDA_TRY(alloc_async(&out->perm, n, s));
    IRR_CUDA_TRY(alloc_async(&out->inv, n, s));
    IRR_CUDA_TRY(alloc_async(&out->row_off, n + 1, s));
    // + kColPad: bulk copies of an entry segment are widened to 16-byte
    // boundaries and may read up to 3 entries past the last one
    IRR_CUDA_TRY(alloc_async(&out->col, 2 * e + kColPad, s));
    IRR_CUDA_TRY(cudaMemsetAsync(out->col + 2 * e, 0, sizeof(int32_t) * kColPad, s));
    const int g = grid_for(n);
    if (reorder && n > 1) {
        float lo[3], scale[3];
        IRR_CUDA_TRY(bbox_frame(pos_user, n, lo, scale, s));
        uint32_t *keys = nullptr, *keys_tmp = nullptr;
        int32_t* vals_tmp = nullptr;
        IRR_CUDA_TRY(alloc_async(&keys, n, s));
        IRR_CUDA_TRY(alloc_async(&keys_tmp, n, s));
        IRR_CUDA_TRY(alloc_async(&vals_tmp, n, s));
        curve_key_kernel<<<g, 256, 0, s>>>(pos_user, n, make_float3(lo[0], lo[1], lo[2]),
                                           make_float3(scale[0], scale[1], scale[2]), curve, keys,
                                           out->perm);
        IRR_CUDA_TRY(cudaGetLastError());
        IRR_CUDA_TRY(radix_sort_pairs(keys, out->perm, keys_tmp, vals_tmp, n, 30, s));
        IRR_CUDA_TRY(cudaFreeAsync(keys, s));
        IRR_CUDA_TRY(cudaFreeAsync(keys_tmp, s));
        IRR_CUDA_TRY(cudaFreeAsync(vals_tmp, s));
    } else if (n > 0) {
        iota_kernel<<<g, 256, 0, s>>>(out->perm, n);
        IRR_CUDA_TRY(cudaGetLastError());
    }
    if (n > 0) {
        invert_kernel<<<g, 256, 0, s>>>(out->perm, n, out->inv);
        IRR_CUDA_TRY(cudaGetLastError());
    }
    // directed entries, binned by row
    uint32_t* deg = out->row_off;  // counted in place, then scanned
    IRR_CUDA_TRY(cudaMemsetAsync(deg, 0, sizeof(uint32_t) * (size_t)(n + 1), s));
    if (e > 0 && n > 0) {
        // rows of at most kRowSortMax entries (every MD list): count, scan,
        // fill at per-row cursors, sort each row -- the same (row, col) layout
        // as the sorts below, in about a third of the passes
        degree_kernel<<<grid_for(e), 256, 0, s>>>(edges, e, out->inv, deg);
        IRR_CUDA_TRY(cudaGetLastError());
        uint32_t* d_max = nullptr;
        IRR_CUDA_TRY(alloc_async(&d_max, 1, s));
        IRR_CUDA_TRY(cudaMemsetAsync(d_max, 0, sizeof(uint32_t), s));
        max_u32_kernel<<<grid_for(n), 256, 0, s>>>(deg, n, d_max);
        IRR_CUDA_TRY(cudaGetLastError());
        uint32_t max_deg = 0;
        IRR_CUDA_TRY(cudaMemcpyAsync(&max_deg, d_max, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        IRR_CUDA_TRY(cudaFreeAsync(d_max, s));
        IRR_CUDA_TRY(cudaStreamSynchronize(s));
        if (max_deg <= (uint32_t)kRowSortMax) {
            IRR_CUDA_TRY(scan_exclusive_u32(deg, out->row_off, n + 1, nullptr, s));
            uint32_t* cursor = nullptr;
            IRR_CUDA_TRY(alloc_async(&cursor, n, s));
            IRR_CUDA_TRY(cudaMemcpyAsync(cursor, out->row_off, sizeof(uint32_t) * (size_t)n,
                                         cudaMemcpyDeviceToDevice, s));
            fill_rows_kernel<<<grid_for(e), 256, 0, s>>>(edges, e, out->inv, cursor, out->col);
            IRR_CUDA_TRY(cudaGetLastError());
            IRR_CUDA_TRY(cudaFreeAsync(cursor, s));
            IRR_CUDA_TRY(launch_row_sort(out->row_off, n, out->col, s));
            return cudaSuccess;
        }
        IRR_CUDA_TRY(cudaMemsetAsync(deg, 0, sizeof(uint32_t) * (size_t)(n + 1), s));
    }
    if (e > 0) {
        const int64_t m = 2 * e;
        uint32_t *rows = nullptr, *rows_tmp = nullptr;
        int32_t* cols_tmp = nullptr;
        IRR_CUDA_TRY(alloc_async(&rows, m, s));
        IRR_CUDA_TRY(alloc_async(&rows_tmp, m, s));
        IRR_CUDA_TRY(alloc_async(&cols_tmp, m, s));
        entries_kernel<<<grid_for(e), 256, 0, s>>>(edges, e, out->inv, rows, out->col, deg);
        IRR_CUDA_TRY(cudaGetLastError());
        int bits = 1;
        while (bits < 31 && ((int64_t)1 << bits) < n) bits++;
        // (row, col) order: stable by column, then stable by row.  Ascending
        // columns inside a row put the lanes of one gather on fewer cache
        // lines (the rows of a warp are curve neighbours and share most of
        // their neighbourhood), and make the layout independent of the
        // order of the edge list.
        IRR_CUDA_TRY(radix_sort_pairs(reinterpret_cast<uint32_t*>(out->col),
                                      reinterpret_cast<int32_t*>(rows), rows_tmp,
                                      cols_tmp, m, bits, s));
        IRR_CUDA_TRY(radix_sort_pairs(rows, out->col, rows_tmp, cols_tmp, m, bits, s));
        IRR_CUDA_TRY(cudaFreeAsync(rows, s));
        IRR_CUDA_TRY(cudaFreeAsync(rows_tmp, s));
        IRR_CUDA_TRY(cudaFreeAsync(cols_tmp, s));
    }
    IRR_CUDA_TRY(scan_exclusive_u32(deg, out->row_off, n + 1, nullptr, s));
    return cudaSuccess;
}

namespace {

// Row r keeps its entries when its caller id perm[r] is in [lo, hi).
__global__ void kept_degree_kernel(const int32_t* perm, const uint32_t* row_off, int64_t n, int64_t lo,
                                   int64_t hi, uint32_t* deg)
{
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t id = perm[r];
        deg[r] = (id >= lo && id < hi) ? row_off[r + 1] - row_off[r] : 0u;
    }
}

// One warp per row: a kept row's entries, in order, to its new offset.
__global__ void copy_kept_rows_kernel(const uint32_t* old_off, const int32_t* old_col,
                                      const uint32_t* new_off, int64_t n, int32_t* new_col)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        const uint32_t len = new_off[r + 1] - new_off[r];
        const uint32_t src = old_off[r], dst = new_off[r];
        for (uint32_t k = lane; k < len; k += 32) new_col[dst + k] = old_col[src + k];
    }
}

}  // namespace

cudaError_t keep_rows(PartitionOut* p, int64_t n, int64_t lo, int64_t hi, int64_t* m_out, cudaStream_t s)
{
    uint32_t* new_off = nullptr;
    int32_t* new_col = nullptr;
    IRR_CUDA_TRY(alloc_async(&new_off, n + 1, s));
    IRR_CUDA_TRY(cudaMemsetAsync(new_off, 0, sizeof(uint32_t) * (size_t)(n + 1), s));
    if (n > 0) {
        kept_degree_kernel<<<grid_for(n), 256, 0, s>>>(p->perm, p->row_off, n, lo, hi, new_off);
        IRR_CUDA_TRY(cudaGetLastError());
    }
    IRR_CUDA_TRY(scan_exclusive_u32(new_off, new_off, n + 1, nullptr, s));
    uint32_t m = 0;
    IRR_CUDA_TRY(cudaMemcpyAsync(&m, new_off + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    IRR_CUDA_TRY(cudaStreamSynchronize(s));
    IRR_CUDA_TRY(alloc_async(&new_col, (int64_t)m + kColPad, s));
    IRR_CUDA_TRY(cudaMemsetAsync(new_col + m, 0, sizeof(int32_t) * kColPad, s));
    if (n > 0) {
        copy_kept_rows_kernel<<<grid_for(32 * n), 256, 0, s>>>(p->row_off, p->col, new_off, n, new_col);
        IRR_CUDA_TRY(cudaGetLastError());
    }
    IRR_CUDA_TRY(cudaFreeAsync(p->row_off, s));
    IRR_CUDA_TRY(cudaFreeAsync(p->col, s));
    p->row_off = new_off;
    p->col = new_col;
    *m_out = (int64_t)m;
    return cudaSuccess;
}

cudaError_t build_sliced(const uint32_t* row_off, const int32_t* col, int64_t n, int G,
                         Sliced* sl, cudaStream_t s)
{
    free_sliced(sl);
    if (n < 0 || (G != 1 && G != 2 && G != 4 && G != 8 && G != 16 && G != 32))
        return cudaErrorInvalidValue;
    const int R = 32 / G;
    const int64_t slices = (n + R - 1) / R;
    uint32_t* words = nullptr;
    unsigned long long* d_total = nullptr;
    IRR_CUDA_TRY(alloc_async(&sl->slice_off, slices + 1, s));
    IRR_CUDA_TRY(alloc_async(&words, slices + 1, s));
    IRR_CUDA_TRY(alloc_async(&d_total, 1, s));
    IRR_CUDA_TRY(cudaMemsetAsync(words, 0, sizeof(uint32_t) * (size_t)(slices + 1), s));
    IRR_CUDA_TRY(cudaMemsetAsync(d_total, 0, sizeof(unsigned long long), s));
    if (slices > 0) {
        slice_words_kernel<<<grid_for(slices), 256, 0, s>>>(row_off, n, G, slices, words, d_total);
        IRR_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long total = 0;
    IRR_CUDA_TRY(cudaMemcpyAsync(&total, d_total, sizeof(total), cudaMemcpyDeviceToHost, s));
    IRR_CUDA_TRY(cudaStreamSynchronize(s));
    cudaError_t err = cudaSuccess;
    if (total > 0xffffffffull) err = cudaErrorInvalidValue;
    if (err == cudaSuccess) err = scan_exclusive_u32(words, sl->slice_off, slices + 1, nullptr, s);
    if (err == cudaSuccess) err = alloc_async(&sl->col, (int64_t)total, s);
    if (err == cudaSuccess && slices > 0) {
        int lg = 0;
        while ((1 << lg) < G) lg++;
        slice_fill_kernel<<<grid_for(slices * 32), 256, 0, s>>>(row_off, col, n, lg, slices,
                                                                sl->slice_off, sl->col);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) {
        sl->host_off.resize((size_t)slices + 1);
        err = cudaMemcpyAsync(sl->host_off.data(), sl->slice_off,
                              sizeof(uint32_t) * (size_t)(slices + 1), cudaMemcpyDeviceToHost, s);
    }
    cudaFreeAsync(words, s);
    cudaFreeAsync(d_total, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) {
        free_sliced(sl);
        return err;
    }
    sl->slices = slices;
    sl->words = (int64_t)total;
    sl->lanes = G;
    return cudaSuccess;
}

void free_sliced(Sliced* sl, cudaStream_t s)
{
    if (s) {
        if (sl->slice_off) cudaFreeAsync(sl->slice_off, s);
        if (sl->col) cudaFreeAsync(sl->col, s);
    } else {
        if (sl->slice_off) cudaFree(sl->slice_off);
        if (sl->col) cudaFree(sl->col);
    }
    sl->slice_off = nullptr;
    sl->col = nullptr;
    sl->slices = sl->words = 0;
    sl->lanes = 0;
    sl->host_off.clear();
    sl->host_off.shrink_to_fit();
}

cudaError_t launch_load_nodes(const void* raw, int elm_size, const int32_t* perm, int64_t n,
                              float4* dst, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    load_nodes_kernel<<<grid_for(n), 256, 0, s>>>(static_cast<const char*>(raw), elm_size, perm, n,
                                                  dst);
    return cudaGetLastError();
}

cudaError_t launch_store_result(const float4* force, const int32_t* inv, int64_t n,
                                int elm_size, void* out, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int vec12 = elm_size == 12 && (reinterpret_cast<uintptr_t>(out) & 15u) == 0;
    store_result_kernel<<<grid_for(n, kMoveThreads), kMoveThreads, 0, s>>>(force, inv, n, elm_size,
                                                                          vec12, static_cast<char*>(out));
    return cudaGetLastError();
}

cudaError_t launch_load_nodes_scatter(const void* rec, int elm_size, const int32_t* inv, int64_t n,
                                      float4* dst, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int vec12 = elm_size == 12 && (reinterpret_cast<uintptr_t>(rec) & 15u) == 0;
    load_nodes_scatter_kernel<<<grid_for(n, kMoveThreads), kMoveThreads, 0, s>>>(
        static_cast<const char*>(rec), elm_size, vec12, inv, n, dst);
    return cudaGetLastError();
}

void* host_device_view(const void* p)
{
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    // page-locked (or registered) host memory mapped at the same address, at
    // a 16-byte boundary (every record format's loads and stores then align)
    const bool ok = a.type == cudaMemoryTypeHost && a.devicePointer == p &&
                    (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
    return ok ? const_cast<void*>(p) : nullptr;
}

cudaError_t launch_validate_edges(const int2* edges, int64_t e, int64_t n, int* d_status,
                                  cudaStream_t s)
{
    if (e <= 0) return cudaSuccess;
    validate_edges_kernel<<<grid_for(e), 256, 0, s>>>(edges, e, n, d_status);
    return cudaGetLastError();
}

namespace {
constexpr int kMaxPoolDevices = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[kMaxPoolDevices] = {};
}  // namespace

cudaError_t irr_malloc_async(void** p, size_t bytes, cudaStream_t s)
{
    int dev = 0;
    IRR_CUDA_TRY(cudaGetDevice(&dev));
    cudaMemPool_t pool = nullptr;
    if (dev >= 0 && dev < kMaxPoolDevices) {
        std::lock_guard<std::mutex> lock(g_pool_mutex);
        if (!g_pools[dev]) {
            cudaMemPoolProps props{};
            props.allocType = cudaMemAllocationTypePinned;
            props.handleTypes = cudaMemHandleTypeNone;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            cudaMemPool_t made = nullptr;
            if (cudaMemPoolCreate(&made, &props) == cudaSuccess) {
                uint64_t keep = ~0ull;
                cudaMemPoolSetAttribute(made, cudaMemPoolAttrReleaseThreshold, &keep);
                g_pools[dev] = made;
            } else {
                cudaGetLastError();
            }
        }
        pool = g_pools[dev];
    }
    if (!pool) return cudaMallocAsync(p, bytes, s);  // the device's default pool
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

}  // namespace irr
