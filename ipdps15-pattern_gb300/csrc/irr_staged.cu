// irr_staged.cu -- the staged ("halo") entry layout, built on the GPU.
//
// The partitioned reduction gathers every neighbour's position for every
// directed entry.  In the sliced layout those gathers go through L1 and, for
// ~15 % of the lines, to L2: the kernel waits on them and the L1 data pipe
// does ~9.5 wavefronts per 32-lane gather.  Here each work item (a run of up
// to 8 slices of 8 consecutive curve-ordered rows) carries its own table: the
// sorted distinct ids of its rows and of all their neighbours -- ~465 for 64
// rows at ~64 neighbours each, so every staged position is used ~9 times.
// The kernel's producer warp gathers the table's positions into shared memory
// (cp.async) while the consumers work on the item before; the consumers then
// read positions from shared memory by 16-bit table offsets.  A row's entries
// are ordered so that the 8 lanes of each quarter-warp phase of a 128-bit
// shared load mostly hit 8 different bank groups: row i of a slice takes its
// pick (t, h, l) from bank group (2t + h + 4 (i & 1) + l) mod 8 -- the rows of
// a phase take complementary groups, and the window rotates so that a row
// draws on all 8 groups evenly -- else from its fullest group.  On a curve-
// ordered random box at ~64 neighbours that is ~5.4 wavefronts per 128-bit
// gather (8 lanes at random would be ~7.2 with the table sorted, ~9 unsorted).
//
// Layout (the oracle restates it bit for bit, oracle/irr_oracle.c
// orc_staged_layout):
//   items: blocks of 8 consecutive rows, cut into runs of at most
//   kHaloSlicesPerItem blocks and kHaloStreamMax words (a block counted at
//   its longest row), each run cut into the longest prefixes whose table
//   holds at most kHaloTabMax ids;
//   slices: within an item the rows are ordered longest first (ties by row),
//   and slice j takes rows 8j .. 8j + 7 of that order -- rows of similar
//   length, so a slice pads ~8 % instead of ~17 % for 8 consecutive rows (the
//   table, and so every gather, is the item's whatever the order); slice j
//   takes 32 (T_j + 1) words, T_j = ceil(its longest row / 8): a header word
//   own | len << 14 | lrow << 24 per lane (own: the row's byte offset in the
//   table, lrow: its index in the item; 1 << 31 for a padding row), then one
//   word b0 | b1 << 16 per lane and step -- 16-bit byte offsets into the
//   table of the lane's two entries (padding: the row's own offset).
// Build: the host cuts the runs from the row offsets; one CTA per run counts
// each prefix's distinct ids in a shared-memory hash set (more rounds for the
// remainders of runs whose tables overflowed); then one CTA per item rebuilds
// its table (hash set, bitonic sort), maps every entry to its slot by binary
// search and lays out the rows' words, one thread per row.
#include <algorithm>
#include <climits>
#include <vector>

#include "irr_internal.cuh"

namespace irr {
namespace {

constexpr int kHashSlots = 2048;        // > 2 x kHaloTabMax
constexpr int kBuildThreads = 256;
constexpr int kSortCap = 1024;          // >= kHaloTabMax, a power of two
// Entries of one item: every word of a step holds two entries, so at most
// 2 x kHaloStreamMax.
constexpr int kItemEntryCap = 2 * kHaloStreamMax;
static_assert(kHaloTabMax <= kSortCap && 2 * kHaloTabMax < kHashSlots, "table limits");
static_assert(kHaloTabMax * 16 < 65536, "table offsets fit 16 bits");

__device__ __forceinline__ uint32_t hash_of(int32_t id)
{
    return ((uint32_t)id * 2654435761u) >> 21;  // 11 bits: kHashSlots = 2048
}

// Inserts id into the set; returns 1 if it was new, 0 if present, -1 if the
// probe found no room (the set is full).
__device__ __forceinline__ int hash_insert(int32_t* set, int32_t id)
{
    uint32_t h = hash_of(id);
    for (int p = 0; p < kHashSlots; p++) {
        const int32_t old = atomicCAS(set + h, -1, id);
        if (old == -1) return 1;
        if (old == id) return 0;
        h = (h + 1) & (kHashSlots - 1);
    }
    return -1;
}

// The ids slice q contributes to a table: its rows and their columns.
// Inserts them (all threads of the CTA) and counts the new ones.
__device__ void insert_slice(const uint32_t* __restrict__ row_off, const int32_t* __restrict__ col,
                             int64_t n, int64_t q, int32_t* set, int* count, int* full)
{
    const int64_t r0 = 8 * q, r1 = min(8 * q + 8, n);
    const int nrows = (int)(r1 - r0);
    const uint32_t e0 = row_off[r0], e1 = row_off[r1];
    const int64_t m = (int64_t)nrows + (e1 - e0);
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
        const int32_t id = k < nrows ? (int32_t)(r0 + k) : col[e0 + (k - nrows)];
        const int res = hash_insert(set, id);
        if (res > 0) atomicAdd(count, 1);
        if (res < 0) *full = 1;
    }
}

// One CTA per run (q0, slices): counts[run * kHaloSlicesPerItem + j] = distinct
// ids of the first j + 1 slices, or kHaloTabMax + 1 once that is exceeded.
__global__ void __launch_bounds__(kBuildThreads) staged_count_kernel(
    const uint32_t* __restrict__ row_off, const int32_t* __restrict__ col, int64_t n,
    const int2* __restrict__ runs, int* __restrict__ counts)
{
    __shared__ int32_t set[kHashSlots];
    __shared__ int count, full;
    const int2 run = runs[blockIdx.x];
    for (int k = threadIdx.x; k < kHashSlots; k += blockDim.x) set[k] = -1;
    if (threadIdx.x == 0) count = full = 0;
    __syncthreads();
    bool over = false;
    for (int j = 0; j < run.y; j++) {
        if (!over) insert_slice(row_off, col, n, (int64_t)run.x + j, set, &count, &full);
        __syncthreads();
        const int c = count;
        over = over || full || c > kHaloTabMax;
        if (threadIdx.x == 0) counts[(int64_t)blockIdx.x * kHaloSlicesPerItem + j] = over ? kHaloTabMax + 1 : c;
        __syncthreads();
    }
}

__device__ __forceinline__ int slot_of(const int32_t* tab, int ntab, int32_t id)
{
    int lo = 0, hi = ntab;  // first slot with tab[slot] >= id
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (tab[mid] < id) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// One CTA per item: its sorted table into ids[tab0, tab0 + ntab), and the
// words of its slices.
__global__ void __launch_bounds__(kBuildThreads) staged_fill_kernel(
    const uint32_t* __restrict__ row_off, const int32_t* __restrict__ col, int64_t n,
    const WorkItem* __restrict__ items, const uint32_t* __restrict__ slice_off,
    int32_t* __restrict__ ids, uint32_t* __restrict__ words, int* __restrict__ status)
{
    __shared__ int32_t set[kHashSlots];
    __shared__ int32_t tab[kSortCap];
    __shared__ uint16_t slots[kItemEntryCap];  // each entry's slot, in CSR order
    __shared__ uint16_t rs[kItemEntryCap];     // per row: slots bucketed by bank group
    __shared__ int order[8 * kHaloSlicesPerItem];  // the item's rows, longest first
    __shared__ int count, full;
    const WorkItem w = items[blockIdx.x];
    const int64_t q0 = w.row0 / 8;
    const int ns = (w.nrows + 7) / 8;
    for (int k = threadIdx.x; k < kHashSlots; k += blockDim.x) set[k] = -1;
    if (threadIdx.x == 0) count = full = 0;
    __syncthreads();
    for (int j = 0; j < ns; j++) insert_slice(row_off, col, n, q0 + j, set, &count, &full);
    __syncthreads();
    const int ntab = count;
    const uint32_t e0 = row_off[w.row0], e1 = row_off[w.row0 + w.nrows];
    if (full || ntab != (int)w.ntab || (int64_t)(e1 - e0) > kItemEntryCap) {
        if (threadIdx.x == 0) atomicOr(status, 1);  // the cut and the fill disagree
        return;
    }
    // compact and sort the table
    __syncthreads();
    if (threadIdx.x == 0) count = 0;
    for (int k = threadIdx.x; k < kSortCap; k += blockDim.x) tab[k] = INT_MAX;
    __syncthreads();
    for (int k = threadIdx.x; k < kHashSlots; k += blockDim.x)
        if (set[k] != -1) tab[atomicAdd(&count, 1)] = set[k];
    __syncthreads();
    // the INT_MAX padding sorts last, so sorting the first power of two that
    // holds the table gives the same first ntab ids as sorting all kSortCap
    int sort_n = 2;
    while (sort_n < ntab) sort_n <<= 1;
    for (int size = 2; size <= sort_n; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int k = threadIdx.x; k < sort_n / 2; k += blockDim.x) {
                const int lo = 2 * k - (k & (stride - 1));
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const int32_t a = tab[lo], b = tab[hi];
                if ((a > b) == up) {
                    tab[lo] = b;
                    tab[hi] = a;
                }
            }
            __syncthreads();
        }
    for (int k = threadIdx.x; k < ntab; k += blockDim.x) ids[(int64_t)w.tab0 + k] = tab[k];
    // every entry's slot
    for (uint32_t k = threadIdx.x; k < e1 - e0; k += blockDim.x)
        slots[k] = (uint16_t)slot_of(tab, ntab, col[e0 + k]);
    __syncthreads();
    // the rows, longest first (ties by row): each row's rank by counting
    const int tid = threadIdx.x;
    const int m = w.nrows;
    if (tid < m) {
        const int64_t r = (int64_t)w.row0 + tid;
        const uint32_t len_r = row_off[r + 1] - row_off[r];
        int rank = 0;
        for (int k = 0; k < m; k++) {
            const uint32_t len_k = row_off[w.row0 + k + 1] - row_off[w.row0 + k];
            rank += (len_k > len_r || (len_k == len_r && k < tid)) ? 1 : 0;
        }
        order[rank] = tid;
    }
    __syncthreads();
    // one thread per slice position: bucket the row's slots by bank group,
    // then the picks
    if (tid >= 8 * ns) return;
    const int64_t q = q0 + tid / 8;
    const int i = tid & 7;
    const int T = (int)((slice_off[q + 1] - slice_off[q]) / 32) - 1;
    uint32_t* sw = words + slice_off[q];
    int len = 0, own = 0;
    uint32_t hdr = 1u << 31;  // a padding row
    // per bank group: the next unused slot of its bucket in rs and the
    // bucket's end (indexed by compile-time constants only: registers)
    int nxt[8], end[8];
#pragma unroll
    for (int g = 0; g < 8; g++) nxt[g] = end[g] = 0;
    if (tid < m) {
        const int lrow = order[tid];
        const int64_t r = (int64_t)w.row0 + lrow;
        const int base = (int)(row_off[r] - e0);
        len = (int)(row_off[r + 1] - row_off[r]);
        own = slot_of(tab, ntab, (int32_t)r);
        int cnt[8];
#pragma unroll
        for (int g = 0; g < 8; g++) cnt[g] = 0;
        for (int k = 0; k < len; k++) {
            const int g = slots[base + k] & 7;
#pragma unroll
            for (int x = 0; x < 8; x++) cnt[x] += (g == x) ? 1 : 0;
        }
        int acc = base;
#pragma unroll
        for (int g = 0; g < 8; g++) {
            nxt[g] = acc;
            acc += cnt[g];
            end[g] = acc;
        }
        int fill[8];
#pragma unroll
        for (int g = 0; g < 8; g++) fill[g] = nxt[g];
        for (int k = 0; k < len; k++) {
            const uint16_t sl = slots[base + k];
            const int g = sl & 7;
            int at = 0;
#pragma unroll
            for (int x = 0; x < 8; x++)
                if (g == x) at = fill[x]++;
            rs[at] = sl;
        }
        hdr = (uint32_t)(own * 16) | ((uint32_t)len << 14) | ((uint32_t)lrow << 24);
    }
    *reinterpret_cast<uint4*>(sw + 4 * i) = make_uint4(hdr, hdr, hdr, hdr);
    const int p = i & 1;
    for (int t = 0; t < T; t++) {
        uint32_t pk[2][4];
#pragma unroll
        for (int h = 0; h < 2; h++)
#pragma unroll
            for (int l = 0; l < 4; l++) {
                // the window's group if its bucket has slots left, else the
                // group with the most left (the first such on ties), else
                // padding (the row's own slot)
                const int g0 = (2 * t + h + 4 * p + l) & 7;
                int take = -1;
#pragma unroll
                for (int x = 0; x < 8; x++)
                    if (x == g0 && nxt[x] < end[x]) take = x;
                if (take < 0) {
                    int most = 0;
#pragma unroll
                    for (int x = 0; x < 8; x++)
                        if (end[x] - nxt[x] > most) {
                            most = end[x] - nxt[x];
                            take = x;
                        }
                }
                int slot = own;
                if (take >= 0) {
                    int at = 0;
#pragma unroll
                    for (int x = 0; x < 8; x++)
                        if (x == take) at = nxt[x]++;
                    slot = rs[at];
                }
                pk[h][l] = (uint32_t)(slot * 16);
            }
        *reinterpret_cast<uint4*>(sw + 32 * (t + 1) + 4 * i) =
            make_uint4(pk[0][0] | (pk[1][0] << 16), pk[0][1] | (pk[1][1] << 16),
                       pk[0][2] | (pk[1][2] << 16), pk[0][3] | (pk[1][3] << 16));
    }
}

// out[j] = the length at position 8 j of an item's m row lengths in descending
// order (the longest row of slice j once the rows are ordered longest first),
// j < ceil(m / 8).  The lengths of an item's rows span a narrow range, so a
// histogram over [min, max] finds them without sorting; wide ranges sort.
void slice_longest(const uint32_t* lens, int m, uint32_t* out)
{
    static_assert(8 * kHaloSlicesPerItem <= 64, "an item holds at most 64 rows");
    const int ns = (m + 7) / 8;
    uint32_t lo = lens[0], hi = lens[0];
    for (int k = 1; k < m; k++) {
        lo = std::min(lo, lens[k]);
        hi = std::max(hi, lens[k]);
    }
    if (hi - lo < 256) {
        uint16_t cnt[256];
        std::fill(cnt, cnt + (hi - lo + 1), (uint16_t)0);
        for (int k = 0; k < m; k++) cnt[lens[k] - lo]++;
        int pos = 0, j = 0;
        for (uint32_t v = hi + 1; v-- > lo && j < ns;) {
            pos += cnt[v - lo];
            while (j < ns && 8 * j < pos) out[j++] = v;
        }
    } else {
        uint32_t sorted[64];
        std::copy(lens, lens + m, sorted);
        std::sort(sorted, sorted + m, [](uint32_t x, uint32_t y) { return x > y; });
        for (int j = 0; j < ns; j++) out[j] = sorted[8 * j];
    }
}

template <class T>
cudaError_t alloc_n(T** p, int64_t count, cudaStream_t s)
{
    return irr_malloc_async(p, sizeof(T) * (size_t)(count > 0 ? count : 1), s);
}

}  // namespace

void free_staged(Staged* st, cudaStream_t s)
{
    void* ps[3] = {st->slice_off, st->words, st->ids};
    for (void* p : ps)
        if (p) {
            if (s) cudaFreeAsync(p, s);
            else cudaFree(p);
        }
    *st = Staged{};
}

cudaError_t build_staged(const uint32_t* row_off, const int32_t* col, const uint32_t* host_row_off,
                         int64_t n, Staged* st, cudaStream_t s)
{
    free_staged(st, s);
    const int64_t S = (n + 7) / 8;
    // the cut's word counts: blocks of 8 consecutive rows
    std::vector<uint64_t> soff((size_t)S + 1, 0);
    for (int64_t q = 0; q < S; q++) {
        uint32_t longest = 0;
        for (int64_t r = 8 * q; r < std::min<int64_t>(8 * q + 8, n); r++)
            longest = std::max(longest, host_row_off[r + 1] - host_row_off[r]);
        const uint64_t wq = 32ull * ((longest + 7) / 8 + 1);
        if (wq > (uint64_t)kHaloStreamMax) return cudaErrorNotSupported;
        soff[(size_t)q + 1] = soff[(size_t)q] + wq;
    }
    // tentative runs, then the longest prefixes whose tables fit
    std::vector<int2> pending;
    for (int64_t q0 = 0; q0 < S;) {
        int64_t q1 = q0 + 1;
        while (q1 < S && q1 - q0 < kHaloSlicesPerItem &&
               soff[(size_t)q1 + 1] - soff[(size_t)q0] <= (uint64_t)kHaloStreamMax)
            q1++;
        pending.push_back(make_int2((int)q0, (int)(q1 - q0)));
        q0 = q1;
    }
    std::vector<WorkItem> items;
    cudaError_t e = cudaSuccess;
    std::vector<int> counts;
    while (!pending.empty()) {
        const int nr = (int)pending.size();
        int2* d_runs = nullptr;
        int* d_counts = nullptr;
        e = alloc_n(&d_runs, nr, s);
        if (e == cudaSuccess) e = alloc_n(&d_counts, (int64_t)nr * kHaloSlicesPerItem, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_runs, pending.data(), sizeof(int2) * nr, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
            staged_count_kernel<<<nr, kBuildThreads, 0, s>>>(row_off, col, n, d_runs, d_counts);
            e = cudaGetLastError();
        }
        counts.assign((size_t)nr * kHaloSlicesPerItem, 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(counts.data(), d_counts, sizeof(int) * counts.size(), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (d_runs) cudaFreeAsync(d_runs, s);
        if (d_counts) cudaFreeAsync(d_counts, s);
        if (e != cudaSuccess) return e;
        std::vector<int2> next;
        for (int k = 0; k < nr; k++) {
            const int2 run = pending[(size_t)k];
            const int* c = counts.data() + (size_t)k * kHaloSlicesPerItem;
            if (c[0] > kHaloTabMax) return cudaErrorNotSupported;  // one slice's table is too large
            int b = 1;
            while (b < run.y && c[b] <= kHaloTabMax) b++;
            WorkItem w{};
            w.inst = 0;
            w.row0 = 8 * run.x;
            w.nrows = (int32_t)(std::min<int64_t>(8 * (int64_t)(run.x + b), n) - 8 * (int64_t)run.x);
            w.flags = kItemStaged;
            w.ntab = (uint32_t)c[b - 1];
            items.push_back(w);
            if (b < run.y) next.push_back(make_int2(run.x + b, run.y - b));
        }
        pending.swap(next);
    }
    std::sort(items.begin(), items.end(), [](const WorkItem& a, const WorkItem& b) { return a.row0 < b.row0; });
    // the slices' word offsets, rows ordered longest first within each item
    std::vector<uint32_t> fin((size_t)S + 1, 0);
    uint64_t acc = 0, tab = 0;
    uint32_t lens[64], longest_of[kHaloSlicesPerItem];
    for (WorkItem& w : items) {
        w.tab0 = (uint32_t)tab;
        tab += w.ntab;
        if (tab > 0x7fffffffull) return cudaErrorNotSupported;
        for (int k = 0; k < w.nrows; k++) lens[k] = host_row_off[w.row0 + k + 1] - host_row_off[w.row0 + k];
        slice_longest(lens, w.nrows, longest_of);
        const int64_t q0 = w.row0 / 8, ns = (w.nrows + 7) / 8;
        w.ent0 = (uint32_t)acc;
        for (int64_t j = 0; j < ns; j++) {
            const uint32_t longest = longest_of[j];  // the first of a slice is its longest
            acc += 32ull * ((longest + 7) / 8 + 1);
            if (acc > 0xffffffffull) return cudaErrorNotSupported;
            fin[(size_t)(q0 + j) + 1] = (uint32_t)acc;
        }
        w.nent = (uint32_t)(acc - w.ent0);
    }
    Staged out;
    out.slices = S;
    out.nwords = (int64_t)acc;
    soff.clear();
    out.nids = (int64_t)tab;
    WorkItem* d_items = nullptr;
    int* d_status = nullptr;
    e = alloc_n(&out.slice_off, S + 1, s);
    if (e == cudaSuccess) e = alloc_n(&out.words, out.nwords, s);
    // 4 ids of slack: the kernel bulk-copies each item's ids in whole 16-byte words
    if (e == cudaSuccess) e = alloc_n(&out.ids, out.nids + 4, s);
    if (e == cudaSuccess) e = alloc_n(&d_items, (int64_t)items.size(), s);
    if (e == cudaSuccess) e = alloc_n(&d_status, 1, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out.slice_off, fin.data(), sizeof(uint32_t) * fin.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !items.empty())
        e = cudaMemcpyAsync(d_items, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, sizeof(int), s);
    if (e == cudaSuccess && !items.empty()) {
        staged_fill_kernel<<<(unsigned)items.size(), kBuildThreads, 0, s>>>(
            row_off, col, n, d_items, out.slice_off, out.ids, out.words, d_status);
        e = cudaGetLastError();
    }
    int status = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (d_items) cudaFreeAsync(d_items, s);
    if (d_status) cudaFreeAsync(d_status, s);
    if (e == cudaSuccess && status) e = cudaErrorInvalidValue;
    if (e != cudaSuccess) {
        free_staged(&out, s);
        return e;
    }
    out.host_off.swap(fin);
    out.items.swap(items);
    *st = std::move(out);
    return cudaSuccess;
}

}  // namespace irr
