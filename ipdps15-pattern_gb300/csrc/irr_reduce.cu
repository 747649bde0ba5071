// irr_reduce.cu -- the edge-reduction kernels.
//
// plain_kernel: the reference's per-edge semantics as written -- one thread
//   per edge of the caller's half list, both endpoint contributions added with
//   float4 atomics into a zeroed result.  It replaces compute_gpu
//   (moldyn/irregular/gpu_kernel.cu:21-103), whose shared-memory hash object
//   Sobject (ros.cu:10-68) and global hash Gobject (rog.cu:11-88) become a
//   direct per-node array.
//
// tiled_kernel: owner computes.  The partitioner hands each node a row of
//   directed entries (one per incident edge); a group of G lanes walks the
//   row, evaluates the law for every entry, keeps FP32 partial sums in
//   registers and combines the G partials with error-free TwoSum steps.  Each
//   edge is evaluated from both ends -- the reference duplicates cross-part
//   edges the same way (moldyn/irregular/partitioner.cpp:142-297, paper
//   Sec. II-A) -- so no atomics are needed and every result is bitwise
//   reproducible.  The grid is persistent: CTAs claim node blocks (work
//   items) from a queue, the reference's per-part atomicAdd queue
//   (gpu_kernel.cu:60-77) generalised to (instance, block) items for the
//   batched form.  A block's entries are contiguous, so one bulk (TMA) copy
//   per item moves them into a ring of shared-memory stages a few items
//   ahead of the consumers: the entry stream, which is most of the traffic,
//   is kept in flight while positions are gathered through L1.
//   Entries come in one of two layouts.  CSR rows (consume_item): the rows
//   of a warp start at unrelated offsets, so its reads of the stage collide
//   in shared-memory banks.  Slices (consume_sliced, struct Sliced): the
//   rows of a warp are interleaved and padded, so each step of the warp is
//   one contiguous 256-byte read and the trip count is uniform; with curve-
//   ordered rows whose columns ascend, the lanes of one gather also land on
//   few cache lines.
#include <algorithm>
#include <type_traits>
#include <vector>

#include "irr_internal.cuh"

namespace irr {
namespace {

template <bool PERIODIC>
__global__ void __launch_bounds__(256) plain_kernel(const float4* __restrict__ pos,
                                                    const int2* __restrict__ edges, int64_t e,
                                                    float4* __restrict__ force, LawParams law)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < e; t += stride) {
        const int2 ed = __ldcs(edges + t);
        const float4 a = __ldg(pos + ed.x);
        const float4 b = __ldg(pos + ed.y);
        float dx, dy, dz;
        const float s = lj_scalar<PERIODIC>(a, b, law, dx, dy, dz);
        if (s == 0.0f) continue;  // outside the cutoff (NaN still propagates)
        const float fx = __fmul_rn(dx, s), fy = __fmul_rn(dy, s), fz = __fmul_rn(dz, s);
        atomicAdd(force + ed.x, make_float4(fx, fy, fz, 0.0f));
        atomicAdd(force + ed.y, make_float4(-fx, -fy, -fz, 0.0f));
    }
}

// ---- bulk copy + mbarrier helpers (inline PTX, sm_90+) ----
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src, uint32_t bytes,
                                          uint64_t* bar)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst_smem)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// One test of phase `parity`; a thread whose phase is not complete may be
// suspended for up to kSuspendNs (it resumes as soon as the phase completes),
// so a waiting warp does not keep issuing polls.
constexpr uint32_t kSuspendNs = 100000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kSuspendNs)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for phase `parity` of the barrier; gives up after `limit_ns`
// nanoseconds of wall-clock time (whatever the suspension granted per test).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// The same bound, polling with a growing sleep (32 ns doubling up to MAX_NS)
// between tests: a warp that waits long -- the producer, waiting for the
// consumers to free a stage -- then takes few issue slots from the warps
// that work on its SM sub-partition (without the sleep a waiting producer
// polled ~450 times per work item).
template <uint32_t MAX_NS>
__device__ __forceinline__ bool mbar_wait_backoff(uint64_t* bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    uint32_t ns = 32;
    for (;;) {
        __nanosleep(ns);
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
        if (ns < MAX_NS) ns <<= 1;
    }
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Law parameters the inner loop keeps in registers; the rest (box side as a
// float pair, FP64 cutoff) is read from the instance descriptor on the rare
// paths that need it.
struct HotLaw {
    float half2;   // just under (side/2)^2: rd at or below it never needs a wrap
    float rc2;
    float band;    // |rd - rc2| < band: take the reference's FP64 decision
};

// What the consumers read of an instance.  Batched launches keep it in
// registers across the work items of one instance (its items are
// consecutive); single-instance launches rebuild it from the launch
// parameter for every item, which costs no registers across items.
struct InstHot {
    const float4* __restrict__ pos;
    const uint32_t* __restrict__ row_off;
    const uint32_t* __restrict__ slice_off;
    float4* __restrict__ force;
    const LawParams* __restrict__ cold;
    int64_t n;
    HotLaw H;
};

__device__ __forceinline__ InstHot load_hot(const InstDesc* __restrict__ I)
{
    InstHot h;
    h.pos = I->pos;
    h.row_off = I->row_off;
    h.slice_off = I->slice_off;
    h.force = I->force;
    h.cold = &I->law;
    h.n = I->n;
    h.H.half2 = I->law.half2;
    h.H.rc2 = I->law.rc2;
    h.H.band = I->law.band;
    return h;
}

// Where a launch's consumers find the instance fields (the kernel's last
// parameter, in the constant bank: its fields are read as operands where they
// are used, so they need no registers across items -- at the 56-register
// bound of 4 CTAs x 288 threads that is what removes the spills):
//   SrcGlobal: from the descriptor table in global memory (any batch size);
//   SrcOne:    every item belongs to instance 0, whose descriptor is the
//              parameter;
//   SrcTable:  up to kTableInsts instances, the fields the step loop reads
//              (positions, law constants) of each in the parameter; the
//              per-slice fields, the producer's col / scol and the rare
//              path's law come from the global table.
struct SrcGlobal {
    int unused;
};
struct SrcOne {
    InstDesc d;
};
struct HotEntry {
    const float4* pos;
    HotLaw H;
    float pad;
};
constexpr int kTableInsts = 1024;  // 1024 x 24 B stays inside the 32 KB of kernel parameters
struct SrcTable {
    HotEntry h[kTableInsts];
};

__device__ __forceinline__ InstHot hot_from(const SrcTable& t, const InstDesc* insts, int inst)
{
    const HotEntry& e = t.h[inst];
    const InstDesc* __restrict__ I = insts + inst;
    InstHot h;
    h.pos = e.pos;
    h.row_off = I->row_off;
    h.slice_off = I->slice_off;
    h.force = I->force;
    h.cold = &I->law;
    h.n = I->n;
    h.H = e.H;
    return h;
}

// wrap_component (irr_law.cuh) without branches: both shifted forms are
// formed and the one the sign of d calls for is selected.
__device__ __forceinline__ float wrap_select(float a, float b, float d, float half, float shi,
                                             float slo)
{
    const float up = __fsub_rn(__fsub_rn(__fsub_rn(a, shi), b), slo);  // d > half
    const float dn = __fadd_rn(__fsub_rn(a, __fsub_rn(b, shi)), slo);  // d < -half
    return d > half ? up : (d < -half ? dn : d);
}

template <bool PERIODIC>
__device__ __noinline__ bool exact_inside_g(float4 a, float4 b, const LawParams* __restrict__ P)
{
    return exact_inside<PERIODIC>(a, b, *P);
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The rare cases of an entry pair: a pair past half the box (periodic) is
// re-wrapped exactly, and a pair whose rd lies within `band` of the cutoff
// takes the reference's FP64 decision.  Updates d, rd and the in-flags.
template <bool PERIODIC>
__device__ __forceinline__ void rare_pair(float4 a, float4 b0, float4 b1, const HotLaw& H,
                                          const LawParams* __restrict__ cold, float2& dx,
                                          float2& dy, float2& dz, float2& rd, bool& in0, bool& in1)
{
    if (PERIODIC && fmaxf(rd.x, rd.y) > H.half2) {
        // every component of both slots through wrap_select (a component
        // within half the box comes back unchanged, bit for bit)
        const float half = cold->half, shi = cold->side_hi, slo = cold->side_lo;
        dx.x = wrap_select(a.x, b0.x, dx.x, half, shi, slo);
        dy.x = wrap_select(a.y, b0.y, dy.x, half, shi, slo);
        dz.x = wrap_select(a.z, b0.z, dz.x, half, shi, slo);
        dx.y = wrap_select(a.x, b1.x, dx.y, half, shi, slo);
        dy.y = wrap_select(a.y, b1.y, dy.y, half, shi, slo);
        dz.y = wrap_select(a.z, b1.z, dz.y, half, shi, slo);
        rd = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
        in0 = rd.x < H.rc2;
        in1 = rd.y < H.rc2;
    }
    if (fabsf(__fsub_rn(rd.x, H.rc2)) < H.band) in0 = exact_inside_g<PERIODIC>(a, b0, cold);
    if (fabsf(__fsub_rn(rd.y, H.rc2)) < H.band) in1 = exact_inside_g<PERIODIC>(a, b1, cold);
}

// Two entries (b0, b1) of the row of node a, evaluated with packed FP32x2
// arithmetic (each half rounds exactly as the scalar law in irr_law.cuh), and
// accumulated into the lane's packed partials.  A slot with v == false
// contributes 0 (its b is the row's own position or any valid node).
//
// The differences are formed by scalar subtractions written straight into
// register pairs (the two positions come from separate loads, so a packed
// subtraction would first have to move them into pairs).  A component
// |d| > side/2 implies rd > (side/2)^2, so the wrap test is one compare on
// rd; it and the cutoff-band test are folded into one branch to the rare
// path (a pair across the box wall, beyond half the box, or within 2^-18 of
// the cutoff).  (A warp vote in front of it measured slower.)
template <bool PERIODIC>
__device__ __forceinline__ void lj_pair(float4 a, float4 b0, float4 b1, bool v0, bool v1, const HotLaw& H,
                                        const LawParams* __restrict__ cold, float2& ax, float2& ay,
                                        float2& az)
{
    float2 dx = make_float2(__fsub_rn(a.x, b0.x), __fsub_rn(a.x, b1.x));
    float2 dy = make_float2(__fsub_rn(a.y, b0.y), __fsub_rn(a.y, b1.y));
    float2 dz = make_float2(__fsub_rn(a.z, b0.z), __fsub_rn(a.z, b1.z));
    float2 rd = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
    const float2 t = __fadd2_rn(rd, make_float2(-H.rc2, -H.rc2));
    bool rare = fminf(fabsf(t.x), fabsf(t.y)) < H.band;
    if (PERIODIC) rare = rare || fmaxf(rd.x, rd.y) > H.half2;
    bool in0 = rd.x < H.rc2, in1 = rd.y < H.rc2;
    if (rare) rare_pair<PERIODIC>(a, b0, b1, H, cold, dx, dy, dz, rd, in0, in1);
    float2 r = make_float2(rcp_approx(rd.x), rcp_approx(rd.y));
    const float2 e = __ffma2_rn(make_float2(-rd.x, -rd.y), r, make_float2(1.0f, 1.0f));
    r = __ffma2_rn(r, e, r);                                     // rd^-1 (one Newton step)
    const float2 r2 = __fmul2_rn(r, r);                          // rd^-2
    float2 s = __fmul2_rn(__fmul2_rn(r2, r2), __ffma2_rn(r2, r, make_float2(-0.5f, -0.5f)));
    s.x = (in0 && v0) ? s.x : 0.0f;
    s.y = (in1 && v1) ? s.y : 0.0f;
    ax = __ffma2_rn(dx, s, ax);
    ay = __ffma2_rn(dy, s, ay);
    az = __ffma2_rn(dz, s, az);
}

// The row's result from its G lanes' packed partials: the two halves of each
// lane joined by TwoSum, then the G lanes by a TwoSum butterfly.
//
// The x and y components run as one FP32x2 pair, z as a scalar; every
// operation rounds as its scalar form (a - b is fma(b, -1, a), one rounding),
// so the result is bitwise the scalar TwoSum chain's.
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e)
{
    s = __fadd2_rn(a, b);
    const float2 bb = sub2(s, a);
    e = __fadd2_rn(sub2(a, sub2(s, bb)), sub2(b, bb));
}

template <int G>
__device__ __forceinline__ float3 join_partials(float2 ax, float2 ay, float2 az)
{
    float2 h, c;  // (x, y) sums and their carried errors
    float hz, cz;
    two_sum2(make_float2(ax.x, ay.x), make_float2(ax.y, ay.y), h, c);
    two_sum(az.x, az.y, hz, cz);
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
        const float2 o = make_float2(__shfl_xor_sync(0xffffffffu, h.x, off, G),
                                     __shfl_xor_sync(0xffffffffu, h.y, off, G));
        const float oz = __shfl_xor_sync(0xffffffffu, hz, off, G);
        const float2 oc = make_float2(__shfl_xor_sync(0xffffffffu, c.x, off, G),
                                      __shfl_xor_sync(0xffffffffu, c.y, off, G));
        const float ocz = __shfl_xor_sync(0xffffffffu, cz, off, G);
        float2 e;
        two_sum2(h, o, h, e);
        c = __fadd2_rn(__fadd2_rn(c, oc), e);
        float ez;
        two_sum(hz, oz, hz, ez);
        cz = __fadd_rn(__fadd_rn(cz, ocz), ez);
    }
    const float2 r = __fadd2_rn(h, c);
    return make_float3(r.x, r.y, __fadd_rn(hz, cz));
}

// One row: G lanes; each lane takes entry pairs (k, k + G) with stride 2G.
// Entry k of the row is cols[k - shift].
template <bool PERIODIC, int G>
__device__ __forceinline__ float3 row_sum(const float4* __restrict__ pos, const int32_t* cols,
                                          uint32_t shift, float4 a, uint32_t beg, uint32_t end,
                                          int lane, const HotLaw& H,
                                          const LawParams* __restrict__ cold)
{
    float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
    for (uint32_t k = beg + lane; k < end; k += 2 * G) {
        const bool v1 = k + G < end;
        const float4 b0 = __ldg(pos + cols[k - shift]);
        const float4 b1 = v1 ? __ldg(pos + cols[k + G - shift]) : a;
        lj_pair<PERIODIC>(a, b0, b1, true, v1, H, cold, ax, ay, az);
    }
    return join_partials<G>(ax, ay, az);
}

constexpr int kConsumerWarps = kConsumerSlices;
// Items per queue claim (a run of consecutive node blocks on one SM shares
// neighbourhood positions in its L1, but runs of 2, 4 and 8 measured slower
// than single items on the 4M-node workload: load balance wins).
#ifndef IRR_CLAIM_CHUNK
#define IRR_CLAIM_CHUNK 1
#endif
constexpr int kClaimChunk = IRR_CLAIM_CHUNK;
constexpr int kPipeThreads = (kConsumerWarps + 1) * 32;

// The rows of one work item that belong to consumer warp `cw`.
template <bool PERIODIC, int G>
__device__ __forceinline__ void consume_item(const WorkItem& w, const InstHot& I,
                                             const int32_t* cols, uint32_t shift, int cw, int lane32)
{
    constexpr int kGroupsPerWarp = 32 / G;
    constexpr int kGroups = kConsumerWarps * kGroupsPerWarp;
    const int lane = lane32 % G;
    const int gid = cw * kGroupsPerWarp + lane32 / G;
    const float4* __restrict__ pos = I.pos;
    const uint32_t* __restrict__ row_off = I.row_off;
    float4* __restrict__ force = I.force;
    const LawParams* __restrict__ cold = I.cold;
    const HotLaw H = I.H;
    const int rounds = (w.nrows + kGroups - 1) / kGroups;
    for (int q = 0; q < rounds; q++) {
        const int rl = q * kGroups + gid;
        const bool valid = rl < w.nrows;
        const int64_t r = (int64_t)w.row0 + rl;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t beg = 0, end = 0;
        if (valid) {
            a = __ldg(pos + r);
            beg = __ldg(row_off + r);
            end = __ldg(row_off + r + 1);
        }
        const float3 f = row_sum<PERIODIC, G>(pos, cols, shift, a, beg, end, lane, H, cold);
        if (valid && lane == 0) force[r] = make_float4(f.x, f.y, f.z, 0.f);
    }
}

// One lane's entry pair of a slice step, as a single 8-byte load (kept whole
// so the two halves are not split into separately predicated loads).  The
// shared form is volatile: it must stay after the stage's mbarrier wait
// (itself volatile asm), which the compiler could otherwise move it across.
template <bool SHARED>
__device__ __forceinline__ int2 load_pair(const int2* p)
{
    int2 c;
    if (SHARED)
        asm volatile("ld.shared.v2.b32 {%0, %1}, [%2];" : "=r"(c.x), "=r"(c.y) : "r"(smem_u32(p)));
    else
        asm("ld.global.nc.v2.b32 {%0, %1}, [%2];" : "=r"(c.x), "=r"(c.y) : "l"(p));
    return c;
}

// The slices of a sliced work item that belong to consumer warp `cw` (one
// slice per warp at a time: lane i*G + l serves row i of the slice).  Word w
// of the instance's sliced array is words[w - shift] (shared memory when
// SHARED).  Each step is one 8-byte load per lane of a contiguous 256-byte
// line; the trip count is the slice's, uniform across the warp, and slots
// past a row's end (padding: the row's own id) are masked.
template <bool PERIODIC, int G, bool SHARED>
__device__ __forceinline__ void consume_sliced(const WorkItem& w, const InstHot& I,
                                               const int32_t* words, uint32_t shift, int cw,
                                               int lane32)
{
    constexpr int R = 32 / G;
    const int lane = lane32 % G;
    const float4* __restrict__ pos = I.pos;
    const uint32_t* __restrict__ row_off = I.row_off;
    const uint32_t* __restrict__ slice_off = I.slice_off;
    float4* __restrict__ force = I.force;
    const LawParams* __restrict__ cold = I.cold;
    const int64_t n = I.n;
    const HotLaw H = I.H;
    const int s0 = w.row0 / R;
    const int ns = (w.nrows + R - 1) / R;
    for (int q = cw; q < ns; q += kConsumerWarps) {
        const uint32_t o0 = __ldg(slice_off + s0 + q);
        const uint32_t steps = (__ldg(slice_off + s0 + q + 1) - o0) >> 6;
        const int64_t r = (int64_t)(s0 + q) * R + lane32 / G;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t len = 0;
        if (r < n) {
            a = __ldg(pos + r);
            len = __ldg(row_off + r + 1) - __ldg(row_off + r);
        }
        const int2* line = reinterpret_cast<const int2*>(words + (o0 - shift)) + lane32;
        float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
        // entry 2Gt + lane (+ G) of the row exists for t < n0 (n1)
        const uint32_t n0 = len > (uint32_t)lane ? (len - (uint32_t)lane + 2 * G - 1) / (2 * G) : 0u;
        const uint32_t n1 = len > (uint32_t)(lane + G) ? (len - (uint32_t)lane - G + 2 * G - 1) / (2 * G) : 0u;
        if constexpr (SHARED) {
            // step t's pair at shared address base + 256 t: the masks as
            // bounds on it, no index arithmetic in the loop
            uint32_t sa = smem_u32(line);
            const uint32_t lim0 = sa + 256u * n0, lim1 = sa + 256u * n1, send = sa + 256u * steps;
            for (; sa != send; sa += 256u) {
                int2 c;
                asm volatile("ld.shared.v2.b32 {%0, %1}, [%2];" : "=r"(c.x), "=r"(c.y) : "r"(sa));
                const float4 b0 = __ldg(pos + c.x);
                const float4 b1 = __ldg(pos + c.y);
                lj_pair<PERIODIC>(a, b0, b1, sa < lim0, sa < lim1, H, cold, ax, ay, az);
            }
        } else {
            for (uint32_t t = 0; t < steps; t++) {
                const int2 c = load_pair<false>(line + 32 * t);
                const float4 b0 = __ldg(pos + c.x);
                const float4 b1 = __ldg(pos + c.y);
                lj_pair<PERIODIC>(a, b0, b1, t < n0, t < n1, H, cold, ax, ay, az);
            }
        }
        const float3 f = join_partials<G>(ax, ay, az);
        if (r < n && lane == 0) force[r] = make_float4(f.x, f.y, f.z, 0.f);
    }
}

// Persistent owner-computes kernel, warp-specialised.  Warp kConsumerWarps is
// the producer: its lane 0 claims runs of kClaimChunk consecutive work items
// from *queue, and for each item waits until its ring stage is empty,
// publishes the item id and
// either bulk-copies the item's entry segment (widened to 16-byte bounds)
// into the stage -- the stage's `full` mbarrier completes on the byte count --
// or, for items read from global memory, just arrives.  The consumer warps
// walk the ring independently: wait `full`, sum their share of the item's
// rows, arrive on `empty` (kConsumerWarps arrivals free the stage).  Waits
// suspend the thread until the phase completes (mbar_try_wait).  Every
// wait is bounded; a wait that gives up sets kStatusWaitTimeout, waits once
// more (bounded) for a copy that may be in flight, and leaves.  wait_ns
// bounds each wait; withhold != 0 (a test of that path) makes every producer
// leave before publishing its first stage, so every consumer's first wait
// runs out and the launch ends with kStatusWaitTimeout and nothing in flight.
//
// Src (SrcGlobal, SrcOne, SrcTable): where the instance fields come from.
template <bool PERIODIC, int G, class Src>
__global__ void __launch_bounds__(kPipeThreads, kCtasPerSm) tiled_kernel(
    const InstDesc* __restrict__ insts, const WorkItem* __restrict__ items, int num_items,
    int* queue, int* status, int use_stages, uint64_t wait_ns, int withhold,
    const __grid_constant__ Src src)
{
    constexpr bool ONE = std::is_same<Src, SrcOne>::value;
    constexpr bool TABLE = std::is_same<Src, SrcTable>::value;
    extern __shared__ int4 smem_raw[];
    int32_t* stage_base = reinterpret_cast<int32_t*>(smem_raw);
    constexpr int kStageInts = kStageEntries + kColPad;
    __shared__ uint64_t full[kStages];
    __shared__ uint64_t empty[kStages];
    __shared__ int s_item[kStages];
    __shared__ int s_smem[kStages];
    const int warp = threadIdx.x / 32;
    const int lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kConsumerWarps);
        }
    }
    __syncthreads();

    if (warp == kConsumerWarps) {
        if (lane != 0 || withhold) return;
        int next_item = 0, chunk_left = 0;
        for (int k = 0;; k++) {
            const int s = k % kStages;
            const int use = k / kStages;
            if (use > 0 && !mbar_wait_bounded(&empty[s], (uint32_t)(use - 1) & 1u, wait_ns)) {
                atomicOr(status, kStatusWaitTimeout);
                return;  // nothing of this stage is in flight: its last copy was consumed
            }
            if (chunk_left == 0) {  // a run of kClaimChunk consecutive items
                const long long first = (long long)atomicAdd(queue, 1) * kClaimChunk;
                next_item = first < num_items ? (int)first : num_items;
                chunk_left = kClaimChunk;
            }
            const int it = next_item++;
            chunk_left--;
            s_item[s] = it;
            bool issue = false;
            if (it < num_items && use_stages) {
                const WorkItem w = items[it];
                issue = !(w.flags & kItemDirect);
                if (issue) {
                    s_smem[s] = 1;
                    const uint32_t a0 = w.ent0 & ~3u;
                    const uint32_t words = ((w.ent0 + w.nent - a0) + 3u) & ~3u;
                    const InstDesc* I;
                    if constexpr (ONE) I = &src.d;
                    else I = insts + w.inst;
                    const int32_t* ent = (w.flags & kItemSliced) ? I->scol : I->col;
                    bulk_load(stage_base + s * kStageInts, ent + a0, words * 4u, &full[s]);
                }
            }
            if (!issue) {
                s_smem[s] = 0;
                mbar_arrive(&full[s]);
            }
            if (it >= num_items) return;
        }
    }

    int cur = -1;  // instance whose fields `hot` holds
    InstHot hot{};
    for (int k = 0;; k++) {
        const int s = k % kStages;
        if (!mbar_wait_bounded(&full[s], (uint32_t)(k / kStages) & 1u, wait_ns)) {
            if (lane == 0) atomicOr(status, kStatusWaitTimeout);
            mbar_wait_bounded(&full[s], (uint32_t)(k / kStages) & 1u, wait_ns);
            return;
        }
        const int it = s_item[s];
        if (it >= num_items) return;
        const WorkItem w = items[it];
        const InstDesc* I;
        if constexpr (ONE) {
            I = &src.d;
            hot = load_hot(I);
        } else if constexpr (TABLE) {
            I = insts + w.inst;
            hot = hot_from(src, insts, w.inst);
        } else {
            I = insts + w.inst;
            if (w.inst != cur) {
                hot = load_hot(I);
                cur = w.inst;
            }
        }
        if (w.flags & kItemSliced) {
            if (s_smem[s])
                consume_sliced<PERIODIC, G, true>(w, hot, stage_base + s * kStageInts, w.ent0, warp,
                                                  lane);
            else
                consume_sliced<PERIODIC, G, false>(w, hot, I->scol, 0u, warp, lane);
        } else if (s_smem[s]) {
            consume_item<PERIODIC, G>(w, hot, stage_base + s * kStageInts, w.ent0 & ~3u, warp, lane);
        } else {
            consume_item<PERIODIC, G>(w, hot, I->col, 0u, warp, lane);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
}

// ---- staged ("halo") layout: positions staged in shared memory ----
//
// halo_kernel: the same persistent, warp-specialised owner-computes reduction
// over the staged layout (irr_staged.cu).  Per work item the producer warp
// bulk-copies the item's words (headers and 16-bit table offsets) into the
// stage, and its 32 lanes gather the item's table -- the positions of every
// node its rows touch, ~465 for 64 rows -- with 16-byte cp.async copies into
// the stage's table; the stage's `full` barrier completes when the bulk copy's
// bytes and all 32 lanes' copies have landed (1 + 32 arrivals).  The
// consumers read each entry's position from shared memory (a 128-bit load at
// a table offset), so the law's operands arrive in tens of cycles instead of
// an L1 miss's hundreds, and the entry order of the layout spreads each
// quarter-warp's 8 loads over the 8 bank groups.  G = 4 lanes per row.
constexpr int kHaloStageWords = kHaloStreamMax + 4 * kHaloTabMax;  // 32-bit words per stage
// The consumers add a table's address to both 16-bit halves of a word at once,
// which needs every shared address of the CTA below 2^16: the stages, the id
// buffers, the barriers and the system's reserved kilobyte.
#ifndef IRR_HALO_PAIR_ADDR
#define IRR_HALO_PAIR_ADDR 1
#endif
static_assert(!IRR_HALO_PAIR_ADDR ||
                  kHaloStages * kHaloStageWords * 4 + kHaloStages * (kHaloTabMax + 8) * 4 + 1024 + 1024 <
                      65536,
              "shared addresses fit 16 bits");
static_assert(8 * kHaloSlicesPerItem <= 64, "a row's index in its item fits the header's 6 bits");

__device__ __forceinline__ void cp_async16(uint32_t dst_smem, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst_smem), "l"(src) : "memory");
}

// One arrival on `bar` once every cp.async this thread issued before has
// landed (noinc: the barrier's expected count includes it).
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar)
{
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Shared loads kept after the stage's barrier wait (volatile, like load_pair).
__device__ __forceinline__ uint32_t lds32(uint32_t addr)
{
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
    return v;
}

__device__ __forceinline__ float4 lds128(uint32_t addr)
{
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(addr));
    return v;
}

// The slices of a staged work item (first row row0, nrows rows) that consumer
// warp `lane32`'s warp claims from the stage's counter *claim (a warp done
// with one slice takes the next unclaimed one, so the item's slices of
// different lengths spread over the warps); `sw` is the stage (words, then
// the table at word kHaloStreamMax) and soff the slices' word offsets within
// it.  Two 16-bit table offsets of a word become shared addresses with one
// add: every address of the CTA's shared window is below 2^16, so the low
// half cannot carry into the high one.
// Build-time variants (each an equal amount of work):
//   IRR_HALO_DYNAMIC   1: warps claim slices from the stage's counter;
//                      0: warp w takes slices w, w + 8, ...
//   IRR_HALO_PAIR_ADDR 1: one add forms both table addresses of a word;
//   IRR_HALO_UNROLL    the step loop's unroll factor;
//   IRR_HALO_CWAIT     the consumers' stage wait polls with a sleep of up to
//                      this many ns (0: suspend-hinted polls, no sleep);
//   IRR_HALO_PWAIT     the same for the producer's wait for a free stage.
// On the 4M-node workload (ms per step): static 0.396 vs dynamic 0.414 slice
// claims; pair addresses 0.391 vs 0.396; 7 consumer warps 0.455 and 3 CTAs
// per SM 0.415 vs 8 warps x 4 CTAs 0.396; rotated claims 0.3877 vs 0.3899;
// the step loop unrolled by 2 (spills) 0.421; the steps that every row of a
// slice fills split off into a loop without the entry masks (spills) 0.410;
// sleep-free waits 0.393, and polls that sleep up to 128 ns to 2 us between
// tests all 0.3875-0.3878; the entry masks as per-slice step-count bounds
// (t < n0, t < n1 instead of 8t + lane < len) 0.4163, but as bounds on the
// step's word address, which the loop advances anyway (no step counter or
// index add left), 0.3736 vs 0.3876 -- the loop below; 3-stage
// rings (3 CTAs per SM, or smaller items at 4) 0.395-0.431; 4 or 6 consumer
// warps with 6 or 7 CTAs per SM 0.413-0.418; each item's steps cut evenly
// across the warps (slices split between warps, piece sums joined in shared
// memory) 0.722: the extra state around the step loop doubled its
// instructions.  The words prefetched into L2 one item ahead: 0.3907 vs
// 0.3873.  A table ring one buffer deeper than the word ring, each item's
// table gathered one item ahead (limits 3072 words / 576 ids to fit 4 CTAs
// per SM): 0.403, vs 0.3888 for this kernel at those limits and 0.3874 at
// 3584 / 640 -- the refill is not bounded by the table gather alone.  What the warps still lose is the ring's coupling: a stage is
// refilled only when its slowest warp is done (~4.3K cycles after the first),
// and the refill takes ~3.6K cycles, so the first warps wait ~1.2K of each
// item's ~7.6K cycles.
#ifndef IRR_HALO_DYNAMIC
#define IRR_HALO_DYNAMIC 0
#endif
// IRR_HALO_ROTATE 1: with static claims, warp w takes slice (w + k) mod 8 of
// the CTA's k-th item (slice 0 holds an item's longest rows, so a fixed
// assignment would always give warp 0 the longest slice).
#ifndef IRR_HALO_ROTATE
#define IRR_HALO_ROTATE 1
#endif
// IRR_HALO_PREFETCH 1: when the producer claims an item (one item ahead), it
// also prefetches the item's words into L2, so that their bulk copy, issued
// once a stage is free, reads L2 rather than DRAM.
#ifndef IRR_HALO_PREFETCH
#define IRR_HALO_PREFETCH 0
#endif

#ifndef IRR_HALO_UNROLL
#define IRR_HALO_UNROLL 1
#endif
constexpr int kHaloUnroll = IRR_HALO_UNROLL;
#ifndef IRR_HALO_CWAIT
#define IRR_HALO_CWAIT 128
#endif
#ifndef IRR_HALO_PWAIT
#define IRR_HALO_PWAIT 256
#endif

// A bounded wait that sleeps up to MAX_NS between polls, or (MAX_NS == 0)
// polls with the suspend hint only.
template <uint32_t MAX_NS>
__device__ __forceinline__ bool mbar_wait_policy(uint64_t* bar, uint32_t parity, uint64_t limit_ns)
{
    if constexpr (MAX_NS == 0) return mbar_wait_bounded(bar, parity, limit_ns);
    else return mbar_wait_backoff<MAX_NS>(bar, parity, limit_ns);
}

// The two neighbours of a lane's step: one word of two 16-bit table byte
// offsets, then the two positions from the table.
__device__ __forceinline__ void halo_operands(uint32_t addr, uint32_t tab_u32, uint32_t tab_pair, float4& b0,
                                              float4& b1)
{
    if (IRR_HALO_PAIR_ADDR) {
        const uint32_t wd = lds32(addr) + tab_pair;
        b0 = lds128(wd & 0xffffu);
        b1 = lds128(wd >> 16);
    } else {
        const uint32_t wd = lds32(addr);
        b0 = lds128(tab_u32 + (wd & 0xffffu));
        b1 = lds128(tab_u32 + (wd >> 16));
    }
}

template <bool PERIODIC>
__device__ __forceinline__ void consume_halo(int row0, int nrows, const uint32_t* soff, int* claim,
                                             const InstHot& I, const uint32_t* sw, int lane32,
                                             int first)
{
    const int lane = lane32 & 3;
    float4* __restrict__ force = I.force;
    const LawParams* __restrict__ cold = I.cold;
    const HotLaw H = I.H;
    const uint32_t words_u32 = smem_u32(sw);
    const uint32_t tab_u32 = smem_u32(sw + kHaloStreamMax);
    const uint32_t tab_pair = tab_u32 * 0x10001u;  // the table's address in both halves
    const int ns = (nrows + 7) / 8;
    for (int qs = first;; qs += kConsumerWarps) {
        int q = qs;
        if (IRR_HALO_DYNAMIC) {
            if (lane32 == 0) q = atomicAdd(claim, 1);
            q = __shfl_sync(0xffffffffu, q, 0);
        }
        if (q >= ns) break;
        const uint32_t o0 = soff[q];
        const uint32_t steps = ((soff[q + 1] - o0) >> 5) - 1;
        uint32_t addr = words_u32 + 4u * (o0 + (uint32_t)lane32);
        // header: own byte offset | len << 14 | row-in-item << 24 (1 << 31: padding)
        const uint32_t hdr = lds32(addr);
        const float4 a = lds128(tab_u32 + (hdr & 0x3fffu));
        const uint32_t len = (hdr >> 14) & 0x3ffu;
        const int64_t r = (int64_t)row0 + ((hdr >> 24) & 0x3fu);
        float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
        // entry 8t + lane (+ 4) of the row exists for t < n0 (n1): as bounds on
        // step t's word address, base + 128 (t + 1), they cost no index
        // arithmetic in the loop (8t + lane < len per step measured 3.5 %
        // slower at 4M nodes)
        const uint32_t n0 = len > (uint32_t)lane ? (len - (uint32_t)lane + 7u) >> 3 : 0u;
        const uint32_t n1 = len > (uint32_t)lane + 4u ? (len - (uint32_t)lane + 3u) >> 3 : 0u;
        const uint32_t lim0 = addr + 128u * n0, lim1 = addr + 128u * n1, end = addr + 128u * steps;
#pragma unroll kHaloUnroll
        for (; addr != end;) {
            addr += 128u;
            float4 b0, b1;
            halo_operands(addr, tab_u32, tab_pair, b0, b1);
            lj_pair<PERIODIC>(a, b0, b1, addr <= lim0, addr <= lim1, H, cold, ax, ay, az);
        }
        const float3 f = join_partials<4>(ax, ay, az);
        if (!(hdr >> 31) && lane == 0) force[r] = make_float4(f.x, f.y, f.z, 0.f);
    }
}

template <bool PERIODIC, class Src>
__global__ void __launch_bounds__(kPipeThreads, kCtasPerSm) halo_kernel(
    const InstDesc* __restrict__ insts, const WorkItem* __restrict__ items, int num_items,
    int* queue, int* status, uint64_t wait_ns, int withhold, const __grid_constant__ Src src)
{
    constexpr bool ONE = std::is_same<Src, SrcOne>::value;
    constexpr bool TABLE = std::is_same<Src, SrcTable>::value;
    extern __shared__ int4 smem_raw[];
    uint32_t* stage_base = reinterpret_cast<uint32_t*>(smem_raw);
    __shared__ uint64_t full[kHaloStages];
    __shared__ uint64_t empty[kHaloStages];
    __shared__ int s_item[kHaloStages];
    // per stage: the item's (instance, first row, rows) and its slices' word
    // offsets within the stage, so that the consumers read no global memory
    __shared__ int4 s_meta[kHaloStages];
    __shared__ uint32_t s_soff[kHaloStages][kHaloSlicesPerItem + 1];
    // per stage: the item's table ids (bulk-copied in whole 16-byte words, so
    // up to 3 ids before and after them), read by the producer's lanes
    __shared__ __align__(16) int32_t s_ids[kHaloStages][kHaloTabMax + 8];
    __shared__ uint64_t idsbar[kHaloStages];
    __shared__ int s_claim[kHaloStages];  // the next unclaimed slice of the stage's item
    const int warp = threadIdx.x / 32;
    const int lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kHaloStages; s++) {
            mbar_init(&full[s], 33);  // the bulk copy's arrive + one per producer lane
            mbar_init(&empty[s], kConsumerWarps);
            mbar_init(&idsbar[s], 1);
        }
    }
    __syncthreads();

    if (warp == kConsumerWarps) {
        if (withhold) return;
        // Item k + 1 is prepared while item k's copies are in flight: its
        // claim, its descriptor, its slices' word offsets (lane j holds the
        // j-th) and the bulk copy of its table ids into s_ids, so that the
        // lanes can issue item k + 1's position copies without waiting on
        // memory once its stage is free.
        int nxt = 0;
        WorkItem wn{};
        uint32_t soff_n = 0;
        auto prepare = [&](int stage) {
            nxt = __shfl_sync(0xffffffffu, nxt, 0);
            if (nxt >= num_items) return;
            wn = items[nxt];
            const InstDesc* In;
            if constexpr (ONE) In = &src.d;
            else In = insts + wn.inst;
            const int ns = (wn.nrows + 7) / 8;
            soff_n = (lane <= ns && lane <= kHaloSlicesPerItem)
                         ? __ldg(In->slice_off + wn.row0 / 8 + lane) - wn.ent0
                         : 0u;
            if (lane == 0) {  // whole 16-byte words around the item's ids
                const uint32_t a0 = wn.tab0 & ~3u;
                const uint32_t cnt = ((wn.tab0 & 3u) + wn.ntab + 3u) & ~3u;
                bulk_load(s_ids[stage], In->tab + a0, cnt * 4u, &idsbar[stage]);
                if (IRR_HALO_PREFETCH)
                    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(In->words + wn.ent0),
                                 "r"(wn.nent * 4u)
                                 : "memory");
            }
        };
        if (lane == 0) nxt = atomicAdd(queue, 1);
        prepare(0);
        for (int k = 0;; k++) {
            const int s = k % kHaloStages;
            const int use = k / kHaloStages;
            const int it = nxt < num_items ? nxt : num_items;
            const WorkItem w = wn;
            const uint32_t so = soff_n;
            int ok = 1;
            if (lane == 0 && use > 0)
                ok = mbar_wait_policy<IRR_HALO_PWAIT>(&empty[s], (uint32_t)(use - 1) & 1u, wait_ns) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {  // a wait gave up: leave with none of this lane's copies in flight
                if (lane == 0) atomicOr(status, kStatusWaitTimeout);
                mbar_wait_backoff<256>(&idsbar[s], (uint32_t)use & 1u, wait_ns);
                asm volatile("cp.async.wait_all;" ::: "memory");
                return;
            }
            if (lane == 0) s_item[s] = it;
            if (it >= num_items) {  // no more work: complete the stage's phase for the consumers
                if (lane == 0) mbar_arrive(&full[s]);
                mbar_arrive(&full[s]);
                asm volatile("cp.async.wait_all;" ::: "memory");
                return;
            }
            if (lane == 0) nxt = atomicAdd(queue, 1);  // item k + 1: the claim is in flight
            const InstDesc* I;
            if constexpr (ONE) I = &src.d;
            else I = insts + w.inst;
            uint32_t* sw = stage_base + s * kHaloStageWords;
            // the metadata, written before the stage is published: lane 0's
            // arrive (release) follows every lane's writes through __syncwarp
            const int ns = (w.nrows + 7) / 8;
            if (lane <= ns && lane <= kHaloSlicesPerItem) s_soff[s][lane] = so;
            if (lane == 0) {
                s_meta[s] = make_int4(w.inst, w.row0, w.nrows, 0);
                s_claim[s] = 0;  // every consumer has left the stage's previous item
            }
            __syncwarp();
            if (lane == 0) bulk_load(sw, I->words + w.ent0, w.nent * 4u, &full[s]);
            // the table: its ids arrived by the bulk copy of the iteration before
            if (!mbar_wait_backoff<64>(&idsbar[s], (uint32_t)use & 1u, wait_ns)) {
                if (lane == 0) atomicOr(status, kStatusWaitTimeout);
                asm volatile("cp.async.wait_all;" ::: "memory");
                return;  // the consumers' wait for this stage runs out too
            }
            const uint32_t tab_u32 = smem_u32(sw + kHaloStreamMax);
            const int32_t* ids = s_ids[s] + (w.tab0 & 3u);
            const float4* __restrict__ pos = I->pos;
            for (uint32_t j = lane; j < w.ntab; j += 32) cp_async16(tab_u32 + 16u * j, pos + ids[j]);
            cp_async_arrive(&full[s]);
            prepare((k + 1) % kHaloStages);
        }
    }

    int cur = -1;
    InstHot hot{};
    for (int k = 0;; k++) {
        const int s = k % kHaloStages;
        if (!mbar_wait_policy<IRR_HALO_CWAIT>(&full[s], (uint32_t)(k / kHaloStages) & 1u, wait_ns)) {
            if (lane == 0) atomicOr(status, kStatusWaitTimeout);
            mbar_wait_policy<IRR_HALO_CWAIT>(&full[s], (uint32_t)(k / kHaloStages) & 1u, wait_ns);
            return;
        }
        const int it = s_item[s];
        if (it >= num_items) return;
        const int4 m = s_meta[s];  // instance, first row, rows
        if constexpr (ONE) {
            hot = load_hot(&src.d);
        } else if constexpr (TABLE) {
            hot = hot_from(src, insts, m.x);
        } else if (m.x != cur) {
            hot = load_hot(insts + m.x);
            cur = m.x;
        }
        consume_halo<PERIODIC>(m.y, m.z, s_soff[s], &s_claim[s], hot, stage_base + s * kHaloStageWords, lane,
                               IRR_HALO_ROTATE ? (warp + k) % kConsumerWarps : warp);
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
}

template <bool PERIODIC, class Src>
cudaError_t launch_halo_src(const InstDesc* d_insts, const WorkItem* d_items, int num_items,
                            int* d_queue, int grid, int* d_status, cudaStream_t s, const Src& src,
                            const WaitPolicy& wp)
{
    auto kern = halo_kernel<PERIODIC, Src>;
    const size_t smem = (size_t)kHaloStages * kHaloStageWords * sizeof(uint32_t);
    IRR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (grid <= 0 || num_items <= 0) return cudaSuccess;
    kern<<<grid, kPipeThreads, smem, s>>>(d_insts, d_items, num_items, d_queue, d_status,
                                          wp.wait_ns, wp.withhold, src);
    return cudaGetLastError();
}

template <bool PERIODIC>
cudaError_t launch_halo_p(const InstDesc* d_insts, const WorkItem* d_items, int num_items,
                          int* d_queue, int grid, int* d_status, cudaStream_t s,
                          const InstDesc* host_insts, int num_insts, const WaitPolicy& wp)
{
    if (host_insts && num_insts == 1)
        return launch_halo_src<PERIODIC>(d_insts, d_items, num_items, d_queue, grid, d_status, s,
                                         SrcOne{host_insts[0]}, wp);
    if (host_insts && num_insts > 1 && num_insts <= kTableInsts) {
        static thread_local SrcTable t;
        for (int k = 0; k < num_insts; k++) {
            const InstDesc& d = host_insts[k];
            t.h[k] = HotEntry{d.pos, HotLaw{d.law.half2, d.law.rc2, d.law.band}, 0.f};
        }
        return launch_halo_src<PERIODIC>(d_insts, d_items, num_items, d_queue, grid, d_status, s, t,
                                         wp);
    }
    return launch_halo_src<PERIODIC>(d_insts, d_items, num_items, d_queue, grid, d_status, s,
                                     SrcGlobal{0}, wp);
}

template <bool PERIODIC, int G, class Src>
cudaError_t launch_tiled_src(const TiledShape& shape, const InstDesc* d_insts,
                             const WorkItem* d_items, int num_items, int* d_queue, int grid,
                             int* d_status, cudaStream_t s, const Src& src, const WaitPolicy& wp)
{
    auto kern = tiled_kernel<PERIODIC, G, Src>;
    const size_t smem =
        shape.stage_smem ? (size_t)kStages * (kStageEntries + kColPad) * sizeof(int32_t) : 0;
    if (smem > 48 * 1024)
        IRR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    if (grid <= 0 || num_items <= 0) return cudaSuccess;
    kern<<<grid, kPipeThreads, smem, s>>>(d_insts, d_items, num_items, d_queue, d_status,
                                          shape.stage_smem, wp.wait_ns, wp.withhold, src);
    return cudaGetLastError();
}

template <bool PERIODIC, int G>
cudaError_t launch_tiled_g(const TiledShape& shape, const InstDesc* d_insts,
                           const WorkItem* d_items, int num_items, int* d_queue, int grid,
                           int* d_status, cudaStream_t s, const InstDesc* host_insts,
                           int num_insts, const WaitPolicy& wp)
{
    if (host_insts && num_insts == 1)
        return launch_tiled_src<PERIODIC, G>(shape, d_insts, d_items, num_items, d_queue, grid,
                                             d_status, s, SrcOne{host_insts[0]}, wp);
    if (host_insts && num_insts > 1 && num_insts <= kTableInsts) {
        static thread_local SrcTable t;  // 28 KB: kept off the stack
        for (int k = 0; k < num_insts; k++) {
            const InstDesc& d = host_insts[k];
            t.h[k] = HotEntry{d.pos, HotLaw{d.law.half2, d.law.rc2, d.law.band}, 0.f};
        }
        return launch_tiled_src<PERIODIC, G>(shape, d_insts, d_items, num_items, d_queue, grid,
                                             d_status, s, t, wp);
    }
    return launch_tiled_src<PERIODIC, G>(shape, d_insts, d_items, num_items, d_queue, grid,
                                         d_status, s, SrcGlobal{0}, wp);
}

template <bool PERIODIC>
cudaError_t launch_tiled_p(const TiledShape& sh, const InstDesc* a, const WorkItem* b, int n,
                           int* q, int grid, int* st, cudaStream_t s, const InstDesc* hi, int ni,
                           const WaitPolicy& wp)
{
    switch (sh.lanes_per_row) {
    case 1: return launch_tiled_g<PERIODIC, 1>(sh, a, b, n, q, grid, st, s, hi, ni, wp);
    case 2: return launch_tiled_g<PERIODIC, 2>(sh, a, b, n, q, grid, st, s, hi, ni, wp);
    case 4: return launch_tiled_g<PERIODIC, 4>(sh, a, b, n, q, grid, st, s, hi, ni, wp);
    case 8: return launch_tiled_g<PERIODIC, 8>(sh, a, b, n, q, grid, st, s, hi, ni, wp);
    case 16: return launch_tiled_g<PERIODIC, 16>(sh, a, b, n, q, grid, st, s, hi, ni, wp);
    case 32: return launch_tiled_g<PERIODIC, 32>(sh, a, b, n, q, grid, st, s, hi, ni, wp);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_plain(const float4* pos, const int2* edges, int64_t e, float4* force,
                         const LawParams& law, cudaStream_t s)
{
    if (e <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    IRR_CUDA_TRY(cudaGetDevice(&dev));
    IRR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t want = (e + 255) / 256;
    const int grid = (int)(want < (int64_t)sms * 32 ? want : (int64_t)sms * 32);
    if (law.periodic)
        plain_kernel<true><<<grid, 256, 0, s>>>(pos, edges, e, force, law);
    else
        plain_kernel<false><<<grid, 256, 0, s>>>(pos, edges, e, force, law);
    return cudaGetLastError();
}

cudaError_t launch_tiled(const TiledShape& shape, const InstDesc* d_insts,
                         const WorkItem* d_items, int num_items, int* d_queue, int grid,
                         int* d_status, cudaStream_t s, const InstDesc* host_insts, int num_insts,
                         const WaitPolicy& wp)
{
    if (!d_queue) return cudaErrorInvalidValue;
    if (shape.staged) {
        if (shape.lanes_per_row != 4) return cudaErrorInvalidValue;
        return shape.periodic ? launch_halo_p<true>(d_insts, d_items, num_items, d_queue, grid,
                                                    d_status, s, host_insts, num_insts, wp)
                              : launch_halo_p<false>(d_insts, d_items, num_items, d_queue, grid,
                                                     d_status, s, host_insts, num_insts, wp);
    }
    return shape.periodic ? launch_tiled_p<true>(shape, d_insts, d_items, num_items, d_queue, grid,
                                                 d_status, s, host_insts, num_insts, wp)
                          : launch_tiled_p<false>(shape, d_insts, d_items, num_items, d_queue,
                                                  grid, d_status, s, host_insts, num_insts, wp);
}

void make_work_items(const uint32_t* row_off, int64_t n, int inst, int max_rows, int staged,
                     std::vector<WorkItem>& out, int round_rows)
{
    int64_t r = 0;
    while (r < n) {
        WorkItem w{};
        w.inst = inst;
        w.row0 = (int32_t)r;
        w.ent0 = row_off[r];
        int64_t q = r + 1;
        if ((int64_t)(row_off[q] - row_off[r]) > kStageEntries) {
            w.flags = kItemDirect;  // one long row: read from global memory
        } else {
            while (q < n && q - r < max_rows && (int64_t)(row_off[q + 1] - row_off[r]) <= kStageEntries)
                q++;
            if (q < n && q - r > round_rows) q = r + (q - r) / round_rows * round_rows;
        }
        w.nrows = (int32_t)(q - r);
        w.nent = row_off[q] - row_off[r];
        if (!staged || w.nent == 0) w.flags |= kItemDirect;
        out.push_back(w);
        r = q;
    }
}

void make_instance_items(const uint32_t* host_row_off, const Sliced& sl, int64_t n, int inst,
                         const TiledShape& shape, std::vector<WorkItem>& out)
{
    if (sl.lanes != 0 && sl.lanes == shape.lanes_per_row)
        make_sliced_items(sl, n, inst, shape.block_nodes, shape.stage_smem, out);
    else
        make_work_items(host_row_off, n, inst, shape.block_nodes, shape.stage_smem, out,
                        kConsumerSlices * (32 / shape.lanes_per_row));
}

void make_sliced_items(const Sliced& sl, int64_t n, int inst, int max_rows, int staged,
                       std::vector<WorkItem>& out)
{
    const int R = 32 / sl.lanes;
    const int64_t max_slices = std::max<int64_t>(1, max_rows / R);
    const uint32_t* off = sl.host_off.data();
    int64_t q = 0;
    while (q < sl.slices) {
        int64_t e = q + 1;
        if ((int64_t)(off[e] - off[q]) <= kStageEntries) {
            while (e < sl.slices && e - q < max_slices &&
                   (int64_t)(off[e + 1] - off[q]) <= kStageEntries)
                e++;
            // whole rounds of the consumer warps where the item allows it
            if (e < sl.slices && e - q > kConsumerSlices) e = q + (e - q) / kConsumerSlices * kConsumerSlices;
        }
        WorkItem w{};
        w.inst = inst;
        w.row0 = (int32_t)(q * R);
        w.nrows = (int32_t)(std::min<int64_t>(n, e * R) - q * R);
        w.ent0 = off[q];
        w.nent = off[e] - off[q];
        w.flags = kItemSliced;
        if (!staged || w.nent == 0 || (int64_t)w.nent > kStageEntries) w.flags |= kItemDirect;
        out.push_back(w);
        q = e;
    }
}

}  // namespace irr
