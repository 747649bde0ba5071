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
//   registers and combines the G partials with error-free TwoSum steps.  A
//   CTA takes a node block (a work item); optionally the block's positions
//   are first copied into shared memory with one bulk (TMA) copy.  Each edge
//   is evaluated from both ends -- the reference duplicates cross-part edges
//   the same way (moldyn/irregular/partitioner.cpp:142-297, paper Sec. II-A)
//   -- so no atomics are needed and every result is bitwise reproducible.
//   With a queue it is the persistent (instance, block) work-queue kernel of
//   the batched form, generalising the reference's per-part atomicAdd queue
//   (gpu_kernel.cu:60-77).
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

// Waits for phase `parity` of the barrier; gives up after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit)
{
    for (int i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

constexpr int kWaitPolls = 1 << 20;

template <bool PERIODIC, int G, bool STAGE, int UNROLL>
__global__ void __launch_bounds__(kTiledThreads) tiled_kernel(const InstDesc* __restrict__ insts,
                                                              const WorkItem* __restrict__ items,
                                                              int num_items, int* queue,
                                                              int* status)
{
    extern __shared__ float4 spos[];
    __shared__ uint64_t bar;
    __shared__ int s_item;
    constexpr int kGroups = kTiledThreads / G;
    const int tid = threadIdx.x;
    const int lane = tid % G;
    const int gid = tid / G;

    bool staged = STAGE;
    if (STAGE) {
        if (tid == 0) mbar_init(&bar, 1);
        __syncthreads();
    }
    uint32_t parity = 0;
    int it = blockIdx.x;
    for (;;) {
        if (queue) {
            if (tid == 0) s_item = atomicAdd(queue, 1);
            __syncthreads();
            it = s_item;
            __syncthreads();
        }
        if (it >= num_items) break;
        const WorkItem w = items[it];
        const float4* __restrict__ pos = insts[w.inst].pos;
        const uint32_t* __restrict__ row_off = insts[w.inst].row_off;
        const int32_t* __restrict__ col = insts[w.inst].col;
        float4* __restrict__ force = insts[w.inst].force;
        const LawParams law = insts[w.inst].law;
        const int nr = w.nrows;

        bool use_smem = false;
        if (STAGE && staged) {
            if (tid == 0) bulk_load(spos, pos + w.row0, (uint32_t)nr * 16u, &bar);
            const bool ok = mbar_wait_bounded(&bar, parity, kWaitPolls);
            parity ^= 1u;
            // Uniform decision: if any thread gave up, the CTA stops staging
            // for good (a copy may still be in flight into spos).
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicOr(status, kStatusWaitTimeout);
                staged = false;
            } else {
                use_smem = true;
            }
        }

        const int rounds = (nr + kGroups - 1) / kGroups;
        for (int q = 0; q < rounds; q++) {
            const int rl = q * kGroups + gid;
            const bool valid = rl < nr;
            const int64_t r = (int64_t)w.row0 + rl;
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
            uint32_t beg = 0, end = 0;
            if (valid) {
                a = use_smem ? spos[rl] : __ldg(pos + r);
                beg = __ldg(row_off + r);
                end = __ldg(row_off + r + 1);
            }
            float ax = 0.f, ay = 0.f, az = 0.f;
            for (uint32_t k = beg + lane; k < end; k += G * UNROLL) {
                int32_t j[UNROLL];
#pragma unroll
                for (int u = 0; u < UNROLL; u++) {
                    const uint32_t kk = k + u * G;
                    j[u] = kk < end ? __ldcs(col + kk) : -1;
                }
                float4 b[UNROLL];
#pragma unroll
                for (int u = 0; u < UNROLL; u++) {
                    if (j[u] >= 0) {
                        const uint32_t jl = (uint32_t)(j[u] - w.row0);
                        b[u] = (use_smem && jl < (uint32_t)nr) ? spos[jl] : __ldg(pos + j[u]);
                    }
                }
#pragma unroll
                for (int u = 0; u < UNROLL; u++) {
                    if (j[u] >= 0) {
                        float dx, dy, dz;
                        const float s = lj_scalar<PERIODIC>(a, b[u], law, dx, dy, dz);
                        ax = fmaf(dx, s, ax);
                        ay = fmaf(dy, s, ay);
                        az = fmaf(dz, s, az);
                    }
                }
            }
            // Combine the G lane partials: TwoSum keeps each rounding error,
            // which is carried in (cx, cy, cz) and added back at the end.
            float cx = 0.f, cy = 0.f, cz = 0.f;
#pragma unroll
            for (int off = G / 2; off > 0; off >>= 1) {
                const float ox = __shfl_xor_sync(0xffffffffu, ax, off, G);
                const float oy = __shfl_xor_sync(0xffffffffu, ay, off, G);
                const float oz = __shfl_xor_sync(0xffffffffu, az, off, G);
                const float ocx = __shfl_xor_sync(0xffffffffu, cx, off, G);
                const float ocy = __shfl_xor_sync(0xffffffffu, cy, off, G);
                const float ocz = __shfl_xor_sync(0xffffffffu, cz, off, G);
                float e;
                two_sum(ax, ox, ax, e);
                cx = __fadd_rn(__fadd_rn(cx, ocx), e);
                two_sum(ay, oy, ay, e);
                cy = __fadd_rn(__fadd_rn(cy, ocy), e);
                two_sum(az, oz, az, e);
                cz = __fadd_rn(__fadd_rn(cz, ocz), e);
            }
            if (valid && lane == 0)
                force[r] = make_float4(__fadd_rn(ax, cx), __fadd_rn(ay, cy), __fadd_rn(az, cz),
                                       0.f);
        }
        if (!queue) break;
        __syncthreads();  // every thread is done with spos before it is refilled
    }
}

template <bool PERIODIC, int G, bool STAGE>
cudaError_t launch_tiled_t(const TiledShape& shape, const InstDesc* d_insts,
                           const WorkItem* d_items, int num_items, int* d_queue, int grid,
                           int* d_status, cudaStream_t s)
{
    constexpr int kUnroll = 2;
    auto kern = tiled_kernel<PERIODIC, G, STAGE, kUnroll>;
    const size_t smem = STAGE ? (size_t)shape.block_nodes * sizeof(float4) : 0;
    if (STAGE && smem > 48 * 1024)
        IRR_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    const int blocks = d_queue ? grid : num_items;
    if (blocks <= 0) return cudaSuccess;
    kern<<<blocks, kTiledThreads, smem, s>>>(d_insts, d_items, num_items, d_queue, d_status);
    return cudaGetLastError();
}

template <bool PERIODIC, int G>
cudaError_t launch_tiled_g(const TiledShape& sh, const InstDesc* a, const WorkItem* b, int n,
                           int* q, int grid, int* st, cudaStream_t s)
{
    return sh.stage_smem ? launch_tiled_t<PERIODIC, G, true>(sh, a, b, n, q, grid, st, s)
                         : launch_tiled_t<PERIODIC, G, false>(sh, a, b, n, q, grid, st, s);
}

template <bool PERIODIC>
cudaError_t launch_tiled_p(const TiledShape& sh, const InstDesc* a, const WorkItem* b, int n,
                           int* q, int grid, int* st, cudaStream_t s)
{
    switch (sh.lanes_per_row) {
    case 4: return launch_tiled_g<PERIODIC, 4>(sh, a, b, n, q, grid, st, s);
    case 8: return launch_tiled_g<PERIODIC, 8>(sh, a, b, n, q, grid, st, s);
    case 16: return launch_tiled_g<PERIODIC, 16>(sh, a, b, n, q, grid, st, s);
    case 32: return launch_tiled_g<PERIODIC, 32>(sh, a, b, n, q, grid, st, s);
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
                         int* d_status, cudaStream_t s)
{
    if (shape.stage_smem && (shape.block_nodes > kMaxStageNodes || shape.block_nodes < 1))
        return cudaErrorInvalidValue;
    return shape.periodic
               ? launch_tiled_p<true>(shape, d_insts, d_items, num_items, d_queue, grid, d_status, s)
               : launch_tiled_p<false>(shape, d_insts, d_items, num_items, d_queue, grid, d_status, s);
}

}  // namespace irr
