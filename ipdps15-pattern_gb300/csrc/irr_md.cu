// irr_md.cu -- Lennard-Jones molecular dynamics around the irregular reduction.
//
// The drivers' step loops (moldyn/moldyn.cu:331-407; miniMD/ljs.cu:171-176,
// whose integrator is commented out at ljs.cu:39) move positions on the host
// and call IrregularStart once per step.  Here the whole loop stays on the GPU:
//   kick + drift   v += dt/2 * F/m, x += dt * v, x wrapped into [0, L)   (FP64)
//   rebuild        every `rebuild_every` steps: GPU neighbour list at
//                  cutforce + skin, GPU partition (the atoms re-sorted along
//                  the Hilbert curve every reorder_every-th rebuild), state
//                  permuted into the new order
//   force          the owner-computes reduction (FP32 per edge, compensated)
//   kick           v += dt/2 * F/m                                       (FP64)
// F = 48 * (the reduction's d * (r^-14 - r^-8/2)), the LJ force at eps = sigma
// = 1, m = 1.  Energies and the virial are FP64 sums of FP32 per-edge terms.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "irr_md.cuh"
#include "irr_trace.cuh"

using namespace irr;

namespace {

int md_fail(irr_md* m, int code, const char* what, cudaError_t e = cudaSuccess)
{
    if (m) {
        m->err = what;
        if (e != cudaSuccess) {
            m->err += ": ";
            m->err += cudaGetErrorString(e);
        }
    }
    cudaGetLastError();
    return code;
}

#define MD_CUDA(m, expr, what)                                                            \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return md_fail((m), e_ == cudaErrorMemoryAllocation ? IRR_ERR_NOMEM : IRR_ERR_CUDA, \
                           what, e_);                                                     \
    } while (0)

int grid_of(int64_t n)
{
    int64_t g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 8192 ? 8192 : g));
}

// KICKS = 1: kick + drift of a step; KICKS = 2: also the closing kick of
// the step before (the same forces).
template <int KICKS>
__global__ void kick_drift_kernel(double* __restrict__ x, double* __restrict__ v,
                                  const float4* __restrict__ f, int64_t n, double dt, double L,
                                  float4* __restrict__ pos4)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        md_kick_drift_atom<KICKS>(x, v, f, i, dt, L, pos4);
}

// cnt[t] = entries of row t with a column above t (rows ascending: a suffix).
__global__ void half_count_kernel(const uint32_t* __restrict__ row_off, const int32_t* __restrict__ col,
                                  int64_t n, uint32_t* __restrict__ cnt)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t b = row_off[t], e = row_off[t + 1];
        uint32_t k = b;
        while (k < e && col[k] <= (int32_t)t) k++;
        cnt[t] = e - k;
    }
}

// half[off[t] ..] = (t, j) for the entries j > t of row t.
__global__ void half_write_kernel(const uint32_t* __restrict__ row_off, const int32_t* __restrict__ col,
                                  int64_t n, const uint32_t* __restrict__ off, int2* __restrict__ half)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t e = row_off[t + 1];
        const uint32_t k0 = e - (off[t + 1] - off[t]);
        for (uint32_t k = k0; k < e; k++) half[off[t] + (k - k0)] = make_int2((int)t, col[k]);
    }
}

__global__ void kick_kernel(double* __restrict__ v, const float4* __restrict__ f, int64_t n,
                            double dt)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        md_kick_atom(v, f, i, dt);
}

__global__ void to_float4_kernel(const double* __restrict__ x, int64_t n, double L,
                                 float4* __restrict__ pos4)
{
    const float Lf = (float)L;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float fx = (float)x[3 * i], fy = (float)x[3 * i + 1], fz = (float)x[3 * i + 2];
        if (fx >= Lf) fx = 0.f;
        if (fy >= Lf) fy = 0.f;
        if (fz >= Lf) fz = 0.f;
        pos4[i] = make_float4(fx, fy, fz, 0.f);
    }
}

// dst[k] = src[perm[k]] for 3-vectors and ids
__global__ void gather3_kernel(const double* __restrict__ src, const int32_t* __restrict__ perm,
                               int64_t n, double* __restrict__ dst)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = perm[k];
        dst[3 * k] = src[3 * s];
        dst[3 * k + 1] = src[3 * s + 1];
        dst[3 * k + 2] = src[3 * s + 2];
    }
}

__global__ void iota_ids_kernel(int32_t* __restrict__ ids, int64_t n)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        ids[k] = (int32_t)k;
}

__global__ void gather_ids_kernel(const int32_t* __restrict__ src, const int32_t* __restrict__ perm,
                                  int64_t n, int32_t* __restrict__ dst)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        dst[k] = src[perm[k]];
}

// out[ids[k]] = src[k]: back to the caller's atom order
__global__ void scatter3_kernel(const double* __restrict__ src, const int32_t* __restrict__ ids,
                                int64_t n, double* __restrict__ dst)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = ids[k];
        dst[3 * d] = src[3 * k];
        dst[3 * d + 1] = src[3 * k + 1];
        dst[3 * d + 2] = src[3 * k + 2];
    }
}

// SplitMix64's output mix (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014).
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// Digest of the positions by atom: the sum mod 2^64, over atoms k and
// components c, of mix64(bits(x) + golden * (3 * id + c + 1)).  Integer sums
// do not depend on their order, so the digest is a function of the state in
// the caller's atom order, whatever the execution order.
__global__ void state_digest_kernel(const double* __restrict__ x, const int32_t* __restrict__ ids,
                                    int64_t n, unsigned long long* out)
{
    uint64_t acc = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = 3ull * (uint64_t)ids[k];
#pragma unroll
        for (int c = 0; c < 3; c++)
            acc += mix64((uint64_t)__double_as_longlong(x[3 * k + c]) +
                         0x9e3779b97f4a7c15ull * (key + (uint64_t)c + 1ull));
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, (unsigned long long)acc);
}

__device__ __forceinline__ double block_sum(double v, double* red)
{
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    v = 0.0;
    if (threadIdx.x < blockDim.x / 32) v = red[threadIdx.x];
    if (w == 0)
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Energies are summed in a fixed order (per-block partials, then one final
// pass), so they are bitwise reproducible.
constexpr int kEnergyBlocks = 1024;

__global__ void kinetic_kernel(const double* __restrict__ v, int64_t n, double* part)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        s += v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2];
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[3 * blockIdx.x] = 0.5 * s;
}

__global__ void energy_final_kernel(const double* __restrict__ part, int blocks, double* acc)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double k = 0.0, p = 0.0, w = 0.0;
    for (int b = 0; b < blocks; b++) {
        k += part[3 * b];
        p += part[3 * b + 1];
        w += part[3 * b + 2];
    }
    acc[0] = k;
    acc[1] = p;
    acc[2] = w;
}

// Potential energy 4(r^-12 - r^-6) and virial r.F = 48 r^2 s over every
// directed entry (each pair counted twice, halved), FP32 per entry, FP64 sums.
__global__ void potential_kernel(const float4* __restrict__ pos, const uint32_t* __restrict__ row_off,
                                 const int32_t* __restrict__ col, int64_t n, LawParams law,
                                 double* part)
{
    __shared__ double red[32];
    double pe = 0.0, vir = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = pos[i];
        float pe_i = 0.f, vir_i = 0.f;
        for (uint32_t k = row_off[i]; k < row_off[i + 1]; k++) {
            const float4 b = pos[col[k]];
            float dx, dy, dz;
            const float s = lj_scalar<true>(a, b, law, dx, dy, dz);
            if (s == 0.0f) continue;
            const float rd = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float r = 1.0f / rd;
            const float r6 = r * r * r;
            pe_i += 4.0f * r6 * (r6 - 1.0f);
            vir_i += 48.0f * s * rd;
        }
        pe += 0.5 * (double)pe_i;
        vir += 0.5 * (double)vir_i;
    }
    pe = block_sum(pe, red);
    __syncthreads();
    vir = block_sum(vir, red);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x + 1] = pe;
        part[3 * blockIdx.x + 2] = vir;
    }
}

// Stream-ordered frees (on s): no device-wide synchronisation, so the set-up
// of several systems can overlap (the serving loop rebuilds them on their
// own streams from several host threads).
void free_part(irr_md* m, cudaStream_t s)
{
    if (m->part.perm) cudaFreeAsync(m->part.perm, s);
    if (m->part.inv) cudaFreeAsync(m->part.inv, s);
    if (m->part.row_off) cudaFreeAsync(m->part.row_off, s);
    if (m->part.col) cudaFreeAsync(m->part.col, s);
    m->part = PartitionOut{};
    free_sliced(&m->sl, s);
    if (m->d_items) cudaFreeAsync(m->d_items, s);
    m->d_items = nullptr;
    m->num_items = 0;
    if (m->half) cudaFreeAsync(m->half, s);
    m->half = nullptr;
}

}  // namespace

namespace irr {

// New neighbour list, partition and execution order from the current positions.
int md_rebuild(irr_md* m)
{
    cudaStream_t s = m->stream;
    const double lc = m->cfg.cutforce + m->cfg.skin;
    const float list_cut2 = (float)(lc * lc);
    int64_t e = 0;
    free_part(m, s);
    // A box of at least 3 cells per axis: the atoms are re-sorted by cell
    // along a Hilbert curve of the cells at every rebuild, and each row is
    // written already in (row, col) order straight from the cell search.
    PartitionOut p;
    // Rows change little between rebuilds: slots a quarter longer than the
    // last build's longest row let one search pass write them.
    uint32_t longest = 0;
    cudaError_t pe = build_rows_by_cell(m->pos4, m->n, (float)m->cfg.side, list_cut2, &p, &e, &longest,
                                        m->cfg.row_slots > 0 ? (uint32_t)m->cfg.row_slots : m->row_cap, s);
    if (pe == cudaSuccess) m->row_cap = (longest + longest / 4 + 8 + 7) & ~7u;
    bool reorder = true;
    if (pe == cudaErrorNotSupported) {
        // Smaller boxes: the half list, then the partition's node order and
        // (row, col) layout.  The node order only decides locality: atoms
        // move a fraction of the skin between rebuilds, so the curve order of
        // an earlier rebuild stays nearly as local, and the atoms are
        // re-sorted only every reorder_every-th rebuild (the first one
        // included); the others keep the execution order.
        int2* d_edges = nullptr;
        MD_CUDA(m, build_neighbor_list(m->pos4, m->n, (float)m->cfg.side, list_cut2, &d_edges, &e, s,
                                       true, false),
                "neighbour build");
        reorder = m->rebuilds % (m->cfg.reorder_every > 1 ? m->cfg.reorder_every : 1) == 0;
        pe = build_partition(m->pos4, m->n, d_edges, e, reorder ? 1 : 0, &p, s);
        if (d_edges) cudaFreeAsync(d_edges, s);
    }
    m->part = p;
    if (pe != cudaSuccess)
        return md_fail(m, pe == cudaErrorMemoryAllocation ? IRR_ERR_NOMEM
                          : pe == cudaErrorInvalidValue  ? IRR_ERR_CAPACITY
                                                         : IRR_ERR_CUDA,
                       "neighbour rows", pe);
    if (reorder) {
        // state into the new order
        const int g = grid_of(m->n);
        gather3_kernel<<<g, 256, 0, s>>>(m->x, m->part.perm, m->n, m->tmp);
        std::swap(m->x, m->tmp);
        gather3_kernel<<<g, 256, 0, s>>>(m->v, m->part.perm, m->n, m->tmp);
        std::swap(m->v, m->tmp);
        gather_ids_kernel<<<g, 256, 0, s>>>(m->ids, m->part.perm, m->n, m->ids_tmp);
        std::swap(m->ids, m->ids_tmp);
        to_float4_kernel<<<g, 256, 0, s>>>(m->x, m->n, m->cfg.side, m->pos4);
        MD_CUDA(m, cudaGetLastError(), "permute state");
    }
    // the sliced layout's work items are cut from its slice offsets (which
    // build_sliced brings to the host); only the CSR fallback needs the row
    // offsets on the host
    if (build_sliced(m->part.row_off, m->part.col, m->n, m->shape.lanes_per_row, &m->sl, s) != cudaSuccess) {
        cudaGetLastError();
        free_sliced(&m->sl, s);  // CSR
    } else if (!sliced_pays(m->sl, 2 * e)) {
        free_sliced(&m->sl, s);
    }
    std::vector<uint32_t> ro;
    if (!m->sl.lanes) {
        ro.resize((size_t)m->n + 1);
        MD_CUDA(m, cudaMemcpyAsync(ro.data(), m->part.row_off, sizeof(uint32_t) * (m->n + 1),
                                   cudaMemcpyDeviceToHost, s), "row offsets");
        MD_CUDA(m, cudaStreamSynchronize(s), "row offsets");
    }
    std::vector<WorkItem> items;
    make_instance_items(ro.data(), m->sl, m->n, 0, m->shape, items);
    m->num_items = (int)items.size();
    MD_CUDA(m, irr_malloc_async(&m->d_items, sizeof(WorkItem) * (items.empty() ? 1 : items.size()), s),
            "work items");
    if (!items.empty())
        MD_CUDA(m, cudaMemcpyAsync(m->d_items, items.data(), sizeof(WorkItem) * items.size(),
                                   cudaMemcpyHostToDevice, s), "work items");
    InstDesc d{};
    d.pos = m->pos4;
    d.row_off = m->part.row_off;
    d.col = m->part.col;
    d.force = m->force;
    d.slice_off = m->sl.lanes ? m->sl.slice_off : nullptr;
    d.scol = m->sl.lanes ? m->sl.col : nullptr;
    d.law = m->law;
    d.n = m->n;
    m->inst = d;
    MD_CUDA(m, cudaMemcpyAsync(m->d_inst, &d, sizeof(d), cudaMemcpyHostToDevice, s), "instance");
    if (m->cfg.exec_plain && e > 0) {
        // the plain kernel's edge list: each pair once, (i, j) with i < j
        uint32_t* off = nullptr;
        MD_CUDA(m, irr_malloc_async(&off, sizeof(uint32_t) * (m->n + 1), s), "half list");
        MD_CUDA(m, irr_malloc_async(&m->half, sizeof(int2) * e, s), "half list");
        half_count_kernel<<<grid_of(m->n), 256, 0, s>>>(m->part.row_off, m->part.col, m->n, off);
        MD_CUDA(m, cudaMemsetAsync(off + m->n, 0, sizeof(uint32_t), s), "half list");
        MD_CUDA(m, scan_exclusive_u32(off, off, m->n + 1, nullptr, s), "half list");
        half_write_kernel<<<grid_of(m->n), 256, 0, s>>>(m->part.row_off, m->part.col, m->n, off, m->half);
        MD_CUDA(m, cudaGetLastError(), "half list");
        cudaFreeAsync(off, s);
    }
    MD_CUDA(m, cudaStreamSynchronize(s), "rebuild");
    m->edges = e;
    m->rebuilds++;
    m->since_rebuild = 0;
    return IRR_OK;
}

int md_forces(irr_md* m)
{
    if (m->cfg.exec_plain) {
        MD_CUDA(m, cudaMemsetAsync(m->force, 0, sizeof(float4) * m->n, m->stream), "clear forces");
        MD_CUDA(m, launch_plain(m->pos4, m->half, m->edges, m->force, m->law, m->stream), "plain kernel");
        return IRR_OK;
    }
    MD_CUDA(m, cudaMemsetAsync(m->d_queue, 0, sizeof(int), m->stream), "queue");
    MD_CUDA(m, launch_tiled(m->shape, m->d_inst, m->d_items, m->num_items, m->d_queue,
                            m->sms * kCtasPerSm, m->d_status, m->stream, &m->inst, 1), "force kernel");
    return IRR_OK;
}

int md_kick_drift(irr_md* m)
{
    kick_drift_kernel<1><<<grid_of(m->n), 256, 0, m->stream>>>(m->x, m->v, m->force, m->n,
                                                               m->cfg.dt, m->cfg.side, m->pos4);
    MD_CUDA(m, cudaGetLastError(), "kick-drift");
    m->since_rebuild++;
    return IRR_OK;
}

// md_kick of the previous step and md_kick_drift of this one in one pass.
int md_kick_kick_drift(irr_md* m)
{
    kick_drift_kernel<2><<<grid_of(m->n), 256, 0, m->stream>>>(m->x, m->v, m->force, m->n,
                                                               m->cfg.dt, m->cfg.side, m->pos4);
    MD_CUDA(m, cudaGetLastError(), "kick-drift");
    m->steps++;
    m->since_rebuild++;
    return IRR_OK;
}

int md_kick(irr_md* m)
{
    kick_kernel<<<grid_of(m->n), 256, 0, m->stream>>>(m->v, m->force, m->n, m->cfg.dt);
    MD_CUDA(m, cudaGetLastError(), "kick");
    m->steps++;
    return IRR_OK;
}

int md_state_digest(irr_md* m, uint64_t* digest)
{
    unsigned long long* d = reinterpret_cast<unsigned long long*>(m->d_acc + 3);  // the spare slot
    MD_CUDA(m, cudaMemsetAsync(d, 0, sizeof(*d), m->stream), "digest");
    state_digest_kernel<<<grid_of(m->n), 256, 0, m->stream>>>(m->x, m->ids, m->n, d);
    MD_CUDA(m, cudaGetLastError(), "digest");
    unsigned long long h = 0;
    MD_CUDA(m, cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, m->stream), "digest");
    MD_CUDA(m, cudaStreamSynchronize(m->stream), "digest");
    *digest = h;
    return IRR_OK;
}

InstDesc md_instance(const irr_md* m)
{
    InstDesc d{};
    d.pos = m->pos4;
    d.row_off = m->part.row_off;
    d.col = m->part.col;
    d.force = m->force;
    d.slice_off = m->sl.lanes ? m->sl.slice_off : nullptr;
    d.scol = m->sl.lanes ? m->sl.col : nullptr;
    d.law = m->law;
    d.n = m->n;
    return d;
}

}  // namespace irr

extern "C" {

void irr_md_config_default(irr_md_config* c)
{
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->device = 0;
    c->dt = 0.005;
    c->cutforce = 2.5;
    c->skin = 0.3;
    c->side = 0.0;
    c->rebuild_every = 20;
    c->reorder_every = 10;
}

int irr_md_create(const irr_md_config* cfg, const double* pos, const double* vel, int64_t n,
                  irr_md** out)
{
    irr::TraceRange trace_("irr_md_create");
    if (!cfg || !out || n < 2 || !pos || !vel) return IRR_ERR_ARG;
    *out = nullptr;
    if (!(cfg->side > 0) || !(cfg->dt > 0) || !(cfg->cutforce > 0) || !(cfg->skin >= 0) ||
        cfg->rebuild_every < 1)
        return IRR_ERR_ARG;
    if (2.0 * (cfg->cutforce + cfg->skin) > cfg->side) return IRR_ERR_ARG;  // one image per pair
    if (cfg->exec_plain != 0 && cfg->exec_plain != 1) return IRR_ERR_ARG;
    if (cfg->row_slots < 0 || cfg->row_slots > 4096) return IRR_ERR_ARG;
    if (n > 0x7fffffffLL) return IRR_ERR_CAPACITY;
    irr_md* m = new (std::nothrow) irr_md();
    if (!m) return IRR_ERR_NOMEM;
    m->cfg = *cfg;
    m->device = cfg->device;
    m->n = n;
    int rc = IRR_OK;
    DeviceGuard dev_guard(m->device);
    if (!dev_guard.ok() ||
        cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, m->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&m->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete m;
        return IRR_ERR_CUDA;
    }
    m->stream = m->own_stream;
    const double rc2 = cfg->cutforce * cfg->cutforce;
    LawParams L{};
    L.rc2d = rc2;
    L.rc2 = (float)rc2;
    L.rc2_lo = (float)(rc2 * (1.0 - 1.0 / 262144.0));
    L.rc2_hi = (float)(rc2 * (1.0 + 1.0 / 262144.0));
    L.periodic = 1;
    L.side = cfg->side;
    L.halfd = 0.5 * cfg->side;
    L.half = (float)(0.5 * cfg->side);
    L.side_hi = (float)cfg->side;
    L.side_lo = (float)(cfg->side - (double)L.side_hi);
    L.half2 = (float)(0.25 * cfg->side * cfg->side * (1.0 - 1.0 / 65536.0));
    L.band = (float)(rc2 * (2.0 / 262144.0));
    m->law = L;
    m->shape.lanes_per_row = 4;
    m->shape.block_nodes = 1024;
    m->shape.stage_smem = 1;
    m->shape.periodic = 1;
    const size_t b3 = sizeof(double) * 3 * (size_t)n;
    cudaError_t e = cudaSuccess;
    // stream-ordered (no device-wide synchronisation; see free_part)
    cudaStream_t os = m->own_stream;
    if (e == cudaSuccess) e = irr_malloc_async(&m->x, b3, os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->v, b3, os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->tmp, b3, os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->pos4, sizeof(float4) * n, os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->force, sizeof(float4) * n, os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->ids, sizeof(int32_t) * n, os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->ids_tmp, sizeof(int32_t) * n, os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->d_inst, sizeof(InstDesc), os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->d_queue, sizeof(int), os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->d_status, sizeof(int), os);
    if (e == cudaSuccess) e = irr_malloc_async(&m->d_acc, (4 + 3 * kEnergyBlocks) * sizeof(double), os);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->d_status, 0, sizeof(int), m->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->x, pos, b3, cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->v, vel, b3, cudaMemcpyHostToDevice, m->stream);
    if (e != cudaSuccess) {
        irr_md_destroy(m);
        return e == cudaErrorMemoryAllocation ? IRR_ERR_NOMEM : IRR_ERR_CUDA;
    }
    // execution slot k holds atom k until the first partition; then wrap the
    // initial positions and make their float copy
    iota_ids_kernel<<<grid_of(n), 256, 0, m->stream>>>(m->ids, n);
    to_float4_kernel<<<grid_of(n), 256, 0, m->stream>>>(m->x, n, cfg->side, m->pos4);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        irr_md_destroy(m);
        return IRR_ERR_CUDA;
    }
    rc = md_rebuild(m);
    if (rc == IRR_OK) rc = md_forces(m);
    if (rc == IRR_OK && cudaStreamSynchronize(m->stream) != cudaSuccess) rc = IRR_ERR_CUDA;
    if (rc != IRR_OK) {
        irr_md_destroy(m);
        return rc;
    }
    *out = m;
    return IRR_OK;
}

int irr_md_destroy(irr_md* m)
{
    if (!m) return IRR_ERR_ARG;
    DeviceGuard dev_guard(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    if (m->own_stream) {
        free_part(m, m->own_stream);
        void* ptrs[] = {m->x, m->v, m->tmp, m->pos4, m->force, m->ids, m->ids_tmp,
                        m->d_inst, m->d_queue, m->d_status, m->d_acc};
        for (void* p : ptrs)
            if (p) cudaFreeAsync(p, m->own_stream);
        cudaStreamSynchronize(m->own_stream);
        cudaStreamDestroy(m->own_stream);
    }
    delete m;
    return IRR_OK;
}

const char* irr_md_last_error(const irr_md* m) { return m ? m->err.c_str() : "null handle"; }

int irr_md_set_stream(irr_md* m, void* stream)
{
    if (!m) return IRR_ERR_ARG;
    m->stream = (cudaStream_t)stream;
    return IRR_OK;
}

int irr_md_run(irr_md* m, int steps)
{
    irr::TraceRange trace_("irr_md_run");
    if (!m || steps < 0) return IRR_ERR_ARG;
    DeviceGuard dev_guard(m->device);
    for (int t = 0; t < steps; t++) {
        // a step's closing kick is fused into the next step's kick-drift
        int rc = t == 0 ? md_kick_drift(m) : md_kick_kick_drift(m);
        if (!rc && m->since_rebuild >= m->cfg.rebuild_every) rc = md_rebuild(m);
        if (!rc) rc = md_forces(m);
        if (rc) return rc;
    }
    return steps > 0 ? md_kick(m) : IRR_OK;
}

int irr_md_energy(irr_md* m, double* kinetic, double* potential, double* virial)
{
    if (!m) return IRR_ERR_ARG;
    DeviceGuard dev_guard(m->device);
    const int blocks = grid_of(m->n) < kEnergyBlocks ? grid_of(m->n) : kEnergyBlocks;
    double* part = m->d_acc + 4;
    kinetic_kernel<<<blocks, 256, 0, m->stream>>>(m->v, m->n, part);
    potential_kernel<<<blocks, 256, 0, m->stream>>>(m->pos4, m->part.row_off, m->part.col, m->n,
                                                    m->law, part);
    energy_final_kernel<<<1, 32, 0, m->stream>>>(part, blocks, m->d_acc);
    MD_CUDA(m, cudaGetLastError(), "energy kernels");
    double h[4];
    int st = 0;
    MD_CUDA(m, cudaMemcpyAsync(h, m->d_acc, sizeof(h), cudaMemcpyDeviceToHost, m->stream), "energy");
    MD_CUDA(m, cudaMemcpyAsync(&st, m->d_status, sizeof(int), cudaMemcpyDeviceToHost, m->stream), "status");
    MD_CUDA(m, cudaStreamSynchronize(m->stream), "energy");
    if (kinetic) *kinetic = h[0];
    if (potential) *potential = h[1];
    if (virial) *virial = h[2];
    if (st) return md_fail(m, IRR_ERR_DEVICE, "device status set (a bounded wait gave up)");
    return IRR_OK;
}

int irr_md_get_state(irr_md* m, double* pos, double* vel)
{
    if (!m) return IRR_ERR_ARG;
    DeviceGuard dev_guard(m->device);
    const size_t b3 = sizeof(double) * 3 * (size_t)m->n;
    const int g = grid_of(m->n);
    std::vector<double> host;
    double* outs[2] = {pos, vel};
    double* srcs[2] = {m->x, m->v};
    for (int k = 0; k < 2; k++) {
        if (!outs[k]) continue;
        scatter3_kernel<<<g, 256, 0, m->stream>>>(srcs[k], m->ids, m->n, m->tmp);
        MD_CUDA(m, cudaGetLastError(), "state");
        MD_CUDA(m, cudaMemcpyAsync(outs[k], m->tmp, b3, cudaMemcpyDeviceToHost, m->stream), "state");
        MD_CUDA(m, cudaStreamSynchronize(m->stream), "state");
    }
    return IRR_OK;
}

int irr_md_get_forces(irr_md* m, double* f)
{
    if (!m || !f) return IRR_ERR_ARG;
    DeviceGuard dev_guard(m->device);
    // F = 48 * reduction result, in the caller's atom order
    std::vector<float4> fr((size_t)m->n);
    std::vector<int32_t> ids((size_t)m->n);
    MD_CUDA(m, cudaMemcpyAsync(fr.data(), m->force, sizeof(float4) * m->n, cudaMemcpyDeviceToHost, m->stream), "forces");
    MD_CUDA(m, cudaMemcpyAsync(ids.data(), m->ids, sizeof(int32_t) * m->n, cudaMemcpyDeviceToHost, m->stream), "forces");
    MD_CUDA(m, cudaStreamSynchronize(m->stream), "forces");
    for (int64_t k = 0; k < m->n; k++) {
        const int64_t d = ids[(size_t)k];
        f[3 * d] = 48.0 * fr[(size_t)k].x;
        f[3 * d + 1] = 48.0 * fr[(size_t)k].y;
        f[3 * d + 2] = 48.0 * fr[(size_t)k].z;
    }
    return IRR_OK;
}

int irr_md_get_info(const irr_md* m, irr_md_info* info)
{
    if (!m || !info) return IRR_ERR_ARG;
    memset(info, 0, sizeof(*info));
    info->num_atoms = m->n;
    info->num_edges = m->edges;
    info->steps = m->steps;
    info->rebuilds = m->rebuilds;
    return IRR_OK;
}

}  // extern "C"
