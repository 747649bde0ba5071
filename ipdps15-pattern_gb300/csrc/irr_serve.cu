// irr_serve.cu -- a request loop that serves MD jobs with continuous batching.
//
// No counterpart in the reference, whose runtime serves one edge set per
// process.  Jobs (Lennard-Jones systems of different sizes, each asking for a
// number of velocity-Verlet steps) arrive as a Poisson stream.  The loop:
//   * admits arrived jobs in arrival order while their estimated device memory
//     fits the budget (their state then stays resident until they finish);
//   * every tick advances each resident job by one step: ONE kick/drift launch
//     over all resident jobs (with the previous step's closing kick folded in
//     for the jobs that did not retire); the rebuilds that are due start on
//     worker threads while the other jobs' forces (one batched launch over
//     their (instance, node block) work items, gathered on the device from
//     each job's own table) are queued; then the rebuilt jobs' forces; the
//     jobs that finish get their closing kick at once;
//   * retires finished jobs (their memory frees up for waiting arrivals).
// A job's rows are computed by the same kernel code whatever else shares the
// launch, so its trajectory is bitwise the same alone and in the mix.
// Serial mode runs the same jobs one at a time for comparison.  Each job's
// initial state arrives with the request: it is made before the clock starts.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <random>
#include <thread>
#include <vector>

#include "irr_md.cuh"
#include "irr_trace.cuh"

using namespace irr;

namespace {

struct JobSpec {
    double arrival;
    int cells;
    int64_t atoms;
    uint64_t seed;
    double side;
    size_t est_bytes;
};

// A request's initial state (3n positions, 3n velocities), in page-locked
// host memory when the driver grants it, else in ordinary memory.
struct Payload {
    double* pos = nullptr;
    double* vel = nullptr;
    bool locked = false;
    void fill(const std::vector<double>& p, const std::vector<double>& v)
    {
        const size_t bytes = sizeof(double) * p.size();
        locked = cudaHostAlloc((void**)&pos, bytes, cudaHostAllocDefault) == cudaSuccess &&
                 cudaHostAlloc((void**)&vel, bytes, cudaHostAllocDefault) == cudaSuccess;
        if (!locked) {
            cudaGetLastError();
            if (pos) cudaFreeHost(pos);
            pos = static_cast<double*>(malloc(bytes));
            vel = static_cast<double*>(malloc(bytes));
        }
        if (pos && vel) {
            memcpy(pos, p.data(), bytes);
            memcpy(vel, v.data(), bytes);
        }
    }
    void release()
    {
        if (locked) {
            if (pos) cudaFreeHost(pos);
            if (vel) cudaFreeHost(vel);
        } else {
            free(pos);
            free(vel);
        }
        pos = vel = nullptr;
    }
};

// A job being set up (upload, first neighbour build, partition and forces)
// on a worker thread while the resident jobs keep stepping.
struct Admission {
    int id = 0;
    irr_md* made = nullptr;
    int rc = IRR_OK;
    std::atomic<bool> done{false};
    std::thread worker;
};

struct Live {
    int id;
    irr_md* md;
    int steps;
    double admit_s;
    double pair_evals;
    bool kick_pending;  // the last step's closing kick is left to the next kick-drift
};

// One resident job in a tick's device tables.  Its atoms occupy whole
// 256-thread blocks [block0, block0 + ceil(n / 256)) of the integrator
// launches; its work items are [item0, item0 + num_items) of the batch.
struct TickJob {
    double* x;
    double* v;
    const float4* force;
    float4* pos4;
    const WorkItem* items;
    int64_t n;
    double side;
    int32_t block0;
    int32_t item0;
    int32_t num_items;
    int32_t kicks;  // kick-drift: 2 when the job's previous closing kick is folded in
};
constexpr int kTickThreads = 256;

// The job a block (or an item) belongs to: the last k with start(k) <= x.
template <class Start>
__device__ __forceinline__ int find_job(int njobs, int64_t x, Start start)
{
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start(mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Each job's kick-drift; a job that did not retire last tick had its closing
// kick left to this pass (kicks == 2, the same roundings as a separate kick).
__global__ void __launch_bounds__(kTickThreads) tick_kick_drift_kernel(const TickJob* __restrict__ jobs,
                                                                       int njobs, double dt)
{
    const int k = find_job(njobs, blockIdx.x, [&](int j) { return (int64_t)jobs[j].block0; });
    const TickJob& J = jobs[k];
    const int64_t i = (int64_t)(blockIdx.x - J.block0) * kTickThreads + threadIdx.x;
    if (i >= J.n) return;
    if (J.kicks == 2)
        md_kick_drift_atom<2>(J.x, J.v, J.force, i, dt, J.side, J.pos4);
    else
        md_kick_drift_atom<1>(J.x, J.v, J.force, i, dt, J.side, J.pos4);
}

__global__ void __launch_bounds__(kTickThreads) tick_kick_kernel(const TickJob* __restrict__ jobs,
                                                                 int njobs, double dt)
{
    const int k = find_job(njobs, blockIdx.x, [&](int j) { return (int64_t)jobs[j].block0; });
    const TickJob& J = jobs[k];
    const int64_t i = (int64_t)(blockIdx.x - J.block0) * kTickThreads + threadIdx.x;
    if (i < J.n) md_kick_atom(J.v, J.force, i, dt);
}

// The batch's work items: job k's own items with the instance set to k.
__global__ void tick_items_kernel(const TickJob* __restrict__ jobs, int njobs, int64_t total,
                                  WorkItem* __restrict__ out)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int k = find_job(njobs, t, [&](int j) { return (int64_t)jobs[j].item0; });
        WorkItem w = jobs[k].items[t - jobs[k].item0];
        w.inst = k;
        out[t] = w;
    }
}

// Host tables of a tick, in page-locked memory (reused every tick: the tick
// ends with a stream synchronisation).
template <class T>
struct Pinned {
    T* h = nullptr;
    T* d = nullptr;
    size_t cap = 0;
    bool reserve(size_t n)
    {
        if (n <= cap) return true;
        release();
        cap = n * 2;
        if (cudaHostAlloc((void**)&h, sizeof(T) * cap, cudaHostAllocDefault) != cudaSuccess ||
            cudaMalloc((void**)&d, sizeof(T) * cap) != cudaSuccess) {
            cudaGetLastError();
            release();
            return false;
        }
        return true;
    }
    void release()
    {
        if (h) cudaFreeHost(h);
        if (d) cudaFree(d);
        h = nullptr;
        d = nullptr;
        cap = 0;
    }
};

// Fills the job table for the jobs ms (their current arrays: a rebuild swaps a
// job's state buffers; kicks[k] for the kick-drift, 1 if none given) and
// uploads it on s; returns the launch's block count and the batch's item
// count.
bool upload_tick_jobs(const std::vector<irr_md*>& ms, Pinned<TickJob>& T, cudaStream_t s,
                      int* blocks, int64_t* items, const std::vector<int>* kicks = nullptr)
{
    if (!T.reserve(ms.size())) return false;
    int64_t b = 0, it = 0;
    for (size_t k = 0; k < ms.size(); k++) {
        const irr_md* m = ms[k];
        TickJob& J = T.h[k];
        J.x = m->x;
        J.v = m->v;
        J.force = m->force;
        J.pos4 = m->pos4;
        J.items = m->d_items;
        J.n = m->n;
        J.side = m->cfg.side;
        J.block0 = (int32_t)b;
        J.item0 = (int32_t)it;
        J.num_items = m->num_items;
        J.kicks = kicks ? (*kicks)[k] : 1;
        b += (m->n + kTickThreads - 1) / kTickThreads;
        it += m->num_items;
    }
    if (b > 0x7fffffffLL || it > 0x7fffffffLL) return false;
    *blocks = (int)b;
    *items = it;
    return cudaMemcpyAsync(T.d, T.h, sizeof(TickJob) * ms.size(), cudaMemcpyHostToDevice, s) ==
           cudaSuccess;
}

// The device tables of one force launch of a tick.
struct ForceBatch {
    Pinned<TickJob> jobs;
    Pinned<TickJob> closing;  // the jobs that retire this tick (their closing kick)
    Pinned<InstDesc> insts;
    WorkItem* d_items = nullptr;
    size_t items_cap = 0;
    void release()
    {
        jobs.release();
        closing.release();
        insts.release();
        if (d_items) cudaFree(d_items);
        d_items = nullptr;
        items_cap = 0;
    }
};

// The forces of the jobs ms (one persistent launch over their work items,
// gathered on the device from each job's own table) and the closing kick of
// those that retire after this step (one launch over them; the others' kicks
// are folded into the next tick's kick-drift), queued on s.
int force_and_kick(const std::vector<irr_md*>& ms, const std::vector<irr_md*>& retiring,
                   ForceBatch& B, const TiledShape& shape, int* d_queue, int* d_status, int sms,
                   double dt, cudaStream_t s, bool plain)
{
    if (ms.empty()) return IRR_OK;
    if (plain) {  // each job by its own plain force launch
        for (irr_md* m : ms) {
            const int frc = md_forces(m);
            if (frc != IRR_OK) return frc;
        }
    } else {
        int blocks = 0;
        int64_t nitems = 0;
        if (!upload_tick_jobs(ms, B.jobs, s, &blocks, &nitems) || !B.insts.reserve(ms.size()))
            return IRR_ERR_CUDA;
        for (size_t k = 0; k < ms.size(); k++) B.insts.h[k] = md_instance(ms[k]);
        if ((size_t)nitems > B.items_cap) {
            if (B.d_items) cudaFree(B.d_items);
            B.items_cap = (size_t)nitems * 2;
            if (cudaMalloc(&B.d_items, sizeof(WorkItem) * B.items_cap) != cudaSuccess) {
                B.d_items = nullptr;
                B.items_cap = 0;
                return IRR_ERR_NOMEM;
            }
        }
        if (cudaMemcpyAsync(B.insts.d, B.insts.h, sizeof(InstDesc) * ms.size(), cudaMemcpyHostToDevice, s) !=
            cudaSuccess)
            return IRR_ERR_CUDA;
        if (nitems > 0) {
            const int64_t want = (nitems + 255) / 256;
            tick_items_kernel<<<(unsigned)(want < 4096 ? want : 4096), 256, 0, s>>>(B.jobs.d, (int)ms.size(),
                                                                                    nitems, B.d_items);
        }
        if (cudaGetLastError() != cudaSuccess || cudaMemsetAsync(d_queue, 0, sizeof(int), s) != cudaSuccess ||
            launch_tiled(shape, B.insts.d, B.d_items, (int)nitems, d_queue, sms * kCtasPerSm, d_status, s,
                         B.insts.h, (int)ms.size()) != cudaSuccess)
            return IRR_ERR_CUDA;
    }
    if (retiring.empty()) return IRR_OK;
    int kblocks = 0;
    int64_t unused = 0;
    if (!upload_tick_jobs(retiring, B.closing, s, &kblocks, &unused)) return IRR_ERR_CUDA;
    tick_kick_kernel<<<kblocks, kTickThreads, 0, s>>>(B.closing.d, (int)retiring.size(), dt);
    return cudaGetLastError() == cudaSuccess ? IRR_OK : IRR_ERR_CUDA;
}

// Starts f(0..count-1) on up to `workers` host threads and returns them
// (join them before using what f produces).
template <class F>
std::vector<std::thread> start_parallel(size_t count, unsigned workers, int device, F f)
{
    std::vector<std::thread> pool;
    if (count == 0) return pool;
    auto next = std::make_shared<std::atomic<size_t>>(0);
    const size_t nth = std::min<size_t>(count, std::max(1u, workers));
    for (size_t t = 0; t < nth; t++)
        pool.emplace_back([=]() {
            cudaSetDevice(device);
            for (size_t i; (i = next->fetch_add(1)) < count;) f(i);
        });
    return pool;
}

// Runs f(0..count-1) on up to `workers` host threads (count small: inline).
// Each call issues work on its own job's stream, so the GPU overlaps the
// jobs' set-up kernels while each thread waits only for its own.
template <class F>
void run_parallel(size_t count, unsigned workers, int device, F f)
{
    if (count <= 1 || workers <= 1) {
        for (size_t i = 0; i < count; i++) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    const unsigned nth = (unsigned)std::min<size_t>(count, workers);
    for (unsigned t = 0; t < nth; t++)
        pool.emplace_back([&]() {
            cudaSetDevice(device);
            for (size_t i = next++; i < count; i = next++) f(i);
        });
    for (auto& th : pool) th.join();
}

uint64_t mix64(uint64_t x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Job k's size, seed and arrival derive from (config seed, k) alone.
std::vector<JobSpec> make_jobs(const irr_serve_config* c)
{
    std::vector<JobSpec> jobs;
    std::mt19937_64 arr(c->seed);
    std::exponential_distribution<double> gap(c->arrival_rate > 0 ? c->arrival_rate : 1.0);
    double t = 0.0;
    const double alat = std::cbrt(4.0 / c->density);
    const int min_cells = (int)std::ceil(2.0 * (c->cutforce + c->skin) / alat + 1e-9);
    for (int k = 0; k < c->num_jobs; k++) {
        t += c->arrival_rate > 0 ? gap(arr) : 0.0;
        std::mt19937_64 g(mix64(c->seed ^ (0x51ed2701ull * (uint64_t)(k + 1))));
        std::uniform_real_distribution<double> u(std::log((double)c->min_atoms), std::log((double)c->max_atoms));
        const double n = std::floor(std::exp(u(g)));
        int cells = (int)std::lround(std::cbrt(n / 4.0));
        cells = std::max(cells, min_cells);
        JobSpec j;
        j.arrival = t;
        j.cells = cells;
        j.atoms = 4ll * cells * cells * cells;
        j.seed = g();
        j.side = cells * alat;
        // resident state + list + partition temporaries, per atom (bytes)
        j.est_bytes = (size_t)j.atoms * 1600 + (64u << 20);
        jobs.push_back(j);
    }
    return jobs;
}

// FCC lattice (miniMD's site order), a small Gaussian jitter, Maxwell
// velocities at the temperature with zero total momentum.
void initial_state(const JobSpec& j, const irr_serve_config* c, std::vector<double>& pos,
                   std::vector<double>& vel)
{
    const double alat = std::cbrt(4.0 / c->density);
    const int m = 2 * j.cells;
    pos.clear();
    for (int k = 0; k < m; k++)
        for (int jj = 0; jj < m; jj++)
            for (int i = 0; i < m; i++)
                if ((i + jj + k) % 2 == 0) {
                    pos.push_back(0.5 * alat * i);
                    pos.push_back(0.5 * alat * jj);
                    pos.push_back(0.5 * alat * k);
                }
    std::mt19937_64 g(j.seed);
    std::normal_distribution<double> jit(0.0, 0.03);
    for (double& x : pos) {
        x += jit(g);
        x -= j.side * std::floor(x / j.side);
        if (x >= j.side) x = 0.0;
    }
    const int64_t n = j.atoms;
    vel.assign(3 * n, 0.0);
    std::normal_distribution<double> mv(0.0, std::sqrt(c->temperature));
    double mean[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            vel[3 * i + d] = mv(g);
            mean[d] += vel[3 * i + d];
        }
    double ke = 0.0;
    for (int64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            vel[3 * i + d] -= mean[d] / n;
            ke += vel[3 * i + d] * vel[3 * i + d];
        }
    const double s = std::sqrt(c->temperature * (3 * n - 3) / ke);
    for (double& v : vel) v *= s;
}

double pct(std::vector<double> v, double q)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double r = q * (v.size() - 1);
    const size_t lo = (size_t)std::floor(r), hi = (size_t)std::ceil(r);
    return v[lo] + (v[hi] - v[lo]) * (r - lo);
}

}  // namespace

extern "C" {

void irr_serve_config_default(irr_serve_config* c)
{
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->device = 0;
    c->num_jobs = 100;
    c->steps_per_job = 50;
    c->rebuild_every = 20;
    c->mode = IRR_SERVE_CONTINUOUS;
    c->only_job = -1;
    // A tick advances every resident job, so its time grows with the resident
    // set and every resident job waits for it.  The 200-job stream (200
    // jobs/s, 2K-2M atoms): p50 / p99 / makespan 0.51 / 0.60 / 1.36 s with no
    // limit, 0.51 / 0.60 / 1.38 s with 96 slots, 0.41 / 0.54 / 1.37 s with 64,
    // 0.40 / 0.53 / 1.40 s with 48, 0.38 / 0.53 / 1.45 s with 32.
    c->max_resident = 64;
    c->arrival_rate = 200.0;
    c->density = 0.8442;
    c->cutforce = 2.5;
    c->skin = 0.3;
    c->dt = 0.005;
    c->temperature = 1.44;
    c->min_atoms = 2048;
    c->max_atoms = 2097152;
    c->budget_bytes = 120e9;
    c->seed = 20260005;
}

int irr_serve_job_state(const irr_serve_config* cfg, int job, int64_t* atoms, double* side,
                        double* pos, double* vel)
{
    if (!cfg || job < 0 || job >= cfg->num_jobs || cfg->min_atoms < 32 ||
        cfg->max_atoms < cfg->min_atoms || !(cfg->density > 0) || !(cfg->temperature > 0))
        return IRR_ERR_ARG;
    const std::vector<JobSpec> jobs = make_jobs(cfg);
    const JobSpec& j = jobs[(size_t)job];
    if (atoms) *atoms = j.atoms;
    if (side) *side = j.side;
    if (pos || vel) {
        std::vector<double> p, v;
        initial_state(j, cfg, p, v);
        if (pos) std::copy(p.begin(), p.end(), pos);
        if (vel) std::copy(v.begin(), v.end(), vel);
    }
    return IRR_OK;
}

int irr_serve_run(const irr_serve_config* cfg, irr_serve_stats* st, irr_serve_job* out)
{
    irr::TraceRange trace_("irr_serve_run");
    if (!cfg || !st) return IRR_ERR_ARG;
    if (cfg->num_jobs < 0 || cfg->steps_per_job < 1 || cfg->rebuild_every < 1 ||
        cfg->min_atoms < 32 || cfg->max_atoms < cfg->min_atoms || !(cfg->density > 0) ||
        !(cfg->budget_bytes > 0) || cfg->max_resident < 1)
        return IRR_ERR_ARG;
    if (cfg->only_job >= cfg->num_jobs) return IRR_ERR_ARG;
    if (cfg->policy != IRR_SERVE_FIFO && cfg->policy != IRR_SERVE_SJF) return IRR_ERR_ARG;
    if (cfg->mode != IRR_SERVE_CONTINUOUS && cfg->mode != IRR_SERVE_SERIAL && cfg->mode != IRR_SERVE_SERIAL_PLAIN)
        return IRR_ERR_ARG;
    memset(st, 0, sizeof(*st));
    DeviceGuard dev_guard(cfg->device);
    if (!dev_guard.ok()) return IRR_ERR_CUDA;
    int sms = 0;
    cudaStream_t s = nullptr;
    int *d_queue = nullptr, *d_status = nullptr;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&d_queue, sizeof(int)) != cudaSuccess || cudaMalloc(&d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(d_status, 0, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return IRR_ERR_CUDA;
    }
    std::vector<JobSpec> jobs = make_jobs(cfg);
    std::vector<int> order;
    if (cfg->only_job >= 0) {
        order.push_back(cfg->only_job);
        jobs[cfg->only_job].arrival = 0.0;
    } else {
        for (int k = 0; k < cfg->num_jobs; k++) order.push_back(k);
    }
    const bool serial = cfg->mode == IRR_SERVE_SERIAL || cfg->mode == IRR_SERVE_SERIAL_PLAIN;
    const bool plain = cfg->mode == IRR_SERVE_SERIAL_PLAIN;
    const int max_res = serial ? 1 : cfg->max_resident;
    std::vector<double> latency;
    std::vector<Live> live;
    Pinned<TickJob> tick_a;        // every resident job (the kick-drift)
    ForceBatch keep_b, due_b;      // the jobs without and with a rebuild this tick
    double used = 0.0, peak = 0.0, pair_evals = 0.0;
    size_t next = 0;
    int rc = IRR_OK;
    TiledShape shape{};
    shape.lanes_per_row = 4;
    shape.block_nodes = 1024;
    shape.stage_smem = 1;
    shape.periodic = 1;
    // Each request carries its initial state (FCC lattice, jitter, Maxwell
    // velocities): made before the serving clock starts, on all host cores,
    // so the loop times admission, upload and the GPU work, not the host RNG.
    // A request's payload arrives in page-locked host memory, as a server's
    // receive buffers would be, so its upload runs at the host link's speed.
    std::vector<Payload> req(jobs.size());
    {
        unsigned nth = std::thread::hardware_concurrency();
        nth = std::max(1u, std::min(nth, 64u));
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < nth; t++)
            pool.emplace_back([&, t]() {
                cudaSetDevice(cfg->device);
                std::vector<double> pos, vel;
                for (size_t q = t; q < order.size(); q += nth) {
                    const int k = order[q];
                    if ((double)jobs[k].est_bytes > cfg->budget_bytes) continue;
                    initial_state(jobs[k], cfg, pos, vel);
                    req[k].fill(pos, vel);
                }
            });
        for (auto& th : pool) th.join();
    }
    const auto t0 = std::chrono::steady_clock::now();
    auto now = [&]() { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    const unsigned workers = serial
                                 ? 1u
                                 : std::max(1u, std::min(std::thread::hardware_concurrency(), 16u));
    cudaEvent_t ev_kd = nullptr;
    cudaEventCreateWithFlags(&ev_kd, cudaEventDisableTiming);
    std::vector<int> waiting;  // arrived, not yet admitted, in arrival order
    std::vector<std::unique_ptr<Admission>> creating;
    auto harvest = [&]() {  // jobs whose set-up has finished join the resident set
        for (size_t i = 0; i < creating.size();) {
            Admission& a = *creating[i];
            if (!a.done.load(std::memory_order_acquire)) {
                i++;
                continue;
            }
            a.worker.join();
            if (a.rc != IRR_OK) {
                if (rc == IRR_OK) rc = a.rc;
            } else {
                a.made->stream = s;
                live.push_back(Live{a.id, a.made, 0, now(), 0.0, false});
            }
            creating.erase(creating.begin() + (std::ptrdiff_t)i);
        }
        st->max_resident = std::max<int64_t>(st->max_resident, (int64_t)live.size());
    };
    while (rc == IRR_OK &&
           (next < order.size() || !waiting.empty() || !creating.empty() || !live.empty())) {
        harvest();
        if (rc) break;
        // arrivals (a job larger than the whole budget is rejected)
        while (next < order.size() && jobs[order[next]].arrival <= now()) {
            const int k = order[next++];
            if ((double)jobs[k].est_bytes > cfg->budget_bytes) {
                if (out) {
                    out[k] = irr_serve_job{};
                    out[k].atoms = jobs[k].atoms;
                    out[k].arrival_s = jobs[k].arrival;
                    out[k].status = IRR_ERR_BUDGET;
                }
                st->rejected++;
                continue;
            }
            waiting.push_back(k);
        }
        // admission within the budget and the slot limit: the earliest
        // arrival first (FIFO), or the smallest job first (SJF; ties by
        // arrival) -- in either order, the first job that does not fit stops it
        if (cfg->policy == IRR_SERVE_SJF)
            std::stable_sort(waiting.begin(), waiting.end(),
                             [&](int a, int b) { return jobs[a].atoms < jobs[b].atoms; });
        // an admitted job's set-up (upload, first neighbour build, partition,
        // forces) runs on a worker thread on its own stream -- at most
        // `workers` at a time -- while the resident jobs keep stepping; it
        // joins them at the first tick after its set-up has finished
        size_t taken = 0;
        while (taken < waiting.size() && creating.size() < workers) {
            const JobSpec& j = jobs[waiting[taken]];
            if ((int)(live.size() + creating.size()) >= max_res ||
                used + (double)j.est_bytes > cfg->budget_bytes)
                break;
            const int id = waiting[taken++];
            used += (double)j.est_bytes;
            peak = std::max(peak, used);
            creating.push_back(std::make_unique<Admission>());
            Admission* a = creating.back().get();
            a->id = id;
            a->worker = std::thread([a, &jobs, &req, cfg, plain]() {
                cudaSetDevice(cfg->device);
                const JobSpec& js = jobs[a->id];
                irr_md_config mc;
                irr_md_config_default(&mc);
                mc.device = cfg->device;
                mc.dt = cfg->dt;
                mc.cutforce = cfg->cutforce;
                mc.skin = cfg->skin;
                mc.side = js.side;
                mc.rebuild_every = cfg->rebuild_every;
                mc.exec_plain = plain ? 1 : 0;
                a->rc = irr_md_create(&mc, req[a->id].pos, req[a->id].vel, js.atoms, &a->made);
                a->done.store(true, std::memory_order_release);
            });
        }
        waiting.erase(waiting.begin(), waiting.begin() + (std::ptrdiff_t)taken);
        if (live.empty()) {
            if (!creating.empty()) {
                std::this_thread::sleep_for(std::chrono::microseconds(50));
            } else if (next < order.size()) {
                const double wait = jobs[order[next]].arrival - now();
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
            }
            continue;
        }
        // one tick: every resident job advances one step
        std::vector<irr_md*> all, keep, due, keep_retiring, due_retiring;
        std::vector<int> kicks;
        for (auto& L : live) {
            all.push_back(L.md);
            kicks.push_back(L.kick_pending ? 2 : 1);
            if (L.kick_pending) L.md->steps++;  // the bookkeeping of md_kick
            L.kick_pending = false;
        }
        int blocks = 0;
        int64_t nitems = 0;
        if (!upload_tick_jobs(all, tick_a, s, &blocks, &nitems, &kicks)) { rc = IRR_ERR_CUDA; break; }
        tick_kick_drift_kernel<<<blocks, kTickThreads, 0, s>>>(tick_a.d, (int)all.size(), cfg->dt);
        if (cudaGetLastError() != cudaSuccess) { rc = IRR_ERR_CUDA; break; }
        for (size_t k = 0; k < live.size(); k++) {
            irr_md* m = live[k].md;
            m->since_rebuild++;  // the bookkeeping of md_kick_drift
            const bool d = m->since_rebuild >= m->cfg.rebuild_every;
            (d ? due : keep).push_back(m);
            if (live[k].steps + 1 >= cfg->steps_per_job) (d ? due_retiring : keep_retiring).push_back(m);
        }
        // the rebuilds that are due start on worker threads, each on its
        // job's own stream after this tick's kick-drift, while this thread
        // queues the forces and kicks of the other jobs; the rebuilt jobs'
        // forces and kicks follow once their rebuilds have returned
        std::vector<int> due_rc(due.size(), IRR_OK);
        if (!due.empty()) cudaEventRecord(ev_kd, s);
        std::vector<std::thread> rebuilding = start_parallel(due.size(), workers, cfg->device, [&](size_t i) {
            irr_md* m = due[i];
            m->stream = m->own_stream;
            cudaStreamWaitEvent(m->stream, ev_kd, 0);
            due_rc[i] = md_rebuild(m);
            m->stream = s;
        });
        const int krc =
            force_and_kick(keep, keep_retiring, keep_b, shape, d_queue, d_status, sms, cfg->dt, s, plain);
        for (auto& th : rebuilding) th.join();
        if (krc != IRR_OK) rc = krc;
        for (int r : due_rc)
            if (r != IRR_OK && rc == IRR_OK) rc = r;
        if (rc) break;
        rc = force_and_kick(due, due_retiring, due_b, shape, d_queue, d_status, sms, cfg->dt, s, plain);
        if (rc) break;
        for (auto& L : live) {
            L.pair_evals += (double)L.md->edges;
            L.steps++;
            if (L.steps >= cfg->steps_per_job)
                L.md->steps++;  // kicked this tick (the bookkeeping of md_kick)
            else
                L.kick_pending = true;
        }
        // the host copies of the tables are reused next tick: wait for this one
        if (cudaStreamSynchronize(s) != cudaSuccess) { rc = IRR_ERR_CUDA; break; }
        // retire finished jobs: their results (final state hash, energy) are
        // read back and their memory freed concurrently, each on its own stream
        std::vector<size_t> fin;
        for (size_t k = 0; k < live.size(); k++)
            if (live[k].steps >= cfg->steps_per_job) fin.push_back(k);
        if (!fin.empty()) {
            const double done = now();
            run_parallel(fin.size(), workers, cfg->device, [&](size_t i) {
                const Live& L = live[fin[i]];
                const JobSpec& j = jobs[L.id];
                L.md->stream = L.md->own_stream;
                if (out) {
                    irr_serve_job r{};
                    r.atoms = j.atoms;
                    r.edges = L.md->edges;
                    r.arrival_s = j.arrival;
                    r.admit_s = L.admit_s;
                    r.done_s = done;
                    md_state_digest(L.md, &r.state_hash);
                    double ke = 0, pe = 0;
                    irr_md_energy(L.md, &ke, &pe, nullptr);
                    r.energy = ke + pe;
                    r.status = IRR_OK;
                    out[L.id] = r;
                }
                irr_md_destroy(L.md);
            });
            for (size_t i = fin.size(); i-- > 0;) {
                const Live& L = live[fin[i]];
                const JobSpec& j = jobs[L.id];
                latency.push_back(done - j.arrival);
                pair_evals += L.pair_evals;
                used -= (double)j.est_bytes;
                live.erase(live.begin() + fin[i]);
                st->jobs_done++;
            }
        }
    }
    const double makespan = now();
    for (auto& a : creating) {  // set-ups still running after an error
        if (a->worker.joinable()) a->worker.join();
        if (a->made) irr_md_destroy(a->made);
    }
    for (auto& r : req) r.release();
    for (auto& L : live) irr_md_destroy(L.md);
    if (ev_kd) cudaEventDestroy(ev_kd);
    int dev_status = 0;
    cudaMemcpy(&dev_status, d_status, sizeof(int), cudaMemcpyDeviceToHost);
    tick_a.release();
    keep_b.release();
    due_b.release();
    cudaFree(d_queue);
    cudaFree(d_status);
    cudaStreamDestroy(s);
    if (rc == IRR_OK && dev_status) rc = IRR_ERR_DEVICE;
    st->makespan_s = makespan;
    st->p50_ms = 1e3 * pct(latency, 0.50);
    st->p99_ms = 1e3 * pct(latency, 0.99);
    st->mean_ms = latency.empty() ? 0.0 : 1e3 * std::accumulate(latency.begin(), latency.end(), 0.0) / latency.size();
    st->max_ms = latency.empty() ? 0.0 : 1e3 * *std::max_element(latency.begin(), latency.end());
    st->pair_evals = pair_evals;
    st->edges_per_s = makespan > 0 ? pair_evals / makespan : 0.0;
    st->peak_budget_bytes = peak;
    return rc;
}

}  // extern "C"
