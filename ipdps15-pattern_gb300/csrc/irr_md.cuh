// irr_md.cuh -- the MD object, shared with the serving loop.
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

// ---- the integrator, per atom (shared by the per-system kernels of
// irr_md.cu and the batched ones of the serving loop, so a system's
// trajectory does not depend on which of them ran it)

// x into [0, L).  An atom moves much less than a box per step, so one shift
// of +-L covers the step (FP64 division is slow here); the floor form is the
// fallback and gives the same value for x in [-L, 2L).
__device__ __forceinline__ double md_wrap_box(double x, double L)
{
    // the common case, +0 <= x < L, decided on the bit patterns with integer
    // compares (FP64 compares issue at the FP64 rate, a small fraction of the
    // FP32 one on this part): for x with the sign bit clear the IEEE order is
    // the integer order; -0, negatives, NaN and x >= L take the path below
    const long long bx = __double_as_longlong(x);
    if (bx >= 0 && bx < __double_as_longlong(L)) return x;
    if (x >= L) {
        x = x < 2.0 * L ? x - L : x - L * floor(x / L);
    } else if (x < 0.0) {
        x = x >= -L ? x + L : x - L * floor(x / L);
    }
    if (x >= L) x -= L;  // x = -tiny rounds up to L
    if (x < 0.0) x = 0.0;
    return x;
}

// Atom i: KICKS half kicks v += dt/2 * 48 f (KICKS = 2 fuses the closing
// kick of the step before, with the same forces: each kick rounds as a
// separate one would), then the drift x += dt v wrapped into [0, L), and the
// float copy for the reduction (a value that rounds up to L wraps to 0).
template <int KICKS>
__device__ __forceinline__ void md_kick_drift_atom(double* __restrict__ x, double* __restrict__ v,
                                                   const float4* __restrict__ f, int64_t i,
                                                   double dt, double L, float4* __restrict__ pos4)
{
    const double hk = 0.5 * dt * 48.0;
    const float4 fi = f[i];
    double* xi = x + 3 * i;
    double* vi = v + 3 * i;
    const double gx = (double)fi.x, gy = (double)fi.y, gz = (double)fi.z;
    double vx = vi[0], vy = vi[1], vz = vi[2];
#pragma unroll
    for (int k = 0; k < KICKS; k++) {
        vx = __fma_rn(hk, gx, vx);
        vy = __fma_rn(hk, gy, vy);
        vz = __fma_rn(hk, gz, vz);
    }
    const double px = md_wrap_box(__fma_rn(dt, vx, xi[0]), L);
    const double py = md_wrap_box(__fma_rn(dt, vy, xi[1]), L);
    const double pz = md_wrap_box(__fma_rn(dt, vz, xi[2]), L);
    vi[0] = vx;
    vi[1] = vy;
    vi[2] = vz;
    xi[0] = px;
    xi[1] = py;
    xi[2] = pz;
    float fx = (float)px, fy = (float)py, fz = (float)pz;
    const float Lf = (float)L;
    if (fx >= Lf) fx = 0.f;
    if (fy >= Lf) fy = 0.f;
    if (fz >= Lf) fz = 0.f;
    pos4[i] = make_float4(fx, fy, fz, 0.f);
}

// Atom i: the closing half kick of a step.
__device__ __forceinline__ void md_kick_atom(double* __restrict__ v, const float4* __restrict__ f,
                                             int64_t i, double dt)
{
    const double hk = 0.5 * dt * 48.0;
    const float4 fi = f[i];
    double* vi = v + 3 * i;
    vi[0] = __fma_rn(hk, (double)fi.x, vi[0]);
    vi[1] = __fma_rn(hk, (double)fi.y, vi[1]);
    vi[2] = __fma_rn(hk, (double)fi.z, vi[2]);
}

struct irr_md {
    irr_md_config cfg{};
    int device = 0;
    int sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t n = 0;
    LawParams law{};
    TiledShape shape{};
    double* x = nullptr;       // [3n] positions, execution order
    double* v = nullptr;       // [3n] velocities
    double* tmp = nullptr;     // [3n] permutation scratch
    float4* pos4 = nullptr;    // float copy of x for the reduction
    float4* force = nullptr;   // reduction result (F / 48)
    int32_t* ids = nullptr;    // execution slot -> caller's atom id
    int32_t* ids_tmp = nullptr;
    PartitionOut part{};
    irr::Sliced sl{};          // sliced entry layout (when it pays)
    InstDesc* d_inst = nullptr;
    InstDesc inst{};           // host copy of *d_inst (the force launch's parameter)
    WorkItem* d_items = nullptr;
    int num_items = 0;
    int* d_queue = nullptr;
    int* d_status = nullptr;
    double* d_acc = nullptr;   // [4] KE, PE, virial, spare
    int64_t edges = 0;
    int64_t steps = 0;
    int64_t rebuilds = 0;
    int64_t since_rebuild = 0;
    uint32_t row_cap = 0;      // per-node slots for the next rebuild's one-pass search (0: two passes)
    int2* half = nullptr;      // exec_plain: the half list (i < j, execution order) of the rows
};


namespace irr {
// One step of one system, split so a server can batch the force launch:
// md_kick_drift, md_rebuild (when due), the forces (md_forces, or one
// batched launch over md_instance() of many systems), md_kick.
int md_rebuild(irr_md* m);
int md_forces(irr_md* m);
int md_kick_drift(irr_md* m);
int md_kick(irr_md* m);
InstDesc md_instance(const irr_md* m);
// Digest of the final positions by atom id (a sum of per-atom 64-bit mixes).
int md_state_digest(irr_md* m, uint64_t* digest);
}  // namespace irr
