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
    std::vector<WorkItem> host_items;  // this system's node blocks (for batched launches)
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
