// irregular_plugin.cuh -- compiles an application's per-edge function (the
// reference's irregular.h plugin) into a kernel that a partitioned handle
// runs at every step (irr_set_user_map, irregular_gb300.h).
//
// The reference builds its executors around the application's irregular.h:
// `map(object, point_data, part_index, edge_data, parameter, task_id,
// part_id, reduce_ptr)` is called once per edge of a part and inserts its
// contributions into a reduction object keyed by node, which combines equal
// keys with `reduce` (moldyn/irregular.h:22-118, moldyn/irregular/
// gpu_kernel.cu:44-102, moldyn/irregular/ros.cu:10-68).  Here the object is
// a node's row: one thread owns a row of the handle's CSR (rows in execution
// order, neighbours ascending) and calls the map once per entry with the edge
// (row, neighbour), part_id = row and part_index[x] = x, so that the map's
// own "is this end mine" tests keep the row's end; the object keeps only
// inserts keyed by its row.  No atomics and a fixed order per row: results
// are bitwise reproducible.
//
// Use, from a .cu file compiled with nvcc for sm_103a:
//   * the reference's table form -- compat/irregular/irr_user_map.cu compiles
//     an unchanged irregular.h (GPU_KERNEL: DEVICE/OBJECT/CONSTANT, namespace
//     FGPU, map_function_table / reduce_function_table) against the
//     Reduction_Object_S of compat/irregular/ros.h and exports a launch
//     function that calls map_function_table[map_idx] (an indirect call, as
//     the reference makes);
//   * one map, inlined -- a functor calling the map directly and
//     irr_plugin::launch_rows<Object>(view, stream, functor).
#ifndef IRREGULAR_PLUGIN_CUH_
#define IRREGULAR_PLUGIN_CUH_

#include <cuda_runtime.h>
#include <stdint.h>

#include "irregular_gb300.h"

namespace irr_plugin {

constexpr int kRowThreads = 256;

// Knuth's TwoSum (error-free float addition): s + e == a + b exactly.
// __fadd_rn keeps the compiler from contracting or reassociating the steps.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float bb = __fadd_rn(s, -a);
    e = __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb));
}

// A row's reduction object over VALUE records with the application's reduce:
// the first insert keyed by the row is copied, later ones are combined as
// reduce(&acc, value), in the row's entry order (the reference's reduction
// objects copy a key's first value and reduce the rest into it,
// moldyn/irregular/ros.cu:10-68).  Inserts of other keys are dropped: that
// end's own row keeps its contribution.  A row without inserts stores zero
// bytes.
template <class Key, class Value, class ReduceFp>
struct RowObject {
    typedef Value value_type;
    Key row_;
    int has_;
    Value acc_;

    __device__ void begin(Key row)
    {
        row_ = row;
        has_ = 0;
    }
    __device__ void first_init() {}
    __device__ void init() { has_ = 0; }
    __device__ bool insert(Key* key, Value* value, ReduceFp reduce_ptr)
    {
        if (!(*key == row_)) return true;
        if (!has_) {
            acc_ = *value;
            has_ = 1;
        } else {
            reduce_ptr(&acc_, value);
        }
        return true;
    }
    __device__ void store(void* dst) const
    {
        static_assert(sizeof(Value) % 4 == 0, "VALUE must be a whole number of 4-byte words");
        uint32_t* d = static_cast<uint32_t*>(dst);
        const uint32_t* a = reinterpret_cast<const uint32_t*>(&acc_);
#pragma unroll
        for (int w = 0; w < (int)(sizeof(Value) / 4); w++) d[w] = has_ ? a[w] : 0u;
    }
};

// The same object for VALUEs that are tuples of floats combined by +: each
// float is summed with a TwoSum-compensated accumulator (the row's sum is
// then the FP64 sum of its float terms rounded once, up to second-order
// terms), and reduce_ptr is not called.
template <class Key, class Value, class ReduceFp>
struct RowSumObject {
    typedef Value value_type;
    static constexpr int kWords = (int)(sizeof(Value) / 4);
    static_assert(sizeof(Value) % 4 == 0, "VALUE must be a tuple of floats");
    Key row_;
    float s_[kWords];
    float c_[kWords];

    __device__ void begin(Key row)
    {
        row_ = row;
#pragma unroll
        for (int w = 0; w < kWords; w++) s_[w] = c_[w] = 0.0f;
    }
    __device__ void first_init() {}
    __device__ void init() { begin(row_); }
    __device__ bool insert(Key* key, Value* value, ReduceFp)
    {
        if (!(*key == row_)) return true;
        const float* v = reinterpret_cast<const float*>(value);
#pragma unroll
        for (int w = 0; w < kWords; w++) {
            float s, e;
            two_sum(s_[w], v[w], s, e);
            s_[w] = s;
            c_[w] = __fadd_rn(c_[w], e);
        }
        return true;
    }
    __device__ void store(void* dst) const
    {
        float* d = static_cast<float*>(dst);
#pragma unroll
        for (int w = 0; w < kWords; w++) d[w] = __fadd_rn(s_[w], c_[w]);
    }
};

// One thread per row, rows strided over a grid of whole blocks.  call(obj,
// point_data, part_index, edge_data, parameter, task_id, part_id) applies the
// map; edge_data holds the pair (row, neighbour) and task_id is 0.
template <class Object, class Call>
__global__ void __launch_bounds__(kRowThreads) rows_kernel(irr_user_view v, Call call)
{
    typedef typename Object::value_type Value;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < v.num_nodes; r += stride) {
        Object obj;
        obj.begin((int)r);
        const uint32_t b = v.row_off[r], e = v.row_off[r + 1];
        for (uint32_t k = b; k < e; k++) {
            int edge[2] = {(int)r, v.col[k]};
            call(&obj, v.node_data, v.part_index, (void*)edge, v.param, 0u, (unsigned int)r);
        }
        obj.store(static_cast<char*>(v.values) + (size_t)r * sizeof(Value));
    }
}

// Launches rows_kernel on stream; IRR_ERR_ARG when the handle's record size
// is not sizeof(VALUE).
template <class Object, class Call>
int launch_rows(const irr_user_view* v, void* stream, Call call)
{
    if (!v || v->value_size != (int)sizeof(typename Object::value_type)) return IRR_ERR_ARG;
    if (v->num_nodes <= 0) return IRR_OK;
    const int64_t want = (v->num_nodes + kRowThreads - 1) / kRowThreads;
    const int64_t cap = (int64_t)(v->num_sms > 0 ? v->num_sms : 1) * 8;
    const int grid = (int)(want < cap ? want : cap);
    rows_kernel<Object, Call><<<grid, kRowThreads, 0, (cudaStream_t)stream>>>(*v, call);
    return cudaGetLastError() == cudaSuccess ? IRR_OK : IRR_ERR_CUDA;
}

}  // namespace irr_plugin

#endif
