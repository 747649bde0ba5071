// irr_user.cu -- data movement for handles bound to a user map (the
// irregular.h plugin, include/irregular_plugin.cuh): node and result records
// of the application's own sizes gathered between the caller's node order and
// execution order, result floats widened to doubles, the identity part_index,
// and coordinates turned into the positions the partitioner orders by.
//
// The reference keeps node records in its own order after reorder_satellite_
// data (moldyn/irregular/partitioner.cpp:299-346) and copies VALUE records
// back per device range (irregular_runtime.cu:393-411); here records are
// opaque words moved by one gather per call.
#include "irr_internal.cuh"

namespace irr {
namespace {

constexpr int kThreads = 256;

int grid_of(int64_t work)
{
    const int64_t b = (work + kThreads - 1) / kThreads;
    return (int)(b < 65535 * 16 ? (b > 0 ? b : 1) : 65535 * 16);
}

// dst record k = src record idx[k] (idx == nullptr: k), words words each.
// One thread per word: consecutive threads copy consecutive words of a
// record, so each record is one contiguous read and one contiguous write.
__global__ void gather_words_kernel(const uint32_t* __restrict__ src, int words,
                                    const int32_t* __restrict__ idx, int64_t n,
                                    uint32_t* __restrict__ dst)
{
    const int64_t total = n * words;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / words;
        const int w = (int)(t - k * words);
        const int64_t from = idx ? (int64_t)idx[k] : k;
        dst[t] = src[from * words + w];
    }
}

// dst (doubles) record k = src (floats) record idx[k], each float widened.
__global__ void widen_kernel(const float* __restrict__ src, int words, const int32_t* __restrict__ idx,
                             int64_t n, double* __restrict__ dst)
{
    const int64_t total = n * words;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / words;
        const int w = (int)(t - k * words);
        const int64_t from = idx ? (int64_t)idx[k] : k;
        dst[t] = (double)src[from * words + w];
    }
}

__global__ void iota_kernel(int32_t* __restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)i;
}

// Coordinates (dims components of float or double) -> float4 (x, y, z, 0);
// a 2-D point gets z = 0.
template <class T>
__global__ void coords_kernel(const T* __restrict__ c, int dims, int64_t n, float4* __restrict__ dst)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const T* p = c + i * dims;
        dst[i] = make_float4((float)p[0], (float)p[1], dims > 2 ? (float)p[2] : 0.0f, 0.0f);
    }
}

}  // namespace

cudaError_t launch_gather_records(const void* src, int elm_size, const int32_t* idx, int64_t n,
                                  void* dst, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (elm_size <= 0 || (elm_size & 3)) return cudaErrorInvalidValue;
    const int words = elm_size / 4;
    gather_words_kernel<<<grid_of(n * words), kThreads, 0, s>>>(
        static_cast<const uint32_t*>(src), words, idx, n, static_cast<uint32_t*>(dst));
    return cudaGetLastError();
}

cudaError_t launch_widen_records(const void* src, int elm_size, const int32_t* idx, int64_t n,
                                 void* dst, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (elm_size <= 0 || (elm_size & 3)) return cudaErrorInvalidValue;
    const int words = elm_size / 4;
    widen_kernel<<<grid_of(n * words), kThreads, 0, s>>>(static_cast<const float*>(src), words, idx,
                                                         n, static_cast<double*>(dst));
    return cudaGetLastError();
}

cudaError_t launch_iota(int32_t* out, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    iota_kernel<<<grid_of(n), kThreads, 0, s>>>(out, n);
    return cudaGetLastError();
}

cudaError_t launch_coords_to_pos(const void* coords, int coord_size, int dims, int64_t n, float4* dst,
                                 cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (dims != 2 && dims != 3) return cudaErrorInvalidValue;
    if (coord_size == 8)
        coords_kernel<double><<<grid_of(n), kThreads, 0, s>>>(static_cast<const double*>(coords), dims, n, dst);
    else if (coord_size == 4)
        coords_kernel<float><<<grid_of(n), kThreads, 0, s>>>(static_cast<const float*>(coords), dims, n, dst);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

}  // namespace irr
