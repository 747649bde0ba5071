// irr_static.cu -- Morton node ordering that allocates no device memory.
//
// irr_morton_order_static computes the same permutation as the partitioner's
// node ordering (perm[new] = old, bit for bit what irr_get_partition returns
// for reorder = 1), for callers that must not allocate: for example a host
// application that reserves the GPU's memory for its own pool at start-up,
// or a latency-bound loop in which a cudaMalloc/cudaFree -- which may
// synchronise the device -- is not acceptable.  The caller passes the
// positions and the output; all scratch lives in g_morton_scratch below.
//
// g_morton_scratch is a file-scope device array: every GPU that loads this
// library holds kStaticScratchBytes (12,886,272 bytes, about 12.3 MiB) of it
// until the process exits.  Host code cannot use its name as a device
// address, so the address is looked up with the device current, by
// cudaGetSymbolAddress: on every call whose stream is not capturing (so a
// device reset, which gives the array a new address, is picked up), and
// taken from the last look-up on that device while a capture is under way
// (so make the first call on a device before any stream capture, and none
// after a device reset while capturing).  Calls share the array and it keeps
// the previous call's contents: everything this code reads from it is written
// earlier in the same call, and calls that overlap on the GPU (from two
// streams or two threads) race on it, so callers must order them.
#include <cmath>
#include <mutex>

#include "irr_internal.cuh"
#include "../../include/irregular_gb300.h"

namespace irr {
namespace {

constexpr int64_t kStaticMaxNodes = IRR_MORTON_STATIC_MAX_NODES;
constexpr int64_t kMaxTiles = (kStaticMaxNodes + kSortTile - 1) / kSortTile;
constexpr int kBboxParts = 1024;

// Scratch layout (offsets in bytes, 256-aligned).
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffKeys = 0;
constexpr size_t kOffKeysTmp = align256(kOffKeys + 4 * kStaticMaxNodes);
constexpr size_t kOffValsTmp = align256(kOffKeysTmp + 4 * kStaticMaxNodes);
constexpr size_t kOffHist = align256(kOffValsTmp + 4 * kStaticMaxNodes);
constexpr size_t kOffScan = align256(kOffHist + 4 * 256 * kMaxTiles);
constexpr size_t kScanWords = 4096;  // block sums of every scan level
constexpr size_t kOffBbox = align256(kOffScan + 4 * kScanWords);
constexpr size_t kOffFrame = align256(kOffBbox + 4 * 6 * kBboxParts);
constexpr size_t kStaticScratchBytes = align256(kOffFrame + 4 * 8);
static_assert(kStaticScratchBytes == IRR_MORTON_STATIC_SCRATCH_BYTES,
              "the header states the scratch array's size");

__device__ __align__(256) unsigned char g_morton_scratch[kStaticScratchBytes];

std::mutex g_addr_mutex;
void* g_addr[64] = {};

// Device address of g_morton_scratch on `device` (the current device): looked
// up again unless `s` is capturing, when the last look-up on the device is
// used (a capture may not be the place for a first look-up, which can load
// the module).
cudaError_t scratch_address(int device, cudaStream_t s, unsigned char** out)
{
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;  // unknown: do not risk a look-up
    }
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_morton_scratch);
        if (e != cudaSuccess) return e;
        g_addr[device] = p;
    }
    if (!g_addr[device]) return cudaErrorStreamCaptureUnsupported;
    *out = static_cast<unsigned char*>(g_addr[device]);
    return cudaSuccess;
}

__device__ __forceinline__ float3 record_xyz(const char* raw, int elm, int64_t i)
{
    const float* f = reinterpret_cast<const float*>(raw + i * elm);
    return make_float3(f[0], f[1], f[2]);
}

__global__ void static_bbox_kernel(const char* raw, int elm, int64_t n, float* part)
{
    __shared__ float red[6][256];
    float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float3 p = record_xyz(raw, elm, i);
        v[0] = fminf(v[0], p.x);
        v[1] = fminf(v[1], p.y);
        v[2] = fminf(v[2], p.z);
        v[3] = fmaxf(v[3], p.x);
        v[4] = fmaxf(v[4], p.y);
        v[5] = fmaxf(v[5], p.z);
    }
    for (int c = 0; c < 6; c++) red[c][threadIdx.x] = v[c];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int c = 0; c < 6; c++)
                red[c][threadIdx.x] = c < 3 ? fminf(red[c][threadIdx.x], red[c][threadIdx.x + s])
                                            : fmaxf(red[c][threadIdx.x], red[c][threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = red[threadIdx.x][0];
}

// frame[0..2] = per-axis min, frame[3..5] = 1024 / (max - min) (0 for a flat
// axis): the partitioner's frame, formed with the same float operations.
__global__ void static_frame_kernel(const float* part, int nparts, float* frame)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int b = 0; b < nparts; b++)
        for (int c = 0; c < 3; c++) {
            v[c] = fminf(v[c], part[b * 6 + c]);
            v[3 + c] = fmaxf(v[3 + c], part[b * 6 + 3 + c]);
        }
    for (int c = 0; c < 3; c++) {
        const float ext = __fsub_rn(v[3 + c], v[c]);
        frame[c] = v[c];
        frame[3 + c] = ext > 0.0f ? __fdiv_rn(1024.0f, ext) : 0.0f;
    }
}

__device__ __forceinline__ uint32_t quant10_static(float x, float lo, float scale)
{
    float t = __fsub_rn(x, lo);
    t = __fmul_rn(t, scale);
    if (!(t > 0.0f)) return 0u;
    if (t >= 1023.0f) return 1023u;
    return __float2uint_rz(t);
}

__global__ void static_keys_kernel(const char* raw, int elm, int64_t n, const float* frame,
                                   uint32_t* keys, int32_t* vals)
{
    const float lx = frame[0], ly = frame[1], lz = frame[2];
    const float sx = frame[3], sy = frame[4], sz = frame[5];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float3 p = record_xyz(raw, elm, i);
        keys[i] = spread3(quant10_static(p.x, lx, sx)) | (spread3(quant10_static(p.y, ly, sy)) << 1) |
                  (spread3(quant10_static(p.z, lz, sz)) << 2);
        vals[i] = (int32_t)i;
    }
}

// Exclusive scan with the block sums of every level carved from `ws`.
cudaError_t scan_ws(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* ws, size_t ws_words,
                    cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    if ((size_t)nb > ws_words) return cudaErrorInvalidValue;
    scan_blocks_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, ws);
    IRR_CUDA_TRY(cudaGetLastError());
    if (nb > 1) {
        IRR_CUDA_TRY(scan_ws(ws, ws, nb, ws + nb, ws_words - (size_t)nb, s));
        add_offsets_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(out, n, ws);
        IRR_CUDA_TRY(cudaGetLastError());
    }
    return cudaSuccess;
}

int grid_of(int64_t n)
{
    int64_t g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

}  // namespace
}  // namespace irr

extern "C" int irr_morton_order_static(int device, void* stream, const void* d_pos, int pos_elm,
                                       int64_t n, int32_t* d_perm)
{
    using namespace irr;
    if (n < 0 || (n > 0 && (!d_pos || !d_perm))) return IRR_ERR_ARG;
    if (pos_elm != 12 && pos_elm != 16) return IRR_ERR_ARG;
    if (n > kStaticMaxNodes) return IRR_ERR_CAPACITY;
    // float records and int32 output: both read or written as 4-byte words
    if ((reinterpret_cast<uintptr_t>(d_pos) | reinterpret_cast<uintptr_t>(d_perm)) % 4u)
        return IRR_ERR_ARG;
    DeviceGuard dev_guard(device);  // the caller's current device comes back on return
    if (!dev_guard.ok()) return IRR_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* ws = nullptr;
    if (scratch_address(device, s, &ws) != cudaSuccess) {
        cudaGetLastError();
        return IRR_ERR_CUDA;
    }
    if (n == 0) return IRR_OK;
    const char* raw = static_cast<const char*>(d_pos);
    uint32_t* keys = reinterpret_cast<uint32_t*>(ws + kOffKeys);
    uint32_t* keys_tmp = reinterpret_cast<uint32_t*>(ws + kOffKeysTmp);
    int32_t* vals_tmp = reinterpret_cast<int32_t*>(ws + kOffValsTmp);
    uint32_t* hist = reinterpret_cast<uint32_t*>(ws + kOffHist);
    uint32_t* scan = reinterpret_cast<uint32_t*>(ws + kOffScan);
    float* bbox = reinterpret_cast<float*>(ws + kOffBbox);
    float* frame = reinterpret_cast<float*>(ws + kOffFrame);
    cudaError_t e = cudaSuccess;
    if (n == 1) {
        // one node: the identity, as the partitioner orders it
        e = cudaMemsetAsync(d_perm, 0, sizeof(int32_t), s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return IRR_ERR_CUDA;
        }
        return IRR_OK;
    }
    const int parts = (int)(n < (int64_t)kBboxParts * 256 ? (n + 255) / 256 : kBboxParts);
    static_bbox_kernel<<<parts, 256, 0, s>>>(raw, pos_elm, n, bbox);
    static_frame_kernel<<<1, 1, 0, s>>>(bbox, parts, frame);
    static_keys_kernel<<<grid_of(n), 256, 0, s>>>(raw, pos_elm, n, frame, keys, d_perm);
    e = cudaGetLastError();
    // stable LSD radix sort of (key, node), 30-bit keys: 4 passes, ends in (keys, d_perm)
    const int64_t ntiles = (n + kSortTile - 1) / kSortTile;
    uint32_t *ka = keys, *kb = keys_tmp;
    int32_t *va = d_perm, *vb = vals_tmp;
    for (int shift = 0; shift < 32 && e == cudaSuccess; shift += 8) {
        radix_hist_kernel<<<(unsigned)ntiles, kSortThreads, 0, s>>>(ka, n, shift, hist, ntiles);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = scan_ws(hist, hist, 256 * ntiles, scan, kScanWords, s);
        if (e == cudaSuccess) {
            radix_scatter_kernel<<<(unsigned)ntiles, kSortThreads, 0, s>>>(ka, va, kb, vb, n, shift,
                                                                          hist, ntiles);
            e = cudaGetLastError();
        }
        uint32_t* tk = ka;
        ka = kb;
        kb = tk;
        int32_t* tv = va;
        va = vb;
        vb = tv;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return IRR_ERR_CUDA;
    }
    return IRR_OK;
}
