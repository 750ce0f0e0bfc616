// pf_scan.cu - exclusive prefix sums over uint32 arrays (reduce, scan the block sums, scan-add).
//
// Used to turn per-contour segment counts, per-segment leaf counts, per-tile fill
// counts and per-framebuffer-tile list lengths into offsets, which replaces the
// reference's atomic allocation and linked lists (pathfinder/shaders/d3d11/bin.comp:100-103,
// propagate.comp:179,210) with a deterministic, gap-free layout.
#include "pf_internal.h"

namespace pfc {

namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;  // 4096

__device__ __forceinline__ uint32_t warp_inclusive(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total in *total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t *total) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_inclusive(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
        const uint32_t wi = warp_inclusive(w);
        if (lane < kScanThreads / 32) warp_sums[lane] = wi - w;
        if (lane == kScanThreads / 32 - 1) *total = wi;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + inc - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_reduce(const uint32_t *__restrict__ in, uint32_t n,
                                                         uint32_t *__restrict__ block_sums) {
    const uint32_t base = blockIdx.x * kScanTile;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const uint32_t i = base + k * kScanThreads + threadIdx.x;
        if (i < n) s += in[i];
    }
    __shared__ uint32_t total;
    block_exclusive(s, &total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Exclusive scan of one tile per block, plus an optional per-block offset.
__global__ void __launch_bounds__(kScanThreads) k_scan_tile(const uint32_t *in, uint32_t *out, uint32_t n,
                                                            const uint32_t *__restrict__ block_offsets,
                                                            uint32_t *total_out) {
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const uint32_t i = base + k;
        v[k] = i < n ? in[i] : 0u;
        s += v[k];
    }
    __shared__ uint32_t total;
    uint32_t run = block_exclusive(s, &total);
    if (block_offsets) run += block_offsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const uint32_t i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (total_out && threadIdx.x == 0) *total_out = total;
}

}  // namespace

size_t scan_temp_bytes(uint32_t n) {
    size_t bytes = 0;
    while (n > kScanTile) {
        n = (n + kScanTile - 1) / kScanTile;
        bytes += (size_t(n) + 1) * sizeof(uint32_t);
    }
    return bytes + 64;
}

cudaError_t scan_exclusive_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total, void *temp,
                               cudaStream_t st) {
    if (n == 0) {
        return cudaMemsetAsync(total, 0, sizeof(uint32_t), st);
    }
    if (n <= kScanTile) {
        k_scan_tile<<<1, kScanThreads, 0, st>>>(in, out, n, nullptr, total);
        count_launches(1);
        return cudaGetLastError();
    }
    const uint32_t nb = (n + kScanTile - 1) / kScanTile;
    uint32_t *sums = static_cast<uint32_t *>(temp);
    k_reduce<<<nb, kScanThreads, 0, st>>>(in, n, sums);
    count_launches(2);
    cudaError_t e = scan_exclusive_u32(sums, sums, nb, total, sums + nb + 1, st);
    if (e != cudaSuccess) return e;
    k_scan_tile<<<nb, kScanThreads, 0, st>>>(in, out, n, sums, nullptr);
    return cudaGetLastError();
}

}  // namespace pfc
