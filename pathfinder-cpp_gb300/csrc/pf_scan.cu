// pf_scan.cu - exclusive prefix sums over uint32 arrays: single pass, decoupled look-back.
//
// Used to turn per-contour segment counts, per-segment leaf counts, per-tile fill
// counts and per-row path counts into offsets, which replaces the reference's atomic
// allocation and linked lists (pathfinder/shaders/d3d11/bin.comp:100-103,
// propagate.comp:179,210) with a deterministic, gap-free layout.
//
// Each block scans one tile of kScanTile elements (uint4 loads), publishes its aggregate,
// then resolves its prefix by looking back over the predecessors' published aggregates /
// inclusive prefixes (a status word per tile: flag in the top 2 bits, value below).  Tiles
// are taken in launch order from an atomic ticket so a block only ever waits on tiles that
// started before it.  Every wait is bounded: after kSpinLimit polls the block records an
// error bit and stops.
#include "pf_internal.h"

namespace pfc {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;                               // 4 x uint4 per thread
constexpr uint32_t kScanTile = kScanThreads * kScanItems;  // 4096
constexpr uint64_t kFlagAgg = 1ull << 62, kFlagInc = 2ull << 62, kValMask = (1ull << 62) - 1;
constexpr uint32_t kSpinLimit = 1u << 20;

__device__ __forceinline__ uint32_t warp_inclusive(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

// state[0] = ticket counter, state[1 + t] = status of tile t
__global__ void __launch_bounds__(kScanThreads) k_scan(const uint32_t *in, uint32_t *out, uint32_t n,
                                                       unsigned long long *state, uint32_t *total,
                                                       uint32_t *err) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_prefix;
    if (threadIdx.x == 0) s_tile = (uint32_t)atomicAdd(&state[0], 1ull);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = (uint64_t)tile * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    if (base + kScanItems <= n && ((reinterpret_cast<uintptr_t>(in + base) & 15) == 0)) {
#pragma unroll
        for (int q = 0; q < kScanItems / 4; q++) {
            const uint4 x = *reinterpret_cast<const uint4 *>(in + base + 4 * q);
            v[4 * q + 0] = x.x;
            v[4 * q + 1] = x.y;
            v[4 * q + 2] = x.z;
            v[4 * q + 3] = x.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; k++) v[k] = base + k < n ? in[base + k] : 0u;
    }
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) sum += v[k];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_inclusive(sum);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
        const uint32_t wi = warp_inclusive(w);
        if (lane < kScanThreads / 32) warp_sums[lane] = wi - w;
        const uint32_t agg = __shfl_sync(0xffffffffu, wi, kScanThreads / 32 - 1);
        // publish the aggregate, then look back over a window of 32 predecessors at a time
        // (lane l reads tile `base - l`); stop at the nearest inclusive prefix
        volatile unsigned long long *st = state + 1;
        if (tile == 0) {
            if (lane == 0) {
                st[0] = kFlagInc | agg;
                s_prefix = 0;
            }
        } else {
            if (lane == 0) st[tile] = kFlagAgg | agg;
            uint64_t prefix = 0;
            int64_t base = (int64_t)tile - 1;
            uint32_t spins = 0;
            for (;;) {
                const int64_t idx = base - lane;
                const unsigned long long sv = idx >= 0 ? st[idx] : kFlagInc;
                const uint64_t flag = sv & ~kValMask;
                const uint32_t inc_mask = __ballot_sync(0xffffffffu, flag == kFlagInc);
                const uint32_t wait_mask = __ballot_sync(0xffffffffu, flag == 0);
                const uint32_t upto = inc_mask ? (inc_mask & (0u - inc_mask)) * 2u - 1u : 0xffffffffu;
                if (wait_mask & upto) {
                    if (++spins > kSpinLimit) {
                        if (lane == 0) atomicOr(err, kErrScanWait);
                        break;
                    }
                    continue;
                }
                uint64_t v = (upto >> lane) & 1u ? (sv & kValMask) : 0;
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
                prefix += v;
                if (inc_mask) break;
                base -= 32;
            }
            if (lane == 0) {
                st[tile] = kFlagInc | (prefix + agg);
                s_prefix = (uint32_t)prefix;
            }
        }
    }
    __syncthreads();
    uint32_t run = s_prefix + warp_sums[warp] + inc - sum;
    if (tile == gridDim.x - 1 && threadIdx.x == kScanThreads - 1 && total) {
        total[0] = run + sum;
    }
    if (base + kScanItems <= n && ((reinterpret_cast<uintptr_t>(out + base) & 15) == 0)) {
        uint32_t o[kScanItems];
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            o[k] = run;
            run += v[k];
        }
#pragma unroll
        for (int q = 0; q < kScanItems / 4; q++)
            *reinterpret_cast<uint4 *>(out + base + 4 * q) = make_uint4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            if (base + k < n) out[base + k] = run;
            run += v[k];
        }
    }
}

}  // namespace

size_t scan_temp_bytes(uint32_t n) {
    const size_t tiles = (size_t(n) + kScanTile - 1) / kScanTile;
    return (tiles + 1) * sizeof(unsigned long long) + 64;
}

cudaError_t scan_exclusive_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total, void *temp,
                               cudaStream_t st, uint32_t *err) {
    if (n == 0) return cudaMemsetAsync(total, 0, sizeof(uint32_t), st);
    const uint32_t tiles = (n + kScanTile - 1) / kScanTile;
    cudaError_t e = cudaMemsetAsync(temp, 0, (size_t(tiles) + 1) * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    k_scan<<<tiles, kScanThreads, 0, st>>>(in, out, n, static_cast<unsigned long long *>(temp), total, err);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace pfc
