// atag_pairs.cuh — the per-frame hash table of cluster pairs (key = the
// pair's two label values, smaller one in the high word): open addressing
// with linear probing over a power-of-two table, plus the atomic merge of a
// batch of points' ClusterBounds sums into a slot.
#pragma once

#include "atag_kernels.cuh"

namespace atag {

constexpr unsigned long long EMPTY_KEY = ~0ull;

__device__ __forceinline__ uint32_t hash_key(unsigned long long k) {
    return (uint32_t)((k * 0x9E3779B97F4A7C15ull) >> 32);
}

__device__ __forceinline__ uint32_t global_insert(const FrameDesc& F, unsigned long long key) {
    uint32_t mask = F.pair_cap - 1, h = hash_key(key) & mask;
    for (uint32_t p = 0; p < F.pair_cap; p++) {
        unsigned long long k = atomicCAS(&F.pair_keys[h], EMPTY_KEY, key);
        if (k == EMPTY_KEY || k == key) return h;
        h = (h + 1) & mask;
    }
    return INVALID;
}
__device__ __forceinline__ uint32_t global_lookup(const FrameDesc& F, unsigned long long key) {
    uint32_t mask = F.pair_cap - 1, h = hash_key(key) & mask;
    for (uint32_t p = 0; p < F.pair_cap; p++) {
        unsigned long long k = F.pair_keys[h];
        if (k == key) return h;
        if (k == EMPTY_KEY) return INVALID;
        h = (h + 1) & mask;
    }
    return INVALID;
}
__device__ __forceinline__ uint32_t global_flush(const FrameDesc& F, uint32_t gs, uint32_t cnt, uint32_t xmin,
                                                 uint32_t xmax, uint32_t ymin, uint32_t ymax, int gx, int gy,
                                                 unsigned long long pxgx) {
    uint32_t old = atomicAdd(&F.pair_count[gs], cnt);
    uint32_t* bb = reinterpret_cast<uint32_t*>(&F.pair_bbox[gs]);
    atomicMin(bb + 0, xmin);
    atomicMax(bb + 1, xmax);
    atomicMin(bb + 2, ymin);
    atomicMax(bb + 3, ymax);
    int* gsum = reinterpret_cast<int*>(&F.pair_gsum[gs]);
    if (gx) atomicAdd(gsum + 0, gx);
    if (gy) atomicAdd(gsum + 1, gy);
    if (pxgx) atomicAdd(&F.pair_pxgx[gs], pxgx);
    return old;
}

}  // namespace atag
