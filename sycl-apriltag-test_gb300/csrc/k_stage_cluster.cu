// k_stage_cluster.cu — kernels of the stage entry points that stand in for
// the reference's oneDPL glue between its device functions:
//   atag_cluster       stages 4-11 (src/main.cpp:467-801), from the dense
//                      boundary planes that find_boundaries writes to the
//                      line-fit prefix sums that fit_lines reads;
//   atag_corner_peaks  stages 13-15 (src/main.cpp:832-907), from fit_lines'
//                      dense corner array to do_indexing's inputs.
// atag_cluster shares the fused detector's pair table, filter and cluster
// sorts (k_cluster.cu); only the entry and exit over the dense planes are
// here: the planes are read twice (sums per pair, then the points of the
// surviving clusters), so no compacted point list is ever written.
#include "atag_kernels.cuh"
#include "atag_pairs.cuh"

namespace atag {

// Stages 4 and 6: copy_if(point != 0) and reduce_by_segment of
// ClusterBounds::inital_from_point per pair key (cluster_bounds.h:27-45).
// The sort by key that separates them in the reference only orders the
// pairs, which k_pairs_finalize does on the distinct keys.  A warp first
// merges the entries that share a key (match_any), then one lane adds the
// sums to the pair's slot of the frame's hash table.
__global__ void __launch_bounds__(256) k_planes_pairs(const __grid_constant__ FrameSet fs,
                                                      const uint32_t* __restrict__ points,
                                                      const unsigned long long* __restrict__ keys, uint32_t n) {
    const FrameDesc& F = fs.get(0);
    uint32_t* status = F.counters + CNT_STATUS;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t found = 0;
    // warp-uniform trip count: every lane takes part in the warp collectives
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + lane;
        const uint32_t p = i < n ? __ldg(points + i) : 0u;
        const bool v = p != 0u;
        if (!__any_sync(0xFFFFFFFFu, v)) continue;
        const unsigned long long key = v ? __ldg(keys + i) : EMPTY_KEY;
        found += v ? 1u : 0u;
        const unsigned m = __match_any_sync(0xFFFFFFFFu, key);
        const int leader = __ffs(m) - 1;
        const uint32_t xd = bp_xd(p), yd = bp_yd(p);
        const int gx = bp_gx(p), gy = bp_gy(p);
        const uint32_t xmn = __reduce_min_sync(m, xd), xmx = __reduce_max_sync(m, xd);
        const uint32_t ymn = __reduce_min_sync(m, yd), ymx = __reduce_max_sync(m, yd);
        const int sgx = __reduce_add_sync(m, gx), sgy = __reduce_add_sync(m, gy);
        const int spx = __reduce_add_sync(m, (int)xd * gx + (int)yd * gy);
        if (v && (int)lane == leader) {
            const uint32_t gs = global_insert(F, key);
            if (gs == INVALID) atomicOr(status, ATAG_DEVFLAG_PAIR_OVERFLOW);
            else global_flush(F, gs, (uint32_t)__popc(m), xmn, xmx, ymn, ymx, sgx, sgy,
                              (unsigned long long)(long long)spx);
        }
    }
    found = warp_sum_u32(found);
    if (lane == 0 && found) atomicAdd(F.counters + CNT_ALLPOINTS, found);
}

// Stage 7: each point of a pair that passed the filter goes to its
// cluster's segment with its calc_theta key (main.cpp:621-675); the
// cluster sorts then order each segment by (slope, point).
__global__ void __launch_bounds__(256) k_planes_scatter(const __grid_constant__ FrameSet fs,
                                                        const uint32_t* __restrict__ points,
                                                        const unsigned long long* __restrict__ keys, uint32_t n) {
    const FrameDesc& F = fs.get(0);
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + lane;
        const uint32_t p = i < n ? __ldg(points + i) : 0u;
        if (!__any_sync(0xFFFFFFFFu, p != 0u)) continue;
        uint32_t cid = INVALID;
        if (p != 0u) {
            const uint32_t slot = global_lookup(F, __ldg(keys + i));
            if (slot != INVALID) cid = F.pair_cluster[slot];
        }
        const unsigned mask = __match_any_sync(0xFFFFFFFFu, cid);
        if (cid != INVALID) {
            const int leader = __ffs(mask) - 1;
            uint32_t b = 0;
            if ((int)lane == leader) b = atomicAdd(F.cluster_cursor + cid, (uint32_t)__popc(mask));
            b = __shfl_sync(mask, b, leader);
            const uint32_t rank = __popc(mask & ((1u << lane) - 1u));
            const atag_cluster_extents ext = F.cluster_extents[cid];
            const float2 ctr = F.cluster_center[cid];
            const float theta = calc_theta(p, ctr.x, ctr.y);
            if (b + rank < ext.count)
                F.sortbuf[ext.start + b + rank] = ((unsigned long long)float_order_key(theta) << 32) | p;
        }
    }
}

// The 16-bit cluster index of every sorted point (main.cpp:641), the
// filtered keys if asked, and the counters.  One warp per cluster.
__global__ void __launch_bounds__(256) k_stage_cluster_out(const __grid_constant__ FrameSet fs,
                                                           uint16_t* cluster_indices,
                                                           unsigned long long* cluster_keys_out) {
    const FrameDesc& F = fs.get(0);
    const uint32_t C = F.counters[CNT_CLUSTERS];
    const uint32_t lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (uint32_t c = blockIdx.x * wpb + (threadIdx.x >> 5); c < C; c += gridDim.x * wpb) {
        const atag_cluster_extents ext = F.cluster_extents[c];
        for (uint32_t k = lane; k < ext.count; k += 32) cluster_indices[ext.start + k] = (uint16_t)c;
        if (lane == 0 && cluster_keys_out) cluster_keys_out[c] = F.cluster_keys[c];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        F.stats->n_corners = 0;
        F.stats->n_peak_clusters = 0;
        F.stats->n_fitted = 0;
        F.stats->n_quads = 0;
        F.stats->status = F.counters[CNT_STATUS];
    }
}

// ---------------------------------------------------------------------------
// Stages 13-15: copy_if(error != 0) over the dense corner array, sort by
// (cluster ascending, error descending) and one PeakExtents per cluster
// with corners.  fit_lines writes a cluster's corners inside its extent, so
// the compaction and the sort run per cluster: counts, an exclusive scan
// over the clusters, then each cluster's corners sorted in shared memory.
// The reference's sort leaves ties unordered; here they go by position.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_peaks_count(const atag_corner* __restrict__ found,
                                                     const atag_cluster_extents* __restrict__ ext,
                                                     uint32_t n_clusters, uint32_t* __restrict__ counts) {
    const uint32_t lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (uint32_t c = blockIdx.x * wpb + (threadIdx.x >> 5); c < n_clusters; c += gridDim.x * wpb) {
        const atag_cluster_extents e = ext[c];
        uint32_t k = 0;
        for (uint32_t i0 = 0; i0 < e.count; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool corner = i < e.count && found[(size_t)e.start + i].error != 0.0f;
            k += (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, corner));
        }
        if (lane == 0) counts[c] = k;
    }
}

__global__ void __launch_bounds__(1024) k_peaks_offsets(const uint32_t* __restrict__ counts, uint32_t n_clusters,
                                                        uint32_t* __restrict__ offsets,
                                                        atag_peak_extents* __restrict__ peak_extents,
                                                        uint32_t extents_cap, uint32_t corner_cap,
                                                        uint32_t* __restrict__ d_counts) {
    __shared__ uint32_t red[33];
    uint32_t carry_q = 0, carry_k = 0;
    for (uint32_t c0 = 0; c0 < n_clusters; c0 += blockDim.x) {
        const uint32_t c = c0 + threadIdx.x;
        const uint32_t k = c < n_clusters ? counts[c] : 0u;
        uint32_t tq, tk;
        const uint32_t q = carry_q + block_exclusive_scan_u32(k ? 1u : 0u, red, &tq);
        const uint32_t s = carry_k + block_exclusive_scan_u32(k, red, &tk);
        if (c < n_clusters) offsets[c] = s;
        if (k && q < extents_cap) peak_extents[q] = atag_peak_extents{s, k};
        carry_q += tq;
        carry_k += tk;
    }
    if (threadIdx.x == 0) {
        d_counts[0] = carry_k;
        d_counts[1] = carry_q;
        d_counts[2] = (carry_k > corner_cap || carry_q > extents_cap) ? ATAG_DEVFLAG_QUAD_OVERFLOW : 0u;
    }
}

__global__ void __launch_bounds__(256) k_peaks_sort(const atag_corner* __restrict__ found,
                                                    const atag_cluster_extents* __restrict__ ext,
                                                    uint32_t n_clusters, const uint32_t* __restrict__ counts,
                                                    const uint32_t* __restrict__ offsets,
                                                    atag_corner* __restrict__ out, uint32_t corner_cap,
                                                    uint32_t* __restrict__ d_counts) {
    extern __shared__ unsigned long long pk_keys[];
    __shared__ uint32_t s_n;
    for (uint32_t c = blockIdx.x; c < n_clusters; c += gridDim.x) {
        const uint32_t k = counts[c];
        if (k == 0) continue;  // uniform over the block
        if (k > PK_SORT_CAP) {
            // more corners than a cluster of valid points can have
            if (threadIdx.x == 0) atomicOr(d_counts + 2, ATAG_DEVFLAG_SORT_OVERFLOW);
            continue;
        }
        const atag_cluster_extents e = ext[c];
        if (threadIdx.x == 0) s_n = 0;
        __syncthreads();
        // key: error descending (complemented order key), then position
        for (uint32_t i = threadIdx.x; i < e.count; i += blockDim.x) {
            const float err = found[(size_t)e.start + i].error;
            if (err != 0.0f) {
                const uint32_t at = atomicAdd(&s_n, 1u);
                if (at < k) pk_keys[at] = ((unsigned long long)(~float_order_key(err)) << 32) | i;
            }
        }
        __syncthreads();
        bitonic_sort_u64(pk_keys, k);
        const uint32_t off = offsets[c];
        for (uint32_t j = threadIdx.x; j < k; j += blockDim.x)
            if (off + j < corner_cap) out[off + j] = found[(size_t)e.start + (uint32_t)pk_keys[j]];
        __syncthreads();
    }
}

}  // namespace atag
