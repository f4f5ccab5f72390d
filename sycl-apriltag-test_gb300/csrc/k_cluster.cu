// k_cluster.cu — the fused path from labels to quads.
//
// The reference groups boundary points with a global 64-bit sort_by_key over
// every point (main.cpp:515), reduces ClusterBounds per key (:571-585),
// filters, maps points back to clusters with a binary search (:621-675) and
// sorts again by (cluster, theta) (:737).  Only the ORDER of the surviving
// clusters and the ORDER of points inside a cluster influence the result,
// and both are fixed by keys, so here:
//   1. k_boundaries_pairs: each CTA finds its boundary points, aggregates
//      them per cluster pair in a shared-memory hash table (warp-level
//      reductions first), merges the per-pair ClusterBounds sums into a
//      per-frame global hash table with one set of atomics per (CTA, pair),
//      and appends its points, tagged with their pair slot, to a list
//      (in batches, points of pairs that earlier tiles already pushed over
//      the cluster size limit are skipped);
//   2. k_pairs_finalize: one CTA per frame sorts the distinct pair keys
//      (hundreds to a few thousand), applies ValidBlobFilter and assigns
//      each surviving pair its cluster index and extent;
//   3. k_scatter_points: points of surviving pairs go straight into their
//      cluster's segment with their theta key; the rest are dropped;
//   4. k_cluster_sort: one CTA per cluster sorts by (theta, point) in
//      shared memory and writes ClusterPoints and the line-fit prefix sums;
//      k_cluster_errors: fit_lines (windowed errors, 7-tap filter, peaks)
//      flat over all cluster points; k_cluster_peaks: the 10 best peaks of
//      each cluster;
//   5. k_peaks_scan / k_index_quads / k_compact_quads: peak extents,
//      do_indexing and the corner intersection, quads in reference order.
#include "atag_kernels.cuh"
#include "atag_pairs.cuh"
#include "atag_quads.cuh"

namespace atag {

// ---------------------------------------------------------------------------
// reset
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_reset_frames(const __grid_constant__ FrameSet fs) {
    const FrameDesc& F = fs.get(blockIdx.y);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < F.pair_cap; i += gridDim.x * blockDim.x) {
        F.pair_keys[i] = EMPTY_KEY;
        F.pair_bbox[i] = make_uint4(0xFFFFFFFFu, 0u, 0xFFFFFFFFu, 0u);
        F.pair_gsum[i] = make_int2(0, 0);
        F.pair_pxgx[i] = 0ull;
        F.pair_count[i] = 0u;
        F.pair_cluster[i] = INVALID;
    }
    if (blockIdx.x == 0 && threadIdx.x < CNT_COUNT) F.counters[threadIdx.x] = 0u;
    if (blockIdx.x == 0 && threadIdx.x < DEAD_PAIRS && F.dead_pairs) F.dead_pairs[threadIdx.x] = EMPTY_KEY;
}

// ---------------------------------------------------------------------------
// 1. boundaries + per-pair aggregation
// ---------------------------------------------------------------------------
constexpr int BP_W = 64;                       // tile width; BP_H (8 or 16) rows is a tuning choice
constexpr int BP_SW = BP_W + 8;  // label row: x0 - 4 .. x0 + BP_W + 3 (16-byte aligned body)
constexpr int BP_LC = 64;                      // CTA hash-table entries (a tile has a few dozen pairs; more go straight to the frame's table)
constexpr uint32_t BP_VALUE = 0x3FFFFFFFu;  // label value without the colour bit

struct PairTableSmem {
    unsigned long long key[BP_LC];
    uint32_t cnt[BP_LC], xmin[BP_LC], xmax[BP_LC], ymin[BP_LC], ymax[BP_LC];
    int gx[BP_LC], gy[BP_LC];
    int pxgx[BP_LC];  // a tile's sum fits 32 bits: at most 4096 points, |x| < 2^13
    uint32_t gslot[BP_LC];
};

// Insert-or-find in the CTA's pair table; a plain read first avoids the
// atomic for keys that are already present (the common case).  *fresh is
// set when this call inserted the key.
__device__ __forceinline__ int local_insert(PairTableSmem& T, unsigned long long key, bool* fresh) {
    // a 32-bit multiplicative hash of both labels (the table has 64 slots)
    uint32_t h = (((uint32_t)key ^ ((uint32_t)(key >> 32) * 0x85EBCA6Bu)) * 0x9E3779B1u) >> 26;
    for (int p = 0; p < BP_LC; p++) {
        unsigned long long k = *(volatile unsigned long long*)&T.key[h];
        if (k == key) return (int)h;
        if (k == EMPTY_KEY) {
            k = atomicCAS(&T.key[h], EMPTY_KEY, key);
            if (k == EMPTY_KEY) {
                *fresh = true;
                return (int)h;
            }
            if (k == key) return (int)h;
        }
        h = (h + 1) & (BP_LC - 1);
    }
    return -1;
}
// A staged point: CTA table slot (8 bits), tile-relative x (6) and y (4),
// neighbour test (2) and colour direction (1).
constexpr uint32_t STAGE_DIRECT = 1u << 21; // point already accounted for in global memory
__device__ __forceinline__ uint32_t stage_entry(int ls, int xo, int yo, int t, int dir) {
    return ((uint32_t)ls << 13) | (uint32_t)xo | ((uint32_t)yo << 6) | ((uint32_t)t << 10) | ((uint32_t)dir << 12);
}
__device__ __forceinline__ uint32_t stage_packed(uint32_t e, uint32_t x0, uint32_t y0) {
    // x0 + 63 < 2^14 and y0 + 15 < 2^15: the sums leave the flag bits clear
    const uint32_t xy = (x0 | (y0 << 16)) + (e & 63) + (((e >> 6) & 15) << 16);
    return xy | (((e >> 10) & 3) << 14) | (((e >> 12) & 1) << 31);
}

// find_boundaries (find_boundaries.cpp:10-155) fused with the per-pair
// ClusterBounds reduction (main.cpp:571-585) and the compaction of points.
template <int BP_H>
__device__ __forceinline__ void boundaries_pairs_impl(const FrameSet& fs, uint32_t min_size) {
    constexpr int BP_SH = BP_H + 1;
    constexpr int NW = BP_H / 2;               // warps: two tile rows each
    constexpr int BP_STAGE = BP_W * BP_H * 4;  // at most 4 points per pixel
    constexpr int BP_WSTAGE = 2 * BP_W * 4;    // the part of one warp (two tile rows)
    constexpr unsigned FULL = 0xFFFFFFFFu;
    static_assert(BP_W == 64, "two 32-pixel words per row");
    // frame from blockIdx.x, tile column and row from blockIdx.y and .z:
    // CTAs are dispatched frame-fastest, so the tiles in flight at once span
    // every frame of the batch and a frame's later tiles start after its
    // first ones published their over-limit pairs
    const FrameDesc& F = fs.get(blockIdx.x);
    const int w = F.width, h = F.height;
    const int ntx = (w + BP_W - 1) / BP_W, nty = (h + BP_H - 1) / BP_H;
    if ((int)blockIdx.y >= ntx || (int)blockIdx.z >= nty) return;
    const int x0 = blockIdx.y * BP_W, y0 = blockIdx.z * BP_H;
    uint32_t* status = F.counters + CNT_STATUS;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    // labels of the tile and its halo (column c = pixel x0 + c - 4: 3 = x0 -
    // 1, BP_W + 4 = x0 + BP_W; row BP_H is the row below the tile), and four
    // bit planes of them: per row four words, [0] bit 31 = x0 - 1, [1] and
    // [2] = x0 .. x0 + 63, [3] bit 0 = x0 + 64.  Plane 0: the colour bit
    // (255 pixel), 1: the component has at least min_size pixels, 2 and 3:
    // the label is one of the two labels of the frame's first / second pair
    // known to be over the cluster size limit.
    __shared__ __align__(16) uint32_t lab[BP_SH][BP_SW];
    __shared__ __align__(16) uint32_t planes[4][BP_SH][4];
    __shared__ PairTableSmem T;
    __shared__ uint32_t stage[BP_STAGE];
    __shared__ uint32_t s_nall;
    const bool track_dead = !F.stage_outputs && F.dead_pairs;

    // pairs that earlier tiles already pushed over the cluster size limit
    // (snapshots: a pair published later is simply processed in full;
    // points of a published pair can never survive, so steps and warps that
    // see different snapshots still agree on the result).  Both filter
    // points at emission.
    static_assert(DEAD_PAIRS == 2, "two over-limit pair planes");
    // a pair joins a white label (colour bit | an even root slot) and a
    // black one (an odd root slot, or label 0 of pixels that are neither 0
    // nor 255): its two label words
    auto pair_labels = [&](unsigned long long key, uint32_t& lw, uint32_t& lk) {
        lw = FULL;
        lk = FULL;
        const uint32_t kA = (uint32_t)(key >> 32), kB = (uint32_t)key;
        if ((kA ^ kB) & 1u) {
            lw = LABEL_PIXEL_MASK | ((kA & 1u) ? kB : kA);
            lk = (kA & 1u) ? kA : kB;
        } else if (kA == 0u) {
            lw = LABEL_PIXEL_MASK | kB;
            lk = 0u;
        }
    };
    uint32_t dW, dK, eW, eK;
    pair_labels(track_dead ? __ldcg(F.dead_pairs) : EMPTY_KEY, dW, dK);
    pair_labels(track_dead ? __ldcg(F.dead_pairs + 1) : EMPTY_KEY, eW, eK);
    if (threadIdx.x == 0) s_nall = 0;
    for (int i = threadIdx.x; i < BP_LC; i += blockDim.x) {
        T.key[i] = EMPTY_KEY;
        T.cnt[i] = 0; T.xmin[i] = 0xFFFFFFFFu; T.xmax[i] = 0; T.ymin[i] = 0xFFFFFFFFu; T.ymax[i] = 0;
        T.gx[i] = 0; T.gy[i] = 0; T.pxgx[i] = 0; T.gslot[i] = INVALID;
    }
    // Loads.  Row-word unit u = 2 r + k (row r of the tile and its halo row,
    // 32-pixel word k) belongs to warp u % NW: lane i loads the label of
    // pixel x0 + 32 k + i (one coalesced 128-byte row segment per warp) and
    // gathers its component's size, and four warp ballots of the flags are
    // the unit's four plane words.  The last two warps, which have one unit
    // fewer, also load the left and right halo columns (lane = row).  A
    // lane issues all its label loads before the first size gather.  Labels
    // out of the image are 0, as the reference reads them.
    {
        constexpr int NUNIT = 2 * BP_SH, PER = (NUNIT + NW - 1) / NW;
        static_assert(NUNIT <= NW * (PER - 1) + NW - 2, "the last two warps have a unit fewer");
        // NW is even, so a warp's units share their word k = warp & 1 and
        // their rows are r0 + (NW / 2) j
        static_assert(NW % 2 == 0, "units of a warp share their word");
        const int kk = warp & 1, r0 = warp >> 1;
        const bool xin = x0 + 32 * kk + lane < w;
        const uint32_t* lrow = F.labels + (size_t)(y0 + r0) * w + (x0 + 32 * kk + lane);
        uint32_t lv[PER], sz[PER];
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const bool in = warp + NW * j < NUNIT && xin && y0 + r0 + (NW / 2) * j < h;
            lv[j] = in ? __ldg(lrow + (size_t)j * (NW / 2) * w) : 0u;
        }
        const bool halo = warp >= NW - 2, right = warp == NW - 1;
        const int hx = right ? x0 + BP_W : x0 - 1, hy = y0 + lane;
        const uint32_t hl = (halo && lane < BP_SH && hx >= 0 && hx < w && hy < h) ? __ldg(F.labels + (size_t)hy * w + hx) : 0u;
#pragma unroll
        for (int j = 0; j < PER; j++)
            if (warp + NW * j < NUNIT) sz[j] = __ldg(F.sizes + (lv[j] & LABEL_VALUE_MASK));
        const uint32_t hs = halo ? __ldg(F.sizes + (hl & LABEL_VALUE_MASK)) : 0u;
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const int r = r0 + (NW / 2) * j, k = kk;
            if (warp + NW * j >= NUNIT) break;
            const uint32_t l = lv[j];
            lab[r][4 + 32 * k + lane] = l;
            const unsigned bc = __ballot_sync(FULL, (int)l < 0);
            const unsigned bb = __ballot_sync(FULL, sz[j] >= min_size);
            const unsigned bd = __ballot_sync(FULL, l == dW || l == dK);
            const unsigned be = __ballot_sync(FULL, l == eW || l == eK);
            if (lane == 0) {
                planes[0][r][1 + k] = bc;
                planes[1][r][1 + k] = bb;
                planes[2][r][1 + k] = bd;
                planes[3][r][1 + k] = be;
            }
        }
        if (halo && lane < BP_SH) {
            lab[lane][right ? BP_W + 4 : 3] = hl;
            const int wq = right ? 3 : 0, sh = right ? 0 : 31;
            planes[0][lane][wq] = (hl >> 31) << sh;
            planes[1][lane][wq] = (hs >= min_size ? 1u : 0u) << sh;
            planes[2][lane][wq] = (hl == dW || hl == dK ? 1u : 0u) << sh;
            planes[3][lane][wq] = (hl == eW || hl == eK ? 1u : 0u) << sh;
        }
    }
    __syncthreads();

    // A: enumerate points in the reference's test order (R, BL unless it
    // would duplicate, B, BR: find_boundaries.cpp:128-150).  Lane (rl, k,
    // t, half) of warp w takes 16 pixels of the 32-pixel word k of tile row
    // 2 w + rl and test t: a pixel emits test t when it is in the image and
    // big and the tested neighbour is big and of the other colour (BL also
    // not when it duplicates the left pixel's BR), computed for the word at
    // once on the bit planes.  Points of the frame's first over-limit pair
    // are counted but not staged.
    const int rl = lane >> 4, k = (lane >> 3) & 1, t = (lane >> 1) & 3, half = lane & 1;
    const int r = 2 * warp + rl;
    uint32_t mt, st;
    {
        const int xb = x0 + 32 * k;
        // The lane's tested neighbour: the same row for R (t = 0), the row
        // below for BL, B and BR.  Bit i of its plane word is pixel
        // xb + i + dx (dx = +1 for R and BR, -1 for BL, 0 for B): a funnel
        // shift of words lo, lo + 1 of that plane row.
        const int nrow = r + (t != 0 ? 1 : 0), lo = t == 1 ? k : k + 1, amt = t == 1 ? 31 : (t == 2 ? 0 : 1);
        auto nb = [&](int p) { return __funnelshift_r(planes[p][nrow][lo], planes[p][nrow][lo + 1], amt); };
        auto own = [&](int p) { return planes[p][r][k + 1]; };
        const uint32_t c0 = own(0), b0 = own(1);
        uint32_t live = (y0 + r < h) ? (xb + 32 <= w ? FULL : (xb < w ? ((1u << (w - xb)) - 1u) : 0u)) : 0u;
        if (xb == 0) live &= ~1u;  // column 0 is never processed
        live &= b0 & (half ? 0xFFFF0000u : 0x0000FFFFu);
        // BL is not emitted where the left pixel's BR covers the same pair
        uint32_t keep = FULL;
        if (t == 1) {
            const uint32_t c0L = __funnelshift_l(planes[0][r][k], c0, 1), b0L = __funnelshift_l(planes[1][r][k], b0, 1);
            keep = ~((c0L ^ planes[0][r + 1][k + 1]) & b0L & planes[1][r + 1][k + 1]);
        }
        mt = (nb(0) ^ c0) & nb(1) & live & keep;
        // points whose two pixels are both labels of one published pair
        st = mt & ~((own(2) & nb(2)) | (own(3) & nb(3)));
    }
    // Each warp lists its staged points in its own part of the staging
    // array (warp scan) and aggregates them itself, so no CTA barrier
    // separates the masks from the rounds.
    uint32_t* wst = stage + warp * BP_WSTAGE;
    const uint32_t ns = (uint32_t)__popc(st);
    uint32_t incl = ns;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t nst = __shfl_sync(FULL, incl, 31);
    {
        uint32_t pos = incl - ns;
        const uint32_t base = stage_entry(0, 32 * k, r, t, 0) - 1u;  // + ffs: pixel 32 k + ffs - 1 (mod 2^32)
        for (uint32_t mm = st; mm; mm &= mm - 1) wst[pos++] = base + (uint32_t)__ffs(mm);
        const uint32_t nall_w = __reduce_add_sync(FULL, (uint32_t)__popc(mt));
        if (lane == 0 && nall_w) atomicAdd(&s_nall, nall_w);
    }
    __syncwarp();
    // the over-limit pairs again, for the rounds (a later snapshot)
    unsigned long long dead0 = EMPTY_KEY, dead1 = EMPTY_KEY;
    if (track_dead) {
        dead0 = __ldcg(F.dead_pairs);
        dead1 = __ldcg(F.dead_pairs + 1);
    }
    // The warp takes its staged points 32 at a time: pair key, CTA table
    // slot (one insert per distinct key of the round) and the per-pair sums
    // of the round's points, merged into the table by one lane per key.
    for (uint32_t b0 = 0; b0 < nst; b0 += 32) {
        const uint32_t i = b0 + (uint32_t)lane;
        const bool v = i < nst;
        uint32_t e = v ? wst[i] : 0u;
        const int xo = (int)(e & 63), ro = (int)((e >> 6) & 15), t = (int)((e >> 10) & 3);
        // the point's pixel and its tested neighbour in the label tile: R is
        // the next word, BL, B and BR the row below (BP_SW - 1, BP_SW, BP_SW + 1)
        static_assert(BP_SW == 72, "neighbour offsets 1, 71, 72, 73");
        const uint32_t* pl = &lab[0][4] + ro * BP_SW + xo;
        const uint32_t p = pl[0], q = pl[(0x49484701u >> (8 * t)) & 0xFFu];
        const uint32_t lp = p & BP_VALUE, lq = q & BP_VALUE;
        const int dir = (q & LABEL_PIXEL_MASK) > (p & LABEL_PIXEL_MASK) ? 1 : 0;
        const unsigned long long key = v ? (((unsigned long long)min(lp, lq) << 32) | max(lp, lq)) : EMPTY_KEY;
        // a round whose points all belong to pairs already over the limit
        // contributes nothing: its points are neither aggregated nor listed
        static_assert(DEAD_PAIRS == 2, "the test below reads both entries");
        const bool dead = v && (key == dead0 || key == dead1);
        if (__all_sync(0xFFFFFFFFu, dead || !v)) {
            if (v) wst[i] = e | STAGE_DIRECT;
            continue;
        }
        const unsigned m = __match_any_sync(0xFFFFFFFFu, key);
        const int leader = __ffs(m) - 1;
        int ls = 0;
        if (v && lane == leader) {
            // a key new to the tile also takes its slot in the frame's
            // table now, so the merge below needs one round trip less
            bool fresh = false;
            ls = local_insert(T, key, &fresh);
            if (fresh) {
                const uint32_t gs = global_insert(F, key);
                if (gs == INVALID) atomicOr(status, ATAG_DEVFLAG_PAIR_OVERFLOW);
                T.gslot[ls] = gs;
            }
        }
        ls = __shfl_sync(0xFFFFFFFFu, ls, leader);
        const uint32_t xd = 2u * (uint32_t)(x0 + xo) + 1u, yd = 2u * (uint32_t)(y0 + ro);
        const int gx = dir ? 1 : -1;
        e |= (uint32_t)dir << 12;
        if (v && ls < 0) {  // CTA table full: account for and list the point directly
            e |= STAGE_DIRECT;
            const uint32_t gs = global_insert(F, key);
            if (gs == INVALID) {
                atomicOr(status, ATAG_DEVFLAG_PAIR_OVERFLOW);
            } else {
                global_flush(F, gs, 1, xd, xd, yd, yd, gx, 0, (unsigned long long)(long long)((int)xd * gx));
                const uint32_t at = atomicAdd(F.counters + CNT_POINTS, 1u);
                if (at < F.point_cap) F.points[at] = ((unsigned long long)gs << 32) | stage_packed(e, x0, y0);
                else atomicOr(status, ATAG_DEVFLAG_POINT_OVERFLOW);
            }
        } else {
            e |= (uint32_t)ls << 13;
        }
        if (v) wst[i] = e;
        const bool a = v && ls >= 0;
        const uint32_t cnt = __reduce_add_sync(m, a ? 1u : 0u);
        const uint32_t xmn = __reduce_min_sync(m, xd), xmx = __reduce_max_sync(m, xd);
        const uint32_t ymn = __reduce_min_sync(m, yd), ymx = __reduce_max_sync(m, yd);
        const int sgx = __reduce_add_sync(m, a ? gx : 0);
        const int spx = __reduce_add_sync(m, a ? (int)xd * gx : 0);
        if (a && lane == leader) {
            atomicAdd(&T.cnt[ls], cnt);
            atomicMin(&T.xmin[ls], xmn);
            atomicMax(&T.xmax[ls], xmx);
            atomicMin(&T.ymin[ls], ymn);
            atomicMax(&T.ymax[ls], ymx);
            atomicAdd(&T.gx[ls], sgx);
            atomicAdd(&T.pxgx[ls], spx);
        }
    }
    __syncthreads();

    // C: merge into the frame's table.  A pair whose running point count
    // already exceeds ValidBlobFilter's maximum 2 (2w + 2h)
    // (cluster_bounds.h:92-93,102) can never survive; its points are counted
    // but not listed.
    const uint32_t max_pixels = 2u * (2u * (uint32_t)w + 2u * (uint32_t)h);
    if (threadIdx.x == 0 && s_nall) atomicAdd(F.counters + CNT_ALLPOINTS, s_nall);
    for (int i = threadIdx.x; i < BP_LC; i += blockDim.x) {
        unsigned long long key = T.key[i];
        if (key == EMPTY_KEY) continue;
        const uint32_t gs = T.gslot[i];  // INVALID: the frame's table was full (flagged)
        if (gs == INVALID) continue;
        uint32_t old = global_flush(F, gs, T.cnt[i], T.xmin[i], T.xmax[i], T.ymin[i], T.ymax[i], T.gx[i], T.gy[i],
                                    (unsigned long long)(long long)T.pxgx[i]);
        T.gslot[i] = (old + T.cnt[i] > max_pixels) ? INVALID : gs;
        // the flush that crosses the limit publishes the pair, so that later
        // tiles skip its points (its count only grows: it stays rejected)
        if (track_dead && old <= max_pixels && old + T.cnt[i] > max_pixels)
            for (uint32_t d = 0; d < DEAD_PAIRS; d++)
                if (atomicCAS(F.dead_pairs + d, EMPTY_KEY, key) == EMPTY_KEY) break;
    }
    __syncthreads();

    // D: each warp lists the points of live pairs from its own staging
    // part: a count pass, one atomic for the warp's place in the list, then
    // the writes in the same order
    auto live_at = [&](uint32_t i) {
        if (i >= nst) return false;
        const uint32_t e = wst[i];
        return !(e & STAGE_DIRECT) && T.gslot[(e >> 13) & 255] != INVALID;
    };
    // the first round's ballot is kept for the writes (most warps have one)
    const unsigned m_first = __ballot_sync(0xFFFFFFFFu, live_at(lane));
    uint32_t nlive = (uint32_t)__popc(m_first);
    for (uint32_t b0 = 32; b0 < nst; b0 += 32) nlive += (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, live_at(b0 + lane)));
    if (nlive == 0) return;
    uint32_t at = 0;
    if (lane == 0) {
        at = atomicAdd(F.counters + CNT_POINTS, nlive);
        if ((unsigned long long)at + nlive > F.point_cap) atomicOr(status, ATAG_DEVFLAG_POINT_OVERFLOW);
    }
    at = __shfl_sync(0xFFFFFFFFu, at, 0);
    const unsigned lt = (1u << lane) - 1u;
    for (uint32_t b0 = 0; b0 < nst; b0 += 32) {
        const uint32_t i = b0 + (uint32_t)lane;
        const unsigned m = b0 == 0 ? m_first : __ballot_sync(0xFFFFFFFFu, live_at(i));
        const bool lv = (m >> lane) & 1u;
        if (lv) {
            const uint32_t e = wst[i], dst = at + (uint32_t)__popc(m & lt);
            if (dst < F.point_cap) F.points[dst] = ((unsigned long long)T.gslot[(e >> 13) & 255] << 32) | stage_packed(e, x0, y0);
        }
        at += (uint32_t)__popc(m);
    }
}

// ---------------------------------------------------------------------------
// 2. pair finalisation: sort keys, filter, cluster indices and extents
// ---------------------------------------------------------------------------
constexpr int PF_THREADS = 1024;
constexpr int PF_SMEM_KEYS = 6048;  // with the scan words, under 48 KB of static shared memory

// K block-wide exclusive scans at once (one set of barriers for all):
// v[k] becomes its exclusive prefix, tot[k] the block total.  `red` holds
// K x 33 words.
template <int K>
__device__ __forceinline__ void block_exclusive_scan_multi(uint32_t (&v)[K], uint32_t (*red)[33], uint32_t (&tot)[K]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    uint32_t x[K];
#pragma unroll
    for (int k = 0; k < K; k++) x[k] = v[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x[k], o);
            if (lane >= o) x[k] += y;
        }
    __syncthreads();
    if (lane == 31)
#pragma unroll
        for (int k = 0; k < K; k++) red[k][wid] = x[k];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint32_t s = lane < nw ? red[k][lane] : 0u;
            uint32_t q = s;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, q, o);
                if (lane >= o) q += y;
            }
            red[k][lane] = q - s;  // exclusive prefix of warp totals
            if (lane == 31) red[k][32] = q;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) {
        tot[k] = red[k][32];
        v[k] = red[k][wid] + x[k] - v[k];
    }
}

__global__ void __launch_bounds__(PF_THREADS) k_pairs_finalize(const __grid_constant__ FrameSet fs,
                                                               PipelineParams p, uint32_t small_max) {
    const FrameDesc& F = fs.get(blockIdx.x);
    uint32_t* status = F.counters + CNT_STATUS;
    __shared__ unsigned long long s_keys[PF_SMEM_KEYS];
    __shared__ uint32_t red4[4][33];
    uint32_t* red = red4[0];
    __shared__ uint32_t s_n;
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    // the sorted key list lives in shared memory when it fits, else in the
    // frame's cluster_keys buffer's tail (pair_cap entries reserved there)
    uint32_t npairs_upper = 0;
    for (uint32_t i = threadIdx.x; i < F.pair_cap; i += blockDim.x) npairs_upper += F.pair_keys[i] != EMPTY_KEY;
    uint32_t C = block_sum_u32(npairs_upper, red);
    unsigned long long* keys = C <= (uint32_t)PF_SMEM_KEYS ? s_keys : F.cluster_keys + F.cluster_cap;
    for (uint32_t i = threadIdx.x; i < F.pair_cap; i += blockDim.x) {
        unsigned long long k = F.pair_keys[i];
        if (k != EMPTY_KEY) keys[atomicAdd(&s_n, 1u)] = k;
    }
    __syncthreads();
    bitonic_sort_u64(keys, C);
    __syncthreads();
    FilterParams fp;
    fp.min_cluster_pixels = p.min_cluster_pixels;
    fp.max_cluster_pixels = 2u * (2u * F.width + 2u * F.height);
    fp.tag_width = p.tag_width;
    fp.normal_border = p.normal_border;
    fp.reversed_border = p.reversed_border;
    uint32_t carry_start = 0, carry_cluster = 0, carry_fstart = 0, carry_small = 0, carry_large = 0, carry_fit = 0;
    uint32_t carry_runs = 0;
    for (uint32_t c0 = 0; c0 < C; c0 += blockDim.x) {
        uint32_t c = c0 + threadIdx.x;
        uint32_t slot = INVALID, cnt = 0;
        bool keep = false;
        uint4 bb = make_uint4(0, 0, 0, 0);
        int2 gs = make_int2(0, 0);
        long long pxgx = 0;
        if (c < C) {
            slot = global_lookup(F, keys[c]);
            cnt = F.pair_count[slot];
            bb = F.pair_bbox[slot];
            gs = F.pair_gsum[slot];
            pxgx = (long long)F.pair_pxgx[slot];
            keep = valid_blob(fp, cnt, bb.x, bb.y, bb.z, bb.w, gs.x, gs.y, pxgx);
        }
        // the scans in key order, in two rounds (which kept pairs fit
        // depends on the first round's prefixes)
        uint32_t s1[3] = {cnt, keep ? 1u : 0u, keep ? cnt : 0u}, t1[3];
        block_exclusive_scan_multi<3>(s1, red4, t1);
        const uint32_t tot_cnt = t1[0], tot_keep = t1[1], tot_fcnt = t1[2];
        uint32_t start = carry_start + s1[0];
        if (c < C && F.pair_bounds_out) {
            // every pair's bounds in key order (stages 5-6 of the reference)
            if (c < F.pair_out_cap) {
                atag_cluster_bounds b;
                b.x_min = (uint16_t)bb.x; b.x_max = (uint16_t)bb.y;
                b.y_min = (uint16_t)bb.z; b.y_max = (uint16_t)bb.w;
                b.gx_sum = gs.x; b.gy_sum = gs.y;
                b.pxgx_pygy_sum = pxgx;
                b.start = start;
                b.count = cnt;
                F.pair_bounds_out[c] = b;
                if (F.pair_keys_out) F.pair_keys_out[c] = keys[c];
            } else {
                atomicOr(status, ATAG_DEVFLAG_PAIR_OVERFLOW);
            }
        }
        uint32_t cid = carry_cluster + s1[1];
        uint32_t fstart = carry_fstart + s1[2];
        const bool fits = keep && cid < F.cluster_cap && (unsigned long long)fstart + cnt <= F.cpoint_cap;
        const bool small = cnt <= small_max;
        uint32_t s2[4] = {fits && small ? 1u : 0u, fits && !small ? 1u : 0u, fits ? cnt : 0u,
                          fits ? (cnt + CE_RUN - 1) / CE_RUN : 0u}, t2[4];
        block_exclusive_scan_multi<4>(s2, red4, t2);
        const uint32_t tot_small = t2[0], tot_large = t2[1], tot_fit = t2[2], tot_runs = t2[3];
        uint32_t js = carry_small + s2[0];
        uint32_t jl = carry_large + s2[1];
        const uint32_t run0 = carry_runs + s2[3];
        if (fits) F.cluster_work[small ? js : F.cluster_cap - 1 - jl] = cid;
        if (keep) {
            if (!fits) {
                atomicOr(status, ATAG_DEVFLAG_CLUSTER_OVERFLOW);
            } else {
                F.pair_cluster[slot] = cid;
                F.cluster_keys[cid] = keys[c];
                atag_cluster_bounds b;
                b.x_min = (uint16_t)bb.x; b.x_max = (uint16_t)bb.y;
                b.y_min = (uint16_t)bb.z; b.y_max = (uint16_t)bb.w;
                b.gx_sum = gs.x; b.gy_sum = gs.y;
                b.pxgx_pygy_sum = pxgx;
                b.start = start;
                b.count = cnt;
                F.cluster_bounds[cid] = b;
                F.cluster_extents[cid] = atag_cluster_extents{fstart, cnt};
                F.cluster_center[cid] = make_float2(bounds_cx(bb.x, bb.y), bounds_cy(bb.z, bb.w));
                F.cluster_cursor[cid] = 0;
                F.cluster_runs[cid] = run0;
                F.peak_count[cid] = 0;
            }
        }
        carry_start += tot_cnt;
        carry_cluster += tot_keep;
        carry_fstart += tot_fcnt;
        carry_small += tot_small;
        carry_large += tot_large;
        carry_fit += tot_fit;
        carry_runs += tot_runs;
    }
    if (threadIdx.x == 0) {
        // clusters are assigned in order and the capacity checks are
        // monotone, so the clusters that fit are the prefix [0, nfit) and
        // their points the prefix [0, carry_fit) of the cluster point array
        const uint32_t nfit = carry_small + carry_large;
        F.counters[CNT_CLUSTERS] = nfit;
        F.counters[CNT_SMALL] = carry_small;
        F.counters[CNT_LARGE] = carry_large;
        F.counters[CNT_RUNS] = carry_runs;
        F.stats->width = F.width;
        F.stats->height = F.height;
        F.stats->n_points = F.counters[CNT_ALLPOINTS];
        F.stats->n_pairs = C;
        F.stats->n_clusters = nfit;
        F.stats->n_cluster_points = carry_fit;
    }
}

// Prefix offsets of per-frame counts over the batch (the flattened work
// spaces of the per-cluster kernels) and reset of their queue cursors.
__global__ void k_batch_offsets(const __grid_constant__ FrameSet fs, uint32_t n_frames, BatchOffsets a) {
    __shared__ uint32_t red[33];
    for (int k = 0; k < 4; k++) {
        const uint32_t which = a.which[k];
        uint32_t* offsets = a.offsets[k];
        uint32_t* work_counters = a.work_counters;
        if (!offsets) continue;
        uint32_t carry = 0;
        for (uint32_t f0 = 0; f0 < n_frames; f0 += blockDim.x) {
            uint32_t f = f0 + threadIdx.x;
            uint32_t v = f < n_frames ? fs.get(f).counters[which] : 0u;
            uint32_t tot;
            uint32_t e = block_exclusive_scan_u32(v, red, &tot);
            if (f < n_frames) offsets[f] = carry + e;
            carry += tot;
        }
        if (threadIdx.x == 0) {
            offsets[n_frames] = carry;
            work_counters[k] = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// 3. scatter points of surviving pairs into their cluster segments
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_scatter_points(const __grid_constant__ FrameSet fs) {
    const FrameDesc& F = fs.get(blockIdx.y);
    uint32_t n = F.counters[CNT_POINTS];
    if (n > F.point_cap) n = F.point_cap;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        uint32_t i = base + threadIdx.x;
        uint32_t cid = INVALID, packed = 0;
        if (i < n) {
            unsigned long long e = F.points[i];
            uint32_t slot = (uint32_t)(e >> 32);
            packed = (uint32_t)e;
            if (slot != INVALID) cid = F.pair_cluster[slot];
        }
        unsigned mask = __match_any_sync(0xffffffffu, cid);
        if (cid != INVALID) {
            int leader = __ffs(mask) - 1;
            uint32_t b = 0;
            if ((int)lane == leader) b = atomicAdd(F.cluster_cursor + cid, (uint32_t)__popc(mask));
            b = __shfl_sync(mask, b, leader);
            uint32_t rank = __popc(mask & ((1u << lane) - 1u));
            atag_cluster_extents ext = F.cluster_extents[cid];
            float2 ctr = F.cluster_center[cid];
            float theta = calc_theta(packed, ctr.x, ctr.y);
            uint32_t pos = ext.start + b + rank;
            F.sortbuf[pos] = ((unsigned long long)float_order_key(theta) << 32) | packed;
        }
    }
}

// ---------------------------------------------------------------------------
// 4. one cluster per CTA: sort by (theta, point), ClusterPoints, line-fit
// inputs and their prefix sums
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t find_frame(const uint32_t* offsets, uint32_t n_frames, uint32_t item) {
    uint32_t lo = 0, hi = n_frames;  // offsets[lo] <= item < offsets[hi]
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (offsets[mid] <= item) lo = mid; else hi = mid;
    }
    return lo;
}

// Inclusive scan of 6 int64 moment lanes within groups of WIDTH lanes
// (32: the whole warp).  W, Mx and My are scanned in 32 bits: over at most
// 128 points their sums stay below 2^31 (W <= 361, rx, ry < 2^15), so the
// result equals the int64 (wrapping) sums.  Callers keep every partial sum
// within 128 points.
template <int WIDTH>
__device__ __forceinline__ Moment scan_moment(const Moment& v) {
    const int pos = (threadIdx.x & 31) & (WIDTH - 1);
    uint32_t mx = (uint32_t)v.Mx, my = (uint32_t)v.My, mw = (uint32_t)v.W;
    long long xx = v.Mxx, yy = v.Myy, xy = v.Mxy;
#pragma unroll
    for (int o = 1; o < WIDTH; o <<= 1) {
        const uint32_t a = __shfl_up_sync(0xffffffffu, mx, o, WIDTH);
        const uint32_t b = __shfl_up_sync(0xffffffffu, my, o, WIDTH);
        const uint32_t c = __shfl_up_sync(0xffffffffu, mw, o, WIDTH);
        const long long d = (long long)__shfl_up_sync(0xffffffffu, (unsigned long long)xx, o, WIDTH);
        const long long e = (long long)__shfl_up_sync(0xffffffffu, (unsigned long long)yy, o, WIDTH);
        const long long f = (long long)__shfl_up_sync(0xffffffffu, (unsigned long long)xy, o, WIDTH);
        if (pos >= o) {
            mx += a; my += b; mw += c;
            xx = wadd(xx, d); yy = wadd(yy, e); xy = wadd(xy, f);
        }
    }
    return Moment{(long long)mx, (long long)my, xx, yy, xy, (long long)mw};
}
__device__ __forceinline__ Moment warp_sum_moment(Moment v) {
    long long x[6] = {v.Mx, v.My, v.Mxx, v.Myy, v.Mxy, v.W};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int j = 0; j < 6; j++)
            x[j] = wadd(x[j], (long long)__shfl_xor_sync(0xffffffffu, (unsigned long long)x[j], o));
    return Moment{x[0], x[1], x[2], x[3], x[4], x[5]};
}
__device__ __forceinline__ Moment shfl_moment(const Moment& v, int src) {
    auto s = [&](long long x) { return (long long)__shfl_sync(0xffffffffu, (unsigned long long)x, src); };
    return Moment{s(v.Mx), s(v.My), s(v.Mxx), s(v.Myy), s(v.Mxy), s(v.W)};
}

template <bool LARGE>
__device__ __forceinline__ void cluster_sort(const FrameSet& fs, const uint32_t* __restrict__ work_offsets,
                                             uint32_t n_frames, uint32_t* __restrict__ work_counter,
                                             uint32_t sort_cap) {
    constexpr uint32_t THREADS = LARGE ? CF_LARGE_THREADS : CF_SMALL_THREADS;
    extern __shared__ unsigned long long smem_keys[];
    __shared__ long long red_m[32][6];
    __shared__ longlong2 lf_row[THREADS / 32][32][3];  // per warp: one row of LineFitPoints
    __shared__ uint32_t red32[33];
    __shared__ uint32_t s_item, s_flag;
    // radix counters of the global-memory sorts, after the padded key array
    uint32_t* hist = reinterpret_cast<uint32_t*>(smem_keys + kpad_size(sort_cap));
    const uint32_t total = work_offsets[n_frames];
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(work_counter, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= total) return;
        const uint32_t fidx = find_frame(work_offsets, n_frames, item);
        const FrameDesc& F = fs.get(fidx);
        const uint32_t j = item - work_offsets[fidx];
        const uint32_t cid = F.cluster_work[LARGE ? F.cluster_cap - 1 - j : j];
        const atag_cluster_extents ext = F.cluster_extents[cid];
        const uint32_t n = ext.count, start = ext.start;
        // sort by (theta, packed point): the reference's (cluster, slope)
        // order (main.cpp:737-750) with ties fixed by the point.  Up to
        // sort_cap keys sort in shared memory (padded layout, key i at
        // kpad(i)): a register bitonic network for up to 4 keys per thread,
        // a merge sort above; larger clusters (4K frames only) radix-sort
        // in global memory (plain layout).
        unsigned long long* X = smem_keys;
        const unsigned long long* src = F.sortbuf + start;
        uint32_t pad_mask = ~0u;
        if (n <= sort_cap) {
            if (LARGE) {
                if (n <= THREADS * 8) merge_sort_keys<THREADS, 8>(src, n, X);
                else if (n <= THREADS * 16) merge_sort_keys<THREADS, 16>(src, n, X);
                else merge_sort_keys<THREADS, 32>(src, n, X);
            } else {
                if (n <= THREADS * 2) sort_keys_regs<THREADS, 2>(src, n, X);
                else if (n <= THREADS * 4) sort_keys_regs<THREADS, 4>(src, n, X);
                else if (n <= THREADS * 8) merge_sort_keys<THREADS, 8>(src, n, X);
                else merge_sort_keys<THREADS, 16>(src, n, X);
            }
        } else {
            X = block_radix_sort_u64<THREADS>(F.sortbuf + start,
                                              reinterpret_cast<unsigned long long*>(F.errbuf + 2ull * start), n,
                                              hist, red32, &s_flag);
            pad_mask = 0u;
            __syncthreads();
        }
        auto at = [&](uint32_t i) -> unsigned long long& { return X[i + ((i >> 4) & pad_mask)]; };
        // The rest runs per warp over contiguous ranges of 128-point chunks
        // (32 lanes x SEG consecutive points).
        constexpr uint32_t W = THREADS / 32, SEG = 4, CH = 32 * SEG;
        const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const uint32_t nch = (n + CH - 1) / CH, ch0 = nch * w / W, ch1 = nch * (w + 1) / W;
        const uint32_t r0 = ch0 * CH, r1 = min(n, ch1 * CH);
        // ClusterPoints out; the key slot is reused for the line-fit inputs
        // (four rows in flight, so their image reads overlap), and the
        // warp's moment total for the scan below
        Moment t{0, 0, 0, 0, 0, 0};
        for (uint32_t i0 = r0 + lane; i0 < r1; i0 += 4 * 32) {
            unsigned long long k[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t i = i0 + u * 32;
                k[u] = i < r1 ? at(i) : 0ull;
            }
            unsigned long long v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = linefit_rxyw((uint32_t)k[u], F.width, F.height, F.grey);
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t i = i0 + u * 32;
                if (i < r1) {
                    const uint32_t packed = (uint32_t)k[u];
                    atag_cluster_point cp;
                    cp.packed_x = (uint16_t)packed;
                    cp.packed_y = (uint16_t)(packed >> 16);
                    cp.slope = float_from_order_key((uint32_t)(k[u] >> 32));
                    F.cluster_points[start + i] = cp;
                    at(i) = v[u];
                    t = m_add(t, moment_of(v[u]));
                }
            }
        }
        // segmented inclusive scan of the moments (main.cpp:796-801).  The
        // carry into a warp's range is the sum of the earlier warps' totals;
        // per chunk, lane l first sums its SEG points (4l .. 4l + 3), one
        // warp scan of those 32 sums gives each segment's offset, then rows
        // of 32 consecutive points add a scan within their segment to its
        // offset, so consecutive lanes store consecutive LineFitPoints.
        t = warp_sum_moment(t);
        if (lane == 0) {
            red_m[w][0] = t.Mx; red_m[w][1] = t.My; red_m[w][2] = t.Mxx;
            red_m[w][3] = t.Myy; red_m[w][4] = t.Mxy; red_m[w][5] = t.W;
        }
        __syncthreads();
        Moment carry{0, 0, 0, 0, 0, 0};
        for (uint32_t k = 0; k < w; k++)
            carry = m_add(carry, Moment{red_m[k][0], red_m[k][1], red_m[k][2], red_m[k][3], red_m[k][4],
                                        red_m[k][5]});
        for (uint32_t c = ch0; c < ch1; c++) {
            const uint32_t c0 = c * CH;
            Moment seg{0, 0, 0, 0, 0, 0};
#pragma unroll
            for (uint32_t q = 0; q < SEG; q++) {
                const uint32_t i = c0 + lane * SEG + q;
                if (i < n) seg = m_add(seg, moment_of(at(i)));
            }
            const Moment incl = scan_moment<32>(seg);
            const Moment off = m_add(carry, m_sub(incl, seg));
            carry = m_add(carry, shfl_moment(incl, 31));
#pragma unroll
            for (uint32_t r = 0; r < SEG; r++) {
                const uint32_t i = c0 + r * 32 + lane;
                const Moment m = i < n ? moment_of(at(i)) : Moment{0, 0, 0, 0, 0, 0};
                const Moment in_seg = scan_moment<SEG>(m);
                const Moment base = shfl_moment(off, (int)(r * (32 / SEG) + lane / SEG));
                // the row's 32 LineFitPoints go out as 512-byte runs: each
                // lane parks its 48 bytes in shared memory, then stores 16
                // consecutive bytes of the row per instruction
                const Moment lf = m_add(base, in_seg);
                lf_row[w][lane][0] = make_longlong2(lf.Mx, lf.My);
                lf_row[w][lane][1] = make_longlong2(lf.Mxx, lf.Myy);
                lf_row[w][lane][2] = make_longlong2(lf.Mxy, lf.W);
                __syncwarp();
                const uint32_t r0 = c0 + r * 32;
                longlong2* out = reinterpret_cast<longlong2*>(F.line_fit + start + r0);
#pragma unroll
                for (uint32_t q = 0; q < 4; q++) {
                    const uint32_t piece = q * 32 + lane, pt = piece >> 2, f = piece & 3;
                    if (r0 + pt < n) out[piece] = f < 3 ? lf_row[w][pt][f] : make_longlong2(0, 0);
                }
                __syncwarp();
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(CF_SMALL_THREADS, 6) k_cluster_sort_small(const __grid_constant__ FrameSet fs,
                                                                        const uint32_t* __restrict__ work_offsets,
                                                                        uint32_t n_frames,
                                                                        uint32_t* __restrict__ work_counter,
                                                                        uint32_t sort_cap) {
    cluster_sort<false>(fs, work_offsets, n_frames, work_counter, sort_cap);
}
__global__ void __launch_bounds__(CF_LARGE_THREADS, 1) k_cluster_sort_large(const __grid_constant__ FrameSet fs,
                                                                           const uint32_t* __restrict__ work_offsets,
                                                                           uint32_t n_frames,
                                                                           uint32_t* __restrict__ work_counter) {
    cluster_sort<true>(fs, work_offsets, n_frames, work_counter, CF_LARGE_CAP);
}

// ---------------------------------------------------------------------------
// 4b. fit_lines (fit_quad.cpp:153-375) in its cyclic form: the error of the
// window around each point, the 7-tap filter and the strict local maxima.
// One warp per run of up to CE_RUN consecutive points of one cluster, 32
// points per step: the warp keeps the errors of positions [s-4, s+36) and
// the filtered errors of [s-1, s+33) in shared memory (cluster-local,
// cyclic indices), carrying the last 8 errors into the next step.  Maxima
// are appended to their cluster's candidate list, which reuses the
// cluster's segment of the sort-key buffer (a cyclic sequence of n values
// has at most n/2 strict maxima).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t cyclic(int i, int n) {  // i in [-n, 3n)
    if (i < 0) i += n;
    while (i >= n) i -= n;
    return (uint32_t)i;
}

constexpr int CE_WARPS = 8;

__global__ void __launch_bounds__(32 * CE_WARPS) k_cluster_errors(const __grid_constant__ FrameSet fs,
                                                                  const uint32_t* __restrict__ run_offsets,
                                                                  uint32_t n_frames,
                                                                  uint32_t* __restrict__ work_counter) {
    __shared__ float s_err[CE_WARPS][40];
    __shared__ float s_flt[CE_WARPS][34];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float* e = s_err[wid];
    float* f = s_flt[wid];
    const uint32_t total = run_offsets[n_frames];
    for (;;) {
        uint32_t item = 0;
        if (lane == 0) item = atomicAdd(work_counter, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) return;
        const uint32_t fidx = find_frame(run_offsets, n_frames, item);
        const FrameDesc& F = fs.get(fidx);
        const uint32_t r = item - run_offsets[fidx];
        // the cluster whose runs contain r
        uint32_t lo = 0, hi = F.counters[CNT_CLUSTERS];
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (F.cluster_runs[mid] <= r) lo = mid; else hi = mid;
        }
        const uint32_t cid = lo;
        const atag_cluster_extents ext = F.cluster_extents[cid];
        const int n = (int)ext.count;
        const uint32_t k = min(20u, ext.count / 12u);
        const atag_line_fit_point* pts = F.line_fit + ext.start;
        const int li0 = (int)((r - F.cluster_runs[cid]) * CE_RUN);
        const int li1 = min(n, li0 + (int)CE_RUN);
        for (int s = li0; s < li1; s += 32) {
            if (s == li0) {
                e[lane] = window_error_local(pts, n, k, cyclic(s - 4 + (int)lane, n));
                if (lane < 8) e[32 + lane] = window_error_local(pts, n, k, cyclic(s + 28 + (int)lane, n));
            } else {
                const float carry = lane < 8 ? e[32 + lane] : 0.0f;
                __syncwarp();
                if (lane < 8) e[lane] = carry;
                e[8 + lane] = window_error_local(pts, n, k, cyclic(s + 4 + (int)lane, n));
            }
            __syncwarp();
            // cyclic 7-tap filter (fit_quad.cpp:296-324): f[j] is position s - 1 + j
            {
                float acc = 0.0f;
#pragma unroll
                for (int j = 0; j < 7; j++) acc = __fadd_rn(acc, __fmul_rn(e[lane + j], filter_tap(j)));
                f[lane] = acc;
                if (lane < 2) {
                    float a2 = 0.0f;
#pragma unroll
                    for (int j = 0; j < 7; j++) a2 = __fadd_rn(a2, __fmul_rn(e[32 + lane + j], filter_tap(j)));
                    f[32 + lane] = a2;
                }
            }
            __syncwarp();
            // strict local maxima (fit_quad.cpp:341-371) with error != 0
            // (main.cpp:832-835); global point 0 is never a corner (the
            // first work-group's first output is x = 1, fit_quad.cpp:182-190)
            const int li = s + (int)lane;
            if (li < li1) {
                const float cur = f[lane + 1];
                if (cur > f[lane] && cur > f[lane + 2] && cur != 0.0f && !(cid == 0 && li == 0)) {
                    const uint32_t at = atomicAdd(F.peak_count + cid, 1u);
                    F.sortbuf[ext.start + at] =
                        ((unsigned long long)float_order_key(cur) << 32) | (uint32_t)(~(uint32_t)li);
                }
            }
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// 4c. the 10 best peaks of each cluster by (error desc, index asc): the
// corner sort of main.cpp:856-863 restricted to what do_indexing reads
// (fit_quad.cpp:411-414 uses at most 10 corners).  One warp per cluster.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_cluster_peaks(const __grid_constant__ FrameSet fs,
                                                       const uint32_t* __restrict__ cluster_offsets,
                                                       uint32_t n_frames) {
    const uint32_t lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const uint32_t total = cluster_offsets[n_frames];
    for (uint32_t item = blockIdx.x * wpb + (threadIdx.x >> 5); item < total; item += gridDim.x * wpb) {
        const uint32_t fidx = find_frame(cluster_offsets, n_frames, item);
        const FrameDesc& F = fs.get(fidx);
        const uint32_t cid = item - cluster_offsets[fidx];
        const uint32_t npeaks = F.peak_count[cid];
        const unsigned long long* cand = F.sortbuf + F.cluster_extents[cid].start;
        const uint32_t take = npeaks < 10u ? npeaks : 10u;
        unsigned long long last = ~0ull;
        for (uint32_t j = 0; j < take; j++) {
            unsigned long long best = 0;
            for (uint32_t c = lane; c < npeaks; c += 32) {
                const unsigned long long key = cand[c];
                if (key < last && key > best) best = key;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long v = __shfl_xor_sync(0xffffffffu, best, o);
                best = v > best ? v : best;
            }
            if (lane == 0) {
                atag_corner c;
                c.line_fit_point_index = ~(uint32_t)best;
                c.cluster_index = (uint16_t)cid;
                c.error = float_from_order_key((uint32_t)(best >> 32));
                F.peaks[(size_t)cid * 10 + j] = c;
            }
            last = best;
        }
    }
}

// ---------------------------------------------------------------------------
// 5. peak extents (D10-D12), do_indexing + corners, ordered quads
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_peaks_scan(const __grid_constant__ FrameSet fs, PipelineParams p) {
    const FrameDesc& F = fs.get(blockIdx.x);
    __shared__ uint32_t red[33];
    const uint32_t C = F.counters[CNT_CLUSTERS];
    uint32_t carry_q = 0, carry_k = 0;
    for (uint32_t c0 = 0; c0 < C; c0 += blockDim.x) {
        uint32_t c = c0 + threadIdx.x;
        uint32_t k = c < C ? F.peak_count[c] : 0u;
        uint32_t tq, tk;
        uint32_t q = carry_q + block_exclusive_scan_u32(k ? 1u : 0u, red, &tq);
        uint32_t s = carry_k + block_exclusive_scan_u32(k, red, &tk);
        if (k) {
            F.peak_clusters[q] = c;
            F.peak_extents[q] = atag_peak_extents{s, k};
        }
        carry_q += tq;
        carry_k += tk;
    }
    if (threadIdx.x == 0) {
        F.counters[CNT_PEAKCLU] = carry_q;
        F.stats->n_corners = carry_k;
        F.stats->n_peak_clusters = carry_q;
    }
}

__global__ void __launch_bounds__(256) k_index_quads(const __grid_constant__ FrameSet fs,
                                                     const uint32_t* __restrict__ work_offsets, uint32_t n_frames,
                                                     PipelineParams p) {
    __shared__ SegmentTable T[8];  // one per warp
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t total = work_offsets[n_frames];
    for (uint32_t item = blockIdx.x * 8 + wid; item < total; item += gridDim.x * 8) {
        const uint32_t fidx = find_frame(work_offsets, n_frames, item);
        const FrameDesc& F = fs.get(fidx);
        const uint32_t q = item - work_offsets[fidx];
        const uint32_t cid = F.peak_clusters[q];
        const atag_cluster_extents ce = F.cluster_extents[p.compat_peak_index ? q : cid];
        atag_fitted_quad* fq = F.fitted + q;
        const int chosen = index_one_cluster(F.peak_count[cid], F.peaks + (size_t)cid * 10, F.line_fit + ce.start,
                                             ce.count, p.max_line_fit_mse, p.cos_critical_f, T[wid], fq);
        if (chosen < 0) {
            // no combination: the quad stays zero (main.cpp:318-319)
            for (uint32_t k = lane; k < sizeof(atag_fitted_quad) / 4; k += 32) reinterpret_cast<uint32_t*>(fq)[k] = 0u;
            if (lane == 0) F.quad_ok[q] = 0;
        } else if (lane == ((uint32_t)chosen & 31u)) {
            atag_quad_corners qc;
            const bool ok = quad_corners(*fq, p, q, &qc);
            F.quad_tmp[q] = qc;
            F.quad_ok[q] = ok ? 1u : 0u;
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(1024) k_compact_quads(const __grid_constant__ FrameSet fs) {
    const FrameDesc& F = fs.get(blockIdx.x);
    __shared__ uint32_t red[33];
    const uint32_t Cp = F.counters[CNT_PEAKCLU];
    uint32_t carry = 0, nfit = 0;
    for (uint32_t c0 = 0; c0 < Cp; c0 += blockDim.x) {
        uint32_t q = c0 + threadIdx.x;
        uint32_t ok = q < Cp ? F.quad_ok[q] : 0u;
        uint32_t fit = 0;
        if (q < Cp) {
            const atag_fitted_quad& fq = F.fitted[q];
            fit = (fq.indices[0] | fq.indices[1] | fq.indices[2] | fq.indices[3]) != 0;
        }
        uint32_t tot, tf;
        uint32_t pos = carry + block_exclusive_scan_u32(ok, red, &tot);
        block_exclusive_scan_u32(fit, red, &tf);
        if (ok) {
            if (pos < F.quad_cap) F.quads[pos] = F.quad_tmp[q];
        }
        carry += tot;
        nfit += tf;
    }
    if (threadIdx.x == 0) {
        if (carry > F.quad_cap) atomicOr(F.counters + CNT_STATUS, ATAG_DEVFLAG_QUAD_OVERFLOW);
        F.stats->n_fitted = nfit;
        F.stats->n_quads = carry < F.quad_cap ? carry : F.quad_cap;
        F.stats->status = F.counters[CNT_STATUS];
    }
}

__global__ void __launch_bounds__(BP_W / 4 * 8, 16) k_boundaries_pairs_r8(const __grid_constant__ FrameSet fs,
                                                                       uint32_t min_size) {
    boundaries_pairs_impl<8>(fs, min_size);
}
__global__ void __launch_bounds__(BP_W / 4 * 16, 8) k_boundaries_pairs_r16(const __grid_constant__ FrameSet fs,
                                                                        uint32_t min_size) {
    boundaries_pairs_impl<16>(fs, min_size);
}

}  // namespace atag
