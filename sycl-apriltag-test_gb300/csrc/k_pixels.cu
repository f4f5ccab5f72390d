// k_pixels.cu — pixel-parallel stages: decimation, adaptive threshold,
// block-based connected-component labelling and the dense boundary planes.
//
// Every kernel takes a FrameDesc table and a blockIdx.y frame index, so the
// same code serves one frame or a batch of frames of different sizes.
#include "atag_kernels.cuh"

namespace atag {

// ---------------------------------------------------------------------------
// a0: colour removal and point-sampling decimation dst(x, y) = grey(src(f x,
// f y)).  Colour is removed the way the reference's loader does it,
// stbi_load(..., STBI_grey) (src/main.cpp:264-265): luma (77 r + 150 g +
// 29 b) >> 8 with alpha ignored (include/stb_image.h:1834-1836); grey + alpha
// keeps the grey byte.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pixel_grey(const uint8_t* p, uint32_t format) {
    switch (format) {
    case ATAG_PIX_RGB8: case ATAG_PIX_RGBA8:
        return ((uint32_t)p[0] * 77u + (uint32_t)p[1] * 150u + (uint32_t)p[2] * 29u) >> 8;
    case ATAG_PIX_BGR8: case ATAG_PIX_BGRA8:
        return ((uint32_t)p[2] * 77u + (uint32_t)p[1] * 150u + (uint32_t)p[0] * 29u) >> 8;
    default: return p[0];
    }
}

__global__ void k_decimate(const __grid_constant__ FrameSet fs) {
    const FrameDesc& F = fs.get(blockIdx.y);
    if (F.factor <= 1 && F.src_format == ATAG_PIX_GREY8) return;
    const uint32_t w = F.width, h = F.height, f = F.factor, fmt = F.src_format;
    const uint32_t bpp = pixel_bytes(fmt);
    const uint32_t words_per_row = w / 4;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < words_per_row * h;
         i += gridDim.x * blockDim.x) {
        const uint32_t y = i / words_per_row, xw = i % words_per_row;
        const uint8_t* s = F.src + (size_t)y * f * F.src_stride + (size_t)xw * 4 * f * bpp;
        uint32_t v = 0;
#pragma unroll
        for (int b = 0; b < 4; b++) v |= pixel_grey(s + (size_t)b * f * bpp, fmt) << (8 * b);
        reinterpret_cast<uint32_t*>(F.grey)[(size_t)y * words_per_row + xw] = v;
    }
}

// ---------------------------------------------------------------------------
// a1: threshold_image (threshold.cpp:8-95) in one kernel.  A CTA owns
// TH_TX x TH_TY (32 x 16) tiles of 4x4 pixels; it loads those plus a
// one-tile halo into shared memory, takes each tile's min/max, dilates 3x3
// (tiles outside the image are neutral, which is the reference's clipping)
// and thresholds.
// ---------------------------------------------------------------------------
constexpr int TH_TX = 32, TH_TY = 16;
constexpr int TH_EX = TH_TX + 2, TH_EY = TH_TY + 2;

__global__ void __launch_bounds__(256, 8) k_threshold(const __grid_constant__ FrameSet fs,
                                                   int min_diff, int write_extrema) {
    const FrameDesc& F = fs.get(blockIdx.y);
    const int tw = F.width / 4, th = F.height / 4;
    const int ntx = (tw + TH_TX - 1) / TH_TX, nty = (th + TH_TY - 1) / TH_TY;
    if ((int)blockIdx.x >= ntx * nty) return;
    const int tx0 = (blockIdx.x % ntx) * TH_TX, ty0 = (blockIdx.x / ntx) * TH_TY;

    __shared__ uint32_t words[TH_EY][TH_EX][4];  // grey rows of each halo tile
    __shared__ uchar2 ext[TH_EY][TH_EX];

    const uint32_t* g32 = reinterpret_cast<const uint32_t*>(F.grey);
    const int wpr = F.width / 4;
    for (int e = threadIdx.x; e < TH_EY * TH_EX; e += blockDim.x) {
        int ey = e / TH_EX, ex = e % TH_EX;
        int ty = ty0 + ey - 1, tx = tx0 + ex - 1;
        uchar2 mm = make_uchar2(255, 0);
        if (tx >= 0 && tx < tw && ty >= 0 && ty < th) {
            uint32_t mn = 0xFFFFFFFFu, mx = 0;
            const uint32_t* gp = g32 + (size_t)(ty * 4) * wpr + tx;  // the tile's first row word
#pragma unroll
            for (int r = 0; r < 4; r++) {
                uint32_t v = __ldg(gp + (size_t)r * wpr);
                words[ey][ex][r] = v;
                mn = __vminu4(mn, v);
                mx = __vmaxu4(mx, v);
            }
            uint32_t a = min(min(mn & 0xFF, (mn >> 8) & 0xFF), min((mn >> 16) & 0xFF, mn >> 24));
            uint32_t b = max(max(mx & 0xFF, (mx >> 8) & 0xFF), max((mx >> 16) & 0xFF, mx >> 24));
            mm = make_uchar2((uint8_t)a, (uint8_t)b);
            if (write_extrema && ex >= 1 && ex <= TH_TX && ey >= 1 && ey <= TH_TY && F.extrema)
                reinterpret_cast<uchar2*>(F.extrema)[(size_t)ty * tw + tx] = mm;
        }
        ext[ey][ex] = mm;
    }
    __syncthreads();
    for (int o = threadIdx.x; o < TH_TX * TH_TY; o += blockDim.x) {
        int oy = o / TH_TX, ox = o % TH_TX;
        int ty = ty0 + oy, tx = tx0 + ox;
        if (tx >= tw || ty >= th) continue;
        uint32_t mn = 255, mx = 0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                uchar2 v = ext[oy + i][ox + j];
                mn = min(mn, (uint32_t)v.x);
                mx = max(mx, (uint32_t)v.y);
            }
        if (write_extrema && F.filtered_extrema)
            reinterpret_cast<uchar2*>(F.filtered_extrema)[(size_t)ty * tw + tx] =
                make_uchar2((uint8_t)mn, (uint8_t)mx);
        uint32_t comp = (mn + (mx - mn) / 2) & 0xFF;
        bool flat = (int)(mx - mn) < min_diff;
        // per byte: 255 above the tile's threshold, 0 at or below it, 127 in
        // a flat tile (byte-wise unsigned compare of the four pixels at once)
        const uint32_t comp4 = comp * 0x01010101u;
        uint32_t* out = reinterpret_cast<uint32_t*>(F.thr) + (size_t)(ty * 4) * wpr + tx;
#pragma unroll
        for (int r = 0; r < 4; r++)
            out[(size_t)r * wpr] = flat ? 0x7F7F7F7Fu : __vcmpgtu4(words[oy + 1][ox + 1][r], comp4);
    }
}

// ---------------------------------------------------------------------------
// a2/a3: BKE connected components (segmentation.cpp:95-392).
//
// The reference's partition is the set of connected components of a graph
// over "slots" (two per 2x2 block: the 255-slot at pixel index y*w+x and the
// 0-slot at y*w+x+1).  Block C links its 255-slot to the 255-slot of the
// block holding each neighbour test pixel P(-1,-1), Q(-1,0), Q(-1,1),
// R(-1,2), S(0,-1), S(1,-1) that is 255 and whose bit survives the
// `pixels_to_check` mask, and likewise for 0.  The mask is the union over
// *all* valid (0 or 255) pixels of the block, regardless of colour, which
// lets a component link through a block of the other colour (:143-171).
// Roots are the minimum slot index of the set.
//
// Here: (1) per CTA tile of CCL_BX x CCL_BY blocks, union-find in shared
// memory over intra-tile links, then every slot points at its tile-local
// root (global index) and each tile root holds its tile-local pixel count;
// (2) links that cross tile borders are merged in global memory;
// (3) final labels, and tile counts folded into the component root.
// ---------------------------------------------------------------------------
constexpr int CCL_BX = 32;  // blocks per tile row; CCL_BY (8, 16 or 32) rows is a tuning choice

// Iteration caps of the union-find loops.  Every union links a root to a
// smaller slot, so a parent chain strictly decreases and visits each slot at
// most once.  In a tile's shared-memory forest that bounds a chain by the
// tile's slots.  In the frame's forest the local pass leaves every slot one
// step from its tile root, and the border pass only links roots of
// components that touch a tile edge: at most two (one per colour) per edge
// block, 2 (2 CCL_BX + 2 rows) edge blocks per tile, largest for 8-row
// tiles.  So a chain, and the retries of one union (each moves to a
// strictly smaller root), are bounded by uf_bound(w, h); a loop that gets
// there flags ATAG_DEVFLAG_UF_ITERATION_CAP instead of spinning.
// FrameDesc::uf_cap may lower the bound (0 keeps it).
__device__ __forceinline__ uint32_t uf_bound(uint32_t w, uint32_t h) {
    const uint32_t tiles = ((w / 2 + CCL_BX - 1) / CCL_BX) * ((h / 2 + 7) / 8);
    return 2u * (2u * CCL_BX + 2u * 8u) * tiles + 2u;
}
__device__ __forceinline__ uint32_t uf_cap_of(const FrameDesc& F) {
    return F.uf_cap ? F.uf_cap : uf_bound(F.width, F.height);
}

// Which neighbour blocks (bit 0 P, 1 Q, 2 R, 3 S) a block links to in the
// 255 forest (wmask) and the 0 forest (bmask); info = pixel colour bits as
// in BkeBitmap (bits 0-3 = 255 at TL,TR,BL,BR; bits 8-11 = 0).
struct BlockLinks {
    uint32_t info, wmask, bmask;
};

template <typename PixelAt>
__device__ __forceinline__ BlockLinks block_links(PixelAt px, int x, int y, int w, int h) {
    uint32_t v00 = px(0, 0), v01 = px(0, 1), v10 = px(1, 0), v11 = px(1, 1);
    uint32_t info = 0, check = 0;
    if (v00 == 255) { check |= 0x777; info |= 1; } else if (v00 == 0) { check |= 0x777; info |= 1 << 8; }
    if (v01 == 255) { check |= 0x777 << 1; info |= 2; } else if (v01 == 0) { check |= 0x777 << 1; info |= 2 << 8; }
    if (v10 == 255) { check |= 0x777 << 4; info |= 4; } else if (v10 == 0) { check |= 0x777 << 4; info |= 4 << 8; }
    if (v11 == 255) info |= 8; else if (v11 == 0) info |= 8 << 8;
    if (x == 0) check &= 0xEEEE; else if (x + 2 >= w) check &= 0x7777;
    if (y == 0) check &= 0xFFF0; else if (y + 2 >= h) check &= 0x0FFF;
    uint32_t wm = 0, bm = 0;
    // test order and neighbour block of each test bit
    auto test = [&](uint32_t bit, int dy, int dx, uint32_t nb) {
        if (check & (1u << bit)) {
            uint32_t t = px(dy, dx);
            if (t == 255) wm |= nb; else if (t == 0) bm |= nb;
        }
    };
    test(0, -1, -1, 1);
    test(1, -1, 0, 2);
    test(2, -1, 1, 2);
    test(3, -1, 2, 4);
    test(4, 0, -1, 8);
    test(8, 1, -1, 8);
    return BlockLinks{info, wm, bm};
}

// Root of n, following at most `cap` parents; *capped is set when the cap
// ends the walk before a root.
__device__ __forceinline__ uint32_t find_root_volatile(volatile uint32_t* p, uint32_t n, uint32_t cap, bool* capped) {
    // path halving: every write replaces a parent by one of its ancestors,
    // which stays valid under concurrent unions (only roots are re-linked)
    for (uint32_t it = 0; it < cap; it++) {
        uint32_t q = p[n];
        if (q == n) return n;
        uint32_t g = p[q];
        if (g != q) p[n] = g;
        n = g;
    }
    *capped = true;
    return n;
}

// Lock-free union toward the smaller root (union_find.h:50-77) with
// iteration caps; returns false if a cap was hit.  With a non-root in hand
// the union still only lowers parents (atomicMin), so the forest stays
// acyclic and every later walk ends.
template <typename Ptr>
__device__ __forceinline__ bool uf_union(Ptr par, uint32_t a, uint32_t b, uint32_t cap) {
    bool capped = false;
    for (uint32_t it = 0; it < cap; it++) {
        a = find_root_volatile(par, a, cap, &capped);
        b = find_root_volatile(par, b, cap, &capped);
        if (capped) return false;
        if (a == b) return true;
        if (a < b) {
            uint32_t old = atomicMin((uint32_t*)&par[b], a);
            if (old == b) return true;
            b = old;
        } else {
            uint32_t old = atomicMin((uint32_t*)&par[a], b);
            if (old == a) return true;
            a = old;
        }
    }
    return false;
}

__device__ __forceinline__ uint32_t ccl_tiles_x(uint32_t w) { return (w / 2 + CCL_BX - 1) / CCL_BX; }
template <int CCL_BY>
__device__ __forceinline__ uint32_t ccl_tiles_y(uint32_t h) { return (h / 2 + CCL_BY - 1) / CCL_BY; }

template <int CCL_BY>
__device__ __forceinline__ void ccl_local_impl(const FrameSet& fs) {
    constexpr int CCL_THREADS = CCL_BX * CCL_BY;
    constexpr unsigned FULL = 0xFFFFFFFFu;
    // grid (tile column, tile row, frame): the frame's tile from the block
    // indices, no division
    const FrameDesc& F = fs.get(blockIdx.z);
    const int w = F.width, h = F.height;
    const int ntx = ccl_tiles_x(w), nty = ccl_tiles_y<CCL_BY>(h);
    if ((int)blockIdx.x >= ntx || (int)blockIdx.y >= nty) return;
    const int bx0 = blockIdx.x * CCL_BX, by0 = blockIdx.y * CCL_BY;
    const int x0 = bx0 * 2, y0 = by0 * 2;
    const uint32_t tile = blockIdx.y * (uint32_t)ntx + blockIdx.x;  // row-major within the frame

    // words of pixels x0 - 4 .. x0 + 2 CCL_BX + 3 of a row (x0 and w are
    // multiples of 4): pixel x is byte x - x0 + 4
    constexpr int WPR = (2 * CCL_BX + 8) / 4;
    static_assert(WPR <= 32, "one word per lane");
    __shared__ uint32_t par[2 * CCL_THREADS];
    __shared__ uint32_t cnt[2 * CCL_THREADS];
    __shared__ uint32_t row_runs[CCL_BY][2];  // S-link ballots of each tile row (255, 0 forest)
    __shared__ uint32_t ulist[CCL_BY][192];   // per row: unions with the row above (slot << 16 | slot)
    __shared__ uint8_t s_links[CCL_THREADS];  // the blocks' links (edge records)

    const int tx = threadIdx.x % CCL_BX, ty = threadIdx.x / CCL_BX;  // lane, warp
    // the warp's pixel rows y - 1, y, y + 1 (y = y0 + 2 ty) with a one-pixel
    // halo as aligned 32-bit words, one per lane (WPR lanes), that the lanes
    // share by shuffles: no shared-memory staging and no barrier before the
    // links (the rows between two warps are read by both, from L1)
    const int o = 2 * tx + 3, wq = o >> 2, sh = (o & 3) * 8;
    uint32_t vm, v0, v1;
    {
        const uint32_t* thr32 = reinterpret_cast<const uint32_t*>(F.thr);
        const int xw = x0 - 4 + 4 * tx;
        const bool colok = tx < WPR && xw >= 0 && xw < w;
        uint32_t v[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int y = y0 - 1 + 2 * ty + k;
            v[k] = (colok && y >= 0 && y < h) ? __ldg(thr32 + (size_t)y * (uint32_t)(w >> 2) + (xw >> 2)) : 0x7F7F7F7Fu;
        }
        // pixels x - 1 .. x + 2 of a row as one word (x = 2 bx)
        auto win = [&](uint32_t r) { return __funnelshift_r(__shfl_sync(FULL, r, wq), __shfl_sync(FULL, r, wq + 1), sh); };
        vm = win(v[0]);
        v0 = win(v[1]);
        v1 = win(v[2]);
    }
    const int bx = bx0 + tx, by = by0 + ty;
    const bool live = bx < w / 2 && by < h / 2;
    const uint32_t l = threadIdx.x;
    cnt[2 * l] = 0;
    cnt[2 * l + 1] = 0;

    // The block's links, computed on bytes: p(x - 1) .. p(x + 2) of pixel
    // rows y - 1, y and y + 1 (x = 2 bx, y = 2 by) as one word each, and
    // per byte "is 255" / "is 0" masks.  The neighbour test pixels and
    // block_links' check masks become: P (up-left) tests p(x-1, y-1) when
    // TL is valid, Q (up) p(x, y-1) or p(x+1, y-1) when TL or TR is, R
    // (up-right) p(x+2, y-1) when TR is, S (left) p(x-1, y) or p(x-1, y+1)
    // when TL or BL is; image edges drop P and S (x = 0), R (x + 2 >= w)
    // and P, Q, R (y = 0).
    const uint32_t Wm = __vcmpeq4(vm, FULL), Km = __vcmpeq4(vm, 0u);
    const uint32_t W0 = __vcmpeq4(v0, FULL), K0 = __vcmpeq4(v0, 0u);
    const uint32_t W1 = __vcmpeq4(v1, FULL), K1 = __vcmpeq4(v1, 0u);
    const uint32_t V0 = W0 | K0, V1 = W1 | K1;
    const bool tl = V0 & 0xFF00u, tr = V0 & 0xFF0000u, bl = V1 & 0xFF00u;
    const bool gx = bx > 0, gy = by > 0, gr = 2 * bx + 2 < w;
    const bool cP = live && tl && gx && gy, cQ = live && (tl || tr) && gy, cR = live && tr && gr && gy;
    const bool cS = live && (tl || bl) && gx;
    // bit 0 P, 1 Q, 2 R, 3 S
    auto links = [&](uint32_t M, uint32_t X0, uint32_t X1) {
        return (cP && (M & 0xFFu) ? 1u : 0u) | (cQ && (M & 0xFFFF00u) ? 2u : 0u) | (cR && (M & 0xFF000000u) ? 4u : 0u) |
               (cS && ((X0 | X1) & 0xFFu) ? 8u : 0u);
    };
    const uint32_t lw = links(Wm, W0, W1), lb = links(Km, K0, K1);
    s_links[threadIdx.x] = (uint8_t)(lw | (lb << 4));
    // the block's 255 and 0 pixel counts
    const uint32_t cw = live ? (uint32_t)(__popc(W0 & 0x00FFFF00u) + __popc(W1 & 0x00FFFF00u)) >> 3 : 0u;
    const uint32_t cb = live ? (uint32_t)(__popc(K0 & 0x00FFFF00u) + __popc(K1 & 0x00FFFF00u)) >> 3 : 0u;

    // S links (left neighbour) inside the tile row, which is this warp: a run
    // of blocks that each link to their left neighbour points at its first
    // block, a smaller slot, so the root of a set stays its minimum
    const uint32_t lane = (uint32_t)tx;
    const unsigned sw = __ballot_sync(FULL, tx > 0 && (lw & 8u));
    const unsigned sb = __ballot_sync(FULL, tx > 0 && (lb & 8u));
    const unsigned le = (2u << lane) - 1u;  // lanes 0 .. lane (2 << 31 wraps to 0)
    const uint32_t hw = 31 - __clz(~sw & le), hb = 31 - __clz(~sb & le);  // run heads (lanes)
    const unsigned mw = le & ~((1u << hw) - 1u), mb = le & ~((1u << hb) - 1u);  // the run up to this lane
    const uint32_t row0 = (uint32_t)ty * CCL_BX;
    const bool last_w = lane == 31 || !((sw >> (lane + 1)) & 1u);  // last block of its run
    const bool last_b = lane == 31 || !((sb >> (lane + 1)) & 1u);
    par[2 * l] = 2 * (row0 + hw);
    par[2 * l + 1] = 2 * (row0 + hb) + 1;
    if (lane == 0) {
        row_runs[ty][0] = sw;
        row_runs[ty][1] = sb;
    }
    __syncthreads();
    // P, Q, R links (up-left, up, up-right) inside the tile.  Every block
    // of a run shares the run's set, so a run needs one union per run of
    // the row above that any of its blocks links to: from the row's link
    // ballots the run's last lane takes the above-row blocks its run links
    // to, keeps the first linked block of each above run and makes those
    // unions.
    if (ty > 0) {
        const unsigned PW = __ballot_sync(FULL, tx > 0 && (lw & 1u)), QW = __ballot_sync(FULL, lw & 2u);
        const unsigned RW = __ballot_sync(FULL, tx < CCL_BX - 1 && (lw & 4u));
        const unsigned PB = __ballot_sync(FULL, tx > 0 && (lb & 1u)), QB = __ballot_sync(FULL, lb & 2u);
        const unsigned RB = __ballot_sync(FULL, tx < CCL_BX - 1 && (lb & 4u));
        const uint32_t aw = ((PW & mw) >> 1) | (QW & mw) | ((RW & mw) << 1);
        const uint32_t ab = ((PB & mb) >> 1) | (QB & mb) | ((RB & mb) << 1);
        const uint32_t up0 = row0 - CCL_BX;
        uint32_t ew = last_w ? (aw & ~((aw << 1) & row_runs[ty - 1][0])) : 0u;
        uint32_t eb = last_b ? (ab & ~((ab << 1) & row_runs[ty - 1][1])) : 0u;
        // the row's unions go to a list (a run touches at most its length
        // + 2 blocks above, so a row has at most 96 per forest), which the
        // warp's lanes then take one each
        const uint32_t nu = (uint32_t)(__popc(ew) + __popc(eb));
        uint32_t incl = nu;
#pragma unroll
        for (uint32_t o2 = 1; o2 < 32; o2 <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o2);
            if (lane >= o2) incl += y;
        }
        uint32_t at = incl - nu;
        for (; ew; ew &= ew - 1) ulist[ty][at++] = (2 * (row0 + hw)) << 16 | (2 * (up0 + __ffs(ew) - 1));
        for (; eb; eb &= eb - 1) ulist[ty][at++] = (2 * (row0 + hb) + 1) << 16 | (2 * (up0 + __ffs(eb) - 1) + 1);
        __syncwarp();
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        for (uint32_t k = lane; k < total; k += 32) {
            const uint32_t e = ulist[ty][k];
            uf_union((volatile uint32_t*)par, e >> 16, e & 0xFFFFu, 2u * CCL_THREADS);
        }
    }
    __syncthreads();
    // roots: a run's head finds it, its other blocks take it from the head
    bool local_capped = false;  // cannot happen: a tile chain visits at most its 2 CCL_THREADS slots
    uint32_t rw = lane == hw ? find_root_volatile((volatile uint32_t*)par, 2 * l, 2u * CCL_THREADS, &local_capped) : 0u;
    uint32_t rb = lane == hb ? find_root_volatile((volatile uint32_t*)par, 2 * l + 1, 2u * CCL_THREADS, &local_capped) : 0u;
    rw = __shfl_sync(FULL, rw, hw);
    rb = __shfl_sync(FULL, rb, hb);
    // pixel counts per root: the run's last lane adds the run's count, the
    // sum over the run's lanes of the ballots of each count bit
    {
        const unsigned w1 = __ballot_sync(FULL, cw & 1u), w2 = __ballot_sync(FULL, cw & 2u), w4 = __ballot_sync(FULL, cw & 4u);
        const unsigned b1 = __ballot_sync(FULL, cb & 1u), b2 = __ballot_sync(FULL, cb & 2u), b4 = __ballot_sync(FULL, cb & 4u);
        const uint32_t sw_ = (uint32_t)(__popc(w1 & mw) + 2 * __popc(w2 & mw) + 4 * __popc(w4 & mw));
        const uint32_t sb_ = (uint32_t)(__popc(b1 & mb) + 2 * __popc(b2 & mb) + 4 * __popc(b4 & mb));
        if (last_w && sw_) atomicAdd(&cnt[rw], sw_);
        if (last_b && sb_) atomicAdd(&cnt[rb], sb_);
    }
    __syncthreads();
    // tile slot s = 2 (row CCL_BX + col) + forest -> frame slot: the tile's
    // first pixel plus row pixel-row pairs plus s mod 2 CCL_BX
    static_assert(CCL_BX == 32, "a tile row is 64 slots");
    const uint32_t tslot0 = (uint32_t)(by0 * 2) * (uint32_t)w + (uint32_t)(bx0 * 2);
    auto gslot = [&](uint32_t s) { return tslot0 + (s >> 6) * (2u * (uint32_t)w) + (s & 63u); };
    const uint2 parents = make_uint2(gslot(rw), gslot(rb));
    if (F.edges) {
        // the edge record: tile roots of the edge blocks, with the block's
        // links of that forest in bits 24-27 (slots are below 2^24); links
        // that leave the tile are the border pass's work
        uint2* rec = reinterpret_cast<uint2*>(F.edges + (size_t)tile * ccl_edge_words(CCL_BY));
        const uint32_t lk = s_links[threadIdx.x];
        const uint2 e = make_uint2(parents.x | ((lk & 15u) << 24), parents.y | ((lk >> 4) << 24));
        if (ty == 0) rec[tx] = e;
        if (ty == CCL_BY - 1) rec[32 + tx] = e;
        if (tx == 0) rec[64 + ty] = e;
        if (tx == CCL_BX - 1) rec[64 + CCL_BY + ty] = e;
    }
    if (live) {
        size_t id = (size_t)(by * 2) * w + bx * 2;
        *reinterpret_cast<uint2*>(F.scratch + id) = parents;
        uint2 sz = make_uint2(rw == 2 * l ? cnt[2 * l] : 0u, rb == 2 * l + 1 ? cnt[2 * l + 1] : 0u);
        *reinterpret_cast<uint2*>(F.sizes + id) = sz;
        if (F.stage_outputs) {
            *reinterpret_cast<uint2*>(F.sizes + id + w) = make_uint2(0u, 0u);
            // the reference keeps the block's information word at scratch[id + w]:
            // bits 0-3 the pixels (TL, TR, BL, BR) that are 255, bits 8-11 those that are 0
            auto bits = [](uint32_t X0, uint32_t X1) {
                return ((X0 >> 8) & 1u) | ((X0 >> 15) & 2u) | ((X1 >> 6) & 4u) | ((X1 >> 13) & 8u);
            };
            *reinterpret_cast<uint2*>(F.scratch + id + w) = make_uint2(bits(W0, W1) | (bits(K0, K1) << 8), 0u);
        }
    }
}

// Merge the links that cross tile borders: P/Q/R of the tile's top row,
// P/S of its left column and R (up-right) of its right column.  After the
// local pass every slot points at its tile root, so a link is a union of
// two tile roots; a lane skips a union that the lane before it (the
// previous block of the same tile edge) makes too, and the warp's unions go
// to a list that its lanes take one each.
template <int CCL_BY>
__device__ __forceinline__ void ccl_border_impl(const FrameSet& fs) {
    constexpr int CCL_BORDER_PER_TILE = CCL_BX + 2 * (CCL_BY - 1);
    const FrameDesc& F = fs.get(blockIdx.y);
    const int w = F.width, h = F.height;
    const int ntx = ccl_tiles_x(w), nty = ccl_tiles_y<CCL_BY>(h);
    const int per_tile = CCL_BORDER_PER_TILE;
    const int total = ntx * nty * per_tile;
    volatile uint32_t* par = F.scratch;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ uint2 blist[8][8 * 32];  // per warp: the unions of one pass (8 per lane at most)
    const uint32_t cap = uf_cap_of(F);
    bool ok = true;
    // warp-uniform trip count: lanes past the end take part in the votes
    for (int i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); i0 < total; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + lane;
        int tbx = 0, tby = 0, bx = 0, by = 0;
        bool live = i < total;
        if (live) {
            const int tile = i / per_tile, k = i % per_tile;
            tbx = (tile % ntx) * CCL_BX;
            tby = (tile / ntx) * CCL_BY;
            if (k < CCL_BX) { bx = tbx + k; by = tby; }
            else if (k < CCL_BX + CCL_BY - 1) { bx = tbx; by = tby + 1 + (k - CCL_BX); }
            else { bx = tbx + CCL_BX - 1; by = tby + 1 + (k - CCL_BX - (CCL_BY - 1)); }
            live = bx < w / 2 && by < h / 2;
        }
        BlockLinks L{0, 0, 0};
        const int x = bx * 2, y = by * 2;
        if (live) {
            const uint8_t* base = F.thr + (size_t)y * w + x;
            L = block_links([&](int dy, int dx) { return (uint32_t)base[(ptrdiff_t)dy * w + dx]; }, x, y, w, h);
        }
        const int ndx[4] = {-1, 0, 1, -1}, ndy[4] = {-1, -1, -1, 0};
        const uint32_t sid = (uint32_t)y * w + x;
        const uint32_t rsw = live ? par[sid] : 0u, rsb = live ? par[sid + 1] : 0u;
        // the lane's unions (up to 4 neighbours x 2 forests) into the warp's
        // list, then one union per lane
        uint32_t ka[8], kb[8], need = 0;
#pragma unroll
        for (int n = 0; n < 4; n++) {
            const int nbx = bx + ndx[n], nby = by + ndy[n];
            // a neighbour in the same tile was merged by the local pass
            const bool cross = live && !(nbx >= tbx && nbx < tbx + CCL_BX && nby >= tby);
            const uint32_t nid = (uint32_t)(nby * 2) * w + nbx * 2;
            const bool lw = cross && (L.wmask & (1u << n)), lb = cross && (L.bmask & (1u << n));
            ka[2 * n] = rsw;
            kb[2 * n] = lw ? par[nid] : 0u;
            ka[2 * n + 1] = rsb;
            kb[2 * n + 1] = lb ? par[nid + 1] : 0u;
            const unsigned long long kw = lw ? ((unsigned long long)ka[2 * n] << 32 | kb[2 * n]) : ~0ull;
            const unsigned long long kk = lb ? ((unsigned long long)ka[2 * n + 1] << 32 | kb[2 * n + 1]) : ~0ull;
            const unsigned long long pw = __shfl_up_sync(0xFFFFFFFFu, kw, 1), pb = __shfl_up_sync(0xFFFFFFFFu, kk, 1);
            if (lw && (lane == 0 || pw != kw)) need |= 1u << (2 * n);
            if (lb && (lane == 0 || pb != kk)) need |= 2u << (2 * n);
        }
        const uint32_t nu = (uint32_t)__popc(need);
        uint32_t incl = nu;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += v;
        }
        uint32_t at = incl - nu;
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (need & (1u << k)) blist[warp][at++] = make_uint2(ka[k], kb[k]);
        __syncwarp();
        const uint32_t nlist = __shfl_sync(0xFFFFFFFFu, incl, 31);
        for (uint32_t k = (uint32_t)lane; k < nlist; k += 32) {
            const uint2 e = blist[warp][k];
            ok &= uf_union(par, e.x, e.y, cap);
        }
        __syncwarp();
    }
    if (!ok && F.counters) atomicOr(F.counters + CNT_STATUS, ATAG_DEVFLAG_UF_ITERATION_CAP);
}

// The border merge from the tiles' edge records: the same unions as
// ccl_border_impl, with each edge block's links and tile roots, and its
// neighbours' tile roots, read from the records (contiguous per tile edge)
// instead of the image and the forest.  A neighbour across the top edge is
// on the bottom row of the tile above (above-left / above-right for the
// corner blocks' P / R), one across the left edge on the left tile's right
// column, one across the right edge on the right tile's left column.
template <int CCL_BY>
__device__ __forceinline__ void ccl_border_edges_impl(const FrameSet& fs) {
    constexpr int PER = CCL_BX + 2 * (CCL_BY - 1);
    constexpr uint32_t EW = ccl_edge_words(CCL_BY), SLOT = 0xFFFFFFu;
    const FrameDesc& F = fs.get(blockIdx.y);
    const int w = F.width, h = F.height;
    const int ntx = ccl_tiles_x(w), nty = ccl_tiles_y<CCL_BY>(h);
    const int total = ntx * nty * PER;
    volatile uint32_t* par = F.scratch;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ uint2 blist[8][8 * 32];  // per warp: the unions of one pass (8 per lane at most)
    const uint32_t cap = uf_cap_of(F);
    bool ok = true;
    // record entry idx of a tile: [0, 32) top row, [32, 64) bottom row,
    // [64, 64 + rows) left column, [64 + rows, 64 + 2 rows) right column
    auto entry = [&](int tile, int idx) { return reinterpret_cast<const uint2*>(F.edges + (size_t)tile * EW)[idx]; };
    // warp-uniform trip count: lanes past the end take part in the votes
    for (int i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); i0 < total; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + lane;
        uint32_t links = 0;
        uint2 mine = make_uint2(0u, 0u), nbr[4] = {};
        if (i < total) {
            const int tile = i / PER, k = i % PER, up = tile - ntx;
            uint32_t keep;
            if (k < CCL_BX) {  // top row: P, Q, R leave the tile; S too in column 0
                mine = entry(tile, k);
                keep = k == 0 ? 0xFFu : 0x77u;
            } else if (k < CCL_BX + CCL_BY - 1) {  // left column: P and S
                mine = entry(tile, 64 + (k - CCL_BX + 1));
                keep = 0x99u;
            } else {  // right column: R
                mine = entry(tile, 64 + CCL_BY + (k - CCL_BX - CCL_BY + 2));
                keep = 0x44u;
            }
            links = ((mine.x >> 24) | ((mine.y >> 24) << 4)) & keep;
            if (k < CCL_BX) {
                const int tx = k;
                if (links & 0x11u) nbr[0] = tx > 0 ? entry(up, 32 + tx - 1) : entry(up - 1, 32 + CCL_BX - 1);
                if (links & 0x22u) nbr[1] = entry(up, 32 + tx);
                if (links & 0x44u) nbr[2] = tx < CCL_BX - 1 ? entry(up, 32 + tx + 1) : entry(up + 1, 32);
                if (links & 0x88u) nbr[3] = entry(tile - 1, 64 + CCL_BY);
            } else if (k < CCL_BX + CCL_BY - 1) {
                const int ty = k - CCL_BX + 1;
                if (links & 0x11u) nbr[0] = entry(tile - 1, 64 + CCL_BY + ty - 1);
                if (links & 0x88u) nbr[3] = entry(tile - 1, 64 + CCL_BY + ty);
            } else {
                const int ty = k - CCL_BX - CCL_BY + 2;
                if (links & 0x44u) nbr[2] = entry(tile + 1, 64 + ty - 1);
            }
        }
        // the lane's unions (up to 4 neighbours x 2 forests) into the warp's
        // list, skipping one the lane before makes too, then one per lane
        uint32_t ka[8], kb[8], need = 0;
#pragma unroll
        for (int n = 0; n < 4; n++) {
            const bool lw = links & (1u << n), lb = links & (16u << n);
            ka[2 * n] = mine.x & SLOT;
            kb[2 * n] = lw ? nbr[n].x & SLOT : 0u;
            ka[2 * n + 1] = mine.y & SLOT;
            kb[2 * n + 1] = lb ? nbr[n].y & SLOT : 0u;
            const unsigned long long kw = lw ? ((unsigned long long)ka[2 * n] << 32 | kb[2 * n]) : ~0ull;
            const unsigned long long kk = lb ? ((unsigned long long)ka[2 * n + 1] << 32 | kb[2 * n + 1]) : ~0ull;
            const unsigned long long pw = __shfl_up_sync(0xFFFFFFFFu, kw, 1), pb = __shfl_up_sync(0xFFFFFFFFu, kk, 1);
            if (lw && (lane == 0 || pw != kw)) need |= 1u << (2 * n);
            if (lb && (lane == 0 || pb != kk)) need |= 2u << (2 * n);
        }
        const uint32_t nu = (uint32_t)__popc(need);
        uint32_t incl = nu;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += v;
        }
        uint32_t at = incl - nu;
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (need & (1u << k)) blist[warp][at++] = make_uint2(ka[k], kb[k]);
        __syncwarp();
        const uint32_t nlist = __shfl_sync(0xFFFFFFFFu, incl, 31);
        for (uint32_t k = (uint32_t)lane; k < nlist; k += 32) {
            const uint2 e = blist[warp][k];
            ok &= uf_union(par, e.x, e.y, cap);
        }
        __syncwarp();
    }
    if (!ok && F.counters) atomicOr(F.counters + CNT_STATUS, ATAG_DEVFLAG_UF_ITERATION_CAP);
}

// FINAL_LABELLING (segmentation.cpp:316-389): labels, component sizes at
// the root, parent array compressed to roots.  A thread takes two
// horizontally adjacent 2x2 blocks (four slots: 16-byte loads and stores of
// parents, sizes and labels) and follows the four parent chains in lock
// step, so four dependent loads are in flight at once.  The forest is final
// here; the only concurrent writes replace a parent by its root, so any
// value read is an ancestor.
__global__ void __launch_bounds__(CCL_FINAL_THREADS, 2048 / CCL_FINAL_THREADS) k_ccl_final(const __grid_constant__ FrameSet fs) {
    // grid (block pairs of a row / CCL_FINAL_THREADS, block rows, frames):
    // the block pair from the block indices, no division
    const FrameDesc& F = fs.get(blockIdx.z);
    const int w = F.width, h = F.height;
    const int npx = w / 4, by = blockIdx.y, px = blockIdx.x * CCL_FINAL_THREADS + threadIdx.x;  // w % 4 == 0
    const uint32_t* par = F.scratch;
    const uint32_t cap = uf_cap_of(F);
    if (by < h / 2 && px < npx) {
        const size_t id = (size_t)(by * 2) * w + (size_t)px * 4;
        const uint4 p4 = *reinterpret_cast<const uint4*>(F.scratch + id);
        const uint4 s4 = *reinterpret_cast<const uint4*>(F.sizes + id);
        const uint32_t top = *reinterpret_cast<const uint32_t*>(F.thr + id);
        const uint32_t bot = *reinterpret_cast<const uint32_t*>(F.thr + id + w);
        uint32_t r[4] = {p4.x, p4.y, p4.z, p4.w};
        bool capped = true;
        for (uint32_t it = 0; it < cap; it++) {
            uint32_t q[4];
#pragma unroll
            for (int k = 0; k < 4; k++) q[k] = par[r[k]];
            bool done = true;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                done &= q[k] == r[k];
                r[k] = q[k];
            }
            if (done) {
                capped = false;
                break;
            }
        }
        if (capped && F.counters) atomicOr(F.counters + CNT_STATUS, ATAG_DEVFLAG_UF_ITERATION_CAP);
        // every slot ends pointing at its root, as the reference's scratch
        // does after its last compression (segmentation.cpp:309)
        if (F.stage_outputs) *reinterpret_cast<uint4*>(F.scratch + id) = make_uint4(r[0], r[1], r[2], r[3]);
        // fold the tile counts of non-root slots into their roots; a root's
        // own entry is left alone (other threads add to it)
        const uint32_t sz[4] = {s4.x, s4.y, s4.z, s4.w};
        bool any_root = false;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t sid = (uint32_t)id + k;
            if (r[k] == sid) any_root = true;
            else if (sz[k]) atomicAdd(F.sizes + r[k], sz[k]);
        }
        if (!F.stage_outputs) {
        } else if (!any_root) {
            *reinterpret_cast<uint4*>(F.sizes + id) = make_uint4(0u, 0u, 0u, 0u);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (r[k] != (uint32_t)id + k) F.sizes[id + k] = 0u;
        }
        auto lab = [](uint32_t c, uint32_t rw, uint32_t rb) {
            return c == 255u ? (LABEL_PIXEL_MASK | rw) : (c == 0u ? rb : 0u);
        };
        *reinterpret_cast<uint4*>(F.labels + id) =
            make_uint4(lab(top & 255u, r[0], r[1]), lab((top >> 8) & 255u, r[0], r[1]),
                       lab((top >> 16) & 255u, r[2], r[3]), lab(top >> 24, r[2], r[3]));
        *reinterpret_cast<uint4*>(F.labels + id + w) =
            make_uint4(lab(bot & 255u, r[0], r[1]), lab((bot >> 8) & 255u, r[0], r[1]),
                       lab((bot >> 16) & 255u, r[2], r[3]), lab(bot >> 24, r[2], r[3]));
    }
}

// ---------------------------------------------------------------------------
// a4: find_boundaries dense planes (find_boundaries.cpp:10-155).  Column 0
// is never processed (every work-group's local x == 0 is halo-only there),
// out-of-image neighbours read label 0.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_boundaries_dense(const __grid_constant__ FrameSet fs,
                                                          uint32_t min_size) {
    const FrameDesc& F = fs.get(blockIdx.y);
    const int w = F.width, h = F.height;
    const size_t N = (size_t)w * h;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
        int y = (int)(i / w), x = (int)(i % w);
        if (x == 0) continue;
        auto L = [&](int yy, int xx) -> uint32_t {
            return (xx >= 0 && xx < w && yy >= 0 && yy < h) ? __ldg(F.labels + (size_t)yy * w + xx) : 0u;
        };
        uint32_t p = F.labels[i];
        uint32_t lp = p & LABEL_VALUE_MASK, cp = p & LABEL_PIXEL_MASK;
        bool small_p = __ldg(F.sizes + lp) < min_size;
        const int dy[4] = {0, 1, 1, 1}, dx[4] = {1, -1, 0, 1};
#pragma unroll
        for (int t = 0; t < 4; t++) {
            if (t == 1) {
                uint32_t left = L(y, x - 1), down = L(y + 1, x);
                bool dup = (left & LABEL_PIXEL_MASK) != (down & LABEL_PIXEL_MASK) &&
                           __ldg(F.sizes + (left & LABEL_VALUE_MASK)) >= min_size &&
                           __ldg(F.sizes + (down & LABEL_VALUE_MASK)) >= min_size;
                if (dup) continue;
            }
            uint32_t q = L(y + dy[t], x + dx[t]);
            uint32_t cq = q & LABEL_PIXEL_MASK;
            if (cq == cp) continue;
            uint32_t lq = q & LABEL_VALUE_MASK;
            if (small_p || __ldg(F.sizes + lq) < min_size) continue;
            uint32_t px = (uint32_t)x | ((uint32_t)t << 14);
            uint32_t py = cq > cp ? (COLOR_DIR_MASK | (uint32_t)y) : (uint32_t)y;
            uint64_t lo = min(lp, lq), hi = max(lp, lq);
            reinterpret_cast<uint32_t*>(F.dense_points)[t * N + i] = px | (py << 16);
            F.dense_keys[t * N + i] = (lo << 32) | hi;
        }
    }
}

__global__ void __launch_bounds__(CCL_BX * 8, 8) k_ccl_local_r8(const __grid_constant__ FrameSet fs) { ccl_local_impl<8>(fs); }
__global__ void __launch_bounds__(CCL_BX * 16, 4) k_ccl_local_r16(const __grid_constant__ FrameSet fs) { ccl_local_impl<16>(fs); }
__global__ void __launch_bounds__(CCL_BX * 32, 2) k_ccl_local_r32(const __grid_constant__ FrameSet fs) { ccl_local_impl<32>(fs); }
__global__ void __launch_bounds__(256) k_ccl_border_r8(const __grid_constant__ FrameSet fs) { ccl_border_impl<8>(fs); }
__global__ void __launch_bounds__(256) k_ccl_border_r16(const __grid_constant__ FrameSet fs) { ccl_border_impl<16>(fs); }
__global__ void __launch_bounds__(256) k_ccl_border_r32(const __grid_constant__ FrameSet fs) { ccl_border_impl<32>(fs); }
__global__ void __launch_bounds__(256) k_ccl_border_edges_r8(const __grid_constant__ FrameSet fs) { ccl_border_edges_impl<8>(fs); }
__global__ void __launch_bounds__(256) k_ccl_border_edges_r16(const __grid_constant__ FrameSet fs) { ccl_border_edges_impl<16>(fs); }
__global__ void __launch_bounds__(256) k_ccl_border_edges_r32(const __grid_constant__ FrameSet fs) { ccl_border_edges_impl<32>(fs); }

}  // namespace atag
