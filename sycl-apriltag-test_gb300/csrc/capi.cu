// capi.cu — the C ABI (include/atag.h): argument checking, workspace
// layout, and the stream-ordered launch sequence of the detector.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "atag_internal.h"
#include "atag_kernels.cuh"

using namespace atag;

namespace {

thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};

atag_status fail(atag_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return fail(ATAG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define LAUNCHED()                                                                                  \
    do {                                                                                            \
        g_launches.fetch_add(1, std::memory_order_relaxed);                                         \
        cudaError_t e_ = cudaGetLastError();                                                        \
        if (e_ != cudaSuccess) return fail(ATAG_ERR_CUDA, "launch: %s", cudaGetErrorString(e_));   \
    } while (0)

struct DeviceInfo {
    int device = -1;
    int num_sms = 0;
    size_t smem_optin = 0;
};

std::mutex g_init_mutex;
DeviceInfo g_dev[64];


atag_status ensure_device(DeviceInfo** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(ATAG_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(ATAG_ERR_NO_DEVICE, "device ordinal %d unsupported", dev);
    std::lock_guard<std::mutex> lk(g_init_mutex);
    DeviceInfo& d = g_dev[dev];
    if (d.device != dev) {
        cudaDeviceProp prop;
        CK(cudaGetDeviceProperties(&prop, dev));
        if (!(prop.major == 10 && prop.minor == 3))
            return fail(ATAG_ERR_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a only", dev,
                        prop.major, prop.minor);
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, k_threshold);
        if (e != cudaSuccess) return fail(ATAG_ERR_NO_DEVICE, "kernels do not load: %s", cudaGetErrorString(e));
        CK(cudaFuncSetAttribute(k_cluster_sort_large, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CF_LARGE_SMEM));
        CK(cudaFuncSetAttribute(k_cluster_sort_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CF_SMALL_SMEM));
        CK(cudaFuncSetAttribute(k_peaks_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PK_SMEM));
        d.num_sms = prop.multiProcessorCount;
        d.smem_optin = prop.sharedMemPerBlockOptin;
        d.device = dev;
    }
    *out = &d;
    return ATAG_OK;
}

bool valid_dims(size_t w, size_t h) { return w >= 4 && h >= 4 && w % 4 == 0 && h % 4 == 0 && w <= 4096 && h <= 4096; }

PipelineParams make_params(const atag_config& c) {
    PipelineParams p;
    p.min_white_black_diff = c.min_white_black_diff;
    p.min_component_size = (uint32_t)c.min_component_size;
    p.min_cluster_pixels = (uint32_t)c.min_cluster_pixels;
    p.tag_width = (uint32_t)c.tag_width;
    p.normal_border = c.normal_border;
    p.reversed_border = c.reversed_border;
    p.max_line_fit_mse = c.max_line_fit_mse;
    double cr = std::cos((double)c.critical_angle_deg * M_PI / 180);
    p.cos_critical_f = (float)cr;
    p.cos_critical_d = cr;
    p.min_area = 0.95 * c.min_tag_width * c.min_tag_width;
    p.compat_peak_index = c.compat_peak_index;
    return p;
}

dim3 grid2(size_t x, size_t y) {
    if (x < 1) x = 1;
    if (x > 65535u * 32) x = 65535u * 32;
    return dim3((unsigned)x, (unsigned)y);
}
size_t cdiv(size_t a, size_t b) { return (a + b - 1) / b; }
// tile CCL grid: (tile columns, tile rows, frames) of the largest frame
dim3 ccl_grid(size_t w, size_t h, size_t rows, size_t frames) {
    return dim3((unsigned)cdiv(w / 2, 32), (unsigned)cdiv(h / 2, rows), (unsigned)frames);
}
// final labelling grid: (pairs of 2x2 blocks of a row, block rows, frames)
dim3 final_grid(size_t w, size_t h, size_t frames) {
    return dim3((unsigned)cdiv(w / 4, CCL_FINAL_THREADS), (unsigned)(h / 2), (unsigned)frames);
}

FrameSet single(const FrameDesc& d) {
    FrameSet s;
    memset(&s, 0, sizeof s);
    s.table = nullptr;
    s.one = d;
    return s;
}
FrameDesc blank() {
    FrameDesc d;
    memset(&d, 0, sizeof d);
    return d;
}

// -------------------------------------------------------------------------
// workspace layout
// -------------------------------------------------------------------------
constexpr size_t ALIGN = 256;
size_t al(size_t v) { return (v + ALIGN - 1) / ALIGN * ALIGN; }
uint32_t pow2_at_least(uint32_t v) {
    uint32_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

struct FrameCaps {
    uint32_t point_cap, pair_cap, cluster_cap, cpoint_cap;
};
FrameCaps caps_for(size_t N) {
    FrameCaps c;
    c.point_cap = (uint32_t)std::max<size_t>(2 * N, 4096);
    size_t pc = std::min<size_t>(std::max<size_t>(N / 512, 1024), 65536);
    c.pair_cap = pow2_at_least((uint32_t)pc);
    c.cluster_cap = (uint32_t)std::min<size_t>(std::max<size_t>(N / 1024, 512), 65535);
    c.cpoint_cap = (uint32_t)std::max<size_t>(N / 2, 4096);
    return c;
}

// Lays out one frame's buffers at `base` (device address, may be 0 to only
// measure).  Returns the bytes used.
// own_grey: the frame needs its own grey buffer (decimated or colour input)
size_t layout_frame(char* base, uint32_t w, uint32_t h, uint32_t factor, bool own_grey, FrameDesc* d) {
    size_t N = (size_t)w * h;
    FrameCaps c = caps_for(N);
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        char* p = base ? base + off : nullptr;
        off += al(bytes);
        return p;
    };
    FrameDesc f = blank();
    f.width = w;
    f.height = h;
    f.factor = factor;
    f.grey = own_grey ? (uint8_t*)take(N) : nullptr;
    f.thr = (uint8_t*)take(N);
    f.scratch = (uint32_t*)take(4 * N);
    f.labels = (uint32_t*)take(4 * N);
    f.sizes = (uint32_t*)take(4 * N);
    f.point_cap = c.point_cap;
    f.points = (unsigned long long*)take(8ull * c.point_cap);
    f.pair_cap = c.pair_cap;
    f.pair_keys = (unsigned long long*)take(8ull * c.pair_cap);
    f.pair_bbox = (uint4*)take(16ull * c.pair_cap);
    f.pair_gsum = (int2*)take(8ull * c.pair_cap);
    f.pair_pxgx = (unsigned long long*)take(8ull * c.pair_cap);
    f.pair_count = (uint32_t*)take(4ull * c.pair_cap);
    f.pair_cluster = (uint32_t*)take(4ull * c.pair_cap);
    f.cluster_cap = c.cluster_cap;
    f.cluster_keys = (unsigned long long*)take(8ull * ((size_t)c.cluster_cap + c.pair_cap));
    f.cluster_bounds = (atag_cluster_bounds*)take(sizeof(atag_cluster_bounds) * c.cluster_cap);
    f.cluster_extents = (atag_cluster_extents*)take(sizeof(atag_cluster_extents) * c.cluster_cap);
    f.cluster_center = (float2*)take(8ull * c.cluster_cap);
    f.cluster_cursor = (uint32_t*)take(4ull * c.cluster_cap);
    f.peak_count = (uint32_t*)take(4ull * c.cluster_cap);
    f.peaks = (atag_corner*)take(sizeof(atag_corner) * 10ull * c.cluster_cap);
    f.peak_clusters = (uint32_t*)take(4ull * c.cluster_cap);
    f.peak_extents = (atag_peak_extents*)take(sizeof(atag_peak_extents) * c.cluster_cap);
    f.fitted = (atag_fitted_quad*)take(sizeof(atag_fitted_quad) * c.cluster_cap);
    f.quad_tmp = (atag_quad_corners*)take(sizeof(atag_quad_corners) * c.cluster_cap);
    f.quad_ok = (uint32_t*)take(4ull * c.cluster_cap);
    f.cpoint_cap = c.cpoint_cap;
    f.sortbuf = (unsigned long long*)take(8ull * c.cpoint_cap);
    f.cluster_points = (atag_cluster_point*)take(sizeof(atag_cluster_point) * c.cpoint_cap);
    f.line_fit = (atag_line_fit_point*)take(sizeof(atag_line_fit_point) * c.cpoint_cap);
    f.errbuf = (float*)take(8ull * c.cpoint_cap);
    f.cluster_work = (uint32_t*)take(4ull * c.cluster_cap);
    f.cluster_runs = (uint32_t*)take(4ull * c.cluster_cap);
    f.counters = (uint32_t*)take(4ull * CNT_COUNT);
    f.dead_pairs = (unsigned long long*)take(8ull * DEAD_PAIRS);
    // CCL edge records, sized for the largest of the tile-row choices
    size_t edge_words = 0;
    for (uint32_t rows : {8u, 16u, 32u})
        edge_words = std::max(edge_words, cdiv(w / 2, 32) * cdiv(h / 2, (size_t)rows) * ccl_edge_words(rows));
    f.edges = (uint32_t*)take(4 * edge_words);
    if (d) *d = f;
    return off;
}

constexpr int RING = 16;
constexpr int CAPTURE_SLOTS = 16;  // distinct frame tables that captured graphs may hold
constexpr size_t WORK_LISTS = 5;  // batch-wide work lists of the per-cluster kernels
constexpr int MAX_LANES = 4;      // sub-batches of one call that run concurrently

// Workspace of atag_cluster: the pair table and the cluster scratch of one
// frame (the outputs are the caller's arrays), plus the counters, a stats
// record for callers that pass none and the work offsets of the sorts.
struct StageClusterLayout {
    size_t bytes;
    FrameDesc d;
    atag_frame_stats* stats;
    uint32_t* work;  // small/large offsets (2 words each), then 2 queue cursors
};
StageClusterLayout layout_stage_cluster(char* base, uint32_t w, uint32_t h, uint32_t cluster_cap, uint32_t cpoint_cap) {
    StageClusterLayout L;
    const FrameCaps c = caps_for((size_t)w * h);
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        char* p = base ? base + off : nullptr;
        off += al(bytes);
        return p;
    };
    FrameDesc f = blank();
    f.width = w;
    f.height = h;
    f.factor = 1;
    f.pair_cap = c.pair_cap;
    f.pair_keys = (unsigned long long*)take(8ull * c.pair_cap);
    f.pair_bbox = (uint4*)take(16ull * c.pair_cap);
    f.pair_gsum = (int2*)take(8ull * c.pair_cap);
    f.pair_pxgx = (unsigned long long*)take(8ull * c.pair_cap);
    f.pair_count = (uint32_t*)take(4ull * c.pair_cap);
    f.pair_cluster = (uint32_t*)take(4ull * c.pair_cap);
    f.cluster_cap = cluster_cap;
    f.cluster_keys = (unsigned long long*)take(8ull * ((size_t)cluster_cap + c.pair_cap));
    f.cluster_center = (float2*)take(8ull * cluster_cap);
    f.cluster_cursor = (uint32_t*)take(4ull * cluster_cap);
    f.peak_count = (uint32_t*)take(4ull * cluster_cap);
    f.cluster_work = (uint32_t*)take(4ull * cluster_cap);
    f.cluster_runs = (uint32_t*)take(4ull * cluster_cap);
    f.cpoint_cap = cpoint_cap;
    f.sortbuf = (unsigned long long*)take(8ull * cpoint_cap);
    f.errbuf = (float*)take(8ull * cpoint_cap);
    f.counters = (uint32_t*)take(4ull * CNT_COUNT);
    f.stage_outputs = 1;
    L.stats = (atag_frame_stats*)take(sizeof(atag_frame_stats));
    L.work = (uint32_t*)take(4ull * 6);
    L.d = f;
    L.bytes = off;
    return L;
}

}  // namespace

namespace atag {
atag_status set_error(atag_status s, const char* msg) { return fail(s, "%s", msg); }
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
}  // namespace atag

// ===========================================================================
// detector
// ===========================================================================
struct atag_detector {
    atag_config cfg;
    PipelineParams pp;
    size_t max_w, max_h, max_frames, max_total_pixels;
    DeviceInfo* dev = nullptr;
    char* ws = nullptr;
    size_t ws_bytes = 0;
    bool owns_ws = false;
    // header carve-out
    FrameDesc* d_tables = nullptr;   // RING x max_frames
    FrameDesc* d_captured = nullptr; // CAPTURE_SLOTS x max_frames: tables of captured calls
    uint32_t* d_work = nullptr;      // per lane: offsets (WORK_LISTS x (max_frames + 1)) + WORK_LISTS counters
    cudaStream_t lane_stream[MAX_LANES] = {};    // streams of lanes 1.. (lane 0 runs on the caller's)
    cudaStream_t side[MAX_LANES] = {};           // per lane: stream of the large-cluster kernel
    cudaEvent_t fork[MAX_LANES] = {}, join[MAX_LANES] = {};
    cudaEvent_t lane_fork = nullptr, lane_join[MAX_LANES] = {};
    uint8_t* d_input = nullptr;      // host-upload input region
    size_t input_bytes = 0;
    atag_quad_corners* d_hquads = nullptr;  // host-path quad staging
    atag_frame_stats* d_hstats = nullptr;
    size_t hquad_cap = 0;
    char* frames_base = nullptr;
    size_t frames_bytes = 0;
    // host staging for the frame tables
    FrameDesc* h_staging = nullptr;  // pinned, RING x max_frames
    FrameDesc* h_captured = nullptr; // pinned, CAPTURE_SLOTS x max_frames; never rewritten while in use
    std::vector<std::vector<FrameDesc>> captured;  // contents of the captured slots in use
    cudaEvent_t ev[RING];
    int ring = 0;
    int last_slot = -1;
    std::vector<FrameDesc> last;     // table last uploaded
    std::vector<FrameDesc> cur;      // table of the last call
    std::vector<cudaEvent_t> stage_events;
    atag_tuning tuning{16, 16, (int32_t)CF_SMALL_CAP, 8, 2, 8, 2};
    atag_limits limits{};
    bool keep_intermediates = false;
    bool refine = false;
};

namespace {

constexpr size_t HOST_QUAD_CAP = 4096;

size_t header_bytes(size_t max_frames, size_t input_bytes) {
    size_t b = 0;
    b += al(sizeof(FrameDesc) * RING * max_frames);
    b += al(sizeof(FrameDesc) * CAPTURE_SLOTS * max_frames);
    b += al(4 * MAX_LANES * (WORK_LISTS * (max_frames + 1) + WORK_LISTS));
    b += al(input_bytes);
    b += al(sizeof(atag_quad_corners) * HOST_QUAD_CAP);
    b += al(sizeof(atag_frame_stats));
    return b;
}

size_t frames_bound(size_t max_frames, size_t max_total_pixels) {
    // bytes(N) is bounded by a per-frame constant plus a per-pixel slope
    size_t c0 = layout_frame(nullptr, 4, 4, 2, true, nullptr);
    size_t big = 1 << 22;  // 4 Mpx
    size_t cb = layout_frame(nullptr, 2048, 2048, 2, true, nullptr);
    double slope = (double)(cb) / (double)big;
    return max_frames * (c0 + 64 * ALIGN) + (size_t)(slope * 1.25 * (double)max_total_pixels) + (1 << 20);
}

}  // namespace

extern "C" {

void atag_config_default(atag_config* c) {
    c->decimate = 1;
    c->min_white_black_diff = 5;
    c->min_component_size = 25;
    c->min_cluster_pixels = 5;
    c->tag_width = 4;
    c->normal_border = 1;
    c->reversed_border = 0;
    c->max_line_fit_mse = 10.0f;
    c->critical_angle_deg = 10.0f;
    c->min_tag_width = 8;
    c->compat_peak_index = 1;
}

const char* atag_status_string(atag_status s) {
    switch (s) {
    case ATAG_OK: return "ok";
    case ATAG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case ATAG_ERR_CUDA: return "CUDA error";
    case ATAG_ERR_CAPACITY: return "capacity exceeded";
    case ATAG_ERR_ITERATION_CAP: return "iteration cap reached";
    case ATAG_ERR_NO_DEVICE: return "no suitable device";
    case ATAG_ERR_OUT_OF_MEMORY: return "out of memory";
    }
    return "unknown status";
}

const char* atag_last_error(void) { return g_last_error.c_str(); }

atag_status atag_init(void) {
    DeviceInfo* d;
    return ensure_device(&d);
}

uint64_t atag_launch_count(void) { return g_launches.load(); }

// ------------------------------------------------------------------ stages

atag_status atag_decimate(const uint8_t* src, size_t sw, size_t sh, size_t f, uint8_t* dst, atag_stream_t stream) {
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    if (!src || !dst || f < 1 || f > 64) return fail(ATAG_ERR_INVALID_ARGUMENT, "decimate: bad pointer or factor");
    size_t w = sw / f, h = sh / f;
    if (!valid_dims(w, h)) return fail(ATAG_ERR_INVALID_ARGUMENT, "decimate: %zux%zu after decimation is not a multiple of 4 in [4, 4096]", w, h);
    if (f == 1) {
        CK(cudaMemcpyAsync(dst, src, sw * sh, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
        return ATAG_OK;
    }
    FrameDesc d = blank();
    d.width = (uint32_t)w; d.height = (uint32_t)h; d.factor = (uint32_t)f; d.src_stride = (uint32_t)sw;
    d.src_format = ATAG_PIX_GREY8;
    d.src = src; d.grey = dst;
    k_decimate<<<grid2(std::min<size_t>(cdiv(w / 4 * h, 256), 4096), 1), 256, 0, (cudaStream_t)stream>>>(single(d));
    LAUNCHED();
    return ATAG_OK;
}

atag_status atag_convert_grey(const uint8_t* src, size_t sw, size_t sh, size_t pitch, int format, size_t f,
                              uint8_t* dst, atag_stream_t stream) {
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    const uint32_t bpp = format < 0 ? 0u : pixel_bytes((uint32_t)format);
    if (!src || !dst || f < 1 || f > 64 || bpp == 0)
        return fail(ATAG_ERR_INVALID_ARGUMENT, "convert_grey: bad pointer, factor or pixel format");
    if (pitch == 0) pitch = sw * bpp;
    if (pitch < sw * bpp) return fail(ATAG_ERR_INVALID_ARGUMENT, "convert_grey: row pitch below the width");
    size_t w = sw / f, h = sh / f;
    if (!valid_dims(w, h)) return fail(ATAG_ERR_INVALID_ARGUMENT, "convert_grey: %zux%zu after decimation is not a multiple of 4 in [4, 4096]", w, h);
    FrameDesc d = blank();
    d.width = (uint32_t)w; d.height = (uint32_t)h; d.factor = (uint32_t)f; d.src_stride = (uint32_t)pitch;
    d.src_format = (uint32_t)format;
    d.src = src; d.grey = dst;
    if (f == 1 && format == ATAG_PIX_GREY8) {
        CK(cudaMemcpy2DAsync(dst, w, src, pitch, w, h, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
        return ATAG_OK;
    }
    k_decimate<<<grid2(std::min<size_t>(cdiv(w / 4 * h, 256), 4096), 1), 256, 0, (cudaStream_t)stream>>>(single(d));
    LAUNCHED();
    return ATAG_OK;
}

atag_status atag_threshold_image(const uint8_t* grey, uint8_t* extrema, uint8_t* filtered, uint8_t* thr,
                                 size_t w, size_t h, atag_stream_t stream) {
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    if (!grey || !thr) return fail(ATAG_ERR_INVALID_ARGUMENT, "threshold_image: null pointer");
    if (!valid_dims(w, h)) return fail(ATAG_ERR_INVALID_ARGUMENT, "threshold_image: %zux%zu is not a multiple of 4 in [4, 4096]", w, h);
    FrameDesc d = blank();
    d.width = (uint32_t)w; d.height = (uint32_t)h; d.factor = 1;
    d.grey = const_cast<uint8_t*>(grey); d.thr = thr; d.extrema = extrema; d.filtered_extrema = filtered;
    size_t tiles = cdiv(w / 4, 32) * cdiv(h / 4, 16);
    k_threshold<<<grid2(tiles, 1), 256, 0, (cudaStream_t)stream>>>(single(d), 5, (extrema || filtered) ? 1 : 0);
    LAUNCHED();
    return ATAG_OK;
}

static atag_status launch_segmentation(const FrameSet& fs, size_t max_w, size_t max_h, size_t nf, cudaStream_t s,
                                       int rows = 16) {
    size_t tiles = cdiv(max_w / 2, 32) * cdiv(max_h / 2, (size_t)rows);
    size_t border = tiles * (32 + 2 * (rows - 1));
    if (rows == 8) {
        k_ccl_local_r8<<<ccl_grid(max_w, max_h, 8, nf), 32 * 8, 0, s>>>(fs);
        LAUNCHED();
        k_ccl_border_r8<<<grid2(cdiv(border, 256), nf), 256, 0, s>>>(fs);
        LAUNCHED();
    } else {
        k_ccl_local_r16<<<ccl_grid(max_w, max_h, 16, nf), 32 * 16, 0, s>>>(fs);
        LAUNCHED();
        k_ccl_border_r16<<<grid2(cdiv(border, 256), nf), 256, 0, s>>>(fs);
        LAUNCHED();
    }
    k_ccl_final<<<final_grid(max_w, max_h, nf), CCL_FINAL_THREADS, 0, s>>>(fs);
    LAUNCHED();
    return ATAG_OK;
}

atag_status atag_image_segmentation(const uint8_t* thr, uint32_t* scratch, uint32_t* labels, uint32_t* sizes,
                                    size_t sizes_elem, size_t w, size_t h, atag_stream_t stream) {
    (void)sizes_elem;
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    if (!thr || !scratch || !labels || !sizes) return fail(ATAG_ERR_INVALID_ARGUMENT, "image_segmentation: null pointer");
    if (!valid_dims(w, h)) return fail(ATAG_ERR_INVALID_ARGUMENT, "image_segmentation: %zux%zu is not a multiple of 4 in [4, 4096]", w, h);
    FrameDesc d = blank();
    d.width = (uint32_t)w; d.height = (uint32_t)h; d.factor = 1;
    d.thr = const_cast<uint8_t*>(thr); d.scratch = scratch; d.labels = labels; d.sizes = sizes;
    d.stage_outputs = 1;
    return launch_segmentation(single(d), w, h, 1, (cudaStream_t)stream);
}

atag_status atag_find_boundaries(const uint32_t* labels, const uint32_t* sizes, atag_boundary_point* points,
                                 uint64_t* blob_labels, size_t w, size_t h, atag_stream_t stream) {
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    if (!labels || !sizes || !points || !blob_labels) return fail(ATAG_ERR_INVALID_ARGUMENT, "find_boundaries: null pointer");
    if (!valid_dims(w, h)) return fail(ATAG_ERR_INVALID_ARGUMENT, "find_boundaries: %zux%zu is not a multiple of 4 in [4, 4096]", w, h);
    FrameDesc d = blank();
    d.width = (uint32_t)w; d.height = (uint32_t)h;
    d.labels = const_cast<uint32_t*>(labels); d.sizes = const_cast<uint32_t*>(sizes);
    d.dense_points = points; d.dense_keys = blob_labels;
    k_boundaries_dense<<<grid2(std::min<size_t>(cdiv(w * h, 256), 8192), 1), 256, 0, (cudaStream_t)stream>>>(single(d), 25);
    LAUNCHED();
    return ATAG_OK;
}

atag_status atag_fit_lines(const atag_line_fit_point* points, const uint16_t* cidx, const atag_cluster_extents* extents,
                           size_t n, atag_corner* found, atag_stream_t stream) {
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    if (n == 0) return ATAG_OK;
    if (!points || !cidx || !extents || !found) return fail(ATAG_ERR_INVALID_ARGUMENT, "fit_lines: null pointer");
    size_t groups = cdiv(n, 24);
    k_fit_lines_windowed<<<grid2(cdiv(groups, 4), 1), 128, 0, (cudaStream_t)stream>>>(points, cidx, extents, n, found);
    LAUNCHED();
    return ATAG_OK;
}

atag_status atag_do_indexing(const atag_peak_extents* extents, size_t count, const atag_corner* corners,
                             const atag_line_fit_point* points, const atag_cluster_extents* cluster_extents,
                             atag_fitted_quad* fitted, atag_stream_t stream) {
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    if (count == 0) return ATAG_OK;
    if (!extents || !corners || !points || !cluster_extents || !fitted)
        return fail(ATAG_ERR_INVALID_ARGUMENT, "do_indexing: null pointer");
    float cosc = (float)std::cos(10 * M_PI / 180);
    k_do_indexing<<<grid2(std::min<size_t>(count, 65535), 1), 256, 0, (cudaStream_t)stream>>>(
        extents, count, corners, points, cluster_extents, 10.0f, cosc, fitted);
    LAUNCHED();
    return ATAG_OK;
}

atag_status atag_process_fitted_quads(const atag_fitted_quad* fitted, size_t count, size_t w, size_t h,
                                      const atag_config* cfg, atag_quad_corners* quads, size_t cap, uint32_t* d_count,
                                      atag_stream_t stream) {
    (void)w; (void)h;
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    if (!d_count || (count && (!fitted || !quads))) return fail(ATAG_ERR_INVALID_ARGUMENT, "process_fitted_quads: null pointer");
    atag_config c;
    if (cfg) c = *cfg; else atag_config_default(&c);
    k_process_quads<<<1, 256, 0, (cudaStream_t)stream>>>(fitted, count, make_params(c), quads, cap, d_count);
    LAUNCHED();
    return ATAG_OK;
}

// ------------------------------------------------------------------ stage glue

static bool stage_cluster_caps(size_t w, size_t h, size_t cluster_capacity, size_t point_capacity,
                               uint32_t* ccap, uint32_t* pcap) {
    if (!valid_dims(w, h) || cluster_capacity == 0 || point_capacity == 0) return false;
    *ccap = (uint32_t)std::min<size_t>(cluster_capacity, 65535);  // 16-bit cluster index
    *pcap = (uint32_t)std::min<size_t>(point_capacity, 4 * w * h);  // at most 4 points per pixel
    return true;
}

atag_status atag_cluster_workspace_size(size_t w, size_t h, size_t cluster_capacity, size_t point_capacity,
                                        size_t* bytes) {
    uint32_t cc, pc;
    if (!bytes || !stage_cluster_caps(w, h, cluster_capacity, point_capacity, &cc, &pc))
        return fail(ATAG_ERR_INVALID_ARGUMENT, "cluster_workspace_size: bad size or capacity");
    *bytes = layout_stage_cluster(nullptr, (uint32_t)w, (uint32_t)h, cc, pc).bytes + ALIGN;
    return ATAG_OK;
}

atag_status atag_cluster(const atag_boundary_point* points, const uint64_t* keys, const uint8_t* grey, size_t w,
                         size_t h, void* ws, size_t ws_bytes, const atag_cluster_outputs* o, atag_stream_t stream) {
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    uint32_t cc, pc;
    if (!o || !stage_cluster_caps(w, h, o->cluster_capacity, o->point_capacity, &cc, &pc))
        return fail(ATAG_ERR_INVALID_ARGUMENT, "cluster: bad size or capacity");
    if (!points || !keys || !grey || !ws || !o->filtered_bounds || !o->cluster_extents || !o->cluster_points ||
        !o->cluster_indices || !o->line_fit_points)
        return fail(ATAG_ERR_INVALID_ARGUMENT, "cluster: null pointer");
    if ((o->pair_bounds || o->pair_keys) && o->pair_capacity == 0)
        return fail(ATAG_ERR_INVALID_ARGUMENT, "cluster: pair outputs without a pair capacity");
    char* base = (char*)(((uintptr_t)ws + ALIGN - 1) / ALIGN * ALIGN);
    StageClusterLayout L = layout_stage_cluster(base, (uint32_t)w, (uint32_t)h, cc, pc);
    if ((size_t)(base - (char*)ws) + L.bytes > ws_bytes)
        return fail(ATAG_ERR_OUT_OF_MEMORY, "cluster: workspace of %zu bytes is too small", ws_bytes);
    FrameDesc d = L.d;
    d.grey = const_cast<uint8_t*>(grey);
    d.cluster_bounds = o->filtered_bounds;
    d.cluster_extents = o->cluster_extents;
    d.cluster_points = o->cluster_points;
    d.line_fit = o->line_fit_points;
    d.stats = o->counts ? o->counts : L.stats;
    d.pair_bounds_out = o->pair_bounds;
    d.pair_keys_out = (unsigned long long*)o->pair_keys;
    d.pair_out_cap = (uint32_t)std::min<size_t>(o->pair_capacity, 0xFFFFFFFFu);
    const FrameSet fs = single(d);
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t n = (uint32_t)(4 * w * h);
    const int sms = dev->num_sms;
    uint32_t* off_small = L.work;
    uint32_t* off_large = L.work + 2;
    uint32_t* wc = L.work + 4;
    atag_config c;
    atag_config_default(&c);
    const PipelineParams p = make_params(c);
    k_reset_frames<<<grid2(cdiv(d.pair_cap, 256), 1), 256, 0, s>>>(fs);
    LAUNCHED();
    k_planes_pairs<<<(unsigned)std::min<size_t>(cdiv(n, 256), (size_t)sms * 8), 256, 0, s>>>(
        fs, reinterpret_cast<const uint32_t*>(points), reinterpret_cast<const unsigned long long*>(keys), n);
    LAUNCHED();
    k_pairs_finalize<<<1, 1024, 0, s>>>(fs, p, CF_SMALL_CAP);
    LAUNCHED();
    {
        BatchOffsets bo{{CNT_SMALL, CNT_LARGE, 0, 0}, {off_small, off_large, nullptr, nullptr}, wc};
        k_batch_offsets<<<1, 1024, 0, s>>>(fs, 1, bo);
    }
    LAUNCHED();
    k_planes_scatter<<<(unsigned)std::min<size_t>(cdiv(n, 256), (size_t)sms * 8), 256, 0, s>>>(
        fs, reinterpret_cast<const uint32_t*>(points), reinterpret_cast<const unsigned long long*>(keys), n);
    LAUNCHED();
    k_cluster_sort_large<<<std::max(1, sms / 2), CF_LARGE_THREADS, CF_LARGE_SMEM, s>>>(fs, off_large, 1, wc + 1);
    LAUNCHED();
    k_cluster_sort_small<<<sms * 8, CF_SMALL_THREADS, CF_SMALL_SMEM, s>>>(fs, off_small, 1, wc, CF_SMALL_CAP);
    LAUNCHED();
    k_stage_cluster_out<<<sms * 4, 256, 0, s>>>(fs, o->cluster_indices, (unsigned long long*)o->filtered_keys);
    LAUNCHED();
    return ATAG_OK;
}

atag_status atag_corner_peaks_workspace_size(size_t cluster_count, size_t* bytes) {
    if (!bytes) return fail(ATAG_ERR_INVALID_ARGUMENT, "corner_peaks_workspace_size: null pointer");
    *bytes = al(8 * std::max<size_t>(cluster_count, 1)) + ALIGN;
    return ATAG_OK;
}

atag_status atag_corner_peaks(const atag_corner* found, const atag_cluster_extents* extents, size_t n_clusters,
                              void* ws, size_t ws_bytes, atag_corner* out, size_t corner_cap,
                              atag_peak_extents* peak_extents, size_t extents_cap, uint32_t* d_counts,
                              atag_stream_t stream) {
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    if (!d_counts) return fail(ATAG_ERR_INVALID_ARGUMENT, "corner_peaks: null counts");
    if (n_clusters > 65535) return fail(ATAG_ERR_INVALID_ARGUMENT, "corner_peaks: more than 65535 clusters");
    if (n_clusters && (!found || !extents || !ws || (corner_cap && !out) || (extents_cap && !peak_extents)))
        return fail(ATAG_ERR_INVALID_ARGUMENT, "corner_peaks: null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    if (n_clusters == 0) {
        CK(cudaMemsetAsync(d_counts, 0, 3 * sizeof(uint32_t), s));
        return ATAG_OK;
    }
    uint32_t* counts = (uint32_t*)(((uintptr_t)ws + ALIGN - 1) / ALIGN * ALIGN);
    uint32_t* offsets = counts + n_clusters;
    if ((size_t)((char*)(offsets + n_clusters) - (char*)ws) > ws_bytes)
        return fail(ATAG_ERR_OUT_OF_MEMORY, "corner_peaks: workspace of %zu bytes is too small", ws_bytes);
    const uint32_t nc = (uint32_t)n_clusters;
    const uint32_t ccap = (uint32_t)std::min<size_t>(corner_cap, 0xFFFFFFFFu);
    const uint32_t ecap = (uint32_t)std::min<size_t>(extents_cap, 0xFFFFFFFFu);
    const int sms = dev->num_sms;
    k_peaks_count<<<(unsigned)std::min<size_t>(cdiv(nc, 8), (size_t)sms * 8), 256, 0, s>>>(found, extents, nc, counts);
    LAUNCHED();
    k_peaks_offsets<<<1, 1024, 0, s>>>(counts, nc, offsets, peak_extents, ecap, ccap, d_counts);
    LAUNCHED();
    k_peaks_sort<<<(unsigned)std::min<size_t>(nc, (size_t)sms * 2), 256, PK_SMEM, s>>>(found, extents, nc, counts,
                                                                                        offsets, out, ccap, d_counts);
    LAUNCHED();
    return ATAG_OK;
}

// ------------------------------------------------------------------ host helpers

atag_status atag_get_moment(const atag_line_fit_point* points, size_t n, size_t i0, size_t i1,
                            atag_line_fit_point* out, size_t* num) {
    if (!points || !out || !num) return fail(ATAG_ERR_INVALID_ARGUMENT, "get_moment: null pointer");
    if (i0 >= n || i1 >= n) return fail(ATAG_ERR_INVALID_ARGUMENT, "get_moment: range [%zu, %zu] outside %zu points", i0, i1, n);
    unsigned long long cnt = 0;
    const Moment m = get_moment(points, n, i0, i1, &cnt);
    atag_line_fit_point r;
    memset(&r, 0, sizeof r);
    store_moment(&r, m);
    // the reference copies the leading operand, a and b included
    const atag_line_fit_point* lead = i0 < i1 ? &points[i1] : (i1 < i0 ? &points[n - 1] : nullptr);
    if (lead) {
        r.a = lead->a;
        r.b = lead->b;
    }
    *out = r;
    *num = (size_t)cnt;
    return ATAG_OK;
}

atag_status atag_fit_line(const atag_line_fit_point* moment, size_t num, float* lp, float* err, float* mse) {
    if (!moment) return fail(ATAG_ERR_INVALID_ARGUMENT, "fit_line: null moment");
    fit_line(load_moment(moment), (unsigned long long)num, lp, err, mse);
    return ATAG_OK;
}

atag_line_fit_point atag_compute_initial_linefit(atag_cluster_point p, uint32_t width, uint32_t height,
                                                 const uint8_t* grey) {
    atag_line_fit_point r;
    memset(&r, 0, sizeof r);
    const uint32_t packed = (uint32_t)p.packed_x | ((uint32_t)p.packed_y << 16);
    if (grey) {
        store_moment(&r, initial_linefit(packed, width, height, grey));
    } else {
        // no image: every weight is 1, as outside the image
        store_moment(&r, initial_linefit(packed, 0, 0, nullptr));
    }
    return r;
}

// ------------------------------------------------------------------ detector

atag_status atag_workspace_size(const atag_config* cfg, size_t max_w, size_t max_h, size_t max_frames,
                                size_t max_total_pixels, size_t* bytes) {
    if (!bytes || max_frames == 0) return fail(ATAG_ERR_INVALID_ARGUMENT, "workspace_size: bad argument");
    atag_config c;
    if (cfg) c = *cfg; else atag_config_default(&c);
    if (c.decimate < 1) return fail(ATAG_ERR_INVALID_ARGUMENT, "workspace_size: decimate < 1");
    if (!valid_dims(max_w, max_h)) return fail(ATAG_ERR_INVALID_ARGUMENT, "workspace_size: bad max dimensions");
    if (max_total_pixels == 0) max_total_pixels = max_w * max_h * max_frames;
    size_t input = max_total_pixels * (size_t)c.decimate * (size_t)c.decimate;
    *bytes = header_bytes(max_frames, input) + frames_bound(max_frames, max_total_pixels);
    return ATAG_OK;
}

atag_status atag_detector_create(const atag_config* cfg, size_t max_w, size_t max_h, size_t max_frames,
                                 size_t max_total_pixels, void* d_ws, size_t ws_bytes, atag_detector** out) {
    if (!out) return fail(ATAG_ERR_INVALID_ARGUMENT, "detector_create: null out");
    *out = nullptr;
    DeviceInfo* dev;
    atag_status st = ensure_device(&dev);
    if (st) return st;
    atag_config c;
    if (cfg) c = *cfg; else atag_config_default(&c);
    if (max_total_pixels == 0) max_total_pixels = max_w * max_h * max_frames;
    size_t need;
    st = atag_workspace_size(&c, max_w, max_h, max_frames, max_total_pixels, &need);
    if (st) return st;
    if (d_ws && ws_bytes < need) return fail(ATAG_ERR_OUT_OF_MEMORY, "detector_create: workspace of %zu bytes < %zu needed", ws_bytes, need);
    atag_detector* det = new atag_detector();
    det->cfg = c;
    det->pp = make_params(c);
    det->max_w = max_w; det->max_h = max_h; det->max_frames = max_frames; det->max_total_pixels = max_total_pixels;
    det->dev = dev;
    if (d_ws) {
        det->ws = (char*)d_ws;
        det->ws_bytes = ws_bytes;
    } else {
        cudaError_t e = cudaMalloc(&det->ws, need);
        if (e != cudaSuccess) {
            delete det;
            return fail(ATAG_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu): %s", need, cudaGetErrorString(e));
        }
        det->ws_bytes = need;
        det->owns_ws = true;
    }
    char* p = det->ws;
    det->d_tables = (FrameDesc*)p; p += al(sizeof(FrameDesc) * RING * max_frames);
    det->d_captured = (FrameDesc*)p; p += al(sizeof(FrameDesc) * CAPTURE_SLOTS * max_frames);
    det->d_work = (uint32_t*)p; p += al(4 * MAX_LANES * (WORK_LISTS * (max_frames + 1) + WORK_LISTS));
    det->input_bytes = max_total_pixels * (size_t)c.decimate * (size_t)c.decimate;
    det->d_input = (uint8_t*)p; p += al(det->input_bytes);
    det->d_hquads = (atag_quad_corners*)p; p += al(sizeof(atag_quad_corners) * HOST_QUAD_CAP);
    det->d_hstats = (atag_frame_stats*)p; p += al(sizeof(atag_frame_stats));
    det->hquad_cap = HOST_QUAD_CAP;
    det->frames_base = p;
    det->frames_bytes = det->ws_bytes - (size_t)(p - det->ws);
    cudaError_t e = cudaHostAlloc(&det->h_staging, sizeof(FrameDesc) * RING * max_frames, cudaHostAllocDefault);
    if (e == cudaSuccess)
        e = cudaHostAlloc(&det->h_captured, sizeof(FrameDesc) * CAPTURE_SLOTS * max_frames, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        if (det->h_staging) cudaFreeHost(det->h_staging);
        if (det->owns_ws) cudaFree(det->ws);
        delete det;
        return fail(ATAG_ERR_OUT_OF_MEMORY, "cudaHostAlloc: %s", cudaGetErrorString(e));
    }
    for (int i = 0; i < RING; i++) cudaEventCreateWithFlags(&det->ev[i], cudaEventDisableTiming);
    for (int k = 0; k < MAX_LANES; k++) {
        cudaStreamCreateWithFlags(&det->side[k], cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&det->fork[k], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&det->join[k], cudaEventDisableTiming);
    }
    for (int k = 1; k < MAX_LANES; k++) {
        cudaStreamCreateWithFlags(&det->lane_stream[k], cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&det->lane_join[k], cudaEventDisableTiming);
    }
    cudaEventCreateWithFlags(&det->lane_fork, cudaEventDisableTiming);
    *out = det;
    return ATAG_OK;
}

atag_status atag_detector_destroy(atag_detector* det) {
    if (!det) return ATAG_OK;
    for (int i = 0; i < RING; i++) {
        cudaEventSynchronize(det->ev[i]);
        cudaEventDestroy(det->ev[i]);
    }
    for (int k = 0; k < MAX_LANES; k++) {
        if (det->side[k]) {
            cudaStreamSynchronize(det->side[k]);
            cudaStreamDestroy(det->side[k]);
        }
        if (det->fork[k]) cudaEventDestroy(det->fork[k]);
        if (det->join[k]) cudaEventDestroy(det->join[k]);
    }
    for (int k = 1; k < MAX_LANES; k++) {
        if (det->lane_stream[k]) {
            cudaStreamSynchronize(det->lane_stream[k]);
            cudaStreamDestroy(det->lane_stream[k]);
        }
        if (det->lane_join[k]) cudaEventDestroy(det->lane_join[k]);
    }
    if (det->lane_fork) cudaEventDestroy(det->lane_fork);
    if (det->h_staging) cudaFreeHost(det->h_staging);
    if (det->h_captured) cudaFreeHost(det->h_captured);
    if (det->owns_ws) cudaFree(det->ws);
    delete det;
    return ATAG_OK;
}

// Lowers a frame's capacities to the detector's limits (never raises them:
// the workspace was laid out for the defaults).
static void apply_limits(const atag_limits& L, FrameDesc* d) {
    if (L.point_capacity) d->point_cap = std::min(d->point_cap, L.point_capacity);
    if (L.pair_capacity) {
        uint32_t p = 1;
        while (p * 2 <= std::min(d->pair_cap, L.pair_capacity)) p *= 2;
        d->pair_cap = p;
    }
    if (L.cluster_capacity) d->cluster_cap = std::min(d->cluster_cap, L.cluster_capacity);
    if (L.cluster_point_capacity) d->cpoint_cap = std::min(d->cpoint_cap, L.cluster_point_capacity);
    d->uf_cap = L.uf_iteration_cap;
}

// The device table of frame descriptors a call's kernels read.  Eager calls
// cycle through a ring of RING slots (a slot is rewritten RING uploads
// later).  A call being captured into a CUDA graph gets a slot of its own
// instead, which no later call rewrites: the graph's copy node reloads the
// same pinned host bytes into it on every replay, so the graph keeps
// detecting the frames it captured however many eager calls run in between.
// Captures of identical tables share a slot.
static atag_status upload_captured(atag_detector* det, const std::vector<FrameDesc>& t, cudaStream_t s,
                                   const FrameDesc** d_table) {
    const size_t n = t.size();
    size_t slot = det->captured.size();
    for (size_t k = 0; k < det->captured.size(); k++)
        if (det->captured[k].size() == n && memcmp(det->captured[k].data(), t.data(), n * sizeof(FrameDesc)) == 0)
            slot = k;
    if (slot == det->captured.size()) {
        if (slot == (size_t)CAPTURE_SLOTS)
            return fail(ATAG_ERR_CAPACITY,
                        "detect_batch: %d different frame tables are held by captured graphs; destroy those graphs "
                        "and call atag_detector_release_captures",
                        CAPTURE_SLOTS);
        memcpy(det->h_captured + slot * det->max_frames, t.data(), n * sizeof(FrameDesc));
        det->captured.push_back(t);
    }
    FrameDesc* d = det->d_captured + slot * det->max_frames;
    CK(cudaMemcpyAsync(d, det->h_captured + slot * det->max_frames, n * sizeof(FrameDesc), cudaMemcpyHostToDevice, s));
    *d_table = d;
    return ATAG_OK;
}

static atag_status upload_table(atag_detector* det, const std::vector<FrameDesc>& t, cudaStream_t s,
                                const FrameDesc** d_table) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) return upload_captured(det, t, s, d_table);
    size_t n = t.size();
    if (det->last_slot >= 0 && det->last.size() == n && memcmp(det->last.data(), t.data(), n * sizeof(FrameDesc)) == 0) {
        *d_table = det->d_tables + (size_t)det->last_slot * det->max_frames;
        return ATAG_OK;
    }
    int slot = det->ring;
    det->ring = (det->ring + 1) % RING;
    CK(cudaEventSynchronize(det->ev[slot]));  // the slot's previous upload has been consumed by its copy
    FrameDesc* h = det->h_staging + (size_t)slot * det->max_frames;
    memcpy(h, t.data(), n * sizeof(FrameDesc));
    FrameDesc* d = det->d_tables + (size_t)slot * det->max_frames;
    CK(cudaMemcpyAsync(d, h, n * sizeof(FrameDesc), cudaMemcpyHostToDevice, s));
    CK(cudaEventRecord(det->ev[slot], s));
    det->last = t;
    det->last_slot = slot;
    *d_table = d;
    return ATAG_OK;
}

// The whole path for frames [first, last) of the uploaded table, on stream
// s, with lane `lane`'s work lists and side stream.  Stage events are
// recorded when `timed`.
static atag_status launch_lane(atag_detector* det, const FrameDesc* d_table, const std::vector<FrameDesc>& t,
                               size_t first, size_t last, cudaStream_t s, int lane, bool timed) {
    const size_t n = last - first;
    size_t mw = 0, mh = 0, max_pair = 0, max_points = 0;
    bool any_decim = false;
    for (size_t i = first; i < last; i++) {
        mw = std::max<size_t>(mw, t[i].width);
        mh = std::max<size_t>(mh, t[i].height);
        max_pair = std::max<size_t>(max_pair, t[i].pair_cap);
        max_points = std::max<size_t>(max_points, t[i].point_cap);
        any_decim |= t[i].factor > 1 || t[i].src_format != ATAG_PIX_GREY8;
    }
    FrameSet fs;
    memset(&fs, 0, sizeof fs);
    fs.table = d_table + first;
    const PipelineParams& p = det->pp;
    const int sms = det->dev->num_sms;
    // batch-wide work lists of this lane: small clusters, large clusters,
    // point runs, all clusters, clusters with peaks; one queue cursor each
    uint32_t* work = det->d_work + (size_t)lane * (WORK_LISTS * (det->max_frames + 1) + WORK_LISTS);
    uint32_t* off_small = work;
    uint32_t* off_large = work + (n + 1);
    uint32_t* off_runs = work + 2 * (n + 1);
    uint32_t* off_clusters = work + 3 * (n + 1);
    uint32_t* off_peaks = work + 4 * (n + 1);
    uint32_t* wc = work + WORK_LISTS * (det->max_frames + 1);
    cudaStream_t side = det->side[lane];
    auto mark = [&](int i) -> atag_status {
        if (timed) CK(cudaEventRecord(det->stage_events[i], s));
        return ATAG_OK;
    };
#define STAGE(i) do { atag_status m_ = mark(i); if (m_) return m_; } while (0)
    const atag_tuning& tu = det->tuning;
    const int ccl_rows = tu.ccl_tile_rows == 8 || tu.ccl_tile_rows == 32 ? tu.ccl_tile_rows : 16;
    const int bp_rows = tu.boundary_tile_rows == 8 ? 8 : 16;
    const size_t tiles_ccl = cdiv(mw / 2, 32) * cdiv(mh / 2, (size_t)ccl_rows);
    STAGE(0);
    k_reset_frames<<<grid2(cdiv(max_pair, 256), n), 256, 0, s>>>(fs);
    LAUNCHED();
    STAGE(1);
    if (any_decim) {
        k_decimate<<<grid2(std::min<size_t>(cdiv(mw / 4 * mh, 256), 2048), n), 256, 0, s>>>(fs);
        LAUNCHED();
    }
    STAGE(2);
    k_threshold<<<grid2(cdiv(mw / 4, 32) * cdiv(mh / 4, 16), n), 256, 0, s>>>(fs, p.min_white_black_diff, 0);
    LAUNCHED();
    STAGE(3);
    if (ccl_rows == 8) k_ccl_local_r8<<<ccl_grid(mw, mh, 8, n), 32 * 8, 0, s>>>(fs);
    else if (ccl_rows == 32) k_ccl_local_r32<<<ccl_grid(mw, mh, 32, n), 32 * 32, 0, s>>>(fs);
    else k_ccl_local_r16<<<ccl_grid(mw, mh, 16, n), 32 * 16, 0, s>>>(fs);
    LAUNCHED();
    STAGE(4);
    {
        const size_t border = tiles_ccl * (32 + 2 * (ccl_rows - 1));
        if (ccl_rows == 8) k_ccl_border_edges_r8<<<grid2(cdiv(border, 256), n), 256, 0, s>>>(fs);
        else if (ccl_rows == 32) k_ccl_border_edges_r32<<<grid2(cdiv(border, 256), n), 256, 0, s>>>(fs);
        else k_ccl_border_edges_r16<<<grid2(cdiv(border, 256), n), 256, 0, s>>>(fs);
        LAUNCHED();
    }
    STAGE(5);
    k_ccl_final<<<final_grid(mw, mh, n), CCL_FINAL_THREADS, 0, s>>>(fs);
    LAUNCHED();
    STAGE(6);
    // grid (frames, tile columns, tile rows): at most 64 x 512 tiles of a
    // 4096 x 4096 frame
    if (bp_rows == 8)
        k_boundaries_pairs_r8<<<dim3((unsigned)n, (unsigned)cdiv(mw, 64), (unsigned)cdiv(mh, 8)), 16 * 8, 0, s>>>(fs, p.min_component_size);
    else
        k_boundaries_pairs_r16<<<dim3((unsigned)n, (unsigned)cdiv(mw, 64), (unsigned)cdiv(mh, 16)), 16 * 16, 0, s>>>(fs, p.min_component_size);
    LAUNCHED();
    STAGE(7);
    k_pairs_finalize<<<(unsigned)n, 1024, 0, s>>>(fs, p, (uint32_t)tu.small_cluster_max);
    LAUNCHED();
    {
        BatchOffsets bo{{CNT_SMALL, CNT_LARGE, CNT_RUNS, CNT_CLUSTERS},
                        {off_small, off_large, off_runs, off_clusters}, wc};
        k_batch_offsets<<<1, 1024, 0, s>>>(fs, (uint32_t)n, bo);
    }
    LAUNCHED();
    STAGE(8);
    k_scatter_points<<<grid2(std::min<size_t>(cdiv(max_points, 256), 1024), n), 256, 0, s>>>(fs);
    LAUNCHED();
    STAGE(9);
    // large clusters on the side stream, concurrently with the small ones
    CK(cudaEventRecord(det->fork[lane], s));
    CK(cudaStreamWaitEvent(side, det->fork[lane], 0));
    k_cluster_sort_large<<<std::max(1, sms / std::max(1, tu.large_ctas_divisor)), CF_LARGE_THREADS, CF_LARGE_SMEM,
                           side>>>(fs, off_large, (uint32_t)n, wc + 1);
    LAUNCHED();
    {
        // the small-cluster kernel's key buffers are sized for the tuned split
        const uint32_t cap = (uint32_t)tu.small_cluster_max;
        const uint32_t smem = cf_small_smem(cap);
        k_cluster_sort_small<<<sms * std::max(1, tu.small_ctas_per_sm), CF_SMALL_THREADS, smem, s>>>(
            fs, off_small, (uint32_t)n, wc, cap);
    }
    LAUNCHED();
    CK(cudaEventRecord(det->join[lane], side));
    CK(cudaStreamWaitEvent(s, det->join[lane], 0));
    STAGE(10);
    k_cluster_errors<<<sms * 8, 256, 0, s>>>(fs, off_runs, (uint32_t)n, wc + 2);
    LAUNCHED();
    STAGE(11);
    k_cluster_peaks<<<sms * 4, 256, 0, s>>>(fs, off_clusters, (uint32_t)n);
    LAUNCHED();
    STAGE(12);
    k_peaks_scan<<<(unsigned)n, 1024, 0, s>>>(fs, p);
    LAUNCHED();
    {
        BatchOffsets bo{{CNT_PEAKCLU, 0, 0, 0}, {off_peaks, nullptr, nullptr, nullptr}, wc + 4};
        k_batch_offsets<<<1, 1024, 0, s>>>(fs, (uint32_t)n, bo);
    }
    LAUNCHED();
    STAGE(13);
    k_index_quads<<<sms * std::max(1, tu.index_ctas_per_sm), 256, 0, s>>>(fs, off_peaks, (uint32_t)n, p);
    LAUNCHED();
    STAGE(14);
    k_compact_quads<<<(unsigned)n, 1024, 0, s>>>(fs);
    LAUNCHED();
    STAGE(15);
    if (det->refine) {
        k_refine_detected<<<dim3((unsigned)n, 64), 128, 0, s>>>(fs);
        LAUNCHED();
    }
    STAGE(16);
#undef STAGE
    return ATAG_OK;
}

atag_status atag_detect_batch(atag_detector* det, const atag_frame* frames, size_t n, atag_quad_corners* d_quads,
                              size_t quad_cap, atag_frame_stats* d_stats, atag_stream_t stream) {
    if (!det || !frames || n == 0 || !d_quads || !d_stats) return fail(ATAG_ERR_INVALID_ARGUMENT, "detect_batch: bad argument");
    if (n > det->max_frames) return fail(ATAG_ERR_INVALID_ARGUMENT, "detect_batch: %zu frames > max %zu", n, det->max_frames);
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t f = (uint32_t)det->cfg.decimate;
    std::vector<FrameDesc> t(n);
    size_t off = 0, total_px = 0;
    for (size_t i = 0; i < n; i++) {
        const atag_frame& fr = frames[i];
        if (!fr.d_grey) return fail(ATAG_ERR_INVALID_ARGUMENT, "detect_batch: frame %zu has no image", i);
        const uint32_t bpp = pixel_bytes(fr.format);
        if (bpp == 0) return fail(ATAG_ERR_INVALID_ARGUMENT, "detect_batch: frame %zu has unknown pixel format %u", i, fr.format);
        const size_t pitch = fr.src_pitch ? fr.src_pitch : (size_t)fr.src_width * bpp;
        if (pitch < (size_t)fr.src_width * bpp)
            return fail(ATAG_ERR_INVALID_ARGUMENT, "detect_batch: frame %zu has a row pitch below its width", i);
        size_t w = fr.src_width / f, h = fr.src_height / f;
        if (!valid_dims(w, h) || w > det->max_w || h > det->max_h)
            return fail(ATAG_ERR_INVALID_ARGUMENT, "detect_batch: frame %zu is %ux%u; after decimation by %u it must be a multiple of 4 within %zux%zu",
                        i, fr.src_width, fr.src_height, f, det->max_w, det->max_h);
        total_px += w * h;
        if (total_px > det->max_total_pixels) return fail(ATAG_ERR_INVALID_ARGUMENT, "detect_batch: batch exceeds %zu pixels", det->max_total_pixels);
        const bool convert = f > 1 || fr.format != ATAG_PIX_GREY8;
        size_t bytes = layout_frame(det->frames_base + off, (uint32_t)w, (uint32_t)h, f, convert, &t[i]);
        off += bytes;
        if (off > det->frames_bytes) return fail(ATAG_ERR_OUT_OF_MEMORY, "detect_batch: workspace too small");
        FrameDesc& d = t[i];
        d.src = fr.d_grey;
        d.src_stride = (uint32_t)pitch;
        d.src_format = fr.format;
        if (!convert) d.grey = const_cast<uint8_t*>(fr.d_grey);
        d.quads = d_quads + i * quad_cap;
        d.quad_cap = (uint32_t)quad_cap;
        d.stats = d_stats + i;
        d.stage_outputs = det->keep_intermediates ? 1u : 0u;
        apply_limits(det->limits, &d);
    }
    const FrameDesc* d_table;
    atag_status st = upload_table(det, t, s, &d_table);
    if (st) return st;
    det->cur = t;
    // Lanes: the batch is split into up to MAX_LANES parts of about equal
    // pixel count that run the whole path concurrently on their own streams
    // (branches of one graph when captured), so each part's serial kernels
    // and tails overlap the other parts' work.  Stage timing needs one
    // stream, so it runs one lane.
    const bool timed = det->stage_events.size() == ATAG_STAGE_COUNT + 1;
    const int lanes = timed ? 1 : (int)std::min<size_t>((size_t)std::min(det->tuning.batch_lanes, MAX_LANES), n);
    if (lanes == 1) return launch_lane(det, d_table, t, 0, n, s, 0, timed);
    size_t cut[MAX_LANES + 1];
    cut[0] = 0;
    cut[lanes] = n;
    {
        size_t acc = 0, i = 0;
        for (int k = 1; k < lanes; k++) {
            // first frame index whose prefix reaches k/lanes of the pixels,
            // leaving at least one frame for each later lane
            while (i < n && acc * lanes < total_px * (size_t)k) {
                acc += (size_t)t[i].width * t[i].height;
                i++;
            }
            cut[k] = std::min(std::max(i, cut[k - 1] + 1), n - (size_t)(lanes - k));
            i = cut[k];
            acc = 0;
            for (size_t j = 0; j < i; j++) acc += (size_t)t[j].width * t[j].height;
        }
    }
    CK(cudaEventRecord(det->lane_fork, s));
    for (int k = 1; k < lanes; k++) CK(cudaStreamWaitEvent(det->lane_stream[k], det->lane_fork, 0));
    for (int k = 0; k < lanes; k++) {
        st = launch_lane(det, d_table, t, cut[k], cut[k + 1], k ? det->lane_stream[k] : s, k, false);
        if (st) return st;
    }
    for (int k = 1; k < lanes; k++) {
        CK(cudaEventRecord(det->lane_join[k], det->lane_stream[k]));
        CK(cudaStreamWaitEvent(s, det->lane_join[k], 0));
    }
    return ATAG_OK;
}

atag_status atag_detect(atag_detector* det, const uint8_t* d_grey, size_t sw, size_t sh, atag_quad_corners* d_quads,
                        size_t quad_cap, atag_frame_stats* d_stats, atag_stream_t stream) {
    atag_frame fr{d_grey, (uint32_t)sw, (uint32_t)sh};
    return atag_detect_batch(det, &fr, 1, d_quads, quad_cap, d_stats, stream);
}

atag_status atag_detect_host(atag_detector* det, const uint8_t* h_grey, size_t sw, size_t sh, atag_quad_corners* h_quads,
                             size_t quad_cap, atag_frame_stats* h_stats, atag_stream_t stream) {
    if (!det || !h_grey || !h_stats || (quad_cap && !h_quads)) return fail(ATAG_ERR_INVALID_ARGUMENT, "detect_host: bad argument");
    if (sw * sh > det->input_bytes) return fail(ATAG_ERR_INVALID_ARGUMENT, "detect_host: frame larger than the detector's input region");
    cudaStream_t s = (cudaStream_t)stream;
    size_t cap = std::min(quad_cap, det->hquad_cap);
    CK(cudaMemcpyAsync(det->d_input, h_grey, sw * sh, cudaMemcpyHostToDevice, s));
    atag_status st = atag_detect(det, det->d_input, sw, sh, det->d_hquads, det->hquad_cap, det->d_hstats, stream);
    if (st) return st;
    CK(cudaMemcpyAsync(h_stats, det->d_hstats, sizeof(atag_frame_stats), cudaMemcpyDeviceToHost, s));
    if (cap) CK(cudaMemcpyAsync(h_quads, det->d_hquads, sizeof(atag_quad_corners) * cap, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return ATAG_OK;
}

atag_status atag_detector_views(const atag_detector* det, size_t frame, atag_frame_views* out) {
    if (!det || !out || frame >= det->cur.size()) return fail(ATAG_ERR_INVALID_ARGUMENT, "detector_views: bad frame");
    const FrameDesc& d = det->cur[frame];
    memset(out, 0, sizeof *out);
    out->decimated = d.grey;
    out->thresholded = d.thr;
    out->labels = d.labels;
    out->sizes = d.sizes;
    out->pair_points = (const uint64_t*)d.points;
    uint32_t n_list = 0;
    if (cudaMemcpy(&n_list, d.counters + CNT_POINTS, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(ATAG_ERR_CUDA, "detector_views: reading the point count failed");
    out->n_pair_points = n_list < d.point_cap ? n_list : d.point_cap;
    out->pair_capacity = d.pair_cap;
    out->pair_keys = (const uint64_t*)d.pair_keys;
    out->pair_count = d.pair_count;
    out->pair_bbox = (const uint32_t*)d.pair_bbox;
    out->pair_gsum = (const int32_t*)d.pair_gsum;
    out->pair_pxgx = (const int64_t*)d.pair_pxgx;
    out->cluster_keys = (const uint64_t*)d.cluster_keys;
    out->cluster_bounds = d.cluster_bounds;
    out->cluster_extents = d.cluster_extents;
    out->cluster_points = d.cluster_points;
    out->line_fit_points = d.line_fit;
    out->peak_count = d.peak_count;
    out->peaks = d.peaks;
    out->peak_clusters = d.peak_clusters;
    out->peak_extents = d.peak_extents;
    out->fitted = d.fitted;
    out->point_capacity = d.point_cap;
    out->cluster_capacity = d.cluster_cap;
    out->cluster_point_capacity = d.cpoint_cap;
    return ATAG_OK;
}

atag_status atag_detector_set_refinement(atag_detector* det, int enable) {
    if (!det) return fail(ATAG_ERR_INVALID_ARGUMENT, "set_refinement: null detector");
    det->refine = enable != 0;
    return ATAG_OK;
}

atag_status atag_detector_release_captures(atag_detector* det) {
    if (!det) return fail(ATAG_ERR_INVALID_ARGUMENT, "release_captures: null detector");
    det->captured.clear();
    return ATAG_OK;
}

atag_status atag_detector_set_limits(atag_detector* det, const atag_limits* limits) {
    if (!det || !limits) return fail(ATAG_ERR_INVALID_ARGUMENT, "set_limits: null argument");
    det->limits = *limits;
    return ATAG_OK;
}

atag_status atag_detector_set_stage_events(atag_detector* det, void* const* events, size_t n) {
    if (!det) return fail(ATAG_ERR_INVALID_ARGUMENT, "set_stage_events: null detector");
    det->stage_events.clear();
    if (!events || n == 0) return ATAG_OK;
    if (n != ATAG_STAGE_COUNT + 1)
        return fail(ATAG_ERR_INVALID_ARGUMENT, "set_stage_events: need %d events, got %zu", ATAG_STAGE_COUNT + 1, n);
    for (size_t i = 0; i < n; i++) det->stage_events.push_back((cudaEvent_t)events[i]);
    return ATAG_OK;
}

atag_status atag_detector_keep_intermediates(atag_detector* det, int keep) {
    if (!det) return fail(ATAG_ERR_INVALID_ARGUMENT, "keep_intermediates: null detector");
    det->keep_intermediates = keep != 0;
    return ATAG_OK;
}

atag_status atag_detector_get_tuning(const atag_detector* det, atag_tuning* out) {
    if (!det || !out) return fail(ATAG_ERR_INVALID_ARGUMENT, "get_tuning: null argument");
    *out = det->tuning;
    return ATAG_OK;
}

atag_status atag_detector_set_tuning(atag_detector* det, const atag_tuning* t) {
    if (!det || !t) return fail(ATAG_ERR_INVALID_ARGUMENT, "set_tuning: null argument");
    if ((t->ccl_tile_rows != 8 && t->ccl_tile_rows != 16 && t->ccl_tile_rows != 32) ||
        (t->boundary_tile_rows != 8 && t->boundary_tile_rows != 16))
        return fail(ATAG_ERR_INVALID_ARGUMENT, "set_tuning: CCL tile rows must be 8, 16 or 32, boundary tile rows 8 or 16");
    if (t->small_cluster_max < 1 || t->small_cluster_max > (int32_t)CF_SMALL_CAP)
        return fail(ATAG_ERR_INVALID_ARGUMENT, "set_tuning: small_cluster_max must be in [1, %u]", CF_SMALL_CAP);
    if (t->small_ctas_per_sm < 1 || t->small_ctas_per_sm > 16 || t->large_ctas_divisor < 1 ||
        t->large_ctas_divisor > 64 || t->index_ctas_per_sm < 1 || t->index_ctas_per_sm > 64)
        return fail(ATAG_ERR_INVALID_ARGUMENT, "set_tuning: CTA counts out of range");
    if (t->batch_lanes < 1 || t->batch_lanes > MAX_LANES)
        return fail(ATAG_ERR_INVALID_ARGUMENT, "set_tuning: batch_lanes must be in [1, %d]", MAX_LANES);
    det->tuning = *t;
    return ATAG_OK;
}

const char* atag_stage_name(int i) {
    static const char* names[ATAG_STAGE_COUNT] = {
        "reset", "decimate", "threshold", "ccl_local", "ccl_border", "ccl_final", "boundaries_pairs",
        "pairs_finalize", "scatter_points", "cluster_sort", "cluster_errors", "cluster_peaks", "peaks_scan",
        "index_quads", "compact_quads", "refine"};
    return (i >= 0 && i < ATAG_STAGE_COUNT) ? names[i] : nullptr;
}

atag_status atag_use_device(int ordinal) {
    cudaError_t e = cudaSetDevice(ordinal);
    if (e != cudaSuccess) return fail(ATAG_ERR_NO_DEVICE, "cudaSetDevice(%d): %s", ordinal, cudaGetErrorString(e));
    DeviceInfo* d;
    return ensure_device(&d);
}

}  // extern "C"
