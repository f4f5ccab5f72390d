// noalloc.cu — image_segmentation for callers that must not allocate.
//
// Some callers cannot call cudaMalloc: a thread that is capturing a CUDA
// graph (allocation is not a stream operation and breaks the capture), a
// camera or robotics frame loop that forbids allocator calls after start-up
// because they can block and synchronise the device, or a host application
// that owns every device allocation and gives plugins none.  For them this
// entry point keeps the union-find forest of image segmentation in a
// file-scope device array instead of a caller buffer; the caller still
// passes the thresholded image in and the label and size buffers out.
//
// The array is NOALLOC_MAX_PIXELS words (8 MiB) and every GPU that loads the
// library holds it until the process exits.  All calls share it: calls that
// overlap on the GPU (on different streams, or from different host threads)
// race on it and must be serialised by the caller.  Nothing in it needs to
// start at zero: every slot is written before it is read in each call.
#include <mutex>

#include "atag_internal.h"
#include "atag_kernels.cuh"

namespace atag {

constexpr size_t NOALLOC_MAX_PIXELS = size_t(1) << 21;  // 2,097,152 pixels, e.g. 1920x1088

static __device__ __align__(256) uint32_t g_noalloc_scratch[NOALLOC_MAX_PIXELS];

namespace {
std::mutex g_noalloc_mutex;
uint32_t* g_noalloc_ptr[64] = {};

// In host code g_noalloc_scratch names a host-side stand-in, not device
// memory, so the device address is looked up once per device, with that
// device current, on the first call made on it.
atag_status noalloc_scratch(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(ATAG_ERR_NO_DEVICE, cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return set_error(ATAG_ERR_NO_DEVICE, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return set_error(ATAG_ERR_CUDA, "cudaGetSymbolAddress of the segmentation scratch failed");
        g_noalloc_ptr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return ATAG_OK;
}
}  // namespace
}  // namespace atag

using namespace atag;

extern "C" atag_status atag_image_segmentation_noalloc(const uint8_t* thr, uint32_t* labels, uint32_t* sizes,
                                                       size_t w, size_t h, atag_stream_t stream) {
    atag_status st = atag_init();
    if (st) return st;
    if (!thr || !labels || !sizes) return set_error(ATAG_ERR_INVALID_ARGUMENT, "image_segmentation_noalloc: null pointer");
    if (w < 4 || h < 4 || w % 4 || h % 4 || w > 4096 || h > 4096)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "image_segmentation_noalloc: size is not a multiple of 4 in [4, 4096]");
    if (w * h > NOALLOC_MAX_PIXELS)
        return set_error(ATAG_ERR_INVALID_ARGUMENT,
                         "image_segmentation_noalloc: frame exceeds the 2097152-pixel scratch; use atag_image_segmentation");
    uint32_t* scratch = nullptr;
    st = noalloc_scratch(&scratch);
    if (st) return st;
    FrameSet fs;
    memset(&fs, 0, sizeof fs);
    FrameDesc& d = fs.one;
    d.width = (uint32_t)w;
    d.height = (uint32_t)h;
    d.factor = 1;
    d.thr = const_cast<uint8_t*>(thr);
    d.scratch = scratch;
    d.labels = labels;
    d.sizes = sizes;
    d.stage_outputs = 1;  // the reference's sizes array, zeros away from roots
    cudaStream_t s = (cudaStream_t)stream;
    const size_t tiles = ((w / 2 + 31) / 32) * ((h / 2 + 15) / 16);
    k_ccl_local_r16<<<dim3((unsigned)((w / 2 + 31) / 32), (unsigned)((h / 2 + 15) / 16), 1), 512, 0, s>>>(fs);
    count_launch();
    k_ccl_border_r16<<<dim3((unsigned)((tiles * (32 + 2 * (16 - 1)) + 255) / 256), 1), 256, 0, s>>>(fs);
    count_launch();
    k_ccl_final<<<dim3((unsigned)((w / 4 + CCL_FINAL_THREADS - 1) / CCL_FINAL_THREADS), (unsigned)(h / 2), 1),
                  CCL_FINAL_THREADS, 0, s>>>(fs);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(ATAG_ERR_CUDA, cudaGetErrorString(e));
    return ATAG_OK;
}
