// Colour removal as the reference does it when it loads an image: an image of
// 1-4 channels is encoded as PNG with the reference's vendored
// stb_image_write.h and decoded to one channel with its stb_image.h
// (stbi_load_from_memory(..., STBI_grey), the call of src/main.cpp:264-265),
// so the conversion is stb's own (stbi__compute_y, include/stb_image.h:1834).
// Test infrastructure only: produces golden vectors for the oracle's and the
// CUDA path's colour conversion.
//
// usage: stb_grey in.raw width height channels out.raw
#define STB_IMAGE_IMPLEMENTATION
#define STB_IMAGE_WRITE_IMPLEMENTATION
#include "stb_image.h"
#include "stb_image_write.h"

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s in.raw width height channels out.raw\n", argv[0]);
        return 2;
    }
    const int w = std::atoi(argv[2]), h = std::atoi(argv[3]), c = std::atoi(argv[4]);
    std::vector<unsigned char> in((size_t)w * h * c);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(in.data(), 1, in.size(), f) != in.size()) return 3;
    std::fclose(f);
    int len = 0;
    unsigned char* png = stbi_write_png_to_mem(in.data(), w * c, w, h, c, &len);
    if (!png) return 4;
    int ow = 0, oh = 0, oc = 0;
    unsigned char* grey = stbi_load_from_memory(png, len, &ow, &oh, &oc, STBI_grey);
    if (!grey || ow != w || oh != h) return 5;
    FILE* o = std::fopen(argv[5], "wb");
    if (!o) return 6;
    std::fwrite(grey, 1, (size_t)w * h, o);
    std::fclose(o);
    stbi_image_free(grey);
    STBIW_FREE(png);
    return 0;
}
