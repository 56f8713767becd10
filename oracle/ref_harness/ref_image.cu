// Host-only harness around the reference's image code (test infrastructure):
// Image.h (FasterBackprojection/Image.h:45-66 bilinear interpolate, 92-138
// resize, 160-178 vertical flip) is the reference's own template, compiled
// from its tree.  TransientImage.cpp cannot be compiled here (it includes the
// OpenGL texture class), so the five lines of TransientImage::save
// (TransientImage.cpp:46-64) and normalizeImage (:66-78) that feed it are
// restated below, in the same order.  The PNG encoder is replaced by handing
// the RGBA pixels back to the caller.
#include "Image.h"

#include <cstring>

namespace {

struct HarnessImage : Image<unsigned char> {
    HarnessImage(uint16_t w, uint16_t h) : Image<unsigned char>(w, h, 4) {}
    std::vector<unsigned char>& pixels() { return _image; }
};

}  // namespace

int SOIL_save_image(const char*, int, int, int, int, const unsigned char*) { return 1; }

// TransientImage(width, height).save(-, slice, (out_w, out_h), stride, offset,
// normalize); rgba receives out_w x out_h x 4 bytes (top row first, as the
// PNG rows).  `slice` is modified in place when normalize != 0, like the
// reference.  Returns 0 on success.
extern "C" int refimg_transient_save(float* slice, uint32_t width, uint32_t height, uint32_t out_w, uint32_t out_h,
                                     uint32_t stride, uint32_t offset, int normalize, unsigned char* rgba) {
    HarnessImage img((uint16_t)width, (uint16_t)height);
    if (normalize) {
        float maxVal = .0f;
        const glm::uint size = img.getWidth() * img.getHeight();
        for (glm::uint idx = 0; idx < size; ++idx) maxVal = glm::max(maxVal, slice[idx]);
        for (glm::uint idx = 0; idx < size; ++idx) slice[idx] /= maxVal;
    }
    std::vector<unsigned char>& px = img.pixels();
    for (int idx = 0; idx < (int)(width * height); ++idx) {
        px[idx * 4 + 0] = px[idx * 4 + 1] = px[idx * 4 + 2] = static_cast<unsigned char>(
            glm::clamp(static_cast<glm::uint>(slice[offset + idx * stride] * 255.0f), 0u, 255u));
        px[idx * 4 + 3] = 255;
    }
    Image<unsigned char>::flipImageVertically(px, img.getWidth(), img.getHeight(), img.getDepth());
    if (out_w != width || out_h != height) img.resize((uint16_t)out_w, (uint16_t)out_h, Image<unsigned char>::BILINEAR);
    if (img.getWidth() != out_w || img.getHeight() != out_h) return 1;
    std::memcpy(rgba, img.bits(), (size_t)out_w * out_h * 4);
    return 0;
}
