// The crop of the reference's ROI loaders (CVImageROILoader,
// CVRGBLabelsROILoader; _extractROI at cv_image_loader_impl.hpp:268-289): of the
// outer contours of the pixels whose value is > 0 (the reference's mask img > 0,
// a numeric comparison in the image's element type), the one whose bounding
// rectangle has the largest area gives the crop.  The outer contours are those of the
// 8-connected components of the nonzero pixels (a component inside another's
// hole has a smaller rectangle and never wins), so the rectangle is found here
// by union-find over the components.  As OpenCV 2's contour tracing does, the
// one-pixel image border counts as zero.  Ties go to the component met first in
// raster order (OpenCV's own contour order is not reproduced).
#include <cstdint>
#include <cstring>
#include <vector>

#include "padenti_gb300.h"

namespace pd {
int set_error(int code, const char *fmt, ...);
}

namespace {

uint32_t find(std::vector<uint32_t> &p, uint32_t a) {
  while (p[a] != a) {
    p[a] = p[p[a]];
    a = p[a];
  }
  return a;
}

void unite(std::vector<uint32_t> &p, uint32_t a, uint32_t b) {
  a = find(p, a);
  b = find(p, b);
  if (a == b) return;
  if (a < b) p[b] = a;  // the root is the component's first pixel in raster order
  else p[a] = b;
}

}  // namespace

// Whether element i of the image is > 0 in its own type (a negative value or a
// negative zero is background).
static bool positive(const void *px, int img_type, uint64_t i) {
  switch (img_type) {
    case PD_IMG_U8: return static_cast<const uint8_t *>(px)[i] > 0;
    case PD_IMG_U16: return static_cast<const uint16_t *>(px)[i] > 0;
    case PD_IMG_I16: return static_cast<const int16_t *>(px)[i] > 0;
    case PD_IMG_I32: return static_cast<const int32_t *>(px)[i] > 0;
    default: return static_cast<const float *>(px)[i] > 0.0f;
  }
}

extern "C" int pd_image_roi(const void *image, uint32_t width, uint32_t height, int32_t img_type,
                            uint32_t channels, uint32_t roi[4]) {
  if (!image || !roi) return pd::set_error(PD_ERR_INVALID, "null argument");
  if (width == 0 || height == 0 || channels == 0) return pd::set_error(PD_ERR_INVALID, "empty image");
  if (img_type < PD_IMG_U8 || img_type > PD_IMG_F32)
    return pd::set_error(PD_ERR_INVALID, "unknown image element type %d", img_type);
  const uint64_t n = (uint64_t)width * height;
  if (n >= (1ull << 32) - 1) return pd::set_error(PD_ERR_UNSUPPORTED, "image of %llu pixels", (unsigned long long)n);
  const uint32_t none = 0xFFFFFFFFu;
  auto on = [&](uint32_t x, uint32_t y) {
    if (x == 0 || y == 0 || x + 1 >= width || y + 1 >= height) return false;  // the zero border
    const uint64_t e = ((uint64_t)y * width + x) * channels;
    for (uint32_t c = 0; c < channels; c++)
      if (positive(image, img_type, e + c)) return true;
    return false;
  };
  std::vector<uint32_t> parent(n, none);
  for (uint32_t y = 0; y < height; y++)
    for (uint32_t x = 0; x < width; x++) {
      if (!on(x, y)) continue;
      const uint32_t i = y * width + x;
      parent[i] = i;
      // the neighbours already visited: west, north-west, north, north-east
      if (parent[i - 1] != none) unite(parent, i, i - 1);
      const uint32_t up = i - width;
      if (parent[up - 1] != none) unite(parent, i, up - 1);
      if (parent[up] != none) unite(parent, i, up);
      if (parent[up + 1] != none) unite(parent, i, up + 1);
    }
  struct Box {
    uint32_t x0, y0, x1, y1;
  };
  std::vector<Box> box(n);
  std::vector<uint32_t> roots;
  for (uint32_t y = 0; y < height; y++)
    for (uint32_t x = 0; x < width; x++) {
      const uint32_t i = y * width + x;
      if (parent[i] == none) continue;
      const uint32_t r = find(parent, i);
      if (r == i) {
        box[r] = Box{x, y, x, y};
        roots.push_back(r);
      } else {
        Box &b = box[r];
        if (x < b.x0) b.x0 = x;
        if (x > b.x1) b.x1 = x;
        if (y > b.y1) b.y1 = y;
      }
    }
  if (roots.empty()) return pd::set_error(PD_ERR_INVALID, "no pixel > 0 inside the image border");
  uint64_t best_area = 0;
  Box best{};
  for (uint32_t r : roots) {  // raster order of the components' first pixels
    const Box &b = box[r];
    const uint64_t area = (uint64_t)(b.x1 - b.x0 + 1) * (b.y1 - b.y0 + 1);
    if (area > best_area) {
      best_area = area;
      best = b;
    }
  }
  roi[0] = best.x0;
  roi[1] = best.y0;
  roi[2] = best.x1 - best.x0 + 1;
  roi[3] = best.y1 - best.y0 + 1;
  return PD_OK;
}
