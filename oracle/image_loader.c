/*
 * image_loader.c -- TEST INFRASTRUCTURE ONLY (part of libpadenti_oracle.so).
 *
 * CPU restatement of the colour-to-class step of the reference's label loader
 * (_rgb2label, src/padenti/cv_image_loader_impl.hpp:233-266), the checker for
 * pd_rgb_to_labels: per pixel, the first class whose colour equals the
 * pixel's first three bytes gives label class+1; no match gives 0.  Pixels are
 * `channels` bytes (3 or 4) in R, G, B(, A) order (the reference converts
 * OpenCV's BGR(A) to RGB(A) before this step).  Parity unpinned: the reference
 * function takes OpenCV matrices and OpenCV is absent.
 */
#include <stdint.h>

#include "padenti_oracle.h"

void or_rgb_to_labels(const uint8_t *src, uint64_t n_pix, uint32_t channels, const uint8_t *map, uint32_t n_classes,
                      uint8_t *dst) {
  for (uint64_t p = 0; p < n_pix; p++) {
    const uint8_t *q = src + p * channels;
    uint32_t l = 0;
    for (; l < n_classes; l++)
      if (q[0] == map[3 * l] && q[1] == map[3 * l + 1] && q[2] == map[3 * l + 2]) break;
    dst[p] = l < n_classes ? (uint8_t)(l + 1) : 0;
  }
}
