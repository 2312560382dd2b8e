/*
 * Compiles the reference's own example plugin (test/feature.cl:29-64) as C with
 * a minimal OpenCL-image shim, so the single-offset depth plugin can be checked
 * against the reference code.  read_imageui follows CLK_ADDRESS_CLAMP: outside
 * the image it returns the border colour 0.  feat_t is short, as in
 * test/test_tree_trainer.cpp.  Test infrastructure only.
 */
#include <stdbool.h>
#include <stddef.h>
#include <tgmath.h>

typedef unsigned int uint;
typedef struct { int x, y; } int2;
typedef struct { uint x, y, z, w; } uint4;
typedef struct { const unsigned short *data; uint w, h; } ref_image;
typedef const ref_image *image2d_t;
typedef int sampler_t;
#define CLK_NORMALIZED_COORDS_FALSE 0
#define CLK_ADDRESS_CLAMP 0
#define CLK_FILTER_NEAREST 0
#define __read_only
#define __global
#define __local
#define ACCESS_FEATURE(ptr, idx, size) ((ptr)[(idx)])

static uint4 read_imageui(image2d_t im, sampler_t s, int2 c) {
  (void)s;
  uint4 r = {0, 0, 0, 0};
  if (c.x >= 0 && c.y >= 0 && (uint)c.x < im->w && (uint)c.y < im->h)
    r.x = im->data[(size_t)c.y * im->w + (size_t)c.x];
  return r;
}

#include <feature.cl>

int ref_compute_feature(const unsigned short *data, uint w, uint h, int x, int y,
                        const short *feat) {
  ref_image im = {data, w, h};
  int2 c = {x, y};
  feat_t buf[2] = {feat[0], feat[1]};
  return (int)computeFeature(&im, 1, w, h, c, NULL, NULL, NULL, buf, 2);
}
