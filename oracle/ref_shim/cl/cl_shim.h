/*
 * OpenCL C -> C shim for compiling the reference's own kernels
 * (src/padenti/kernels/hist_update.cl, predict.cl) as C, so the oracle can be
 * checked against them on the host.  TEST INFRASTRUCTURE ONLY.
 *
 * What it provides:
 *   - the vector types the kernels use (int2, int4, uint4) as structs, with
 *     make_int2/make_int4 for the vector literals (the Makefile rewrites
 *     "(int2)(" and "(int4)(" into these calls, and the swizzle "coords.xy"
 *     into "coords", in a generated copy of each kernel);
 *   - images as {data, element type, width, height, channels} with
 *     read_imageui / read_imagei / write_imagei under CLK_ADDRESS_CLAMP
 *     semantics: an out-of-image read returns 0 in .x (the border colour);
 *     in-image reads of a one-channel image return (v, 0, 0, 1);
 *   - work-item functions reading the executor's current work-item;
 *   - barrier() (with CL_SHIM_BARRIERS): a switch back to the work-group
 *     scheduler, which runs every work-item of the group up to the barrier
 *     before any passes it (ucontext coroutines), so local-memory traffic
 *     across a barrier behaves as on a device.
 * Arithmetic is IEEE single precision with correctly rounded division
 * (-ffp-contract=off): where OpenCL allows a less accurate divide or log2,
 * the oracle fixes the IEEE result, and this shim executes the kernels under
 * the same rule.
 */
#ifndef PD_CL_SHIM_H
#define PD_CL_SHIM_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <tgmath.h>
#undef I /* <complex.h>'s imaginary unit; hist_update.cl defines its own I() */

typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef struct { int x, y; } int2;
typedef struct { int x, y, z, w; } int4;
typedef struct { uint x, y, z, w; } uint4;

/* OpenCL's integer min(), as hist_update.cl:83 uses it (int arguments). */
static inline int min(int a, int b) { return a < b ? a : b; }

static inline int2 make_int2(int x, int y) {
  int2 r = {x, y};
  return r;
}
static inline int4 make_int4(int x, int y, int z, int w) {
  int4 r = {x, y, z, w};
  return r;
}

enum { CL_SHIM_U8 = 1, CL_SHIM_U16 = 2, CL_SHIM_I32 = 3 };
typedef struct {
  void *data;
  int type;  /* CL_SHIM_* element type */
  uint w, h, ch;
} cl_shim_image;
typedef cl_shim_image *image2d_t;
typedef int sampler_t;

#define CLK_NORMALIZED_COORDS_FALSE 0
#define CLK_ADDRESS_CLAMP 0
#define CLK_FILTER_NEAREST 0
#define CLK_LOCAL_MEM_FENCE 1
#define __kernel
#define __global
#define __local
#define __read_only
#define __write_only

static inline uint cl_shim_elem(const cl_shim_image *im, size_t i) {
  switch (im->type) {
    case CL_SHIM_U8: return ((const uint8_t *)im->data)[i];
    case CL_SHIM_U16: return ((const uint16_t *)im->data)[i];
    default: return (uint)((const int32_t *)im->data)[i];
  }
}

static inline uint4 read_imageui(image2d_t im, sampler_t s, int2 c) {
  (void)s;
  uint4 r = {0, 0, 0, 0};
  if (c.x < 0 || c.y < 0 || (uint)c.x >= im->w || (uint)c.y >= im->h) return r;
  const size_t e = ((size_t)c.y * im->w + (size_t)c.x) * im->ch;
  r.x = cl_shim_elem(im, e);
  r.y = im->ch > 1 ? cl_shim_elem(im, e + 1) : 0u;
  r.z = im->ch > 2 ? cl_shim_elem(im, e + 2) : 0u;
  r.w = im->ch > 3 ? cl_shim_elem(im, e + 3) : 1u;
  return r;
}

static inline int4 read_imagei(image2d_t im, sampler_t s, int2 c) {
  uint4 u = read_imageui(im, s, c);
  int4 r = {(int)u.x, (int)u.y, (int)u.z, (int)u.w};
  return r;
}

static inline void write_imagei(image2d_t im, int2 c, int4 v) {
  if (c.x < 0 || c.y < 0 || (uint)c.x >= im->w || (uint)c.y >= im->h) return;  /* undefined on a device */
  ((int32_t *)im->data)[(size_t)c.y * im->w + (size_t)c.x] = v.x;
}

/* The executor's current work-item. */
typedef struct {
  size_t gid[2], lid[2];
} cl_shim_item;
static cl_shim_item cl_shim_wi;
static size_t cl_shim_lsize[2], cl_shim_gsize[2];
#define get_global_id(d) (cl_shim_wi.gid[(d)])
#define get_local_id(d) (cl_shim_wi.lid[(d)])
#define get_local_size(d) (cl_shim_lsize[(d)])
#define get_global_size(d) (cl_shim_gsize[(d)])

#ifdef CL_SHIM_BARRIERS
#include <ucontext.h>
static ucontext_t cl_shim_main;
static ucontext_t *cl_shim_ctx;
static size_t cl_shim_cur;
static void barrier(int flags) {
  (void)flags;
  swapcontext(&cl_shim_ctx[cl_shim_cur], &cl_shim_main);
}
#endif

#endif
