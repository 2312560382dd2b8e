#ifndef __IMG_TYPE
#define __IMG_TYPE
typedef image2d_t image_t;
#endif
