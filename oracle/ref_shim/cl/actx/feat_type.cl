#ifndef __FEAT_TYPE
#define __FEAT_TYPE
typedef int feat_t;
#endif
