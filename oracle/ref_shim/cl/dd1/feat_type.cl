#ifndef __FEAT_TYPE
#define __FEAT_TYPE
typedef short feat_t;
#endif
