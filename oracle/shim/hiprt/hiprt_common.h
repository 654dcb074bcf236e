/* Clean-room stand-in for HIPRT's common macros (host compilation only). Test infrastructure. */
#ifndef GBPT_SHIM_HIPRT_COMMON_H
#define GBPT_SHIM_HIPRT_COMMON_H
#include <hiprt/hiprt_vec.h>
#endif
