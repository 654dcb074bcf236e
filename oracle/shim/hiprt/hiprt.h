/* Clean-room stand-in. Test infrastructure. */
#ifndef GBPT_SHIM_HIPRT_H
#define GBPT_SHIM_HIPRT_H
#include <hiprt/hiprt_types.h>
#endif
