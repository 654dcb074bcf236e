/* Clean-room stand-in: the reference's host build only needs the types. Test infrastructure. */
#ifndef GBPT_SHIM_HIPRT_DEVICE_H
#define GBPT_SHIM_HIPRT_DEVICE_H
#include <hiprt/hiprt_types.h>
#endif
