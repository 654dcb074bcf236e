/* Clean-room stand-in: the reference's host build uses only the texture handle type
 * (src/Device/includes/Texture.h:50-197 of the reference). Test infrastructure only. */
#ifndef GBPT_SHIM_OROCHI_H
#define GBPT_SHIM_OROCHI_H
typedef unsigned long long oroTextureObject_t;
typedef void* oroStream_t;
#endif
