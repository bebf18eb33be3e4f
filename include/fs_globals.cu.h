/* Device globals of the file system (the reference keeps a dozen g_* pointers,
 * libgpufs/fs_globals.cu.h:33-54; here one pointer reaches the session). */
#ifndef fs_globals_cu_h
#define fs_globals_cu_h
#include <assert.h>
#include "gfs_types.h"
extern __device__ gfs_state* g_gfs;
#endif
