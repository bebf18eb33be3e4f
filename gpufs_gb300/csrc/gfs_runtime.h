/* Internal host-side declarations shared by the runtime and the workload
 * entry points; the public C ABI is include/gpufs_gb300.h. */
#ifndef GFS_RUNTIME_H
#define GFS_RUNTIME_H
#include <stddef.h>
#include "gpufs_gb300.h"
#include "gfs_types.h"
#ifdef __cplusplus
extern "C" {
#endif
void* gfs__scratch(gfs_ctx* c, size_t bytes);
int gfs__activate(gfs_ctx* c);
/* the session's bound on device-side waits (ns) */
unsigned long long gfs__timeout_ns(gfs_ctx* c);
void gfs__preload_kernels(void);
void gfs__preload_runtime(void);
void gfs__preload_workloads(void);
void gfs__preload_grep(void);
void gfs__preload_apps(void);
const gfs_state* gfs__host_state(gfs_ctx* c);
double _timestamp(void);
#ifdef __cplusplus
}
#endif
#endif
