/* Internal host-side declarations shared by the runtime and the workload
 * entry points; the public C ABI is include/gpufs_gb300.h. */
#ifndef GFS_RUNTIME_H
#define GFS_RUNTIME_H
#include <stddef.h>
#include <cuda_runtime.h>
#include "gpufs_gb300.h"
#include "gfs_types.h"
#ifdef __cplusplus
extern "C" {
#endif
void* gfs__scratch(gfs_ctx* c, size_t bytes);
/* pinned host buffer of at least `bytes` (grown on demand, session-owned;
 * callers on one session must not overlap) */
void* gfs__host_bounce(gfs_ctx* c, size_t bytes);
/* device memory from the session's stream-ordered pool (cudaMalloc when
 * the pool is unavailable), usable on stream s and after; freed on stream s */
void* gfs__dev_alloc(gfs_ctx* c, size_t bytes, cudaStream_t s);
/* kernels of the session's device may address pageable host memory
 * (cudaDevAttrPageableMemoryAccess: host page tables, as on Grace) */
int gfs__pageable_access(gfs_ctx* c);
void gfs__dev_free(gfs_ctx* c, void* p, cudaStream_t s);
/* the registered host mapping of an open file slot, as a device address and
 * its length (0 when the slot has none); valid while the slot stays open */
int gfs__slot_map(gfs_ctx* c, uint32_t slot, unsigned long long* dev_addr, unsigned long long* len);
/* the same mapping's host address (1), or 0 when the slot has none */
int gfs__slot_map_host(gfs_ctx* c, uint32_t slot, const uint8_t** base, unsigned long long* len);
/* pread through an open slot's host fd (reopened by name if it was closed
 * past the open-file limit); bytes read or -errno */
long long gfs__slot_pread(gfs_ctx* c, uint32_t slot, void* buf, size_t n, uint64_t off);
/* where the bytes that the reference's grep chunk walk reads twice start in
 * a file held in memory (its size when there are none): the host walk the
 * grep plans run over each file, callable on its own */
uint64_t gfs__grep_tail_start(const uint8_t* bytes, uint64_t size);
int gfs__activate(gfs_ctx* c);
/* register a file's host mapping from the calling thread before a kernel
 * opens it read-only (the open then makes no CUDA call on a host worker) */
void gfs__premap(gfs_ctx* c, const char* path);
/* the session's bound on device-side waits (ns) */
unsigned long long gfs__timeout_ns(gfs_ctx* c);
/* the session's GFS_CFG_* flags and CUDA device */
uint32_t gfs__config_flags(gfs_ctx* c);
int gfs__device(gfs_ctx* c);
void gfs__preload_kernels(void);
void gfs__preload_runtime(void);
void gfs__preload_workloads(void);
void gfs__preload_grep(void);
void gfs__preload_apps(void);
void gfs__preload_bigmatrix(void);
const gfs_state* gfs__host_state(gfs_ctx* c);
double _timestamp(void);
#ifdef __cplusplus
}
#endif
#endif
