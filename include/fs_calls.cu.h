/*
 * Kernel-callable file API: the names, signatures and calling convention of
 * the reference (libgpufs/fs_calls.cu.h:34-65).  Calls are collective over
 * the thread block (the _warp forms over the warp); single_thread_* are
 * per-thread.  Link with libgpufs.a using relocatable device code
 * (nvcc -rdc=true), as with the reference.
 *
 * gvmmap/FatPointer/TLB (libgpufs/fat_pointer.cu.h) are in fat_pointer.cu.h,
 * included here as in the reference.
 */
#ifndef FS_CALLS_CU
#define FS_CALLS_CU

#include "fs_constants.h"
#include "fs_debug.cu.h"
#include "util.cu.h"
#include "timer.h"
#include "fs_globals.cu.h"
#include "fat_pointer.cu.h"

__device__ int single_thread_fsync(int fd);
__device__ int single_thread_ftruncate(int fd, int size);
__device__ int single_thread_open(const char* filename, int flags);

#define READ 0
#define WRITE 1

__device__ int gclose(int fd);
__device__ int gopen(const char* filename, int flags);
__device__ int gmsync(volatile void* addr, size_t length, int flags);
__device__ int gmunmap(volatile void* addr, size_t length);
__device__ int gmunmap_warp(volatile void* addr, size_t length, int ref = 1);
__device__ volatile void* gmmap(void* addr, size_t size, int prot, int flags, int fd, off_t offset);
__device__ volatile void* gmmap_warp(void* addr, size_t size, int prot, int flags, int fd, off_t offset, int ref = 1);
__device__ size_t gwrite(int fd, size_t offset, size_t size, uchar* buffer);
__device__ size_t gread(int fd, size_t offset, size_t size, uchar* buffer);
__device__ unsigned int gunlink(char* filename);
__device__ size_t fstat(int fd);
__device__ int gfsync(int fd);
__device__ int gftruncate(int fd, int size);

#endif
