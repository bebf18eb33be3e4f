/*
 * run_gpufs_handler of the reference (libgpufs/host_loop.h:559-656).  The
 * session's host workers already serve the kernel; this waits until the
 * kernel stream is idle and reports device-side errors.
 */
#ifndef HOST_LOOP_CPP
#define HOST_LOOP_CPP

/* system headers the reference's host_loop.h brings in, which the samples
 * use without including them (stat, open, pthreads, iostream) */
#include <assert.h>
#include <fcntl.h>
#include <pthread.h>
#include <stdio.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>
#include <iomanip>
#include <iostream>

#include "fs_initializer.cu.h"

static inline void run_gpufs_handler(volatile GPUGlobals* gpuGlobals, int gpuid) {
    gfs_ctx* ctx = gpuGlobals->ctx;
    int e = gfs_run_handler(ctx, gpuid);
    if (e) fprintf(stderr, "gpufs: kernel stream error %d\n", e);
    unsigned int bits = gfs_last_error(ctx, 1);
    if (bits) fprintf(stderr, "gpufs: device error bits 0x%x\n", bits);
}

#endif
