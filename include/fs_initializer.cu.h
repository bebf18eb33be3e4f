/*
 * Host session object of the reference (libgpufs/fs_initializer.cu.h:56-203)
 * over the C ABI.  initializer() creates a session whose page size, pool
 * size and table size come from the including program's FS_LOGBLOCKSIZE,
 * PPOOL_SIZE and MAX_NUM_FILES; its host workers serve requests from then
 * until the object is deleted.
 */
#ifndef FS_INITIALIZER_H
#define FS_INITIALIZER_H

#include <stdio.h>
#include <stdlib.h>
#include <cuda_runtime.h>

#include "fs_constants.h"
#include "fs_debug.cu.h"
#include "util.cu.h"
#include "timer.h"
#include "fs_globals.cu.h"
#include "gpufs_gb300.h"

struct GPUStreamManager {
    cudaStream_t kernelStream;
};

struct GPUGlobals {
    gfs_ctx* ctx;
    GPUStreamManager* streamMgr;

    GPUGlobals() {
        gfs_config c;
        gfs_default_config(&c);
        c.log_page = FS_LOGBLOCKSIZE;
        c.pool_bytes = (uint64_t)(PPOOL_SIZE);
        c.max_files = MAX_NUM_FILES;
        int dev = 0;
        cudaGetDevice(&dev);
        c.device = dev;
        if (gfs_create(&c, &ctx) != 0) {
            fprintf(stderr, "gpufs: session creation failed\n");
            exit(-1);
        }
        streamMgr = new GPUStreamManager();
        streamMgr->kernelStream = (cudaStream_t)gfs_kernel_stream(ctx);
    }
    ~GPUGlobals() {
        gfs_destroy(ctx);
        delete streamMgr;
    }
};
typedef volatile GPUGlobals* GPUGlobals_ptr;

static inline void initializer(GPUGlobals_ptr* globals) { *globals = new GPUGlobals(); }

#endif
