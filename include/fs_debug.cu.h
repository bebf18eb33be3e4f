/*
 * Statistics and tracing macros of the reference (libgpufs/fs_debug.cu.h).
 * The reference compiles them to nothing unless MALLOC_STATS / TIMING_STATS
 * are defined; here they are always empty and the counters live in the
 * session instead (gfs_get_stats in gpufs_gb300.h).
 */
#ifndef FS_DEBUG_CU_H
#define FS_DEBUG_CU_H

#define DEBUG_NOINLINE __noinline__
#define GPRINT(...)

#define PRINT_MALLOC
#define PRINT_FREE
#define PRINT_PAGE_ALLOC_RETRIES
#define PRINT_LOCKLESS_SUCCESS
#define PRINT_LOCKED_TRIES
#define PRINT_WRONG_FILE_ID
#define PRINT_RT_MALLOC
#define PRINT_RT_FREE
#define PRINT_HT_MISS
#define PRINT_HT_HIT
#define PRINT_PRECLOSE_PUSH
#define PRINT_PRECLOSE_FETCH
#define PRINT_FLUSHED_READ
#define PRINT_FLUSHED_WRITE
#define PRINT_TRY_LOCK_FAILED
#define PRINT_KILL_BUFFER_CACHE
#define PRINT_HM_LOCKLESS
#define PRINT_HM_LOCKED
#define PRINT_DEBUG
#define PRINT_TIMES(...)
#define PRINT_TRACE(...)

#define INIT_ALL_STATS
#define INIT_TIMING_STATS
#define INIT_DEBUG

#define KERNEL_START
#define KERNEL_STOP
#define PAGE_SEARCH_START
#define PAGE_SEARCH_STOP
#define MAP_START
#define MAP_STOP
#define COPY_BLOCK_START
#define COPY_BLOCK_STOP
#define FILE_OPEN_START
#define FILE_OPEN_STOP
#define FILE_CLOSE_START
#define FILE_CLOSE_STOP

#endif
