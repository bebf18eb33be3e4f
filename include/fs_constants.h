/*
 * Compile-time constants of the reference's device API
 * (libgpufs/fs_constants.h), for programs written against it.  In this
 * library page size, pool size and table sizes are run-time settings
 * (gfs_config); the initializer() in fs_initializer.cu.h passes these
 * macros to the session, so a program compiled with -DFS_LOGBLOCKSIZE=21
 * runs on 2 MiB pages.
 */
#ifndef FS_CONSTANTS
#define FS_CONSTANTS

#include <sys/mman.h>
#include <fcntl.h>

#ifndef FS_LOGBLOCKSIZE
#define FS_LOGBLOCKSIZE (12)
#endif
#define FS_BLOCKSIZE (1 << FS_LOGBLOCKSIZE)
#define FS_BLOCKMASK (FS_BLOCKSIZE - 1)

#ifndef PPOOL_SIZE
#define PPOOL_SIZE (1024 * 1024 * 1024 * 2L)
#endif
#define PPOOL_FRAMES (PPOOL_SIZE >> FS_LOGBLOCKSIZE)

#ifndef MAX_NUM_FILES
#define MAX_NUM_FILES (128)
#endif
#define FSTABLE_SIZE MAX_NUM_FILES
#define FILENAME_SIZE 64

#define E_FSTABLE_FULL -1
#define E_IPC_OPEN_ERROR -2

#define O_GRDONLY (O_RDONLY)
#define O_GWRONLY (O_WRONLY)
#define O_GCREAT (O_CREAT)
#define O_GRDWR (O_RDWR)
#define O_GWRONCE (O_GCREAT | O_GWRONLY)

#define GMAP_FAILED MAP_FAILED

#define PAGE_READ_ACCESS 0
#define PAGE_WRITE_ACCESS 1
typedef char Page[FS_BLOCKSIZE];

typedef unsigned char uchar;

#endif
