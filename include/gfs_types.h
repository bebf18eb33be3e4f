/*
 * Layouts shared by the host runtime and the device file-system code.
 *
 * Everything here is plain C so the host C++ runtime, the CUDA device code
 * and the C-ABI header agree byte for byte.  The structures replace the
 * reference's PFrame/PPool (libgpufs/fs_structures.cu.h:24-60,
 * mallocfree.cu.h:36-54), HashMap (hashMap.cu.h:26-38), FTable
 * (fs_structures.cu.h:81-127) and the CPU_IPC_* queues (cpu_ipc.cu.h:34-123,
 * async_ipc.cu.h) with one lock-free design:
 *
 *   frames[]   one 32-byte record per HBM page frame; `st` packs the pin
 *              count, the clock reference bit, the dirty bit and the state
 *              (FREE/CLAIMED/LOADING/VALID/EVICTING/DEAD); `key` packs
 *              (file slot, file generation, page index) in one 64-bit word so
 *              a frame's identity changes atomically.
 *   index[]    set-associative page index: buckets of 16 32-bit ways, each
 *              way = (10-bit tag << 22) | frame, inserted by CAS under a
 *              per-bucket insert lock, looked up lock-free.
 *   files[]    open-file table, open-addressed by name hash; `st` packs
 *              status, slot incarnation and open count for CAS transitions.
 *   ring[]     MPMC request ring in mapped pinned host memory (Vyukov
 *              sequence protocol): device blocks produce, host workers
 *              consume; completions come back as a 32-bit word in mapped
 *              host memory (hdone), stored by the host worker once the copy
 *              that moved the data has completed.
 */
#ifndef GFS_TYPES_H
#define GFS_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GFS_NAME_MAX 64       /* FILENAME_SIZE, libgpufs/fs_constants.h:55 */
#define GFS_WAYS 16           /* page-index ways per bucket */
#define GFS_MAX_FRAMES (1u << 22)
#define GFS_NO_FRAME 0xFFFFFFFFu

/* ---- frame state word ---- */
#define GFS_F_PINS 0x000FFFFFu
#define GFS_F_REF 0x00100000u
#define GFS_F_DIRTY 0x00200000u
#define GFS_F_SHIFT 24
#define GFS_F_STMASK 0x0F000000u
#define GFS_FS_FREE 0u
#define GFS_FS_CLAIMED 1u
#define GFS_FS_LOADING 2u
#define GFS_FS_VALID 3u
#define GFS_FS_EVICTING 4u
#define GFS_FS_DEAD 5u /* a request for it timed out: never reused this session */

/* ---- file slot state word: status:4 | incarnation:8 | open count:20 ---- */
#define GFS_S_CNT 0x000FFFFFu
#define GFS_S_INC_SHIFT 20
#define GFS_S_INC_MASK 0x0FF00000u
#define GFS_S_SHIFT 28
#define GFS_SS_EMPTY 0u
#define GFS_SS_CLAIMING 1u
#define GFS_SS_CLOSED 2u
#define GFS_SS_OPENING 3u
#define GFS_SS_OPEN 4u
#define GFS_SS_CLOSING 5u
#define GFS_SS_BROKEN 6u

/* ---- request ops ---- */
#define GFS_OP_OPEN 1
#define GFS_OP_CLOSE 2
#define GFS_OP_READ 3
#define GFS_OP_WRITE 4
#define GFS_OP_TRUNC 5
#define GFS_OP_UNLINK 6
#define GFS_RF_DIFF 1 /* OR-merge with the bytes already in the file (RW_IPC_DIFF) */
#define GFS_RF_STAGED 2 /* WRITE: the bytes are already in write-stage slot `dev_addr` (host memory) */

/* completion word: 0 pending, 1+result on success, GFS_DONE_ERR|errno */
#define GFS_DONE_ERR 0x80000000u

/* device-side error codes (returned negated by the device API) */
#define GFS_OK 0
#define GFS_ENOENT 2
#define GFS_EIO 5
#define GFS_E2BIG 7
#define GFS_EBADF 9
#define GFS_EAGAIN 11
#define GFS_ENOMEM 12
#define GFS_EINVAL 22
#define GFS_EMFILE 24
#define GFS_ENOSPC 28
#define GFS_ETIMEDOUT 110

/* sticky error bits in gfs_state.error */
#define GFS_ERRB_TIMEOUT 1u
#define GFS_ERRB_IO 2u
#define GFS_ERRB_NOMEM 4u
#define GFS_ERRB_TABLE 8u
#define GFS_ERRB_ARG 16u

typedef struct gfs_frame {
    uint32_t st;      /* pins | REF | DIRTY | state<<24 */
    uint32_t content; /* valid bytes in the frame */
    uint64_t key;     /* file:20 << 44 | gen:12 << 32 | page index:32 */
    uint32_t pad2;
    uint32_t pad0;
    uint64_t pad1;
} gfs_frame;

/* host reply to an OPEN, written into mapped host memory per file slot */
typedef struct gfs_open_reply {
    int32_t host_fd;
    int32_t err;
    uint64_t size;
    int64_t ctime_ns;
    uint64_t map_dev; /* device address of the file's registered host mapping (read-only opens), 0 if none */
} gfs_open_reply;

typedef struct gfs_file {
    uint32_t st;      /* status:4 | incarnation:8 | open count:20 */
    uint32_t gen;     /* page-key generation (12 bits used) */
    int32_t flags;    /* O_G* flags of the current open */
    uint32_t pad3;
    /* -- written by the host reply (gfs_open_reply layout) -- */
    int32_t host_fd;
    int32_t err;
    uint64_t size;    /* file size; grows with writes (atomicMax) */
    int64_t ctime_ns;
    /* -- */
    uint64_t hash;    /* name hash */
    uint64_t cached_ctime; /* ctime the cached pages belong to */
    uint64_t cached_size;
    uint32_t lock;
    uint32_t pad;
    uint64_t map_dev; /* from the reply: the registered host mapping, 0 if none */
    char name[GFS_NAME_MAX];
} gfs_file;

typedef struct gfs_req {
    uint32_t seq; /* ring sequence */
    uint16_t op;
    uint16_t rflags;
    int32_t host_fd;
    uint32_t file;
    uint64_t offset;
    uint64_t length;
    uint64_t dev_addr;  /* data frame, or reply destination */
    uint64_t done_addr; /* completion word (mapped host memory, device address) */
    int32_t oflags;
    uint32_t pad[5];
    char name[GFS_NAME_MAX];
} gfs_req; /* 136 bytes */

typedef struct gfs_stats {
    unsigned long long hits;
    unsigned long long misses;
    unsigned long long evictions;
    unsigned long long writebacks;
    unsigned long long read_rpcs;
    unsigned long long bytes_read_rpc;
    unsigned long long opens;
    unsigned long long closes;
    unsigned long long timeouts;
    unsigned long long errors;
    unsigned long long conflict_evictions;
    unsigned long long err_site; /* first error: site << 16 | errno */
    unsigned long long rpc_submitted;
    unsigned long long pad[3];
} gfs_stats;

typedef struct gfs_state {
    /* configuration */
    uint32_t log_page;
    uint32_t page_size;
    uint32_t n_frames;
    uint32_t n_buckets;   /* power of two */
    uint32_t n_files;     /* power of two */
    uint32_t ring_slots;  /* power of two */
    uint64_t timeout_ns;  /* bound on every device-side wait */
    /* device memory */
    uint8_t* pool;
    gfs_frame* frames;
    uint32_t* index;      /* n_buckets * GFS_WAYS */
    uint32_t* bucket_lock;
    gfs_file* files;
    uint32_t* dirty_bits; /* one bit per frame */
    /* mapped pinned host memory (device view) */
    gfs_req* ring;
    uint32_t* hdone;          /* completion words: [0, n_frames) frames, then files */
    gfs_open_reply* hreply;   /* open replies, one per file slot */
    /* counters */
    uint32_t ring_tail;
    uint32_t clock_hand;
    uint32_t table_lock;
    uint32_t error;       /* sticky GFS_ERRB_* */
    gfs_stats stats;
    /* write-back staging: wstage_slots pages of mapped pinned host memory
     * (device view); a dirty frame's bytes are stored there by the SMs and
     * the host only merges and writes them (no device-to-host copy) */
    uint8_t* wstage;
    uint32_t* wstage_bits;          /* device memory: one bit per slot, set while in use */
    uint32_t wstage_slots;          /* 0 when pages are too large to stage */
    uint32_t wstage_pad;
} gfs_state;

#ifdef __cplusplus
}
static_assert(sizeof(gfs_req) == 136, "gfs_req layout");
static_assert(sizeof(gfs_frame) == 32, "gfs_frame layout");
static_assert(sizeof(gfs_open_reply) == 32, "gfs_open_reply layout");
#endif
#endif
