/*
 * gpufs_gb300 -- C ABI of the GB300 GPU file system.
 *
 * Plain C: pointers, sizes and integers only.  A host program (or an FFI
 * such as Python ctypes) binds these symbols from libgpufs_gb300.so.  Each
 * entry point names the reference interface it replaces (paths relative to
 * the GPUfs source tree).
 *
 * Device memory arguments are raw device addresses (void*); host memory
 * arguments are ordinary host pointers.  Functions return 0 / a non-negative
 * count on success and a negative errno-style code on failure.  Every call
 * that runs a kernel waits for it before returning.  One session may be
 * live per process at a time (the device API reaches it through one
 * __device__ global, as the reference's g_* globals do).
 */
#ifndef GPUFS_GB300_H
#define GPUFS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gfs_ctx gfs_ctx;

/* Session configuration.  Compile-time constants of the reference
 * (libgpufs/fs_constants.h:26-77) become run-time fields here. */
typedef struct gfs_config {
    uint32_t log_page;      /* page = 1 << log_page bytes, 12..21 (FS_LOGBLOCKSIZE) */
    uint32_t max_files;     /* open-file table slots, rounded up to 2^k (MAX_NUM_FILES) */
    uint64_t pool_bytes;    /* HBM buffer cache (PPOOL_SIZE) */
    uint32_t ring_slots;    /* host request ring slots, 2^k (RW_IPC_SIZE) */
    uint32_t host_workers;  /* host I/O threads (RW_HOST_WORKERS) */
    uint32_t staging_depth; /* pinned staging pages per worker (RW_SCRATCH_PER_WORKER) */
    uint32_t flags;         /* GFS_CFG_* */
    uint64_t timeout_ns;    /* bound on every device-side wait (the reference waits forever) */
    int32_t device;         /* CUDA device ordinal */
    uint32_t pad1;
} gfs_config;

/* gfs_config.flags: read files through pread into pinned staging only, never
 * through a registered mapping of the file (see gfs_create) */
#define GFS_CFG_NO_FILE_MAP 1u
/* gfs_config.flags: keep the buffer cache in HBM when the session ends, for
 * the next session of this process with the same page size, pool, file-table
 * size and device, together with the session's registered file mappings.
 * Kept only if every file is closed and every page clean and unpinned at
 * gfs_destroy.  Cross-session counterpart of the reopen
 * check of libgpufs/fs_calls.cu:197-218: a file's first open in the new
 * session compares the host's ctime and size with those its cached pages
 * belong to and drops the pages if they differ. */
#define GFS_CFG_RETAIN_CACHE 2u
/* gfs_config.flags: build grep dictionary tables on the host instead of on
 * the device (the device build falls back to the host build by itself when
 * every seed fails; this flag takes that path directly) */
#define GFS_CFG_HOST_TABLE 4u

#define GFS_NSTATS 21
/* gfs_get_stats order: device hits(page accesses), misses, evictions,
 * writebacks, read_rpcs, bytes_read_rpc, opens, closes, timeouts, errors,
 * conflict_evictions; host requests, reads, read_bytes, writes, write_bytes,
 * opens, errors; first device failure (site << 16 | errno); requests
 * submitted; host reads served by DMA from a registered file mapping */

/* ---- session ---- */
/* defaults: 64 KiB pages, 2 GiB pool, 1024 files, 4096 ring slots, 8 workers */
void gfs_default_config(gfs_config* cfg);
/* replaces initializer() / GPUGlobals::GPUGlobals (libgpufs/fs_initializer.cu:116-167,
 * fs_initializer.cu.h:139-178); host workers start here and serve until destroy.
 * Files opened read-only are mapped and registered with CUDA on their first
 * open (kept across closes while unchanged: same inode, size and ctime, and
 * released at destroy or when over half the host memory is mapped), so a
 * page miss is filled by the missing block's own loads from the host page
 * cache, or by one copy-engine DMA from it into the frame; other files, and
 * any file whose mapping fails, go through pread into pinned staging as the
 * reference does (host_loop.h:431-557).  Dirty pages of at most 256 KiB are
 * staged by the GPU into mapped host slots for write-back. */
int gfs_create(const gfs_config* cfg, gfs_ctx** out);
/* replaces GPUGlobals::~GPUGlobals (libgpufs/fs_initializer.cu.h:180-198) */
int gfs_destroy(gfs_ctx* ctx);
/* replaces run_gpufs_handler (libgpufs/host_loop.h:559-656): waits until the
 * kernel stream is idle; returns the CUDA error code of the stream (0 ok) */
int gfs_run_handler(gfs_ctx* ctx, int gpuid);
/* gpuGlobals->streamMgr->kernelStream (libgpufs/fs_initializer.cu.h:90): a cudaStream_t */
void* gfs_kernel_stream(gfs_ctx* ctx);
/* device address of the session state (for kernels that take it explicitly) */
void* gfs_device_state(gfs_ctx* ctx);
uint32_t gfs_page_size(gfs_ctx* ctx);
uint32_t gfs_num_frames(gfs_ctx* ctx);
void* gfs_pool_base(gfs_ctx* ctx);
/* sticky device error bits (1 timeout, 2 io, 4 no frame, 8 table full, 16 bad argument) */
uint32_t gfs_last_error(gfs_ctx* ctx, int clear);
/* counters; replaces the PRINT_* statistics of libgpufs/fs_debug.cu.h:99-148 */
int gfs_get_stats(gfs_ctx* ctx, unsigned long long* out, int n);
int gfs_reset_stats(gfs_ctx* ctx);
/* empty the buffer cache of clean, unpinned pages (no kernel may be running);
 * returns the number of frames kept (pinned or dirty) */
long long gfs_drop_cache(gfs_ctx* ctx);
/* valid pages this session took over at gfs_create from a cache an earlier
 * session retained (GFS_CFG_RETAIN_CACHE); 0 if it started empty */
long long gfs_retained_pages(gfs_ctx* ctx);
/* free a retained cache that no session has taken over (gfs_create without
 * GFS_CFG_RETAIN_CACHE, or with another geometry, frees it too); returns 1
 * if one was kept.  A retained cache lives in the process's CUDA context; a
 * cudaDeviceReset() frees its memory, after which no session takes it over
 * (its pointers and a token in device memory are checked first) and this
 * call drops it without freeing anything. */
int gfs_release_retained(void);
/* pinned host<->device cudaMemcpyAsync bandwidth, best of `reps` (GB/s) */
int gfs_measure_link(uint64_t bytes, int reps, float* h2d_gbs, float* d2h_gbs);
/* Cold-read ceilings for one file of at least 1 MiB (GB/s, best of reps; no
 * reference counterpart): out[0] pinned host -> device in one copy, out[1]
 * the same as chunk-byte copies over `streams` streams, out[2] those copies
 * from the file's registered mapping, out[3] a kernel reading pinned host
 * memory, out[4] a kernel reading the registered file mapping, out[5] the
 * same with each CTA reading its own contiguous slice, out[6] the same with
 * one warp per CTA.  The file must not change during the call. */
int gfs_measure_cold_paths(const char* path, int streams, uint64_t chunk, int reps, float* out, int n_out);

/* ---- host-side fault injection (tests only; no GPU fault is ever made) ---- */
/* stall (1) or resume (0) the host service: device waits then time out */
int gfs_set_paused(gfs_ctx* ctx, int paused);
/* the next `count` host page reads fail with `err` (errno) */
int gfs_inject_read_errors(gfs_ctx* ctx, int count, int err);

/* ---- device API, driven from the host (each call runs one kernel whose
 * blocks call the reference-named device functions) ---- */
/* gopen(O_GRDONLY) + gread + gclose over [off, off+size) split into page-aligned
 * slices, one per block (libgpufs/fs_calls.cu:227,689,35).  host_out: host buffer.
 * Returns bytes read (clamped at end of file) or -error. */
long long gfs_pread(gfs_ctx* ctx, const char* path, uint64_t off, uint64_t size, void* host_out, int nblocks,
                    int nthreads);
/* same into a device buffer; *kernel_ms (optional) = kernel time (CUDA events) */
long long gfs_pread_dev(gfs_ctx* ctx, const char* path, uint64_t off, uint64_t size, void* dev_out, int nblocks,
                        int nthreads, float* kernel_ms);
/* gopen(oflags) + gwrite + gclose (libgpufs/fs_calls.cu:739); the last close
 * writes the dirty pages back to the host file. */
long long gfs_pwrite(gfs_ctx* ctx, const char* path, int oflags, uint64_t off, uint64_t size, const void* host_in,
                     int nblocks, int nthreads);
/* read through gmmap/gmunmap (use_warp_api: gmmap_warp/gmunmap_warp)
 * (libgpufs/fs_calls.cu:385-481,618-683) */
long long gfs_mmap_read(gfs_ctx* ctx, const char* path, uint64_t off, uint64_t size, void* host_out, int nblocks,
                        int nthreads, int use_warp_api);
/* gopen + fstat + gclose (libgpufs/fs_calls.cu:851) */
long long gfs_fstat_path(gfs_ctx* ctx, const char* path);
/* gopen(O_GRDWR) + gftruncate + gclose (libgpufs/fs_calls.cu:127-149) */
int gfs_truncate_path(gfs_ctx* ctx, const char* path, long long size);
/* gunlink (libgpufs/fs_calls.cu:845; unimplemented there) */
int gfs_unlink_path(gfs_ctx* ctx, const char* path);
/* gopen(O_GRDWR) + gwrite + gfsync (data on the host file while still open) + gclose */
long long gfs_pwrite_fsync(gfs_ctx* ctx, const char* path, uint64_t off, uint64_t size, const void* host_in);

/* memcopy sample, samples/memcopy/cp.cu:73-108 test_cpy: every block copies
 * pages blockIdx*PAGE, stride gridDim*PAGE, from src to a new dst (O_GWRONCE).
 * mode 0: gread/gwrite through a per-block buffer, as the reference;
 * mode 1: gmmap both pages and copy frame to frame (half the HBM traffic).
 * *kernel_ms (optional): kernel time. */
int gfs_memcopy(gfs_ctx* ctx, const char* src, const char* dst, int nblocks, int nthreads, int mode,
                float* kernel_ms);

/* bigmatrix_mmap sample (samples/bigmatrix_mmap/bigmatrix_mmap.cu:66-168):
 * y = A x, A read through gmmap page windows (rows x cols FP32 row-major,
 * cols = size(vec)/4), x mapped once (read with gread when larger than a
 * page), y written through gmmap of out_path (write-once, truncated first).
 * FP32 accumulation, deterministic reduction order.  nthreads: 32 ..
 * GFS_BIGMATRIX_THREADS per block (-GFS_EINVAL beyond). */
#define GFS_BIGMATRIX_THREADS 512
int gfs_bigmatrix(gfs_ctx* ctx, const char* vec_path, const char* mat_path, const char* out_path, int nblocks,
                  int nthreads, float* kernel_ms);
/* The same GEMV read once: when the matrix file has a registered host
 * mapping, the kernel reads it straight from there (SM loads over the host
 * link, no cache pages, as O_DIRECT); x and y go through the cache.  No
 * reference counterpart. */
int gfs_bigmatrix_direct(gfs_ctx* ctx, const char* vec_path, const char* mat_path, const char* out_path, int nblocks,
                         int nthreads, float* kernel_ms);
/* XXH64 (seed 0) of each file, read through the buffer cache; one warp per file */
int gfs_xxh64_files(gfs_ctx* ctx, const char* const* paths, int n, unsigned long long* host_out, float* kernel_ms);

/* Allocation-free form of gfs_xxh64_files (no reference counterpart: the
 * reference has no checksum and allocates per call).  Same results; every
 * per-call buffer lives in a fixed file-scope device array, so a call makes
 * no cudaMalloc/cudaFree or other allocation.  At most
 * GFS_XXH64_NOALLOC_MAX_FILES files per call, else -GFS_E2BIG.  The first
 * call on a device looks the array's address up (cudaGetSymbolAddress): make
 * it before any stream capture.  The array is 90,368 bytes on every device
 * that loads the library, held until exit.  The call runs on the session's
 * device (made current for its duration, the caller's device restored
 * after); a device reset makes the next call look the address up again.
 * The array is shared by all callers on a device, so overlapping calls on
 * one device race: serialise them. */
#define GFS_XXH64_NOALLOC_MAX_FILES 1024
int gfs_xxh64_files_noalloc(gfs_ctx* ctx, const char* const* paths, int n, unsigned long long* host_out);

/* ---- grep_text (samples/grep_text/grep_text_gpu.cu:193-387) ----
 * Whole-word occurrence counts of every record of a dictionary file (32-byte
 * NUL-padded records, the reference's dict.gpu format) in every corpus file,
 * read through the buffer cache.  counts[w * n_files + f] (uint32), equal to
 * the reference's on any input, including the effects of its 16 KiB window
 * walk: letter runs cut at windows whose halo is all letters, and the last
 * 1..31 bytes counted twice when the last window is longer than 16384.
 * gfs_grep_open reads the dictionary, builds its hash table, uploads it and
 * opens the corpus files on the device; gfs_grep_run scans (files stay open
 * and cached between runs); gfs_grep_close closes them. */
typedef struct gfs_grep gfs_grep;
int gfs_grep_open(gfs_ctx* ctx, const char* dict_path, const char* const* paths, int n_files, gfs_grep** out);
/* n_ctas <= 0: one per SM.  *kernel_ms (optional): device time of the scan. */
int gfs_grep_run(gfs_grep* g, int n_ctas, float* kernel_ms);
/* The same scan, read once: chunks of files that have a registered host
 * mapping are loaded by the GPU straight from it (16-byte SM loads over
 * the host link), bypassing the buffer cache, as O_DIRECT does; other files
 * go through the cache.  No reference counterpart (the sample reads through
 * the cache). */
int gfs_grep_run_direct(gfs_grep* g, int n_ctas, float* kernel_ms);
int gfs_grep_counts(gfs_grep* g, uint32_t* host_counts);
/* device address of the counts (n_words * n_files uint32) */
void* gfs_grep_device_counts(gfs_grep* g);
/* out: n_words, n_files, buckets, table in shared memory (0/1), dynamic shared
 * bytes, chunks, last status word, last error site, host microseconds of the
 * dictionary table build, host microseconds of opening the files */
int gfs_grep_info(gfs_grep* g, long long* out, int n);
int gfs_grep_close(gfs_grep* g);
/* `steps` runs back to back on the kernel stream; *total_ms: all of them
 * (CUDA events), *scan_ms: mean duration of one scan kernel */
int gfs_grep_bench(gfs_grep* g, int n_ctas, int steps, float* total_ms, float* scan_ms);
/* Batched form: every file's counts and its XXH64 (seed 0) in one persistent
 * launch, CTAs taking whole files longest first, captured as a CUDA graph on
 * first use (per grid size) and replayed; host_xxh[n_files] (optional).
 * The first call must not run inside another stream capture. */
int gfs_grep_batch(gfs_grep* g, int n_ctas, unsigned long long* host_xxh, float* kernel_ms);
/* ---- served form (no reference counterpart: the reference serves one
 * kernel at a time) ----
 * A persistent kernel whose warps take (file, offset, length, op) requests
 * from a ring in mapped host memory and serve them through the buffer
 * cache; served files are opened once and stay open on the device.
 * Read and grep ranges start at any byte; write ranges must start 16-byte
 * aligned (else -GFS_EINVAL for that request). */
#define GFS_SV_READ 1  /* read the range of a served file; result: its XXH64 (seed 0) */
#define GFS_SV_GREP 2  /* result: tokens of the range (read as a text of its own) that are dictionary words */
#define GFS_SV_WRITE 3 /* write the request's byte pattern over the range of an output file; result: bytes */
typedef struct gfs_serve_req {
    uint32_t op;
    uint32_t file;       /* served file index, or output file index for GFS_SV_WRITE */
    uint64_t offset;
    uint64_t length;
    uint64_t arrival_ns; /* open-loop arrival time from the start of the run */
} gfs_serve_req;
typedef struct gfs_serve_res {
    unsigned long long result;
    int32_t status;      /* 0 or -errno */
    uint32_t pad;
    uint64_t submit_ns;  /* published to the ring (after admission) */
    uint64_t complete_ns; /* completion seen by the host; latency = complete_ns - arrival_ns */
} gfs_serve_res;
typedef struct gfs_server gfs_server;
/* dictionary (grep_text record format), served files, write-once output files */
int gfs_serve_open(gfs_ctx* ctx, const char* dict_path, const char* const* paths, int n_files,
                   const char* const* out_paths, int n_out, gfs_server** out);
/* one open-loop run over requests sorted by arrival; inflight_pages bounds the
 * pages of admitted, unfinished requests (memory-gated admission);
 * warps_per_sm: serving warps per SM asked for, rounded down to whole blocks
 * of 8 and capped at what the device holds at once (gfs_serve_warps_per_sm).
 * Greps longer than 1 MiB are split into parts that idle serving warps take. */
int gfs_serve_run(gfs_server* sv, const gfs_serve_req* reqs, int n, gfs_serve_res* res, uint64_t inflight_pages,
                  int warps_per_sm);
/* the serving warps per SM a run asked for `warps_per_sm` uses */
int gfs_serve_warps_per_sm(gfs_server* sv, int warps_per_sm);
/* the last run's histogram of device service times, counted on the device:
 * out[b] = requests served in [2^b, 2^(b+1)) ns, from the take of the
 * request to its completion (the host-side latency adds queueing, admission
 * and the ring); copies min(n, 64) buckets, returns 64 */
int gfs_serve_service_hist(gfs_server* sv, unsigned long long* out, int n);
/* closes every file (dirty output pages are written back) */
int gfs_serve_close(gfs_server* sv);

/* ---- learned cost model for the autotuner (no reference counterpart) ----
 * A network n_in -> 64 -> 64 -> 1 (tanh hidden units, FP32) that predicts a
 * run's log time from workload features and session parameters, trained on
 * the device by the library's own forward/backward and Adam kernels (mean
 * squared error over the data set, full batch, deterministic).  Parameters
 * are one flat vector: W1 [n_in][64], b1 [64], W2 [64][64], b2 [64], w3 [64],
 * b3.  X is row-major [n][n_in]. */
#define GFS_CM_HIDDEN 64
#define GFS_CM_MAX_INPUTS 64
typedef struct gfs_costmodel gfs_costmodel;
/* Glorot-uniform weights from a seeded stream, zero biases */
int gfs_cm_create(int n_in, int device, unsigned long long seed, gfs_costmodel** out);
int gfs_cm_destroy(gfs_costmodel* cm);
int gfs_cm_n_params(const gfs_costmodel* cm);
int gfs_cm_get_params(gfs_costmodel* cm, float* host_out);
/* also resets the optimiser state */
int gfs_cm_set_params(gfs_costmodel* cm, const float* host_in);
/* the training set (copied to the device) */
int gfs_cm_set_data(gfs_costmodel* cm, const float* X, const float* y, int n);
/* loss and its gradient with respect to every parameter, on the training set */
int gfs_cm_grad(gfs_costmodel* cm, float* host_grad, float* host_loss);
/* `steps` full-batch Adam steps (fresh optimiser state); host_losses, when not
 * NULL, receives the loss before each step */
int gfs_cm_train(gfs_costmodel* cm, int steps, float lr, float* host_losses);
int gfs_cm_predict(gfs_costmodel* cm, const float* X, int n, float* host_y);

/* one call: open + run + counts to host + close (the reference sample's whole run) */
int gfs_grep_text(gfs_ctx* ctx, const char* dict_path, const char* const* paths, int n_files, uint32_t* host_counts,
                  int n_ctas);

#ifdef __cplusplus
}
#endif
#endif
