/*
 * Host runtime of the GB300 GPU file system.
 *
 * Replaces the reference's host side:
 *   GPUGlobals / GPUStreamManager / initializer  libgpufs/fs_initializer.cu(.h)
 *   run_gpufs_handler, open_loop, rw_task,        libgpufs/host_loop.h:156-656
 *   mainLoop, async_close_loop, diff_and_merge
 *
 * The reference runs five busy-polling threads only while
 * run_gpufs_handler() blocks, one 4-byte flag per request, a mutex/condvar
 * hand-off per batch, an extra device staging copy per page, and a D2H copy
 * plus stream synchronisation per written page.  Here:
 *   - `host_workers` threads consume one MPMC request ring (mapped pinned
 *     memory, 136-byte slots, sequence-numbered) for the whole lifetime of
 *     the session, so kernels may run at any time, not only inside the
 *     handler call;
 *   - read-only files are mmap'ed and registered before kernels open them;
 *     most misses of such files are then filled by the SMs themselves, and
 *     those that reach the host are one cudaMemcpyAsync from the mapping
 *     into the page frame; other reads go pread -> pinned staging ->
 *     cudaMemcpyAsync into the frame (no device staging copy); the worker
 *     itself writes the request's completion word, in mapped host memory,
 *     once the copy's event has fired -- nothing in the completion path is
 *     executed by the GPU, so a kernel that occupies every SM while it
 *     waits cannot hold up its own completions;
 *   - open replies are written into mapped host memory, no copy at all;
 *   - writes come either staged by the SMs in mapped write-stage slots or
 *     as a D2H copy, then (OR-merge for write-once files) -> pwrite;
 *   - staging slots are recycled in issue order as their events complete;
 *   - every kernel is loaded at session creation: a lazily loaded kernel
 *     launched while a file-system kernel runs stalls driver calls.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <errno.h>
#include <fcntl.h>
#include <sched.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/prctl.h>
#include <sys/resource.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <time.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <mutex>
#include <random>
#include <unordered_map>
#include <thread>
#include <vector>

#include "gfs_types.h"
#include "gfs_runtime.h"

extern __device__ gfs_state* g_gfs;

struct FileMap;

namespace {

struct Pending { /* a copy in flight: a read's H2D, or a write-back's D2H */
    uint32_t* done; /* host pointer of the completion word */
    uint32_t code;
    int write = 0;  /* write-back: merge and pwrite once the copy landed */
    uint32_t file = 0; /* device file slot */
    uint64_t offset = 0;
    size_t len = 0;
    uint32_t rflags = 0;
};

/* Host side of a device file slot (requests name the slot): the name and
 * flags it was opened with, its host fd -- closed when the process nears its
 * open-file limit and reopened by name when a request needs it -- its
 * registered mapping, its size when opened and the pages written back
 * since (a write-once page landing past the size at open on bytes not
 * written back before needs no OR-merge read: those bytes are zero). */
struct HostSlot {
    std::mutex mu;
    char name[GFS_NAME_MAX + 1] = {0};
    int oflags = 0; /* for reopening: no O_CREAT/O_TRUNC/O_EXCL */
    int fd = -1;
    int users = 0;  /* requests inside a syscall on fd */
    bool open = false;
    uint64_t last = 0;
    std::atomic<FileMap*> map{nullptr};
    uint64_t size_at_open = 0;
    std::vector<uint64_t> written; /* bit per page */
};

struct Worker {
    int id = 0;
    cudaStream_t stream = nullptr;
    uint8_t* staging = nullptr; /* depth * slot_bytes, pinned */
    uint8_t* merge = nullptr;   /* OR-merge scratch */
    size_t slot_bytes = 0;
    int depth = 0;
    std::vector<cudaEvent_t> ev;
    std::vector<Pending> pend; /* per staging slot */
    std::vector<char> busy;    /* slot has a copy in flight */
    int next = 0;              /* next slot to use (ring order = completion order) */
    int oldest = 0;            /* oldest busy slot */
    int nbusy = 0;
    std::thread th;
};

__global__ void k_init_frames(gfs_frame* f, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        gfs_frame z;
        z.st = 0u;
        z.content = 0u;
        z.key = ~0ULL;
        z.pad2 = 0u;
        z.pad0 = 0u;
        z.pad1 = 0ULL;
        f[i] = z;
    }
}

uint32_t next_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return (uint32_t)p;
}

ssize_t pread_full(int fd, uint8_t* buf, size_t len, off_t off) {
    size_t got = 0;
    while (got < len) {
        ssize_t r = pread(fd, buf + got, len - got, off + (off_t)got);
        if (r < 0) {
            if (errno == EINTR) continue;
            return -1;
        }
        if (r == 0) break;
        got += (size_t)r;
    }
    return (ssize_t)got;
}

ssize_t pwrite_full(int fd, const uint8_t* buf, size_t len, off_t off) {
    size_t put = 0;
    while (put < len) {
        ssize_t r = pwrite(fd, buf + put, len - put, off + (off_t)put);
        if (r < 0) {
            if (errno == EINTR) continue;
            return -1;
        }
        put += (size_t)r;
    }
    return (ssize_t)put;
}

} // namespace

/* A read-only file's bytes, mapped from the host page cache and registered
 * with CUDA, so page misses are copy-engine DMA from it (no pread, no
 * staging copy).  Keyed by the file's identity and version. */
struct FileMap {
    uint64_t dev = 0, ino = 0, size = 0;
    int64_t ctime_ns = 0;
    uint8_t* base = nullptr;
    uint64_t dev_addr = 0; /* the same bytes, addressed from the device */
    size_t len = 0;
    int refs = 0;      /* open host fds using it */
    uint64_t last = 0; /* LRU stamp */
};

struct gfs_ctx {
    gfs_config cfg{};
    gfs_state hs{};
    gfs_state* ds = nullptr;
    gfs_req* ring_h = nullptr;
    cudaStream_t kstream = nullptr;
    std::atomic<uint32_t> head{0};
    std::atomic<int> stop{0};
    std::atomic<int> paused{0};
    std::atomic<int> inject_count{0};
    int inject_err = EIO;
    std::vector<Worker*> workers;
    std::atomic<unsigned long long> h_reads{0}, h_read_bytes{0}, h_writes{0}, h_write_bytes{0}, h_opens{0},
        h_errors{0}, h_requests{0};
    char* d_scratch = nullptr; /* small device scratch for names/results of C-ABI calls */
    void* h_bounce = nullptr;  /* pinned host buffer for results copied back to callers' memory */
    size_t h_bounce_cap = 0;
    cudaMemPool_t mem_pool = nullptr; /* stream-ordered device memory of per-call objects (plans, servers) */
    int pageable = 0; /* kernels may address pageable host memory (host page tables) */
    uint8_t* hmap = nullptr;   /* mapped block: completion words + open replies (host view) */
    uint8_t* wstage_h = nullptr; /* write-back staging slots (host view of gfs_state.wstage) */
    size_t wstage_bytes = 0;
    uint8_t* hmap_d = nullptr; /* same, device view */
    size_t hmap_bytes = 0;
    size_t reply_off = 0;
    std::atomic<int> logged{0};
    size_t d_scratch_cap = 0;
    /* registered file mappings */
    std::mutex map_mu;
    std::unordered_multimap<uint64_t, FileMap*> maps; /* by inode */
    size_t map_count_cap = 0; /* mappings, well under the process's map-area limit */
    std::unique_ptr<HostSlot[]> slots; /* one per device file slot */
    std::atomic<int> open_fds{0};
    int fd_cap = 0;
    std::atomic<uint64_t> fd_clock{0};
    std::atomic<uint32_t> evict_hand{0};
    size_t mapped_bytes = 0, map_cap = 0;
    uint64_t map_clock = 0;
    std::atomic<unsigned long long> h_map_reads{0};
    unsigned long long retained_pages = 0; /* valid pages taken over from a retained cache */
};

static uint32_t* host_word(gfs_ctx* c, uint64_t dev_addr) {
    uint64_t base = (uint64_t)(uintptr_t)c->hmap_d;
    if (dev_addr < base || dev_addr + 4 > base + c->hmap_bytes) return nullptr;
    return (uint32_t*)(c->hmap + (dev_addr - base));
}

static void set_done(gfs_ctx* c, uint32_t* d, uint32_t code) {
    if (!d) return;
    if (code & GFS_DONE_ERR) c->h_errors++;
    __atomic_store_n(d, code, __ATOMIC_RELEASE);
}

static void log_failure(gfs_ctx* c, const gfs_req& r, int err) {
    if (c->logged.fetch_add(1) < 8)
        fprintf(stderr, "gpufs_gb300: host op %d failed: %s (fd %d, offset %llu, length %llu)\n", (int)r.op,
                strerror(err), r.host_fd, (unsigned long long)r.offset, (unsigned long long)r.length);
}

/* A write-back whose page has landed in staging slot k: OR-merge with the
 * file's bytes for write-once files (diff_and_merge, host_loop.h:76-137),
 * unless those bytes are known to be zero, then pwrite. */
static int slot_acquire_fd(gfs_ctx* c, uint32_t s);
static void slot_release_fd(gfs_ctx* c, uint32_t s);

/* Write len bytes of buf (the page at file offset `offset` of slot `file`)
 * to the host file, OR-merged with the bytes already there for write-once
 * files (RW_IPC_DIFF, host_loop.h:76-137); buf is merged in place.  Returns
 * 0 or an errno. */
static int write_out(gfs_ctx* c, Worker* w, uint32_t file, uint64_t offset, uint8_t* buf, size_t len, int rflags) {
    bool merge = (rflags & GFS_RF_DIFF) != 0;
    gfs_req r{};
    r.op = GFS_OP_WRITE;
    r.file = file;
    r.offset = offset;
    r.length = len;
    const int fd = slot_acquire_fd(c, file);
    if (fd < 0) {
        log_failure(c, r, -fd);
        return -fd;
    }
    r.host_fd = fd;
    {
        HostSlot& h = c->slots[file];
        const uint64_t pg = offset >> c->hs.log_page;
        std::lock_guard<std::mutex> lk(h.mu);
        if (h.written.size() <= (size_t)(pg >> 6)) h.written.resize((size_t)(pg >> 6) + 1, 0ULL);
        const uint64_t bit = 1ULL << (pg & 63u);
        if (merge && offset >= h.size_at_open && !(h.written[(size_t)(pg >> 6)] & bit)) merge = false;
        h.written[(size_t)(pg >> 6)] |= bit;
    }
    if (merge) {
        ssize_t m = pread_full(fd, w->merge, len, (off_t)offset);
        size_t i = 0;
        for (; m >= 8 && i + 8 <= (size_t)m; i += 8) {
            uint64_t a, b;
            memcpy(&a, buf + i, 8);
            memcpy(&b, w->merge + i, 8);
            a |= b;
            memcpy(buf + i, &a, 8);
        }
        for (; (ssize_t)i < m; i++) buf[i] |= w->merge[i];
    }
    ssize_t put = pwrite_full(fd, buf, len, (off_t)offset);
    int err = put < 0 ? errno : EIO;
    slot_release_fd(c, file);
    c->h_writes++;
    if (put >= 0) c->h_write_bytes += (unsigned long long)put;
    if (put != (ssize_t)len) {
        log_failure(c, r, err);
        return err;
    }
    return 0;
}

static void finish_write(gfs_ctx* c, Worker* w, int k, const Pending& p) {
    uint8_t* buf = w->staging + (size_t)k * w->slot_bytes;
    const int e = write_out(c, w, p.file, p.offset, buf, p.len, p.rflags);
    set_done(c, p.done, e == 0 ? 1u + (uint32_t)p.len : (GFS_DONE_ERR | (uint32_t)e));
}

/* Complete in-flight copies whose data has landed (in issue order). */
static void drain(gfs_ctx* c, Worker* w, bool block) {
    while (w->nbusy) {
        int k = w->oldest;
        if (!w->busy[(size_t)k]) { /* a slot used synchronously (write) */
            w->oldest = (k + 1) % w->depth;
            continue;
        }
        cudaError_t e = block ? cudaEventSynchronize(w->ev[(size_t)k]) : cudaEventQuery(w->ev[(size_t)k]);
        if (e == cudaErrorNotReady) return;
        Pending p = w->pend[(size_t)k];
        if (p.write && e == cudaSuccess) finish_write(c, w, k, p);
        else set_done(c, p.done, e == cudaSuccess ? p.code : (GFS_DONE_ERR | (uint32_t)EIO));
        w->busy[(size_t)k] = 0;
        w->oldest = (k + 1) % w->depth;
        w->nbusy--;
        if (!block) continue;
        return;
    }
}

/* A free staging slot (waits for the oldest copy when all are in flight). */
static int slot_take(gfs_ctx* c, Worker* w) {
    while (w->busy[(size_t)w->next]) drain(c, w, true);
    int k = w->next;
    w->next = (k + 1) % w->depth;
    return k;
}

static void map_release(FileMap* m) {
    cudaHostUnregister(m->base);
    munmap(m->base, m->len);
    delete m;
}

/* Mapping for a file just opened read-only (host fd `fd`, stat `st`), made
 * on first use and kept while unchanged; nullptr when it cannot be made. */
static FileMap* map_attach(gfs_ctx* c, int fd, const struct stat& st) {
    if ((c->cfg.flags & GFS_CFG_NO_FILE_MAP) || !S_ISREG(st.st_mode) || st.st_size < (off_t)(64 << 10)) return nullptr;
    const int64_t ct = (int64_t)st.st_ctim.tv_sec * 1000000000LL + st.st_ctim.tv_nsec;
    const size_t len = (size_t)st.st_size;
    const uint64_t key = (uint64_t)st.st_ino * 0x9E3779B97F4A7C15ULL ^ (uint64_t)st.st_dev;
    {
        std::lock_guard<std::mutex> lk(c->map_mu);
        auto rg = c->maps.equal_range(key);
        for (auto it = rg.first; it != rg.second; ++it) {
            FileMap* m = it->second;
            if (m->dev == (uint64_t)st.st_dev && m->ino == (uint64_t)st.st_ino && m->size == (uint64_t)len &&
                m->ctime_ns == ct) {
                m->refs++;
                m->last = ++c->map_clock;
                return m;
            }
        }
        if (c->mapped_bytes + len > c->map_cap || c->maps.size() + 1 > c->map_count_cap) {
            /* evict unused mappings, least recently used first */
            std::vector<std::pair<uint64_t, FileMap*>> idle;
            for (auto& e : c->maps)
                if (!e.second->refs) idle.push_back({e.second->last, e.second});
            std::sort(idle.begin(), idle.end());
            for (size_t i = 0; i < idle.size() &&
                               (c->mapped_bytes + len > c->map_cap || c->maps.size() + 1 > c->map_count_cap);
                 i++) {
                FileMap* m = idle[i].second;
                const uint64_t k = m->ino * 0x9E3779B97F4A7C15ULL ^ m->dev;
                auto r2 = c->maps.equal_range(k);
                for (auto it = r2.first; it != r2.second; ++it)
                    if (it->second == m) {
                        c->maps.erase(it);
                        break;
                    }
                c->mapped_bytes -= m->len;
                map_release(m);
            }
            if (c->mapped_bytes + len > c->map_cap || c->maps.size() + 1 > c->map_count_cap) return nullptr;
        }
    }
    void* p = mmap(nullptr, len, PROT_READ, MAP_SHARED | MAP_POPULATE, fd, 0);
    if (p == MAP_FAILED) return nullptr;
    /* mapped for the device too: direct scans read it with SM loads */
    bool reg = cudaHostRegister(p, len, cudaHostRegisterMapped | cudaHostRegisterReadOnly) == cudaSuccess;
    if (!reg) {
        cudaGetLastError();
        reg = cudaHostRegister(p, len, cudaHostRegisterMapped) == cudaSuccess;
    }
    void* dp = nullptr;
    if (!reg || cudaHostGetDevicePointer(&dp, p, 0) != cudaSuccess) {
        cudaGetLastError();
        if (reg) cudaHostUnregister(p);
        munmap(p, len);
        return nullptr;
    }
    FileMap* m = new FileMap();
    m->dev_addr = (uint64_t)(uintptr_t)dp;
    m->dev = (uint64_t)st.st_dev;
    m->ino = (uint64_t)st.st_ino;
    m->size = (uint64_t)len;
    m->ctime_ns = ct;
    m->base = (uint8_t*)p;
    m->len = len;
    m->refs = 1;
    std::lock_guard<std::mutex> lk(c->map_mu);
    m->last = ++c->map_clock;
    c->maps.emplace(key, m);
    c->mapped_bytes += len;
    return m;
}

static void map_detach(gfs_ctx* c, FileMap* m) {
    if (!m) return;
    std::lock_guard<std::mutex> lk(c->map_mu);
    m->refs--;
}

/* Register the mapping of a file a kernel is about to open read-only, from
 * the calling thread, so the device's open finds it cached: the host worker
 * that serves the open then makes no CUDA call while kernels run, and the
 * registration's cost stays out of the kernel's time.  A cached mapping
 * costs one stat(). */
extern "C" void gfs__premap(gfs_ctx* c, const char* path) {
    if (!c || !path || (c->cfg.flags & GFS_CFG_NO_FILE_MAP)) return;
    struct stat st;
    if (stat(path, &st) != 0 || !S_ISREG(st.st_mode) || st.st_size < (off_t)(64 << 10)) return;
    const int64_t ct = (int64_t)st.st_ctim.tv_sec * 1000000000LL + st.st_ctim.tv_nsec;
    const uint64_t key = (uint64_t)st.st_ino * 0x9E3779B97F4A7C15ULL ^ (uint64_t)st.st_dev;
    {
        std::lock_guard<std::mutex> lk(c->map_mu);
        auto rg = c->maps.equal_range(key);
        for (auto it = rg.first; it != rg.second; ++it) {
            const FileMap* m = it->second;
            if (m->dev == (uint64_t)st.st_dev && m->ino == (uint64_t)st.st_ino && m->size == (uint64_t)st.st_size &&
                m->ctime_ns == ct)
                return;
        }
    }
    const int fd = open(path, O_RDONLY | O_CLOEXEC);
    if (fd < 0) return;
    struct stat st2;
    if (fstat(fd, &st2) == 0) map_detach(c, map_attach(c, fd, st2));
    close(fd);
}

/* Close the host fds of idle slots (clock order) until the process is
 * comfortably below its open-file limit; `keep` is spared. */
static void fd_evict(gfs_ctx* c, uint32_t keep) {
    const uint32_t n = c->hs.n_files;
    const int target = c->fd_cap - c->fd_cap / 8;
    for (uint32_t tries = 0; tries < 2 * n && c->open_fds.load() > target; tries++) {
        const uint32_t i = c->evict_hand.fetch_add(1) % n;
        if (i == keep) continue;
        HostSlot& h = c->slots[i];
        if (!h.mu.try_lock()) continue;
        if (h.fd >= 0 && h.users == 0) {
            close(h.fd);
            h.fd = -1;
            c->open_fds--;
        }
        h.mu.unlock();
    }
}

/* The host fd of slot s for one syscall (reopened by name if it was
 * closed); -errno when the slot is not open.  Pair with slot_release_fd. */
static int slot_acquire_fd(gfs_ctx* c, uint32_t s) {
    if (s >= c->hs.n_files) return -EBADF;
    HostSlot& h = c->slots[s];
    bool reopened = false;
    int fd;
    {
        std::lock_guard<std::mutex> lk(h.mu);
        if (!h.open) return -EBADF;
        if (h.fd < 0) {
            h.fd = open(h.name, h.oflags | O_CLOEXEC);
            if (h.fd < 0) return -errno;
            reopened = true;
        }
        h.users++;
        h.last = ++c->fd_clock;
        fd = h.fd;
    }
    if (reopened && ++c->open_fds > c->fd_cap) fd_evict(c, s);
    return fd;
}

static void slot_release_fd(gfs_ctx* c, uint32_t s) {
    HostSlot& h = c->slots[s];
    std::lock_guard<std::mutex> lk(h.mu);
    h.users--;
}

static int host_open_flags(int oflags) {
    /* the reference turns write-once into O_RDWR|O_CREAT (host_loop.h:169-173);
     * write-only files are opened read-write as well so partial-page writes
     * can be filled from the file */
    if (oflags == (O_CREAT | O_WRONLY)) return O_RDWR | O_CREAT;
    if ((oflags & O_ACCMODE) == O_WRONLY) return (oflags & ~O_ACCMODE) | O_RDWR;
    return oflags;
}

static void handle(gfs_ctx* c, Worker* w, const gfs_req& r) {
    c->h_requests++;
    uint32_t* done = host_word(c, r.done_addr);
    switch (r.op) {
    case GFS_OP_OPEN: {
        char name[GFS_NAME_MAX + 1];
        memcpy(name, r.name, GFS_NAME_MAX);
        name[GFS_NAME_MAX] = 0;
        const int hflags = host_open_flags(r.oflags);
        int fd = r.file < c->hs.n_files ? open(name, hflags | O_CLOEXEC, 0644) : -1;
        int err = fd < 0 ? (r.file < c->hs.n_files ? errno : EBADF) : 0;
        gfs_open_reply rep{};
        rep.host_fd = fd;
        rep.err = err;
        if (fd >= 0) {
            struct stat st;
            if (fstat(fd, &st) != 0) memset(&st, 0, sizeof st);
            rep.size = (uint64_t)st.st_size;
            rep.ctime_ns = (int64_t)st.st_ctim.tv_sec * 1000000000LL + st.st_ctim.tv_nsec;
            FileMap* fm = (hflags & O_ACCMODE) == O_RDONLY ? map_attach(c, fd, st) : nullptr;
            rep.map_dev = fm ? fm->dev_addr : 0u;
            HostSlot& h = c->slots[r.file];
            {
                std::lock_guard<std::mutex> lk(h.mu);
                if (h.fd >= 0) { close(h.fd); c->open_fds--; } /* left over from an unclean close */
                map_detach(c, h.map.exchange(fm));
                memcpy(h.name, name, sizeof h.name);
                h.oflags = hflags & ~(O_CREAT | O_TRUNC | O_EXCL);
                h.fd = fd;
                h.users = 0;
                h.open = true;
                h.last = ++c->fd_clock;
                h.size_at_open = (uint64_t)st.st_size;
                h.written.clear();
            }
            if (++c->open_fds > c->fd_cap) fd_evict(c, r.file);
        }
        if (r.file < c->hs.n_files) {
            gfs_open_reply* dst = (gfs_open_reply*)(c->hmap + c->reply_off + (size_t)r.file * sizeof(gfs_open_reply));
            *dst = rep;
        }
        c->h_opens++;
        if (fd < 0 && err != ENOENT) log_failure(c, r, err);
        set_done(c, done, fd >= 0 ? 1u : (GFS_DONE_ERR | (uint32_t)err));
        break;
    }
    case GFS_OP_CLOSE: {
        int rc = 0, e = 0;
        if (r.file < c->hs.n_files) {
            HostSlot& h = c->slots[r.file];
            std::lock_guard<std::mutex> lk(h.mu);
            if (h.fd >= 0) {
                rc = close(h.fd);
                e = errno;
                h.fd = -1;
                c->open_fds--;
            }
            map_detach(c, h.map.exchange(nullptr));
            h.open = false;
            h.written.clear();
        }
        set_done(c, done, rc == 0 ? 1u : (GFS_DONE_ERR | (uint32_t)e));
        break;
    }
    case GFS_OP_READ: {
        if (c->inject_count.load() > 0 && c->inject_count.fetch_sub(1) > 0) {
            set_done(c, done, GFS_DONE_ERR | (uint32_t)c->inject_err);
            break;
        }
        size_t len = (size_t)r.length;
        if (len > w->slot_bytes) len = w->slot_bytes;
        int k = slot_take(c, w);
        FileMap* fm = r.file < c->hs.n_files ? c->slots[r.file].map.load(std::memory_order_acquire) : nullptr;
        if (fm && r.offset < fm->len) {
            /* DMA straight from the registered page-cache mapping */
            const size_t n = len < fm->len - (size_t)r.offset ? len : fm->len - (size_t)r.offset;
            size_t cp = (n + 4095u) & ~(size_t)4095u;
            if (cp > w->slot_bytes) cp = w->slot_bytes;
            cudaError_t e = cudaMemcpyAsync((void*)(uintptr_t)r.dev_addr, fm->base + r.offset, n,
                                            cudaMemcpyHostToDevice, w->stream);
            if (e == cudaSuccess && cp > n)
                e = cudaMemsetAsync((void*)(uintptr_t)(r.dev_addr + n), 0, cp - n, w->stream);
            if (e == cudaSuccess) e = cudaEventRecord(w->ev[(size_t)k], w->stream);
            if (e != cudaSuccess) {
                log_failure(c, r, EIO);
                set_done(c, done, GFS_DONE_ERR | (uint32_t)EIO);
                break;
            }
            c->h_reads++;
            c->h_map_reads++;
            c->h_read_bytes += (unsigned long long)n;
            w->pend[(size_t)k] = Pending{done, 1u + (uint32_t)n};
            w->busy[(size_t)k] = 1;
            w->nbusy++;
            drain(c, w, false);
            break;
        }
        uint8_t* buf = w->staging + (size_t)k * w->slot_bytes;
        const int fd = slot_acquire_fd(c, r.file);
        if (fd < 0) {
            log_failure(c, r, -fd);
            set_done(c, done, GFS_DONE_ERR | (uint32_t)(-fd));
            break;
        }
        ssize_t n = pread_full(fd, buf, len, (off_t)r.offset);
        const int rerr = errno;
        slot_release_fd(c, r.file);
        if (n < 0) {
            log_failure(c, r, rerr);
            set_done(c, done, GFS_DONE_ERR | (uint32_t)rerr);
            break;
        }
        size_t cp = ((size_t)n + 4095u) & ~(size_t)4095u;
        if (cp > w->slot_bytes) cp = w->slot_bytes;
        if (cp > (size_t)n) memset(buf + n, 0, cp - (size_t)n);
        c->h_reads++;
        c->h_read_bytes += (unsigned long long)n;
        if (!cp) {
            set_done(c, done, 1u);
            break;
        }
        /* copy-engine copy straight into the page frame; the completion
         * word is written by this thread once the copy's event has fired */
        cudaError_t e = cudaMemcpyAsync((void*)(uintptr_t)r.dev_addr, buf, cp, cudaMemcpyHostToDevice, w->stream);
        if (e == cudaSuccess) e = cudaEventRecord(w->ev[(size_t)k], w->stream);
        if (e != cudaSuccess) {
            log_failure(c, r, EIO);
            set_done(c, done, GFS_DONE_ERR | (uint32_t)EIO);
            break;
        }
        w->pend[(size_t)k] = Pending{done, 1u + (uint32_t)n};
        w->busy[(size_t)k] = 1;
        w->nbusy++;
        drain(c, w, false);
        break;
    }
    case GFS_OP_WRITE: {
        if (r.rflags & GFS_RF_STAGED) {
            /* the SMs stored the bytes in a write-stage slot: merge and
             * pwrite now, no copy to wait for */
            const size_t page = (size_t)c->hs.page_size;
            const uint64_t k = r.dev_addr;
            if (k * page >= c->wstage_bytes) {
                log_failure(c, r, EINVAL);
                set_done(c, done, GFS_DONE_ERR | (uint32_t)EINVAL);
                break;
            }
            size_t len = (size_t)r.length < page ? (size_t)r.length : page;
            const int e = write_out(c, w, r.file, r.offset, c->wstage_h + k * page, len, r.rflags);
            set_done(c, done, e == 0 ? 1u + (uint32_t)len : (GFS_DONE_ERR | (uint32_t)e));
            break;
        }
        /* device -> staging now; merge and pwrite when the copy has landed */
        size_t len = (size_t)r.length;
        if (len > w->slot_bytes) len = w->slot_bytes;
        int k = slot_take(c, w);
        uint8_t* buf = w->staging + (size_t)k * w->slot_bytes;
        cudaError_t e = cudaMemcpyAsync(buf, (const void*)(uintptr_t)r.dev_addr, len, cudaMemcpyDeviceToHost,
                                        w->stream);
        if (e == cudaSuccess) e = cudaEventRecord(w->ev[(size_t)k], w->stream);
        if (e != cudaSuccess) {
            log_failure(c, r, EIO);
            set_done(c, done, GFS_DONE_ERR | (uint32_t)EIO);
            break;
        }
        Pending pw{done, 0u};
        pw.write = 1;
        pw.file = r.file;
        pw.offset = r.offset;
        pw.len = len;
        pw.rflags = r.rflags;
        w->pend[(size_t)k] = pw;
        w->busy[(size_t)k] = 1;
        w->nbusy++;
        drain(c, w, false);
        break;
    }
    case GFS_OP_TRUNC: {
        const int fd = slot_acquire_fd(c, r.file);
        if (fd < 0) {
            set_done(c, done, GFS_DONE_ERR | (uint32_t)(-fd));
            break;
        }
        int rc = ftruncate(fd, (off_t)r.length);
        const int e = errno;
        slot_release_fd(c, r.file);
        set_done(c, done, rc == 0 ? 1u : (GFS_DONE_ERR | (uint32_t)e));
        break;
    }
    case GFS_OP_UNLINK: {
        char name[GFS_NAME_MAX + 1];
        memcpy(name, r.name, GFS_NAME_MAX);
        name[GFS_NAME_MAX] = 0;
        int rc = unlink(name);
        set_done(c, done, rc == 0 ? 1u : (GFS_DONE_ERR | (uint32_t)errno));
        break;
    }
    default:
        set_done(c, done, GFS_DONE_ERR | (uint32_t)EINVAL);
    }
}

static uint64_t mono_ns() {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

/* A worker waits for the request of its own ring ticket.  It spins, then
 * yields the CPU while requests came recently (GFS_HOT_NS after the last
 * one it served: a kernel's next request, such as the close after its
 * reads, is then picked up within microseconds), then naps 10 us at a time
 * with a 1 us timer slack (the default 50 us slack would stretch every
 * nap, and with it the latency of the first request after a quiet spell). */
#define GFS_HOT_NS 2000000ull
static void worker_main(gfs_ctx* c, Worker* w) {
    cudaSetDevice(c->cfg.device);
    cudaFree(nullptr);
    prctl(PR_SET_TIMERSLACK, 1000UL, 0, 0, 0);
    const uint32_t R = c->cfg.ring_slots, mask = R - 1;
    uint64_t last_busy = mono_ns();
    while (!c->stop.load(std::memory_order_relaxed)) {
        uint32_t t = c->head.fetch_add(1);
        gfs_req* slot = &c->ring_h[t & mask];
        unsigned spins = 0;
        bool hot = mono_ns() - last_busy < GFS_HOT_NS;
        while (__atomic_load_n(&slot->seq, __ATOMIC_ACQUIRE) != t + 1u) {
            if (c->stop.load(std::memory_order_relaxed)) return;
            if (w->nbusy) {
                /* copies in flight: complete them as they land (a device
                 * thread may be waiting on one); no backing off meanwhile */
                drain(c, w, false);
                spins = 0;
                continue;
            }
            if (spins++ < 4096u) continue;
            if (hot) {
                sched_yield();
                if ((spins & 255u) == 0u && mono_ns() - last_busy >= GFS_HOT_NS) hot = false;
                continue;
            }
            struct timespec ts = {0, 10000};
            nanosleep(&ts, nullptr);
        }
        last_busy = mono_ns();
        while (c->paused.load(std::memory_order_relaxed) && !c->stop.load(std::memory_order_relaxed)) {
            struct timespec ts = {0, 200000};
            nanosleep(&ts, nullptr);
        }
        if (c->stop.load(std::memory_order_relaxed)) return;
        gfs_req r;
        memcpy(&r, (const void*)slot, sizeof r);
        __atomic_store_n(&slot->seq, t + R, __ATOMIC_RELEASE);
        handle(c, w, r);
    }
}

#define CK(x)                                                                                     \
    do {                                                                                          \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess) {                                                                  \
            fprintf(stderr, "gpufs_gb300: %s failed: %s (%s:%d)\n", #x, cudaGetErrorString(e_), __FILE__, \
                    __LINE__);                                                                    \
            rc = -(int)e_;                                                                        \
            goto fail;                                                                            \
        }                                                                                         \
    } while (0)

static gfs_ctx* g_current = nullptr; /* session g_gfs points at */

/* CUDA maps streams onto a fixed set of hardware work queues (8 unless
 * CUDA_DEVICE_MAX_CONNECTIONS says otherwise).  A worker stream that shares
 * a queue with the stream of a running file-system kernel has its copies
 * ordered behind that kernel, which is waiting for them.  Ask for 32 queues
 * before any context exists (the library is loaded before the first CUDA
 * call in the programs and bindings that use it); host_workers is capped at
 * GFS_MAX_WORKERS so a session's streams fit. */
#define GFS_CONNECTIONS "32"
#define GFS_MAX_WORKERS 24
__attribute__((constructor)) static void gfs_set_connections() { setenv("CUDA_DEVICE_MAX_CONNECTIONS", GFS_CONNECTIONS, 0); }

void gfs__preload_runtime();

/* A buffer cache kept in HBM after its session ended (GFS_CFG_RETAIN_CACHE)
 * for the next session of this process with the same geometry: page pool,
 * frames, page index and file table, every page clean and unpinned and
 * every file closed, and the session's registered file mappings.  File slots keep their names, generations and the
 * ctime and size their pages belong to, so the next session's first open of
 * a file compares those with the host's reply, as a reopen within a session
 * does (the version check of fs_calls.cu:197-218), and drops the pages of a
 * file that changed in between. */
struct RetainedCache {
    int device = -1;
    uint32_t log_page = 0, n_frames = 0, n_buckets = 0, n_files = 0;
    uint8_t* pool = nullptr;
    gfs_frame* frames = nullptr;
    uint32_t* index = nullptr;
    uint32_t* bucket_lock = nullptr;
    gfs_file* files = nullptr;
    uint32_t* dirty_bits = nullptr;
    unsigned long long pages = 0; /* valid pages */
    /* the registered file mappings, none in use (keyed by file identity and
     * ctime, so a changed file is never served from an old one) */
    std::unordered_multimap<uint64_t, FileMap*> maps;
    size_t mapped_bytes = 0;
    uint64_t map_clock = 0;
    /* a token in device memory of its own, written when the cache is kept:
     * after a cudaDeviceReset the kept allocations are gone (and a new
     * allocation may take their addresses), so the cache is only touched if
     * every kept pointer is still device memory of this device and the
     * token reads back unchanged */
    uint64_t* token_d = nullptr;
    uint64_t token = 0;
};
static std::mutex g_retained_mu;
static RetainedCache* g_retained = nullptr; /* under g_retained_mu */

/* the kept allocations still belong to this process's context on r's
 * device (the caller has made that device current) */
static bool retained_alive(const RetainedCache* r) {
    const void* ptrs[] = {r->pool, r->frames, r->index, r->bucket_lock, r->files, r->dirty_bits, r->token_d};
    for (const void* p : ptrs) {
        cudaPointerAttributes a;
        if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeDevice ||
            a.device != r->device) {
            cudaGetLastError();
            return false;
        }
    }
    uint64_t t = 0;
    if (cudaMemcpy(&t, r->token_d, sizeof t, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return t == r->token;
}

/* Free a kept cache; one whose allocations did not survive (a device
 * reset in between) is dropped without freeing what is no longer ours. */
static void retained_free(RetainedCache* r) {
    if (!r) return;
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) cur = -1;
    cudaSetDevice(r->device);
    if (retained_alive(r)) {
        cudaFree(r->pool);
        cudaFree(r->frames);
        cudaFree(r->index);
        cudaFree(r->bucket_lock);
        cudaFree(r->files);
        cudaFree(r->dirty_bits);
        cudaFree(r->token_d);
    }
    for (auto& e : r->maps) map_release(e.second);
    if (cur >= 0) cudaSetDevice(cur);
    cudaGetLastError();
    delete r;
}

/* What keeps a cache from being retained: frames pinned, dirty, or in a
 * state other than FREE and VALID (a DEAD frame had a request time out);
 * files other than EMPTY or CLOSED without openers; held locks.
 * out[0] += such objects, out[1] += valid pages. */
__global__ void k_retain_check(const gfs_state* S, unsigned long long* out) {
    unsigned long long bad = 0, valid = 0;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, T = gridDim.x * blockDim.x;
    for (uint32_t i = tid; i < S->n_frames; i += T) {
        const uint32_t st = S->frames[i].st, s = (st >> GFS_F_SHIFT) & 0xFu;
        if (st & (GFS_F_PINS | GFS_F_DIRTY)) bad++;
        else if (s == GFS_FS_VALID) valid++;
        else if (s != GFS_FS_FREE) bad++;
    }
    for (uint32_t i = tid; i < S->n_files; i += T) {
        const uint32_t st = S->files[i].st, s = st >> GFS_S_SHIFT;
        if (!(s == GFS_SS_EMPTY || (s == GFS_SS_CLOSED && (st & GFS_S_CNT) == 0u))) bad++;
    }
    for (uint32_t i = tid; i < S->n_buckets; i += T)
        if (S->bucket_lock[i]) bad++;
    if (tid == 0 && S->table_lock) bad++;
    if (bad) atomicAdd(&out[0], bad);
    if (valid) atomicAdd(&out[1], valid);
}

/* At the end of a session (device idle, host workers stopped): keep its
 * cache for a later session if nothing in it is owned or in flight.  The
 * kept objects leave the session and are not freed with it; a cache kept
 * earlier and not taken over is freed. */
static void retain_cache(gfs_ctx* c) {
    gfs_state& s = c->hs;
    unsigned long long* d = nullptr;
    unsigned long long h[2] = {1ull, 0ull};
    if (cudaMalloc(&d, sizeof h) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    bool ok = cudaMemset(d, 0, sizeof h) == cudaSuccess;
    if (ok) {
        k_retain_check<<<152, 256>>>(c->ds, d);
        ok = cudaGetLastError() == cudaSuccess && cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost) == cudaSuccess;
    }
    cudaFree(d);
    cudaGetLastError();
    if (!ok || h[0] != 0) return;
    RetainedCache* r = new RetainedCache();
    r->device = c->cfg.device;
    r->log_page = s.log_page;
    r->n_frames = s.n_frames;
    r->n_buckets = s.n_buckets;
    r->n_files = s.n_files;
    r->pool = s.pool;
    r->frames = s.frames;
    r->index = s.index;
    r->bucket_lock = s.bucket_lock;
    r->files = s.files;
    r->dirty_bits = s.dirty_bits;
    r->pages = h[1];
    r->token = ((uint64_t)std::random_device{}() << 32) ^ (uint64_t)std::random_device{}() ^
               (uint64_t)(uintptr_t)r ^ 0x9E3779B97F4A7C15ull;
    if (cudaMalloc(&r->token_d, sizeof r->token) != cudaSuccess ||
        cudaMemcpy(r->token_d, &r->token, sizeof r->token, cudaMemcpyHostToDevice) != cudaSuccess) {
        /* no token, no keeping: nothing has left the session yet, which
         * frees its cache as usual */
        cudaGetLastError();
        if (r->token_d) cudaFree(r->token_d);
        delete r;
        return;
    }
    {
        std::lock_guard<std::mutex> lk(c->map_mu);
        for (auto& e : c->maps) {
            if (e.second->refs == 0) {
                r->maps.emplace(e.first, e.second);
                r->mapped_bytes += e.second->len;
            } else {
                map_release(e.second);
            }
        }
        c->maps.clear();
        c->mapped_bytes = 0;
        r->map_clock = c->map_clock;
    }
    s.pool = nullptr;
    s.frames = nullptr;
    s.index = nullptr;
    s.bucket_lock = nullptr;
    s.files = nullptr;
    s.dirty_bits = nullptr;
    std::lock_guard<std::mutex> lk(g_retained_mu);
    retained_free(g_retained);
    g_retained = r;
}

/* drop clean, unpinned, valid frames: first their index ways, then the frames */
__global__ void k_drop_ways(gfs_state* S) {
    size_t n = (size_t)S->n_buckets * GFS_WAYS;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t v = S->index[i];
        if (!v) continue;
        uint32_t st = S->frames[v & 0x3FFFFFu].st;
        if (((st >> GFS_F_SHIFT) & 0xFu) == GFS_FS_VALID && !(st & (GFS_F_PINS | GFS_F_DIRTY))) S->index[i] = 0u;
    }
}
__global__ void k_drop_frames(gfs_state* S, unsigned long long* kept) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < S->n_frames; i += gridDim.x * blockDim.x) {
        gfs_frame* F = &S->frames[i];
        uint32_t st = F->st;
        uint32_t s = (st >> GFS_F_SHIFT) & 0xFu;
        if (s == GFS_FS_VALID && !(st & (GFS_F_PINS | GFS_F_DIRTY))) {
            F->key = ~0ULL;
            F->st = 0u;
        } else if (s != GFS_FS_FREE) {
            atomicAdd(kept, 1ULL);
        }
    }
}

extern "C" {

/* Point the device API (g_gfs) at this session, in stream order. */
int gfs__activate(gfs_ctx* c) {
    if (g_current == c) return 0;
    cudaError_t e = cudaMemcpyToSymbolAsync(g_gfs, &c->ds, sizeof(gfs_state*), 0, cudaMemcpyHostToDevice, c->kstream);
    if (e != cudaSuccess) return -GFS_EIO;
    cudaStreamSynchronize(c->kstream);
    g_current = c;
    return 0;
}

void gfs_default_config(gfs_config* c) {
    memset(c, 0, sizeof *c);
    c->log_page = 16;
    c->pool_bytes = 2ull << 30;
    c->max_files = 1024;
    c->ring_slots = 4096;
    c->host_workers = 8;
    c->staging_depth = 8;
    c->timeout_ns = 30ull * 1000000000ull;
    c->device = 0;
}

int gfs_create(const gfs_config* cfg_in, gfs_ctx** out) {
    int rc = 0;
    gfs_ctx* c = new gfs_ctx();
    c->cfg = *cfg_in;
    gfs_config& cfg = c->cfg;
    *out = nullptr;
    if (cfg.log_page < 12 || cfg.log_page > 21) { delete c; return -GFS_EINVAL; }
    if (cfg.host_workers < 1) cfg.host_workers = 1;
    if (cfg.host_workers > GFS_MAX_WORKERS) cfg.host_workers = GFS_MAX_WORKERS;
    if (cfg.staging_depth < 2) cfg.staging_depth = 2;
    if (cfg.timeout_ns == 0) cfg.timeout_ns = 30ull * 1000000000ull;
    cfg.ring_slots = next_pow2(cfg.ring_slots < 64 ? 64 : cfg.ring_slots);
    cfg.max_files = next_pow2(cfg.max_files < 64 ? 64 : cfg.max_files);
    if (cfg.max_files > (1u << 20)) { delete c; return -GFS_EINVAL; }
    {
        /* host fds per file slot, below the open-file limit; registered
         * file mappings, at most half the host memory */
        struct rlimit rl;
        size_t nfd = 1u << 16;
        if (getrlimit(RLIMIT_NOFILE, &rl) == 0 && rl.rlim_cur != RLIM_INFINITY && rl.rlim_cur < (1u << 20))
            nfd = (size_t)rl.rlim_cur;
        /* host fds stay below the open-file limit, with room for the process */
        c->fd_cap = nfd > 2048 ? (int)nfd - 1024 : (int)nfd / 2;
        if (c->fd_cap < 16) c->fd_cap = 16;
        const long pages = sysconf(_SC_PHYS_PAGES), psz = sysconf(_SC_PAGESIZE);
        c->map_cap = pages > 0 && psz > 0 ? (size_t)pages * (size_t)psz / 2 : (size_t)8 << 30;
        long mm = 65530;
        if (FILE* f = fopen("/proc/sys/vm/max_map_count", "r")) {
            if (fscanf(f, "%ld", &mm) != 1) mm = 65530;
            fclose(f);
        }
        c->map_count_cap = mm > 8192 ? (size_t)(mm / 2) : 4096;
    }
    {
        uint64_t page = 1ull << cfg.log_page;
        uint64_t nf = cfg.pool_bytes / page;
        if (nf < 64) nf = 64;
        if (nf > GFS_MAX_FRAMES - 1) nf = GFS_MAX_FRAMES - 1;
        gfs_state& s = c->hs;
        s.log_page = cfg.log_page;
        s.page_size = (uint32_t)page;
        s.n_frames = (uint32_t)nf;
        s.n_buckets = next_pow2((nf + 3) / 4 < 64 ? 64 : (nf + 3) / 4);
        s.n_files = cfg.max_files;
        c->slots.reset(new HostSlot[cfg.max_files]);
        s.ring_slots = cfg.ring_slots;
        s.timeout_ns = cfg.timeout_ns;
        CK(cudaSetDevice(cfg.device));
        cudaSetDeviceFlags(cudaDeviceMapHost);
        cudaGetLastError();
        /* load every kernel of the library now: a lazily loaded kernel
         * launched while a file-system kernel waits on the host would stall
         * the driver calls the host workers make */
        gfs__preload_kernels();
        /* a retained cache of the same geometry is taken over; any other is
         * freed (a session without GFS_CFG_RETAIN_CACHE frees it too) */
        RetainedCache* adopt = nullptr;
        {
            std::lock_guard<std::mutex> lk(g_retained_mu);
            if (RetainedCache* r = g_retained) {
                g_retained = nullptr;
                if ((cfg.flags & GFS_CFG_RETAIN_CACHE) && r->device == cfg.device && r->log_page == s.log_page &&
                    r->n_frames == s.n_frames && r->n_buckets == s.n_buckets && r->n_files == s.n_files &&
                    retained_alive(r)) {
                    adopt = r;
                } else {
                    retained_free(r);
                }
            }
        }
        if (adopt) {
            s.pool = adopt->pool;
            s.frames = adopt->frames;
            s.index = adopt->index;
            s.bucket_lock = adopt->bucket_lock;
            s.files = adopt->files;
            s.dirty_bits = adopt->dirty_bits;
            c->retained_pages = adopt->pages;
            c->maps.swap(adopt->maps);
            c->mapped_bytes = adopt->mapped_bytes;
            c->map_clock = adopt->map_clock;
            cudaFree(adopt->token_d);
            delete adopt;
        } else {
            CK(cudaMalloc(&s.pool, nf * page));
            CK(cudaMalloc(&s.frames, nf * sizeof(gfs_frame)));
            CK(cudaMalloc(&s.index, (size_t)s.n_buckets * GFS_WAYS * sizeof(uint32_t)));
            CK(cudaMemset(s.index, 0, (size_t)s.n_buckets * GFS_WAYS * sizeof(uint32_t)));
            CK(cudaMalloc(&s.bucket_lock, (size_t)s.n_buckets * sizeof(uint32_t)));
            CK(cudaMemset(s.bucket_lock, 0, (size_t)s.n_buckets * sizeof(uint32_t)));
            CK(cudaMalloc(&s.files, (size_t)s.n_files * sizeof(gfs_file)));
            CK(cudaMemset(s.files, 0, (size_t)s.n_files * sizeof(gfs_file)));
            CK(cudaMalloc(&s.dirty_bits, ((nf + 31) / 32) * sizeof(uint32_t)));
            CK(cudaMemset(s.dirty_bits, 0, ((nf + 31) / 32) * sizeof(uint32_t)));
            k_init_frames<<<256, 256>>>(s.frames, (uint32_t)nf);
            CK(cudaGetLastError());
        }
        CK(cudaHostAlloc((void**)&c->ring_h, (size_t)cfg.ring_slots * sizeof(gfs_req),
                         cudaHostAllocMapped | cudaHostAllocPortable));
        memset(c->ring_h, 0, (size_t)cfg.ring_slots * sizeof(gfs_req));
        for (uint32_t i = 0; i < cfg.ring_slots; i++) c->ring_h[i].seq = i;
        CK(cudaHostGetDevicePointer((void**)&s.ring, c->ring_h, 0));
        const size_t reply_off = ((size_t)(nf + s.n_files) * 4 + 15) & ~(size_t)15;
        c->hmap_bytes = reply_off + (size_t)s.n_files * sizeof(gfs_open_reply);
        CK(cudaHostAlloc((void**)&c->hmap, c->hmap_bytes, cudaHostAllocMapped | cudaHostAllocPortable));
        memset(c->hmap, 0, c->hmap_bytes);
        CK(cudaHostGetDevicePointer((void**)&c->hmap_d, c->hmap, 0));
        s.hdone = (uint32_t*)c->hmap_d;
        s.hreply = (gfs_open_reply*)(c->hmap_d + reply_off);
        c->reply_off = reply_off;
        s.wstage = nullptr;
        s.wstage_bits = nullptr;
        s.wstage_slots = 0;
        {
            /* write-back staging for frames the SMs stage themselves (at
             * most 256 KiB of valid bytes each): 64 MiB of host memory in
             * page-sized slots, 32 to 1024 of them */
            uint64_t slots = (64ull << 20) / page;
            slots = slots > 1024 ? 1024 : (slots < 32 ? 32 : slots);
            c->wstage_bytes = (size_t)slots * page;
            CK(cudaHostAlloc((void**)&c->wstage_h, c->wstage_bytes, cudaHostAllocMapped | cudaHostAllocPortable));
            CK(cudaHostGetDevicePointer((void**)&s.wstage, c->wstage_h, 0));
            CK(cudaMalloc(&s.wstage_bits, ((slots + 31) / 32) * 4));
            CK(cudaMemset(s.wstage_bits, 0, ((slots + 31) / 32) * 4));
            s.wstage_slots = (uint32_t)slots;
        }
        CK(cudaMalloc(&c->ds, sizeof(gfs_state)));
        CK(cudaMemcpy(c->ds, &s, sizeof(gfs_state), cudaMemcpyHostToDevice));
        CK(cudaMemcpyToSymbol(g_gfs, &c->ds, sizeof(gfs_state*)));
        g_current = c;
        CK(cudaStreamCreateWithFlags(&c->kstream, cudaStreamNonBlocking));
        if (cudaDeviceGetAttribute(&c->pageable, cudaDevAttrPageableMemoryAccess, cfg.device) != cudaSuccess) {
            cudaGetLastError();
            c->pageable = 0;
        }
        {
            /* the session's own pool, kept warm (nothing returned to the
             * driver at synchronisation points) */
            cudaMemPoolProps pp = {};
            pp.allocType = cudaMemAllocationTypePinned;
            pp.handleTypes = cudaMemHandleTypeNone;
            pp.location.type = cudaMemLocationTypeDevice;
            pp.location.id = cfg.device;
            if (cudaMemPoolCreate(&c->mem_pool, &pp) == cudaSuccess) {
                uint64_t keep = ~0ull;
                cudaMemPoolSetAttribute(c->mem_pool, cudaMemPoolAttrReleaseThreshold, &keep);
            } else {
                cudaGetLastError();
                c->mem_pool = nullptr;
            }
        }
        c->d_scratch_cap = 1 << 20;
        CK(cudaMalloc(&c->d_scratch, c->d_scratch_cap));
        CK(cudaDeviceSynchronize());
        for (uint32_t i = 0; i < cfg.host_workers; i++) {
            Worker* w = new Worker();
            w->id = (int)i;
            w->depth = (int)cfg.staging_depth;
            w->slot_bytes = (size_t)page;
            c->workers.push_back(w);
            CK(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
            CK(cudaHostAlloc((void**)&w->staging, (size_t)w->depth * w->slot_bytes, cudaHostAllocPortable));
            w->merge = (uint8_t*)malloc(w->slot_bytes);
            w->ev.resize((size_t)w->depth);
            w->pend.resize((size_t)w->depth);
            w->busy.assign((size_t)w->depth, 0);
            for (int k = 0; k < w->depth; k++) CK(cudaEventCreateWithFlags(&w->ev[(size_t)k], cudaEventDisableTiming));
        }
        for (Worker* w : c->workers) w->th = std::thread(worker_main, c, w);
    }
    *out = c;
    return 0;
fail:
    gfs_destroy(c);
    return rc ? rc : -1;
}

int gfs_destroy(gfs_ctx* c) {
    if (!c) return 0;
    if (c->kstream) cudaStreamSynchronize(c->kstream);
    c->stop.store(1);
    for (Worker* w : c->workers)
        if (w->th.joinable()) w->th.join();
    cudaDeviceSynchronize();
    if ((c->cfg.flags & GFS_CFG_RETAIN_CACHE) && c->ds && c->hs.pool) retain_cache(c);
    for (Worker* w : c->workers) {
        for (cudaEvent_t e : w->ev)
            if (e) cudaEventDestroy(e);
        if (w->stream) cudaStreamDestroy(w->stream);
        if (w->staging) cudaFreeHost(w->staging);
        free(w->merge);
        delete w;
    }
    c->workers.clear();
    if (c->slots)
        for (uint32_t i = 0; i < c->hs.n_files; i++)
            if (c->slots[i].fd >= 0) close(c->slots[i].fd);
    for (auto& e : c->maps) map_release(e.second);
    c->maps.clear();
    if (c->h_bounce) cudaFreeHost(c->h_bounce);
    c->h_bounce = nullptr;
    if (c->wstage_h) cudaFreeHost(c->wstage_h);
    c->wstage_h = nullptr;
    if (c->hs.wstage_bits) cudaFree(c->hs.wstage_bits);
    c->hs.wstage_bits = nullptr;
    if (c->mem_pool) {
        cudaDeviceSynchronize();
        cudaMemPoolDestroy(c->mem_pool);
        c->mem_pool = nullptr;
    }
    gfs_state& s = c->hs;
    gfs_state* none = nullptr;
    if (c->ds && g_current == c) {
        cudaMemcpyToSymbol(g_gfs, &none, sizeof none);
        g_current = nullptr;
    }
    cudaFree(s.pool);
    cudaFree(s.frames);
    cudaFree(s.index);
    cudaFree(s.bucket_lock);
    cudaFree(s.files);
    cudaFree(s.dirty_bits);
    cudaFree(c->ds);
    cudaFree(c->d_scratch);
    if (c->ring_h) cudaFreeHost(c->ring_h);
    if (c->hmap) cudaFreeHost(c->hmap);
    if (c->kstream) cudaStreamDestroy(c->kstream);
    delete c;
    return 0;
}

void* gfs_kernel_stream(gfs_ctx* c) { return (void*)c->kstream; }
unsigned long long gfs__timeout_ns(gfs_ctx* c) { return c->cfg.timeout_ns; }
uint32_t gfs__config_flags(gfs_ctx* c) { return c->cfg.flags; }
int gfs__device(gfs_ctx* c) { return c->cfg.device; }
void* gfs_device_state(gfs_ctx* c) { return (void*)c->ds; }
uint32_t gfs_page_size(gfs_ctx* c) { return c->hs.page_size; }
uint32_t gfs_num_frames(gfs_ctx* c) { return c->hs.n_frames; }
void* gfs_pool_base(gfs_ctx* c) { return (void*)c->hs.pool; }

int gfs_run_handler(gfs_ctx* c, int gpuid) {
    (void)gpuid;
    cudaError_t e = cudaStreamSynchronize(c->kstream);
    return (int)e;
}

uint32_t gfs_last_error(gfs_ctx* c, int clear) {
    uint32_t v = 0;
    cudaMemcpy(&v, &c->ds->error, sizeof v, cudaMemcpyDeviceToHost);
    if (clear) {
        uint32_t z = 0;
        cudaMemcpy(&c->ds->error, &z, sizeof z, cudaMemcpyHostToDevice);
    }
    return v;
}

int gfs_get_stats(gfs_ctx* c, unsigned long long* out, int n) {
    gfs_stats st;
    if (cudaMemcpy(&st, &c->ds->stats, sizeof st, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    unsigned long long v[GFS_NSTATS] = {
        st.hits, st.misses, st.evictions, st.writebacks, st.read_rpcs, st.bytes_read_rpc, st.opens, st.closes,
        st.timeouts, st.errors, st.conflict_evictions, c->h_requests.load(), c->h_reads.load(),
        c->h_read_bytes.load(), c->h_writes.load(), c->h_write_bytes.load(), c->h_opens.load(), c->h_errors.load(),
        st.err_site, st.rpc_submitted, c->h_map_reads.load()};
    int k = n < GFS_NSTATS ? n : GFS_NSTATS;
    for (int i = 0; i < k; i++) out[i] = v[i];
    return k;
}

int gfs_reset_stats(gfs_ctx* c) {
    gfs_stats z;
    memset(&z, 0, sizeof z);
    cudaMemcpy(&c->ds->stats, &z, sizeof z, cudaMemcpyHostToDevice);
    c->h_requests = 0;
    c->h_reads = 0;
    c->h_read_bytes = 0;
    c->h_writes = 0;
    c->h_write_bytes = 0;
    c->h_opens = 0;
    c->h_errors = 0;
    c->h_map_reads = 0;
    return 0;
}

int gfs_set_paused(gfs_ctx* c, int paused) {
    c->paused.store(paused ? 1 : 0);
    return 0;
}

int gfs_inject_read_errors(gfs_ctx* c, int count, int err) {
    c->inject_err = err > 0 ? err : EIO;
    c->inject_count.store(count);
    return 0;
}

/* device scratch for the C-ABI helpers (names, per-block results) */
void* gfs__scratch(gfs_ctx* c, size_t bytes) {
    if (bytes > c->d_scratch_cap) {
        cudaFree(c->d_scratch);
        size_t cap = c->d_scratch_cap;
        while (cap < bytes) cap <<= 1;
        if (cudaMalloc(&c->d_scratch, cap) != cudaSuccess) {
            c->d_scratch = nullptr;
            c->d_scratch_cap = 0;
            return nullptr;
        }
        c->d_scratch_cap = cap;
    }
    return c->d_scratch;
}

int gfs__pageable_access(gfs_ctx* c) { return c && c->pageable; }

void* gfs__dev_alloc(gfs_ctx* c, size_t bytes, cudaStream_t s) {
    void* p = nullptr;
    if (c->mem_pool && cudaMallocFromPoolAsync(&p, bytes, c->mem_pool, s) == cudaSuccess) return p;
    cudaGetLastError();
    return cudaMalloc(&p, bytes) == cudaSuccess ? p : nullptr;
}

void gfs__dev_free(gfs_ctx* c, void* p, cudaStream_t s) {
    if (!p) return;
    if (c->mem_pool && cudaFreeAsync(p, s) == cudaSuccess) return;
    cudaGetLastError();
    cudaFree(p);
}

int gfs__slot_map(gfs_ctx* c, uint32_t slot, unsigned long long* dev_addr, unsigned long long* len) {
    *dev_addr = 0;
    *len = 0;
    if (!c || !c->slots || slot >= c->hs.n_files) return -GFS_EINVAL;
    HostSlot& h = c->slots[slot];
    std::lock_guard<std::mutex> lk(h.mu);
    FileMap* m = h.open ? h.map.load(std::memory_order_acquire) : nullptr;
    if (!m) return 0;
    *dev_addr = m->dev_addr;
    *len = m->len;
    return 1;
}

int gfs__slot_map_host(gfs_ctx* c, uint32_t slot, const uint8_t** base, unsigned long long* len) {
    *base = nullptr;
    *len = 0;
    if (!c || !c->slots || slot >= c->hs.n_files) return -GFS_EINVAL;
    HostSlot& h = c->slots[slot];
    std::lock_guard<std::mutex> lk(h.mu);
    FileMap* m = h.open ? h.map.load(std::memory_order_acquire) : nullptr;
    if (!m) return 0;
    *base = m->base;
    *len = m->len;
    return 1;
}

long long gfs__slot_pread(gfs_ctx* c, uint32_t slot, void* buf, size_t n, uint64_t off) {
    if (!c || !c->slots || slot >= c->hs.n_files) return -GFS_EINVAL;
    const int fd = slot_acquire_fd(c, slot);
    if (fd < 0) return fd;
    const ssize_t r = pread_full(fd, (uint8_t*)buf, n, (off_t)off);
    const int e = errno;
    slot_release_fd(c, slot);
    return r < 0 ? -(long long)e : (long long)r;
}

void* gfs__host_bounce(gfs_ctx* c, size_t bytes) {
    if (bytes > c->h_bounce_cap) {
        if (c->h_bounce) cudaFreeHost(c->h_bounce);
        c->h_bounce = nullptr;
        c->h_bounce_cap = 0;
        /* powers of two up to 64 MiB (small requests grow rarely); above,
         * the request rounded up to 2 MiB, so a large count matrix pins
         * about its own size and no more */
        size_t cap = (size_t)1 << 20;
        while (cap < bytes && cap < ((size_t)64 << 20)) cap <<= 1;
        if (cap < bytes) cap = (bytes + ((size_t)2 << 20) - 1) & ~(((size_t)2 << 20) - 1);
        if (cudaHostAlloc(&c->h_bounce, cap, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            c->h_bounce = nullptr;
            return nullptr;
        }
        c->h_bounce_cap = cap;
    }
    return c->h_bounce;
}

const gfs_state* gfs__host_state(gfs_ctx* c) { return &c->hs; }

void gfs__preload_runtime() {
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, k_init_frames);
    cudaFuncGetAttributes(&a, k_drop_ways);
    cudaFuncGetAttributes(&a, k_drop_frames);
    cudaFuncGetAttributes(&a, k_retain_check);
}

void gfs__preload_kernels() {
    gfs__preload_runtime();
    gfs__preload_workloads();
    gfs__preload_grep();
    gfs__preload_apps();
    gfs__preload_bigmatrix();
}

long long gfs_retained_pages(gfs_ctx* c) { return c ? (long long)c->retained_pages : -GFS_EINVAL; }

int gfs_release_retained(void) {
    RetainedCache* r;
    {
        std::lock_guard<std::mutex> lk(g_retained_mu);
        r = g_retained;
        g_retained = nullptr;
    }
    if (!r) return 0;
    retained_free(r);
    return 1;
}

/* Empty the buffer cache (clean, unpinned pages); returns frames kept. */
long long gfs_drop_cache(gfs_ctx* c) {
    cudaStream_t s = c->kstream;
    cudaStreamSynchronize(s);
    unsigned long long* kept = nullptr;
    if (cudaMalloc(&kept, sizeof *kept) != cudaSuccess) return -GFS_ENOMEM;
    cudaMemsetAsync(kept, 0, sizeof *kept, s);
    k_drop_ways<<<1024, 256, 0, s>>>(c->ds);
    k_drop_frames<<<1024, 256, 0, s>>>(c->ds, kept);
    unsigned long long h = 0;
    cudaMemcpyAsync(&h, kept, sizeof h, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    cudaFree(kept);
    return e == cudaSuccess ? (long long)h : -GFS_EIO;
}

/* Pinned host <-> device copy bandwidth (best of `reps`), the cold-read
 * roofline: copy-engine cudaMemcpyAsync of `bytes` each way. */
int gfs_measure_link(uint64_t bytes, int reps, float* h2d_gbs, float* d2h_gbs) {
    void* h = nullptr;
    void* d = nullptr;
    if (cudaHostAlloc(&h, bytes, cudaHostAllocDefault) != cudaSuccess) return -GFS_ENOMEM;
    if (cudaMalloc(&d, bytes) != cudaSuccess) {
        cudaFreeHost(h);
        return -GFS_ENOMEM;
    }
    memset(h, 1, bytes);
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best_h2d = 0, best_d2h = 0;
    for (int dir = 0; dir < 2; dir++) {
        for (int r = 0; r < reps + 1; r++) {
            cudaEventRecord(a, s);
            if (dir == 0) cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s);
            else cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s);
            cudaEventRecord(b, s);
            cudaEventSynchronize(b);
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            float gbs = (float)((double)bytes / (ms * 1e-3) / 1e9);
            if (r == 0) continue; /* warm-up */
            if (dir == 0 && gbs > best_h2d) best_h2d = gbs;
            if (dir == 1 && gbs > best_d2h) best_d2h = gbs;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(s);
    cudaFree(d);
    cudaFreeHost(h);
    if (h2d_gbs) *h2d_gbs = best_h2d;
    if (d2h_gbs) *d2h_gbs = best_d2h;
    return 0;
}

/* One SM-driven copy of n16 16-byte vectors from src (host memory mapped
 * for the device) to dst, four loads in flight per thread. */
__global__ void k_host_read(const uint4* __restrict__ src, uint64_t n16, uint4* __restrict__ dst) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n16; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n16; i += stride) dst[i] = src[i];
}

/* The same copy, each CTA reading its own contiguous slice front to back
 * (as a scan with a static run of chunks per CTA does), 8 loads in flight
 * per thread. */
__global__ void k_host_read_slices(const uint4* __restrict__ src, uint64_t n16, uint4* __restrict__ dst) {
    const uint64_t per = (n16 + gridDim.x - 1) / gridDim.x;
    const uint64_t lo = per * blockIdx.x, hi = lo + per < n16 ? lo + per : n16;
    const uint32_t nt = blockDim.x;
    uint64_t i = lo + threadIdx.x;
    for (; i + 7u * nt < hi; i += 8u * nt) {
        uint4 v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = src[i + (uint64_t)u * nt];
#pragma unroll
        for (int u = 0; u < 8; u++) dst[i + (uint64_t)u * nt] = v[u];
    }
    for (; i < hi; i += nt) dst[i] = src[i];
}

/* Cold-read ceilings for one file (best of `reps` after a warm-up, GB/s):
 * out[0] pinned host -> device, one cudaMemcpyAsync; out[1] the same bytes
 * as `chunk`-byte copies over `streams` streams; out[2] those copies from
 * the file's registered mapping (the session's cold path); out[3] a kernel
 * reading the pinned buffer; out[4] a kernel reading the registered file
 * mapping; out[5] the same, each CTA (one per SM, 1024 threads) reading its
 * own contiguous slice; out[6] the same with one warp per CTA.  The file is
 * mapped read-only and must not change meanwhile. */
int gfs_measure_cold_paths(const char* path, int streams, uint64_t chunk, int reps, float* out, int n_out) {
    if (!path || streams < 1 || streams > 64 || chunk < 4096 || reps < 1 || !out || n_out < 1) return -GFS_EINVAL;
    int fd = open(path, O_RDONLY | O_CLOEXEC);
    if (fd < 0) return -errno;
    struct stat st;
    if (fstat(fd, &st) != 0 || st.st_size < (off_t)(1 << 20)) {
        close(fd);
        return -GFS_EINVAL;
    }
    const size_t len = (size_t)st.st_size & ~(size_t)15;
    void* map = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_SHARED | MAP_POPULATE, fd, 0);
    close(fd);
    if (map == MAP_FAILED) return -errno;
    int rc = 0;
    void *h = nullptr, *d = nullptr, *hd = nullptr, *md = nullptr;
    bool reg = false;
    std::vector<cudaStream_t> ss((size_t)streams, nullptr);
    cudaEvent_t a = nullptr, b = nullptr;
    float best[7] = {0, 0, 0, 0, 0, 0, 0};
    if (cudaHostAlloc(&h, len, cudaHostAllocMapped) == cudaSuccess && cudaMalloc(&d, len) == cudaSuccess) {
        reg = cudaHostRegister(map, (size_t)st.st_size, cudaHostRegisterMapped | cudaHostRegisterReadOnly) ==
              cudaSuccess;
        if (!reg) {
            cudaGetLastError();
            reg = cudaHostRegister(map, (size_t)st.st_size, cudaHostRegisterMapped) == cudaSuccess;
        }
    }
    if (!reg) {
        cudaGetLastError();
        rc = -GFS_ENOMEM;
    } else {
        memcpy(h, map, len);
        cudaHostGetDevicePointer(&hd, h, 0);
        cudaHostGetDevicePointer(&md, map, 0);
        for (auto& x : ss) cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking);
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        int sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        for (int kind = 0; kind < 7 && kind < n_out; kind++) {
            for (int r = 0; r < reps + 1; r++) {
                cudaDeviceSynchronize();
                cudaEventRecord(a, ss[0]);
                if (kind == 0) {
                    cudaMemcpyAsync(d, h, len, cudaMemcpyHostToDevice, ss[0]);
                } else if (kind <= 2) {
                    const uint8_t* src = kind == 1 ? (const uint8_t*)h : (const uint8_t*)map;
                    /* every stream starts after the first event and the
                     * closing event waits for every stream */
                    for (size_t i = 0, k = 0; i < len; i += chunk, k++) {
                        cudaStream_t x = ss[k % ss.size()];
                        if (k < ss.size() && k) cudaStreamWaitEvent(x, a, 0);
                        cudaMemcpyAsync((uint8_t*)d + i, src + i, len - i < chunk ? len - i : chunk,
                                        cudaMemcpyHostToDevice, x);
                    }
                    for (size_t k = 1; k < ss.size(); k++) {
                        cudaEvent_t j;
                        cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
                        cudaEventRecord(j, ss[k]);
                        cudaStreamWaitEvent(ss[0], j, 0);
                        cudaEventDestroy(j);
                    }
                } else if (kind <= 4) {
                    const uint4* src = (const uint4*)(kind == 3 ? hd : md);
                    k_host_read<<<sms * 4, 512, 0, ss[0]>>>(src, (uint64_t)(len / 16), (uint4*)d);
                } else {
                    k_host_read_slices<<<sms, kind == 5 ? 1024 : 32, 0, ss[0]>>>((const uint4*)md,
                                                                                  (uint64_t)(len / 16), (uint4*)d);
                }
                cudaEventRecord(b, ss[0]);
                if (cudaEventSynchronize(b) != cudaSuccess) {
                    rc = -GFS_EIO;
                    break;
                }
                float ms = 0;
                cudaEventElapsedTime(&ms, a, b);
                const float gbs = (float)((double)len / (ms * 1e-3) / 1e9);
                if (r > 0 && gbs > best[kind]) best[kind] = gbs;
            }
            if (rc) break;
        }
    }
    cudaGetLastError();
    for (auto& x : ss)
        if (x) cudaStreamDestroy(x);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (reg) cudaHostUnregister(map);
    cudaGetLastError();
    munmap(map, (size_t)st.st_size);
    cudaFree(d);
    if (h) cudaFreeHost(h);
    for (int i = 0; i < n_out && i < 7; i++) out[i] = best[i];
    return rc;
}

double _timestamp() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return 1e6 * (double)tv.tv_sec + (double)tv.tv_usec;
}

} /* extern "C" */
