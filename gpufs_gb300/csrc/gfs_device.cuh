/*
 * Device-side internals of the GB300 GPU file system.
 *
 * Replaces the reference's page-fault core and its supporting structures:
 *   getRwLockedPage            libgpufs/fs_calls.cu:238-383   -> pin_page()
 *   HashMap read/get/remove    libgpufs/hashMap.cu:41-218     -> index_*()
 *   PFrame state machine       libgpufs/fs_structures.cu:25-174
 *   PPool::allocPage + swapper libgpufs/mallocfree.cu:55-235  -> alloc_frame()
 *   read_cpu / RW queue        libgpufs/cpu_ipc.cu:163-299    -> rpc_call()
 *   async write-back ring      libgpufs/async_ipc.cu:89-159   -> flush_frame()
 *   FTable open/close          libgpufs/fs_structures.cu:335-378, fs_calls.cu:35-236
 *
 * Design (GB300-first):
 *   - no global or per-frame spinlocks on the read path: a page is found by
 *     a lock-free probe of one 64-byte bucket and pinned with one atomic on
 *     the frame's state word; identity is re-checked after the pin (the key
 *     is a single 64-bit word written while the frame is unpinnable);
 *   - misses allocate with a clock (second-chance) sweep that evicts clean
 *     frames and writes dirty ones back through the host when it must;
 *   - a miss of a file with a registered host mapping can come back fresh
 *     (GFS_PIN_SMFILL) for the caller's own threads to fill from the
 *     mapping, with no request to the host; dirty frames of at most 256 KiB
 *     are staged by the SMs into mapped host slots for write-back;
 *   - every wait is bounded by %globaltimer and returns -GFS_ETIMEDOUT with
 *     a sticky error bit instead of spinning forever (the reference's
 *     WAIT_ON_MEM, util.cu.h:28, never gives up); once the bit is set,
 *     waits on the host fail at once;
 *   - requests to the host are 136-byte slots of an MPMC ring in mapped
 *     pinned host memory, published by one release store of the slot's
 *     sequence word; completions come back as a word in mapped host memory
 *     that the host worker writes after the data has landed.
 */
#ifndef GFS_DEVICE_CUH
#define GFS_DEVICE_CUH

#include <stdint.h>
#include <stddef.h>
#include "gfs_types.h"

/* reference open flags (libgpufs/fs_constants.h:86-90) */
#include <fcntl.h>
#ifndef O_GRDONLY
#define O_GRDONLY (O_RDONLY)
#define O_GWRONLY (O_WRONLY)
#define O_GCREAT (O_CREAT)
#define O_GRDWR (O_RDWR)
#define O_GWRONCE (O_GCREAT | O_GWRONLY)
#endif

namespace gfsd {
namespace { /* internal linkage: every TU gets its own copy */

/* ------------------------------------------------------------------ */
/* memory-model primitives                                             */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t ld_acq(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_rlx(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_rlx64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int64_t ld_rlxs64(const int64_t* p) {
    return (int64_t)ld_rlx64((const uint64_t*)p);
}
__device__ __forceinline__ void st_rel(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_rlx(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_rlx64(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acq_sys(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_rel_sys(uint32_t* p, uint32_t v) {
    asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_rlx_sys(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_rlx_sys64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_rlx_sys(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t atom_add_ar(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint32_t atom_cas_ar(uint32_t* p, uint32_t cmp, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.cas.b32 %0, [%1], %2, %3;"
                 : "=r"(old) : "l"(p), "r"(cmp), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint32_t atom_or_rel(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.release.gpu.global.or.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint32_t atom_and_ar(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.and.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint4 ld_cg4(const void* p) {
    uint4 v;
    asm volatile("ld.global.cg.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}
/* 16 bytes of a caller's buffer: cache-global when it is global memory, a
 * generic load otherwise (a block's shared-memory buffer; global-space
 * loads of a shared address are an error) */
__device__ __forceinline__ uint4 ld_user4(const void* p, bool global) {
    return global ? ld_cg4(p) : *(const uint4*)p;
}

/* Bounded wait: exponential back-off with __nanosleep, deadline on the
 * global timer.  tick() returns false once the deadline has passed. */
struct Waiter {
    uint64_t deadline;
    uint32_t ns;
    __device__ __forceinline__ explicit Waiter(uint64_t timeout_ns) : deadline(gtimer() + timeout_ns), ns(20) {}
    __device__ __forceinline__ bool tick(uint32_t cap = 1024) {
        if (gtimer() > deadline) return false;
        __nanosleep(ns);
        if (ns < cap) ns <<= 1;
        return true;
    }
};

__device__ __forceinline__ void count(gfs_state* S, unsigned long long* c, unsigned long long v = 1) {
    atomicAdd(c, v);
}
__device__ __forceinline__ void set_error(gfs_state* S, uint32_t bit) { atomicOr(&S->error, bit); }
/* record the first failure's site (for diagnosis) and set the sticky bit */
__device__ __forceinline__ void fail_at(gfs_state* S, uint32_t bit, uint32_t site, int err) {
    atomicOr(&S->error, bit);
    atomicCAS(&S->stats.err_site, 0ULL, ((unsigned long long)site << 16) | (unsigned long long)(err < 0 ? -err : err));
}

/* ------------------------------------------------------------------ */
/* keys and hashing                                                    */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ uint64_t page_key(uint32_t file, uint32_t gen, uint32_t block) {
    return ((uint64_t)file << 44) | ((uint64_t)(gen & 0xFFFu) << 32) | (uint64_t)block;
}
__device__ __forceinline__ uint32_t key_file(uint64_t k) { return (uint32_t)(k >> 44); }
__device__ __forceinline__ uint32_t key_gen(uint64_t k) { return (uint32_t)(k >> 32) & 0xFFFu; }
__device__ __forceinline__ uint32_t key_block(uint64_t k) { return (uint32_t)k; }

__device__ __forceinline__ uint64_t fmix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}
__device__ __forceinline__ uint32_t key_tag(uint64_t h) { return (uint32_t)((h >> 40) % 1023u) + 1u; }

__device__ __forceinline__ uint32_t fstate(uint32_t st) { return (st >> GFS_F_SHIFT) & 0xFu; }
__device__ __forceinline__ uint32_t sstatus(uint32_t st) { return st >> GFS_S_SHIFT; }

/* ------------------------------------------------------------------ */
/* page index: set-associative, 16 ways per 64-byte bucket             */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ uint32_t index_find(gfs_state* S, uint64_t key, uint64_t h) {
    const uint32_t* b = S->index + (size_t)(h & (S->n_buckets - 1)) * GFS_WAYS;
    uint32_t tag = key_tag(h);
#pragma unroll
    for (int q = 0; q < GFS_WAYS / 4; q++) {
        uint4 v = ld_cg4(b + 4 * q);
        uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            if ((w[i] >> 22) == tag) {
                uint32_t fr = w[i] & 0x3FFFFFu;
                if (ld_rlx64(&S->frames[fr].key) == key) return fr;
            }
        }
    }
    return GFS_NO_FRAME;
}

/* caller holds the bucket's insert lock */
__device__ __forceinline__ bool index_insert(gfs_state* S, uint64_t h, uint32_t fr) {
    uint32_t* b = S->index + (size_t)(h & (S->n_buckets - 1)) * GFS_WAYS;
    uint32_t v = (key_tag(h) << 22) | fr;
    for (int i = 0; i < GFS_WAYS; i++)
        if (ld_rlx(&b[i]) == 0 && atomicCAS(&b[i], 0u, v) == 0u) return true;
    return false;
}

__device__ __forceinline__ void index_remove(gfs_state* S, uint64_t key, uint32_t fr) {
    uint64_t h = fmix64(key);
    uint32_t* b = S->index + (size_t)(h & (S->n_buckets - 1)) * GFS_WAYS;
    uint32_t v = (key_tag(h) << 22) | fr;
    for (int i = 0; i < GFS_WAYS; i++)
        if (ld_rlx(&b[i]) == v) { atomicCAS(&b[i], v, 0u); return; }
}

__device__ __forceinline__ bool spin_lock(uint32_t* l, Waiter& w) {
    while (atomicCAS(l, 0u, 1u) != 0u)
        if (!w.tick(256)) return false;
    __threadfence();
    return true;
}
__device__ __forceinline__ void spin_unlock(uint32_t* l) {
    __threadfence();
    atomicExch(l, 0u);
}

/* ------------------------------------------------------------------ */
/* RPC to the host                                                     */
/* ------------------------------------------------------------------ */
struct Req {
    uint16_t op, rflags;
    int32_t host_fd;
    uint32_t file;
    int32_t oflags;
    uint64_t offset, length, dev_addr;
    const char* name; /* device pointer, <= GFS_NAME_MAX bytes, may be null */
};

/* completion words in mapped host memory, written by the host CPU */
__device__ __forceinline__ uint32_t* frame_done(gfs_state* S, uint32_t fr) { return S->hdone + fr; }
__device__ __forceinline__ uint32_t* file_done(gfs_state* S, uint32_t slot) { return S->hdone + S->n_frames + slot; }

/* A wait on the host already ran out in this session: later waits on it
 * give up at once (one stalled host frees the GPU within about one
 * timeout, not one timeout per request); gfs_last_error(ctx, 1) clears it */
__device__ __forceinline__ bool host_stalled(gfs_state* S) {
    return (ld_rlx(&S->error) & GFS_ERRB_TIMEOUT) != 0u;
}

/* Publish one request and wait for its completion word (in mapped host
 * memory; the host CPU writes it once the data has landed).  Returns the
 * non-negative result (bytes moved, or 0) or -errno / -GFS_ETIMEDOUT. */
__device__ __noinline__ int rpc_call(gfs_state* S, const Req& r, uint32_t* done) {
    if (host_stalled(S)) return -GFS_ETIMEDOUT;
    /* the completion word is cleared before the request is published: the
     * release store of the sequence word below orders both this store and
     * the request's fields before it at system scope, so no separate fence
     * is needed (each costs a round trip to host memory) */
    st_rlx_sys(done, 0u);
    Waiter w(S->timeout_ns);
    /* the lanes of a warp that call together (a lane-per-page miss burst)
     * take consecutive ring tickets with one atomic by their leader */
    const unsigned act = __activemask();
    uint32_t lane_id;
    asm("mov.u32 %0, %%laneid;" : "=r"(lane_id));
    const int lane = (int)lane_id, leader = __ffs(act) - 1;
    uint32_t t = 0;
    if (lane == leader) t = atomicAdd(&S->ring_tail, (uint32_t)__popc(act));
    t = __shfl_sync(act, t, leader) + (uint32_t)__popc(act & ((1u << lane) - 1u));
    gfs_req* slot = S->ring + (t & (S->ring_slots - 1));
    while (ld_acq_sys(&slot->seq) != t) {
        if (!w.tick(2048)) {
            count(S, &S->stats.timeouts);
            fail_at(S, GFS_ERRB_TIMEOUT, 1, GFS_ETIMEDOUT); /* ring slot never freed */
            return -GFS_ETIMEDOUT;
        }
    }
    volatile gfs_req* vs = slot;
    vs->op = r.op;
    vs->rflags = r.rflags;
    vs->host_fd = r.host_fd;
    vs->file = r.file;
    vs->offset = r.offset;
    vs->length = r.length;
    vs->dev_addr = r.dev_addr;
    vs->done_addr = (uint64_t)(uintptr_t)done;
    vs->oflags = r.oflags;
    if (r.name) {
        for (int i = 0; i < GFS_NAME_MAX; i += 4) {
            uint32_t v = 0;
            for (int b = 0; b < 4; b++) v |= (uint32_t)(uint8_t)r.name[i + b] << (8 * b);
            ((volatile uint32_t*)vs->name)[i / 4] = v;
        }
    }
    st_rel_sys(&slot->seq, t + 1u);
    count(S, &S->stats.rpc_submitted);
    uint32_t c;
    while ((c = ld_acq_sys(done)) == 0u) {
        if (!w.tick(1024) || host_stalled(S)) {
            count(S, &S->stats.timeouts);
            fail_at(S, GFS_ERRB_TIMEOUT, 2 + 16 * (uint32_t)r.op, GFS_ETIMEDOUT); /* no completion */
            return -GFS_ETIMEDOUT;
        }
    }
    if (c & GFS_DONE_ERR) {
        count(S, &S->stats.errors);
        set_error(S, GFS_ERRB_IO);
        int e = (int)(c & ~GFS_DONE_ERR);
        return -(e ? e : GFS_EIO);
    }
    return (int)(c - 1u);
}

/* ------------------------------------------------------------------ */
/* frames                                                              */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ uint8_t* frame_data(gfs_state* S, uint32_t fr) {
    return S->pool + ((size_t)fr << S->log_page);
}
__device__ __forceinline__ void unpin(gfs_state* S, uint32_t fr, uint32_t n = 1) {
    __threadfence();
    atomicSub(&S->frames[fr].st, n);
}
__device__ __forceinline__ bool key_stale(gfs_state* S, uint64_t key) {
    uint32_t f = key_file(key);
    if (f >= S->n_files) return true;
    return (ld_rlx(&S->files[f].gen) & 0xFFFu) != key_gen(key);
}
__device__ __forceinline__ void dirty_bit_set(gfs_state* S, uint32_t fr) {
    atomicOr(&S->dirty_bits[fr >> 5], 1u << (fr & 31));
}
__device__ __forceinline__ void dirty_bit_clear(gfs_state* S, uint32_t fr) {
    atomicAnd(&S->dirty_bits[fr >> 5], ~(1u << (fr & 31)));
}
/* Mark a frame dirty after its bytes were written (data first, then bit). */
__device__ __forceinline__ void mark_dirty(gfs_state* S, uint32_t fr) {
    __threadfence();
    uint32_t old = atom_or_rel(&S->frames[fr].st, GFS_F_DIRTY);
    if (!(old & GFS_F_DIRTY)) dirty_bit_set(S, fr);
}

__device__ __noinline__ int writeback_frame(gfs_state* S, uint32_t fr, uint64_t key, int host_fd, int oflags,
                                            int stage_slot = -1);

/* Take a frame out of VALID (refcount 0) into EVICTING and then CLAIMED:
 * drop it from the index, wait out transient pins.  Dirty frames must have
 * been written back by the caller (or be stale). */
__device__ __forceinline__ bool finish_evict(gfs_state* S, uint32_t fr, uint64_t key, bool was_dirty) {
    gfs_frame* F = &S->frames[fr];
    index_remove(S, key, fr);
    if (was_dirty) dirty_bit_clear(S, fr);
    /* pinners that raced the CAS see EVICTING and back off at once; the
     * drain has its own bound, independent of the caller's budget */
    Waiter w(S->timeout_ns);
    while ((ld_rlx(&F->st) & GFS_F_PINS) != 0u) {
        if (!w.tick(256)) {
            /* never reuse a frame somebody still holds: retire it */
            atomicAdd(&F->st, (GFS_FS_DEAD - GFS_FS_EVICTING) << GFS_F_SHIFT);
            fail_at(S, GFS_ERRB_TIMEOUT, 3, GFS_ETIMEDOUT); /* pins never drained */
            return false;
        }
    }
    atomicAnd(&F->st, ~(GFS_F_DIRTY | GFS_F_REF));
    atomicAdd(&F->st, (GFS_FS_CLAIMED - GFS_FS_EVICTING) << GFS_F_SHIFT);
    count(S, &S->stats.evictions);
    return true;
}

/* Clock (second-chance) allocation.  Returns a frame in state CLAIMED with
 * no pins, owned by the caller, or GFS_NO_FRAME once `budget_ns` is spent.
 * Clean, unpinned, unreferenced (or stale) frames are evicted in passing;
 * dirty frames are written back and evicted only after two full sweeps
 * found nothing clean. */
__device__ __noinline__ uint32_t alloc_frame(gfs_state* S, uint64_t budget_ns) {
    Waiter w(budget_ns);
    const uint32_t n = S->n_frames;
    uint32_t scanned = 0;
    for (;;) {
        uint32_t h = atomicAdd(&S->clock_hand, 1u) % n;
        gfs_frame* F = &S->frames[h];
        uint32_t st = ld_rlx(&F->st);
        uint32_t s = fstate(st);
        if (s == GFS_FS_FREE && (st & GFS_F_PINS) == 0u) {
            if (atomicCAS(&F->st, st, GFS_FS_CLAIMED << GFS_F_SHIFT) == st) return h;
        } else if (s == GFS_FS_VALID && (st & GFS_F_PINS) == 0u) {
            uint64_t key = ld_rlx64(&F->key);
            bool stale = key_stale(S, key);
            if (!stale && (st & GFS_F_REF)) {
                atomicAnd(&F->st, ~GFS_F_REF);
            } else if (!stale && (st & GFS_F_DIRTY)) {
                if (scanned >= 2u * n) {
                    uint32_t f = key_file(key);
                    gfs_file* fe = &S->files[f];
                    uint32_t fst = ld_acq(&fe->st);
                    if (sstatus(fst) == GFS_SS_OPEN &&
                        atomicCAS(&F->st, st, (GFS_FS_EVICTING << GFS_F_SHIFT) | GFS_F_DIRTY) == st) {
                        int rc = writeback_frame(S, h, key, ld_rlx((const uint32_t*)&fe->host_fd),
                                                 ld_rlx((const uint32_t*)&fe->flags));
                        if (rc >= 0) {
                            count(S, &S->stats.writebacks);
                            if (finish_evict(S, h, key, true)) return h;
                        } else {
                            /* put it back: still dirty */
                            atomicAdd(&F->st, (GFS_FS_VALID - GFS_FS_EVICTING) << GFS_F_SHIFT);
                        }
                    }
                }
            } else {
                if (atomicCAS(&F->st, st, GFS_FS_EVICTING << GFS_F_SHIFT | (st & GFS_F_DIRTY)) == st) {
                    if (finish_evict(S, h, key, (st & GFS_F_DIRTY) != 0u)) return h;
                }
            }
        }
        if ((++scanned % n) == 0u || (scanned & 1023u) == 0u) {
            if (!w.tick(4096)) return GFS_NO_FRAME;
        }
    }
}

/* Return a CLAIMED (or LOADING, unpublished) frame we own to FREE. */
__device__ __forceinline__ void release_owned(gfs_state* S, uint32_t fr, uint32_t from_state, uint32_t our_pins) {
    gfs_frame* F = &S->frames[fr];
    st_rlx64(&F->key, ~0ULL);
    __threadfence();
    atomicAdd(&F->st, (uint32_t)(0u - (from_state << GFS_F_SHIFT)) - our_pins);
}

/* pin modes */
#define GFS_PIN_READ 0      /* fill from the host file */
#define GFS_PIN_WFULL 1     /* the caller overwrites the whole page: no fill */
#define GFS_PIN_WPART 2     /* partial write: fill if the file has bytes there */
#define GFS_PIN_WONCE 3     /* write-once file (O_GWRONCE): never fill, zero */
#define GFS_PIN_NOALLOC 8   /* flag: fail with -GFS_ENOMEM quickly instead of waiting long */
#define GFS_PIN_SMFILL 16   /* flag (with READ): the caller fills a missed page of a file with a
                               registered host mapping itself (SM loads from the mapping) instead
                               of a host copy; pin_page then returns it fresh.  A page another
                               caller is still loading is not waited for: -GFS_EAGAIN (a caller
                               holding frames it has yet to fill must not wait on others) */

struct PinFile {
    uint32_t slot, gen;
    int host_fd, oflags;
    uint64_t size;
    uint64_t map_dev; /* the file's registered host mapping (read-only opens), 0 if none */
};

__device__ __forceinline__ PinFile pin_file(gfs_state* S, int fd) {
    PinFile p;
    gfs_file* fe = &S->files[fd];
    p.slot = (uint32_t)fd;
    p.gen = ld_rlx(&fe->gen);
    p.host_fd = (int)ld_rlx((const uint32_t*)&fe->host_fd);
    p.oflags = (int)ld_rlx((const uint32_t*)&fe->flags);
    p.size = ld_rlx64(&fe->size);
    p.map_dev = ld_rlx64(&fe->map_dev);
    return p;
}

/* Page-fault handler (single thread).  On success returns the frame index
 * (>= 0) holding one pin for the caller; *fresh is set when the caller owns
 * a frame that is still LOADING and must initialise it (zero or overwrite)
 * and then call publish_valid().  Negative return = -error. */
__device__ __noinline__ int pin_page(gfs_state* S, const PinFile& pf, uint32_t block, int mode, bool* fresh) {
    *fresh = false;
    const uint64_t key = page_key(pf.slot, pf.gen, block);
    const uint64_t h = fmix64(key);
    const uint32_t bidx = (uint32_t)(h & (S->n_buckets - 1));
    const bool soft = (mode & GFS_PIN_NOALLOC) != 0;
    const bool smfill = (mode & GFS_PIN_SMFILL) != 0;
    mode &= 7;
    Waiter w(S->timeout_ns);
    for (;;) {
        uint32_t fr = index_find(S, key, h);
        if (fr != GFS_NO_FRAME) {
            gfs_frame* F = &S->frames[fr];
            uint32_t old = atom_add_ar(&F->st, 1u);
            uint32_t s = fstate(old);
            if ((s == GFS_FS_VALID || s == GFS_FS_LOADING) && ld_rlx64(&F->key) == key) {
                if (s == GFS_FS_LOADING && smfill) {
                    atomicSub(&F->st, 1u);
                    return -GFS_EAGAIN;
                }
                if (s == GFS_FS_LOADING) {
                    for (;;) {
                        uint32_t cur = ld_acq(&F->st);
                        uint32_t cs = fstate(cur);
                        if (cs == GFS_FS_VALID) break;
                        if (cs != GFS_FS_LOADING || ld_rlx64(&F->key) != key) {
                            atomicSub(&F->st, 1u);
                            return -GFS_EIO; /* the loader failed */
                        }
                        if (!w.tick(1024) || host_stalled(S)) {
                            atomicSub(&F->st, 1u);
                            count(S, &S->stats.timeouts);
                            fail_at(S, GFS_ERRB_TIMEOUT, 4, GFS_ETIMEDOUT); /* LOADING never ended */
                            return -GFS_ETIMEDOUT;
                        }
                    }
                }
                if (!(old & GFS_F_REF)) atomicOr(&F->st, GFS_F_REF);
                return (int)fr;
            }
            atomicSub(&F->st, 1u);
            if (!w.tick(256)) break;
            continue;
        }
        /* miss: allocate outside the bucket lock, insert under it */
        uint32_t nf = alloc_frame(S, soft ? 2000000ull : S->timeout_ns);
        if (nf == GFS_NO_FRAME) {
            if (!soft) { fail_at(S, GFS_ERRB_NOMEM, 5, GFS_ENOMEM); count(S, &S->stats.errors); }
            return -GFS_ENOMEM;
        }
        gfs_frame* F = &S->frames[nf];
        st_rlx64(&F->key, key);
        st_rlx(&F->content, 0u);
        __threadfence();
        /* CLAIMED -> LOADING with our pin */
        atomicAdd(&F->st, ((GFS_FS_LOADING - GFS_FS_CLAIMED) << GFS_F_SHIFT) + 1u);
        if (!spin_lock(&S->bucket_lock[bidx], w)) {
            release_owned(S, nf, GFS_FS_LOADING, 1u);
            count(S, &S->stats.timeouts);
            fail_at(S, GFS_ERRB_TIMEOUT, 6, GFS_ETIMEDOUT);
            return -GFS_ETIMEDOUT;
        }
        if (index_find(S, key, h) != GFS_NO_FRAME) {
            spin_unlock(&S->bucket_lock[bidx]);
            release_owned(S, nf, GFS_FS_LOADING, 1u);
            continue; /* somebody else inserted it first: pin theirs */
        }
        bool ok = index_insert(S, h, nf);
        if (!ok) {
            /* bucket full: evict a clean, unpinned resident of this bucket */
            uint32_t* b = S->index + (size_t)bidx * GFS_WAYS;
            for (int i = 0; i < GFS_WAYS && !ok; i++) {
                uint32_t v = ld_rlx(&b[i]);
                if (!v) continue;
                uint32_t vf = v & 0x3FFFFFu;
                gfs_frame* V = &S->frames[vf];
                uint32_t vst = ld_rlx(&V->st);
                if (fstate(vst) != GFS_FS_VALID || (vst & GFS_F_PINS)) continue;
                uint64_t vkey = ld_rlx64(&V->key);
                bool vstale = key_stale(S, vkey);
                if ((vst & GFS_F_DIRTY) && !vstale) continue;
                if (atomicCAS(&V->st, vst, GFS_FS_EVICTING << GFS_F_SHIFT | (vst & GFS_F_DIRTY)) != vst) continue;
                if (finish_evict(S, vf, vkey, (vst & GFS_F_DIRTY) != 0u)) {
                    /* finish_evict left it CLAIMED and ours: free it */
                    release_owned(S, vf, GFS_FS_CLAIMED, 0u);
                    count(S, &S->stats.conflict_evictions);
                    ok = index_insert(S, h, nf);
                }
            }
        }
        spin_unlock(&S->bucket_lock[bidx]);
        if (!ok) {
            release_owned(S, nf, GFS_FS_LOADING, 1u);
            if (!w.tick(4096)) break;
            continue;
        }
        count(S, &S->stats.misses);
        /* we own the load */
        uint64_t foff = (uint64_t)block << S->log_page;
        bool need_fill = false;
        if (pf.host_fd >= 0 && foff < pf.size) {
            if (mode == GFS_PIN_READ || mode == GFS_PIN_WPART) need_fill = true;
        }
        if (need_fill && smfill && pf.map_dev && pf.oflags == O_GRDONLY) {
            /* the caller copies the page's bytes from the mapping */
            *fresh = true;
            return (int)nf;
        }
        if (need_fill) {
            Req r = {};
            r.op = GFS_OP_READ;
            r.host_fd = pf.host_fd;
            r.file = pf.slot;
            r.offset = foff;
            uint64_t left = pf.size - foff;
            r.length = left < S->page_size ? left : S->page_size;
            r.dev_addr = (uint64_t)(uintptr_t)frame_data(S, nf);
            count(S, &S->stats.read_rpcs);
            int got = rpc_call(S, r, frame_done(S, nf));
            if (got < 0) {
                index_remove(S, key, nf);
                if (got == -GFS_ETIMEDOUT) {
                    /* the host may still complete it later: never reuse */
                    atomicAdd(&F->st, ((GFS_FS_DEAD - GFS_FS_LOADING) << GFS_F_SHIFT) - 1u);
                } else {
                    release_owned(S, nf, GFS_FS_LOADING, 1u);
                }
                return got;
            }
            count(S, &S->stats.bytes_read_rpc, (unsigned long long)got);
            st_rlx(&F->content, (uint32_t)got);
            __threadfence();
            atomicAdd(&F->st, (GFS_FS_VALID - GFS_FS_LOADING) << GFS_F_SHIFT);
            return (int)nf;
        }
        *fresh = true;
        return (int)nf;
    }
    count(S, &S->stats.timeouts);
    fail_at(S, GFS_ERRB_TIMEOUT, 7, GFS_ETIMEDOUT); /* stale pins / full bucket retries */
    return -GFS_ETIMEDOUT;
}

__device__ __forceinline__ void publish_valid(gfs_state* S, uint32_t fr) {
    __threadfence();
    atomicAdd(&S->frames[fr].st, (GFS_FS_VALID - GFS_FS_LOADING) << GFS_F_SHIFT);
}

/* Most valid bytes of a frame the SMs stage for write-back themselves (one
 * warp copies them into a write-stage slot); fuller frames are copied by the
 * host's copy engine, which moves a large page faster than one warp. */
#define GFS_WSTAGE_MAX_BYTES (256u << 10)

/* A free write-stage slot for a frame of `content` valid bytes, or -1 when
 * the frame is too full to stage or no slot is free (the caller then has the
 * host copy the frame).  The bitmap's words are scanned once from a word
 * chosen by `hint`, so concurrent claimers start apart. */
__device__ __forceinline__ int wstage_claim(gfs_state* S, uint32_t hint, uint32_t content) {
    if (content > GFS_WSTAGE_MAX_BYTES || !S->wstage || !S->wstage_slots) return -1;
    const uint32_t nw = (S->wstage_slots + 31u) >> 5;
    for (uint32_t t = 0; t < nw; t++) {
        const uint32_t wi = (hint + t) % nw;
        const uint32_t valid = wi == nw - 1u && (S->wstage_slots & 31u) ? (1u << (S->wstage_slots & 31u)) - 1u : ~0u;
        uint32_t free_ = ~ld_rlx(&S->wstage_bits[wi]) & valid;
        while (free_) {
            const int b = __ffs(free_) - 1;
            if (!(atomicOr(&S->wstage_bits[wi], 1u << b) & (1u << b))) return (int)(wi * 32u + (uint32_t)b);
            free_ &= ~(1u << b);
        }
    }
    return -1;
}
__device__ __forceinline__ void wstage_release(gfs_state* S, int k) {
    atomicAnd(&S->wstage_bits[k >> 5], ~(1u << (k & 31)));
}

/* Write one frame's valid bytes back to the host file (single thread; the
 * caller owns the frame by a pin or by EVICTING).  stage_slot >= 0: the
 * caller has stored the bytes in that write-stage slot (mapped pinned host
 * memory) and the host only merges and writes them -- no device-to-host
 * copy is issued while kernels run; the slot is released here.  Otherwise
 * the host copies the frame. */
__device__ __noinline__ int writeback_frame(gfs_state* S, uint32_t fr, uint64_t key, int host_fd, int oflags,
                                            int stage_slot) {
    gfs_frame* F = &S->frames[fr];
    uint32_t content = ld_rlx(&F->content);
    const int slot = stage_slot;
    if (content == 0u) {
        if (slot >= 0) wstage_release(S, slot);
        return 0;
    }
    Req r = {};
    r.op = GFS_OP_WRITE;
    r.rflags = (oflags == O_GWRONCE) ? GFS_RF_DIFF : 0;
    r.host_fd = host_fd;
    r.file = key_file(key);
    r.offset = (uint64_t)key_block(key) << S->log_page;
    r.length = content;
    r.dev_addr = (uint64_t)(uintptr_t)frame_data(S, fr);
    if (slot >= 0) {
        r.rflags |= GFS_RF_STAGED;
        r.dev_addr = (uint64_t)slot;
    }
    const int rc = rpc_call(S, r, frame_done(S, fr));
    /* the host has finished with the slot once the request completed; after
     * a timeout it may still read it: the slot is then never reused */
    if (slot >= 0 && rc != -GFS_ETIMEDOUT) wstage_release(S, slot);
    return rc;
}

/* First half of a flush of one dirty frame of file `slot` (single thread):
 * 1 = the frame is pinned, its dirty bit cleared and *key_out holds its
 * key (the caller writes it back and calls flush_finish); 0 = nothing to
 * write; < 0 = error. */
__device__ __forceinline__ int flush_prepare(gfs_state* S, uint32_t fr, uint32_t slot, uint32_t gen,
                                             uint64_t* key_out) {
    gfs_frame* F = &S->frames[fr];
    Waiter w(S->timeout_ns);
    for (;;) {
        uint64_t key = ld_rlx64(&F->key);
        if (key_file(key) != slot) return 0;
        uint32_t st = ld_acq(&F->st);
        uint32_t s = fstate(st);
        if (s == GFS_FS_EVICTING) {
            if (!w.tick(1024)) { fail_at(S, GFS_ERRB_TIMEOUT, 8, GFS_ETIMEDOUT); return -GFS_ETIMEDOUT; }
            continue;
        }
        if (s != GFS_FS_VALID || !(st & GFS_F_DIRTY)) return 0;
        if (key_gen(key) != (gen & 0xFFFu)) { /* truncated/invalidated: drop */
            dirty_bit_clear(S, fr);
            atomicAnd(&F->st, ~GFS_F_DIRTY);
            return 0;
        }
        uint32_t old = atom_add_ar(&F->st, 1u);
        if (fstate(old) != GFS_FS_VALID || ld_rlx64(&F->key) != key) { atomicSub(&F->st, 1u); continue; }
        dirty_bit_clear(S, fr);
        uint32_t prev = atom_and_ar(&F->st, ~GFS_F_DIRTY);
        if (!(prev & GFS_F_DIRTY)) {
            unpin(S, fr);
            return 0;
        }
        *key_out = key;
        return 1;
    }
}

/* Second half: after the write-back's result rc, keep the frame dirty on
 * failure and drop the pin. */
__device__ __forceinline__ int flush_finish(gfs_state* S, uint32_t fr, int rc) {
    if (rc < 0) mark_dirty(S, fr); /* keep it for a later attempt */
    else count(S, &S->stats.writebacks);
    unpin(S, fr);
    return rc < 0 ? rc : 0;
}

/* Flush one dirty frame of file `slot` (single thread; the host copies the
 * frame).  Returns 0 or -err. */
__device__ __noinline__ int flush_frame(gfs_state* S, uint32_t fr, uint32_t slot, uint32_t gen, int host_fd, int oflags) {
    uint64_t key = 0;
    const int p = flush_prepare(S, fr, slot, gen, &key);
    if (p <= 0) return p;
    return flush_finish(S, fr, writeback_frame(S, fr, key, host_fd, oflags));
}

/* ------------------------------------------------------------------ */
/* open-file table                                                     */
/* ------------------------------------------------------------------ */
/* A file name as 16 little-endian words, zero padded: read once with
 * independent byte loads (no early exit), so a lookup costs one memory
 * latency instead of one per character. */
struct Name {
    uint32_t w[GFS_NAME_MAX / 4];
    int len;
    uint64_t h;
};
__device__ __forceinline__ void name_load(const char* n, Name& nm) {
#pragma unroll
    for (int i = 0; i < GFS_NAME_MAX / 4; i++)
        nm.w[i] = (uint32_t)(uint8_t)n[4 * i] | ((uint32_t)(uint8_t)n[4 * i + 1] << 8) |
                  ((uint32_t)(uint8_t)n[4 * i + 2] << 16) | ((uint32_t)(uint8_t)n[4 * i + 3] << 24);
    int len = GFS_NAME_MAX;
#pragma unroll
    for (int i = GFS_NAME_MAX / 4 - 1; i >= 0; i--) {
        const uint32_t z = (nm.w[i] - 0x01010101u) & ~nm.w[i] & 0x80808080u; /* lowest set bit: first NUL */
        if (z) len = 4 * i + ((__ffs(z) - 1) >> 3);
    }
    uint64_t h = 1469598103934665603ULL;
#pragma unroll
    for (int i = 0; i < GFS_NAME_MAX / 4; i++) {
        const int keep = len - 4 * i; /* bytes of this word inside the name */
        nm.w[i] &= keep >= 4 ? 0xFFFFFFFFu : (keep <= 0 ? 0u : (1u << (8 * keep)) - 1u);
        for (int k = 0; k < 4 && k < keep; k++) {
            h ^= (nm.w[i] >> (8 * k)) & 0xFFu;
            h *= 1099511628211ULL;
        }
    }
    nm.len = len;
    nm.h = h | 1ULL;
}
/* the slot's stored name (written under the table lock, published by the
 * release store of its state word) against nm, 16 bytes at a time */
__device__ __forceinline__ bool name_eq(const Name& nm, const char* slot_name) {
    const uint4* q = (const uint4*)slot_name;
    bool eq = true;
#pragma unroll
    for (int i = 0; i < GFS_NAME_MAX / 16; i++) {
        uint4 v;
        asm volatile("ld.relaxed.gpu.global.v4.u32 {%0,%1,%2,%3}, [%4];"
                     : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(q + i) : "memory");
        eq = eq && v.x == nm.w[4 * i] && v.y == nm.w[4 * i + 1] && v.z == nm.w[4 * i + 2] && v.w == nm.w[4 * i + 3];
    }
    return eq;
}

__device__ __forceinline__ int file_find(gfs_state* S, const Name& nm) {
    uint32_t mask = S->n_files - 1;
    for (uint32_t p = 0; p < S->n_files; p++) {
        uint32_t i = (uint32_t)(nm.h + p) & mask;
        gfs_file* fe = &S->files[i];
        uint32_t st = ld_acq(&fe->st);
        uint32_t s = sstatus(st);
        if (s == GFS_SS_EMPTY) return -1;
        if (s == GFS_SS_CLAIMING) continue;
        if (ld_rlx64(&fe->hash) == nm.h && name_eq(nm, fe->name)) return (int)i;
    }
    return -1;
}

/* Caller holds the table lock.  Binds `name` to the first empty slot on its
 * probe path, or re-binds a closed, unused, clean slot. */
__device__ __forceinline__ int file_claim(gfs_state* S, const Name& nm) {
    const uint64_t h = nm.h;
    uint32_t mask = S->n_files - 1;
    for (uint32_t p = 0; p < S->n_files; p++) {
        uint32_t i = (uint32_t)(h + p) & mask;
        gfs_file* fe = &S->files[i];
        uint32_t st = ld_acq(&fe->st);
        uint32_t s = sstatus(st);
        bool recyc = (s == GFS_SS_CLOSED && (st & GFS_S_CNT) == 0u);
        if (s != GFS_SS_EMPTY && !recyc) continue;
        uint32_t inc = ((st >> GFS_S_INC_SHIFT) + 1u) & 0xFFu;
        uint32_t claiming = (GFS_SS_CLAIMING << GFS_S_SHIFT) | (inc << GFS_S_INC_SHIFT);
        if (atomicCAS(&fe->st, st, claiming) != st) continue;
#pragma unroll
        for (int k = 0; k < GFS_NAME_MAX / 4; k++) ((volatile uint32_t*)fe->name)[k] = nm.w[k];
        st_rlx64(&fe->hash, h);
        st_rlx((uint32_t*)&fe->host_fd, (uint32_t)-1);
        st_rlx64(&fe->cached_ctime, 0ULL);
        st_rlx64(&fe->cached_size, ~0ULL);
        atomicAdd(&fe->gen, 1u); /* frames of the slot's previous name become stale */
        __threadfence();
        st_rel(&fe->st, (GFS_SS_CLOSED << GFS_S_SHIFT) | (inc << GFS_S_INC_SHIFT));
        return (int)i;
    }
    return -1;
}

/* gopen body (single thread): returns the slot (fd) or -error. */
__device__ __noinline__ int file_open(gfs_state* S, const char* name, int oflags) {
    Name nm;
    name_load(name, nm);
    if (nm.len == 0 || nm.len >= GFS_NAME_MAX) { set_error(S, GFS_ERRB_ARG); return -GFS_EINVAL; }
    const uint64_t h = nm.h;
    Waiter w(S->timeout_ns);
    for (;;) {
        int slot = file_find(S, nm);
        if (slot < 0) {
            if (!spin_lock(&S->table_lock, w)) { set_error(S, GFS_ERRB_TIMEOUT); return -GFS_ETIMEDOUT; }
            slot = file_find(S, nm);
            if (slot < 0) slot = file_claim(S, nm);
            spin_unlock(&S->table_lock);
            if (slot < 0) { set_error(S, GFS_ERRB_TABLE); return -GFS_EMFILE; }
        }
        gfs_file* fe = &S->files[slot];
        for (;;) {
            uint32_t st = ld_acq(&fe->st);
            if (ld_rlx64(&fe->hash) != h || !name_eq(nm, fe->name)) break; /* re-bound: find again */
            uint32_t s = sstatus(st), cnt = st & GFS_S_CNT;
            uint32_t inc_bits = st & GFS_S_INC_MASK;
            if (s == GFS_SS_OPEN) {
                /* fetch-and-add (never retried under contention); it holds if
                 * status and incarnation were unchanged, else it is undone */
                const uint32_t old = atomicAdd(&fe->st, 1u);
                if ((old & ~GFS_S_CNT) == (st & ~GFS_S_CNT)) return slot;
                atomicSub(&fe->st, 1u);
                continue;
            }
            if (s == GFS_SS_CLOSED && cnt == 0u) {
                uint32_t opening = (GFS_SS_OPENING << GFS_S_SHIFT) | inc_bits | 1u;
                if (atomicCAS(&fe->st, st, opening) != st) continue;
                /* we are the opener */
                st_rlx((uint32_t*)&fe->flags, (uint32_t)oflags);
                Req r = {};
                r.op = GFS_OP_OPEN;
                r.file = (uint32_t)slot;
                r.oflags = oflags;
                r.name = fe->name;
                count(S, &S->stats.opens);
                int rc = rpc_call(S, r, file_done(S, (uint32_t)slot));
                if (rc >= 0) {
                    /* the reply sits in mapped host memory: copy it in */
                    const gfs_open_reply* rep = S->hreply + slot;
                    st_rlx((uint32_t*)&fe->host_fd, ld_rlx_sys((const uint32_t*)&rep->host_fd));
                    st_rlx((uint32_t*)&fe->err, 0u);
                    st_rlx64(&fe->size, ld_rlx_sys64(&rep->size));
                    st_rlx64((uint64_t*)&fe->ctime_ns, ld_rlx_sys64((const uint64_t*)&rep->ctime_ns));
                    st_rlx64(&fe->map_dev, ld_rlx_sys64(&rep->map_dev));
                    __threadfence();
                }
                if (rc < 0) {
                    st_rlx((uint32_t*)&fe->err, (uint32_t)(-rc));
                    __threadfence();
                    uint32_t to = (rc == -GFS_ETIMEDOUT) ? GFS_SS_BROKEN : GFS_SS_CLOSED;
                    atomicAdd(&fe->st, ((to - GFS_SS_OPENING) << GFS_S_SHIFT) - 1u);
                    return rc;
                }
                int64_t ct = ld_rlxs64(&fe->ctime_ns);
                uint64_t sz = ld_rlx64(&fe->size);
                if ((uint64_t)ct != ld_rlx64(&fe->cached_ctime) || sz != ld_rlx64(&fe->cached_size)) {
                    atomicAdd(&fe->gen, 1u); /* host copy changed: cached pages are stale */
                    st_rlx64(&fe->cached_ctime, (uint64_t)ct);
                    st_rlx64(&fe->cached_size, sz);
                }
                __threadfence();
                atomicAdd(&fe->st, (GFS_SS_OPEN - GFS_SS_OPENING) << GFS_S_SHIFT);
                return slot;
            }
            if (s == GFS_SS_OPENING) {
                if (atomicCAS(&fe->st, st, st + 1u) != st) continue;
                for (;;) {
                    uint32_t cur = ld_acq(&fe->st);
                    uint32_t cs = sstatus(cur);
                    if (cs == GFS_SS_OPEN) return slot;
                    if (cs != GFS_SS_OPENING) {
                        atomicSub(&fe->st, 1u);
                        int e = (int)ld_rlx((const uint32_t*)&fe->err);
                        return -(e ? e : GFS_EIO);
                    }
                    if (!w.tick(2048)) {
                        atomicSub(&fe->st, 1u);
                        set_error(S, GFS_ERRB_TIMEOUT);
                        return -GFS_ETIMEDOUT;
                    }
                }
            }
            if (s == GFS_SS_BROKEN) return -GFS_EIO;
            if (!w.tick(2048)) { set_error(S, GFS_ERRB_TIMEOUT); return -GFS_ETIMEDOUT; }
        }
        if (!w.tick(256)) { set_error(S, GFS_ERRB_TIMEOUT); return -GFS_ETIMEDOUT; }
    }
}

/* First half of gclose (single thread): 0 = others still hold it, 1 = we are
 * the last closer (status CLOSING), <0 = error. */
__device__ __forceinline__ int file_close_begin(gfs_state* S, int fd) {
    if (fd < 0 || (uint32_t)fd >= S->n_files) return -GFS_EBADF;
    gfs_file* fe = &S->files[fd];
    const uint32_t st = ld_acq(&fe->st);
    if (sstatus(st) != GFS_SS_OPEN || (st & GFS_S_CNT) == 0u) return -GFS_EBADF; /* not open */
    /* The caller holds one count, so the slot stays OPEN until it drops it:
     * fetch-and-subtract; the closer that takes the count to zero then moves
     * the slot to CLOSING, unless an opener came in first (that opener then
     * holds the file and will close it). */
    const uint32_t old = atomicSub(&fe->st, 1u);
    if ((old & GFS_S_CNT) > 1u) return 0;
    const uint32_t zero = old - 1u;
    const uint32_t closing = (GFS_SS_CLOSING << GFS_S_SHIFT) | (zero & GFS_S_INC_MASK);
    return atomicCAS(&fe->st, zero, closing) == zero ? 1 : 0;
}

__device__ __forceinline__ int file_close_finish(gfs_state* S, int fd) {
    gfs_file* fe = &S->files[fd];
    Req r = {};
    r.op = GFS_OP_CLOSE;
    r.host_fd = (int)ld_rlx((const uint32_t*)&fe->host_fd);
    r.file = (uint32_t)fd;
    count(S, &S->stats.closes);
    int rc = rpc_call(S, r, file_done(S, (uint32_t)fd));
    __threadfence();
    uint32_t to = (rc == -GFS_ETIMEDOUT) ? GFS_SS_BROKEN : GFS_SS_CLOSED;
    atomicAdd(&fe->st, (to - GFS_SS_CLOSING) << GFS_S_SHIFT);
    return rc < 0 ? rc : 0;
}

/* ------------------------------------------------------------------ */
/* copies                                                              */
/* ------------------------------------------------------------------ */
/* Warp-cooperative copy of n bytes; 16-byte vectors with cache-global
 * loads when src and dst share their alignment mod 16 (the reference's
 * copy_block_16, util.cu.h:161-236, used ld.cv/st.wt for the same job). */
__device__ __forceinline__ void warp_copy(uint8_t* dst, const uint8_t* src, size_t n, int lane) {
    uintptr_t d = (uintptr_t)dst, s = (uintptr_t)src;
    const bool sg = __isGlobal(src) != 0; /* a user buffer may be in shared memory */
    if (((d ^ s) & 15u) == 0u) {
        size_t head = (16u - (s & 15u)) & 15u;
        if (head > n) head = n;
        if ((size_t)lane < head) dst[lane] = src[lane];
        size_t n4 = (n - head) >> 4;
        uint4* d4 = (uint4*)(dst + head);
        const uint4* s4 = (const uint4*)(src + head);
        size_t i = (size_t)lane;
        for (; i + 96 < n4; i += 128) {
            uint4 a = ld_user4(s4 + i, sg), b = ld_user4(s4 + i + 32, sg), c = ld_user4(s4 + i + 64, sg),
                  e = ld_user4(s4 + i + 96, sg);
            d4[i] = a; d4[i + 32] = b; d4[i + 64] = c; d4[i + 96] = e;
        }
        for (; i < n4; i += 32) d4[i] = ld_user4(s4 + i, sg);
        size_t t0 = head + (n4 << 4);
        for (size_t k = t0 + (size_t)lane; k < n; k += 32) dst[k] = src[k];
    } else if (((d ^ s) & 3u) == 0u) {
        size_t head = (4u - (s & 3u)) & 3u;
        if (head > n) head = n;
        if ((size_t)lane < head) dst[lane] = src[lane];
        size_t n1 = (n - head) >> 2;
        uint32_t* d1 = (uint32_t*)(dst + head);
        const uint32_t* s1 = (const uint32_t*)(src + head);
        for (size_t i = (size_t)lane; i < n1; i += 32) d1[i] = sg ? __ldcg(s1 + i) : s1[i];
        for (size_t k = head + (n1 << 2) + (size_t)lane; k < n; k += 32) dst[k] = src[k];
    } else {
        for (size_t k = (size_t)lane; k < n; k += 32) dst[k] = src[k];
    }
}

__device__ __forceinline__ void warp_zero(uint8_t* dst, size_t n, int lane) {
    uintptr_t d = (uintptr_t)dst;
    size_t head = (16u - (d & 15u)) & 15u;
    if (head > n) head = n;
    if ((size_t)lane < head) dst[lane] = 0;
    size_t n4 = (n - head) >> 4;
    uint4* d4 = (uint4*)(dst + head);
    for (size_t i = (size_t)lane; i < n4; i += 32) d4[i] = make_uint4(0, 0, 0, 0);
    for (size_t k = head + (n4 << 4) + (size_t)lane; k < n; k += 32) dst[k] = 0;
}

} // namespace
} // namespace gfsd

#endif
