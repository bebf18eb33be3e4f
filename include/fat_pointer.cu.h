/*
 * File-backed "fat pointers": gvmmap() and FatPointer<T, N>, the interface of
 * libgpufs/fat_pointer.cu.h and fs_calls.cu.h:55-61.  A fat pointer names a
 * position in an open file; dereferencing it maps the page under that
 * position through the buffer cache and yields a reference into the page,
 * and moving it is pointer arithmetic in elements of T.
 *
 * Design here:
 *   - each thread's pointer holds at most one page pinned; it is remapped
 *     only when a dereference leaves that page;
 *   - lanes of a warp that want the same page of the same file share one
 *     pin request (the pin count is the number of lanes), so a warp that
 *     walks one page costs one lookup;
 *   - TLB<N> is accepted for source compatibility; translations go straight
 *     to the buffer cache's lock-free index, so no translation cache is kept
 *     (N only selects the type);
 *   - on a writable file, releasing a page marks it dirty and extends the
 *     page content and the file size to the furthest byte dereferenced
 *     through the pointer (reads through a writable pointer count too); the
 *     bytes reach the host file at gclose/gfsync, as with gmmap;
 *   - a dereference that cannot be mapped (pool exhausted, read past the end
 *     of a read-only file) returns a reference to a per-lane sink of 128
 *     bytes and records the failure in the session's error bits.
 * Calls may be made from divergent code: each step involves only the lanes
 * that make it.
 */
#ifndef FAT_POINTER_CU
#define FAT_POINTER_CU

#include <stddef.h>
#include <stdint.h>
#include <sys/types.h>

__device__ int gfs_fp_acquire(int fd, unsigned long long off, int ref, int* fresh);
__device__ unsigned char* gfs_fp_data(int frame);
__device__ void gfs_fp_publish(int frame);
__device__ unsigned int gfs_fp_log_page();
__device__ void gfs_fp_release(int frame, int ref, unsigned int touched, unsigned long long page_start);
__device__ unsigned char* gfs_fp_sink();

template <int N>
struct TLB {
    int reserved; /* no translation cache is needed; see above */
};

template <typename T, int N>
class FatPointer {
  public:
    __device__ FatPointer(int fd, off_t start, size_t size, int flags)
        : fd_(fd), flags_(flags), start_((unsigned long long)start), end_((unsigned long long)start + size),
          pos_((unsigned long long)start) {}
    __device__ FatPointer(const FatPointer& o)
        : fd_(o.fd_), flags_(o.flags_), start_(o.start_), end_(o.end_), pos_(o.pos_) {}
    __device__ ~FatPointer() { release(); }

    __device__ FatPointer& operator=(const FatPointer& o) {
        if (this != &o) {
            release();
            fd_ = o.fd_;
            flags_ = o.flags_;
            start_ = o.start_;
            end_ = o.end_;
            pos_ = o.pos_;
        }
        return *this;
    }
    /* absolute position: `offset` bytes from the mapping's start */
    __device__ FatPointer& moveTo(size_t offset) {
        pos_ = start_ + offset;
        return *this;
    }
    /* relative move in elements of T */
    __device__ FatPointer& move(size_t n) {
        pos_ += (unsigned long long)n * sizeof(T);
        return *this;
    }
    __device__ FatPointer& operator+=(size_t n) { return move(n); }
    __device__ FatPointer& operator-=(size_t n) { return move((size_t)0 - n); }
    __device__ FatPointer& operator++() { return move(1); }
    __device__ FatPointer& operator--() { return move((size_t)0 - 1); }

    __device__ T& operator*() {
        const unsigned lp = gfs_fp_log_page();
        const unsigned long long page = pos_ >> lp;
        if (frame_ < 0 || page != page_) acquire(page, lp);
        const unsigned int in_page = (unsigned int)(pos_ & ((1ull << lp) - 1ull));
        if (!base_) return *(T*)gfs_fp_sink();
        const unsigned int end = in_page + (unsigned int)sizeof(T);
        if (end > touched_) touched_ = end;
        return *(T*)(base_ + in_page);
    }
    /* element i from the current position (the pointer's page follows it) */
    __device__ T& operator[](size_t i) {
        pos_ += (unsigned long long)i * sizeof(T);
        T& r = **this;
        pos_ -= (unsigned long long)i * sizeof(T);
        return r;
    }
    /* bytes from the mapping's start */
    __device__ size_t offset() const { return (size_t)(pos_ - start_); }
    /* drop the pinned page now (it is dropped on destruction otherwise) */
    __device__ void release() {
        const unsigned mask = __activemask();
        const unsigned lane = threadIdx.x & 31u;
        unsigned want = __ballot_sync(mask, frame_ >= 0);
        while (want) {
            const int leader = __ffs(want) - 1;
            const int lf = __shfl_sync(mask, frame_, leader);
            const bool mine = frame_ >= 0 && frame_ == lf;
            const unsigned same = __ballot_sync(mask, mine);
            const unsigned touched = __reduce_max_sync(mask, mine ? touched_ : 0u);
            if ((int)lane == leader) gfs_fp_release(lf, __popc(same), touched, page_ << gfs_fp_log_page());
            if (mine) {
                frame_ = -1;
                base_ = nullptr;
                touched_ = 0;
            }
            want &= ~same;
        }
    }

  private:
    /* map the page holding pos_ (warp-aggregated per (file, page)) */
    __device__ void acquire(unsigned long long page, unsigned lp) {
        release();
        const unsigned mask = __activemask();
        const unsigned lane = threadIdx.x & 31u;
        unsigned need = mask;
        while (need) {
            const int leader = __ffs(need) - 1;
            const int lfd = __shfl_sync(mask, fd_, leader);
            const unsigned long long lpage = __shfl_sync(mask, page, leader);
            const bool mine = ((need >> lane) & 1u) && fd_ == lfd && page == lpage;
            const unsigned same = __ballot_sync(mask, mine);
            int fr = -1, fresh = 0;
            if ((int)lane == leader) fr = gfs_fp_acquire(lfd, lpage << lp, __popc(same), &fresh);
            fr = __shfl_sync(mask, fr, leader);
            fresh = __shfl_sync(mask, fresh, leader);
            if (fr >= 0 && fresh) {
                /* a new write-once page: zeroed by its lanes, then published */
                unsigned char* d = gfs_fp_data(fr);
                const unsigned rank = __popc(same & ((1u << lane) - 1u)), cnt = __popc(same);
                if (mine)
                    for (unsigned long long k = (unsigned long long)rank * 16u; k < (1ull << lp); k += cnt * 16ull)
                        *(uint4*)(d + k) = make_uint4(0u, 0u, 0u, 0u);
                __syncwarp(mask);
                if ((int)lane == leader) gfs_fp_publish(fr);
                __syncwarp(mask);
            }
            if (mine) {
                frame_ = fr;
                page_ = lpage;
                base_ = fr >= 0 ? gfs_fp_data(fr) : nullptr;
                touched_ = 0;
            }
            need &= ~same;
        }
    }

    int fd_;
    int flags_;
    unsigned long long start_, end_, pos_;
    int frame_ = -1;
    unsigned long long page_ = ~0ull;
    unsigned char* base_ = nullptr;
    unsigned int touched_ = 0;
};

/* fs_calls.cu.h:55-61: a fat pointer at byte `offset` of fd over `size` bytes */
template <typename T, int N>
__device__ FatPointer<T, N> gvmmap(void* addr, size_t size, int prot, int flags, int fd, off_t offset, TLB<N>* tlb) {
    (void)addr;
    (void)prot;
    (void)tlb;
    return FatPointer<T, N>(fd, offset, size, flags);
}

#endif
