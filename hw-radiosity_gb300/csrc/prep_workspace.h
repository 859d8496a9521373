// Host-side resources of scene preparation and handle creation:
//   PrepWorkspace  per host thread and device, a stream and grow-only device
//                  buffers for the preparation kernels (octree overlap tests,
//                  neighbour links, table expansion), kept between calls;
//   PinnedStage    per host thread, grow-only pinned staging for uploads and
//                  downloads;
//   HostPool       the process's pool of host threads for the packing passes
//                  (split_range, for_each_item, copy_segments);
//   HostLayout, DevBlock  offsets of pieces in one staging buffer or one
//                  device allocation.
// A batch of small scenes then pays neither a stream creation nor a
// synchronising cudaFree per scene.  Each call finishes its work on the
// stream before it returns, so consecutive calls on one thread can share the
// buffers; calls from different threads use their own.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

namespace radgb {

class PrepWorkspace {
public:
    explicit PrepWorkspace(int device) : device_(device) {}
    ~PrepWorkspace() {
        int cur = 0;
        if (cudaGetDevice(&cur) != cudaSuccess) return;   // the runtime is already shutting down
        cudaSetDevice(device_);
        for (auto& b : bufs_)
            if (b.p) cudaFree(b.p);
        if (stream_) cudaStreamDestroy(stream_);
        cudaSetDevice(cur);
    }
    PrepWorkspace(const PrepWorkspace&) = delete;
    PrepWorkspace& operator=(const PrepWorkspace&) = delete;

    // the workspace's stream (created on first use, with the device current)
    cudaError_t stream(cudaStream_t* out) {
        if (!stream_) {
            cudaError_t e = cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking);
            if (e != cudaSuccess) return e;
        }
        *out = stream_;
        return cudaSuccess;
    }
    // buffer k with at least `bytes` bytes; its contents are not kept when it grows
    cudaError_t buffer(std::size_t k, std::size_t bytes, void** out) {
        if (bufs_.size() <= k) bufs_.resize(k + 1);
        Buf& b = bufs_[k];
        if (bytes > b.cap) {
            if (b.p) {
                cudaStreamSynchronize(stream_);
                cudaFree(b.p);
                b.p = nullptr;
                b.cap = 0;
            }
            const std::size_t cap = bytes > 2 * b.cap ? bytes : 2 * b.cap;
            cudaError_t e = cudaMalloc(&b.p, cap ? cap : 16);
            if (e != cudaSuccess) return e;
            b.cap = cap;
        }
        *out = b.p;
        return cudaSuccess;
    }

private:
    struct Buf {
        void* p = nullptr;
        std::size_t cap = 0;
    };
    int device_;
    cudaStream_t stream_ = nullptr;
    std::vector<Buf> bufs_;
};

// Pinned host staging for uploads and downloads, per host thread, grow-only
// and kept between calls.  The records a handle uploads are packed into it
// and copied from it: packing into fresh pageable vectors paid a page fault
// per 4 KB, and copying straight from the scene's pageable memory made the
// host's next writes to those pages fault instead.  A call finishes its copies
// before it returns, so the next call on the thread may reuse the buffer.
class PinnedStage {
public:
    ~PinnedStage() {
        int cur = 0;
        if (p_ && cudaGetDevice(&cur) == cudaSuccess) cudaFreeHost(p_);
    }
    cudaError_t get(std::size_t bytes, void** out) {
        if (bytes > cap_) {
            const std::size_t cap = bytes > 2 * cap_ ? bytes : 2 * cap_;
            if (p_) cudaFreeHost(p_);
            p_ = nullptr;
            cap_ = 0;
            cudaError_t e = cudaHostAlloc(&p_, cap, cudaHostAllocPortable);
            if (e != cudaSuccess) return e;
            cap_ = cap;
        }
        *out = p_;
        return cudaSuccess;
    }

private:
    void* p_ = nullptr;
    std::size_t cap_ = 0;
};

inline PinnedStage& pinned_stage() {
    thread_local PinnedStage stage;
    return stage;
}

// Host threads for the packing passes of large scenes (the record packing of
// an upload, the unpacking of a download): started on first use and kept for
// the process, so a pass pays a wake-up, not a thread creation per chunk.  One
// pass at a time; a caller that finds the pool busy runs its pass itself.
// The pool is never destroyed: its idle workers wait on a condition variable
// until the process ends, so no exit-time destructor joins threads (which a
// forked child does not have).
class HostPool {
public:
    static HostPool& get() {
        static HostPool* pool = new HostPool();
        return *pool;
    }
    // f(a, b) over [0, n) in `parts` contiguous chunks, claimed in order by
    // the caller and up to threads - 1 workers; false (nothing run) when
    // another pass holds the pool or no worker could be started
    template <typename F>
    bool run(int n, int parts, int threads, F& f) {
        std::unique_lock<std::mutex> busy(busy_, std::try_to_lock);
        if (!busy.owns_lock()) return false;
        try {
            while ((int)workers_.size() < threads - 1) workers_.emplace_back([this] { work(); });
        } catch (...) {
            if (workers_.empty()) return false;
        }
        Pass p;
        {
            std::lock_guard<std::mutex> g(m_);
            pass_ = {[](void* ctx, int a, int b) { (*static_cast<F*>(ctx))(a, b); }, &f, n, parts, ++gen_};
            p = pass_;
            done_.store(0);
            ticket_.store((unsigned long long)p.gen << 32);
        }
        wake_.notify_all();
        take(p);
        while (done_.load(std::memory_order_acquire) < parts) std::this_thread::yield();
        return true;
    }

private:
    struct Pass {
        void (*call)(void*, int, int);
        void* ctx;
        int n, parts;
        unsigned gen;
    };
    HostPool() = default;
    // claim chunks of pass p until none is left; a ticket holds the pass
    // number and its next chunk, so a worker still holding an older pass
    // never claims a chunk of a newer one
    void take(const Pass& p) {
        unsigned long long t = ticket_.load();
        for (;;) {
            if ((unsigned)(t >> 32) != p.gen || (int)(t & 0xffffffffu) >= p.parts) return;
            if (!ticket_.compare_exchange_weak(t, t + 1)) continue;
            const int k = (int)(t & 0xffffffffu);
            p.call(p.ctx, (int)((long long)p.n * k / p.parts), (int)((long long)p.n * (k + 1) / p.parts));
            done_.fetch_add(1, std::memory_order_release);
            t = ticket_.load();
        }
    }
    void work() {
        unsigned seen = 0;
        for (;;) {
            Pass p;
            {
                std::unique_lock<std::mutex> g(m_);
                wake_.wait(g, [&] { return gen_ != seen; });
                p = pass_;
                seen = p.gen;
            }
            take(p);
        }
    }
    std::mutex busy_, m_;
    std::condition_variable wake_;
    std::vector<std::thread> workers_;
    Pass pass_ = {nullptr, nullptr, 0, 0, 0};
    std::atomic<unsigned long long> ticket_{0};
    std::atomic<int> done_{0};
    unsigned gen_ = 0;
};

// f(a, b) over [0, n) in `jobs` contiguous chunks on the host pool, or on the
// caller's thread when jobs is 1 or the pool is busy
template <typename F>
void split_range(int n, int jobs, F f) {
    if (jobs > 64) jobs = 64;
    if (jobs <= 1 || n <= 1 || !HostPool::get().run(n, jobs, jobs, f)) f(0, n);
}

// f(k) for every k in [0, n), items claimed one at a time by `jobs` threads
// of the host pool (for items of uneven cost, such as the scenes of a batch)
template <typename F>
void for_each_item(int n, int jobs, F f) {
    if (jobs > 64) jobs = 64;
    auto chunk = [&](int a, int b) {
        for (int k = a; k < b; k++) f(k);
    };
    if (jobs <= 1 || n <= 1 || !HostPool::get().run(n, n, jobs, chunk)) chunk(0, n);
}

// host threads for a packing pass over n slots: one per 4,096 slots up to
// the -jobs option and 16, none below 16,384 slots
inline int pack_jobs(int n, int opt_jobs) {
    if (n < 16384) return 1;
    int j = n / 4096;
    if (j > opt_jobs) j = opt_jobs;
    if (j > 16) j = 16;
    return j < 1 ? 1 : j;
}

// Offsets of consecutive pieces in one buffer, each at a 256-byte boundary.
struct HostLayout {
    std::size_t size = 0;
    std::size_t add(std::size_t bytes) {
        const std::size_t at = size;
        size += (bytes + 255) & ~std::size_t(255);
        return at;
    }
};

// Arrays carved from one device allocation: add() each pointer with its
// element count, then carve() the allocation of `size` bytes.
struct DevBlock {
    std::size_t size = 0;
    std::vector<std::pair<void**, std::size_t>> at;
    template <typename U>
    void add(U** p, std::size_t count) {
        at.emplace_back(reinterpret_cast<void**>(p), size);
        size += (count * sizeof(U) + 255) & ~std::size_t(255);
    }
    void carve(void* base) {
        for (auto& a : at) *a.first = static_cast<char*>(base) + a.second;
    }
};

// Host copies of several pieces, the bytes split evenly over `jobs` threads
// of the host pool.
struct CopySeg {
    void* dst;
    const void* src;
    std::size_t bytes;
};
inline void copy_segments(const std::vector<CopySeg>& segs, int jobs) {
    std::size_t total = 0;
    for (const CopySeg& g : segs) total += g.bytes;
    if (total < (std::size_t)1 << 20) jobs = 1;        // below 1 MB one thread copies it
    const int parts = jobs < 1 ? 1 : jobs;
    auto part = [&](int a, int b) {
        for (int k = a; k < b; k++) {
            const std::size_t lo = total * k / parts, hi = total * (k + 1) / parts;
            std::size_t base = 0;
            for (const CopySeg& g : segs) {
                const std::size_t s0 = lo > base ? lo - base : 0, s1 = hi - base < g.bytes ? hi - base : g.bytes;
                if (hi > base && s0 < g.bytes && s1 > s0)
                    std::memcpy(static_cast<char*>(g.dst) + s0, static_cast<const char*>(g.src) + s0, s1 - s0);
                base += g.bytes;
                if (base >= hi) break;
            }
        }
    };
    split_range(parts, parts, part);
}

// this thread's workspace for `device` (the device must be current)
inline PrepWorkspace& prep_workspace(int device) {
    thread_local std::vector<std::unique_ptr<PrepWorkspace>> per_device;
    if ((int)per_device.size() <= device) per_device.resize((std::size_t)device + 1);
    if (!per_device[(std::size_t)device]) per_device[(std::size_t)device].reset(new PrepWorkspace(device));
    return *per_device[(std::size_t)device];
}

}  // namespace radgb
