// Scratch of the scene-preparation kernels (octree overlap tests, neighbour
// links): per host thread and device, a stream and grow-only device buffers
// kept between calls.  A batch of small scenes then pays neither a stream
// creation nor a synchronising cudaFree per scene.  Each call finishes its
// work on the stream before it returns, so consecutive calls on one thread
// can share the buffers; calls from different threads use their own.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <memory>
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
            if (p_) cudaFreeHost(p_);
            p_ = nullptr;
            cap_ = 0;
            const std::size_t cap = bytes > 2 * cap_ ? bytes : 2 * cap_;
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

// this thread's workspace for `device` (the device must be current)
inline PrepWorkspace& prep_workspace(int device) {
    thread_local std::vector<std::unique_ptr<PrepWorkspace>> per_device;
    if ((int)per_device.size() <= device) per_device.resize((std::size_t)device + 1);
    if (!per_device[(std::size_t)device]) per_device[(std::size_t)device].reset(new PrepWorkspace(device));
    return *per_device[(std::size_t)device];
}

}  // namespace radgb
