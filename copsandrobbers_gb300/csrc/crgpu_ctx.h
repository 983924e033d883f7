// crgpu_ctx.h - the context object behind the C ABI (shared by the API translation units).
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

// Device blocks a context keeps after the solver that used them is destroyed, so that the next
// solve of a similar size on the same context (the one-call cr_solve in a loop, a solve server's
// worker) takes them instead of calling cudaMalloc and cudaFree, which map and unmap pages and
// synchronise the device.  Only blocks of at least kMinBytes are kept; the free ones are held up
// to `limit` bytes (the largest go first); a block is reused for a request of at least two
// thirds of its size.  Reuse is ordered by the context's stream, the only stream its solvers use;
// blocks come back only from destroyed solvers, whose work has completed.  A solver may be
// destroyed from another thread than the one solving on the context (a solve server's client
// releasing a table), so the cache takes a lock.
struct cr_block_cache {
    static constexpr size_t kMinBytes = 1u << 20;
    struct Block {
        void* p;
        size_t bytes;
        bool used;
    };
    std::vector<Block> blocks;
    size_t limit = 4ull << 30;
    std::mutex mu;

    cudaError_t get(void** out, size_t bytes) {
        std::lock_guard<std::mutex> lock(mu);
        *out = nullptr;
        if (bytes >= kMinBytes) {
            int best = -1;
            for (int i = 0; i < (int)blocks.size(); ++i) {
                const Block& b = blocks[i];
                if (!b.used && b.bytes >= bytes && b.bytes - bytes <= bytes / 2 &&
                    (best < 0 || b.bytes < blocks[best].bytes))
                    best = i;
            }
            if (best >= 0) {
                blocks[best].used = true;
                *out = blocks[best].p;
                return cudaSuccess;
            }
        }
        cudaError_t e = cudaMalloc(out, bytes);
        if (e == cudaErrorMemoryAllocation) {   // give the held blocks back and try once more
            cudaGetLastError();
            release_free();
            e = cudaMalloc(out, bytes);
        }
        if (e == cudaSuccess && bytes >= kMinBytes && limit > 0) blocks.push_back(Block{*out, bytes, true});
        return e;
    }
    void put(void* p) {
        if (!p) return;
        std::lock_guard<std::mutex> lock(mu);
        for (Block& b : blocks)
            if (b.p == p) {
                b.used = false;
                trim();
                return;
            }
        cudaFree(p);
    }
    size_t free_bytes() const {
        size_t t = 0;
        for (const Block& b : blocks)
            if (!b.used) t += b.bytes;
        return t;
    }
    void trim() {
        while (free_bytes() > limit) {
            int big = -1;
            for (int i = 0; i < (int)blocks.size(); ++i)
                if (!blocks[i].used && (big < 0 || blocks[i].bytes > blocks[big].bytes)) big = i;
            cudaFree(blocks[big].p);
            blocks.erase(blocks.begin() + big);
        }
    }
    void set_limit(size_t bytes) {
        std::lock_guard<std::mutex> lock(mu);
        limit = bytes;
        trim();
    }
    void clear() {
        std::lock_guard<std::mutex> lock(mu);
        release_free();
    }
    // (the callers below hold the lock)
    void release_free() {
        for (size_t i = 0; i < blocks.size();) {
            if (!blocks[i].used) {
                cudaFree(blocks[i].p);
                blocks.erase(blocks.begin() + i);
            } else {
                ++i;
            }
        }
    }
};

struct cr_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 1;
    bool profiling = false;
    std::string err;
    cr_block_cache cache;
};
