// crgpu_tables.cu - configuration table and successor CSR on the device.
//
//   k_unrank       AuxGraph::generateCopConfigs (lib/include/AuxGraph.h:117-177): config id ->
//                  sorted cop multiset, the inverse of config_rank().
//   k_trans_count  AuxGraph::createTransitions (lib/include/AuxGraph.h:179-275): per config,
//   k_trans_fill   the successor configs of one simultaneous cop move, sorted and
//                  deduplicated, stored as next id * n (the value the reference's table file
//                  holds).  One warp per config sorts its successor ranks in shared memory.
#include "crgpu_internal.cuh"

namespace crgpu {

// Largest x in [prev, n-1] with B[i][x] >= need (B[i][.] is non-increasing in x).
__device__ __forceinline__ int unrank_step(const uint32_t* B, int np1, int i, int prev, int n,
                                           uint32_t need) {
    int lo = prev, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (B[i * np1 + mid] >= need) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_unrank(const uint32_t* __restrict__ B, int n, int k, uint32_t C, uint16_t* out) {
    const int np1 = n + 1;
    for (uint32_t cid = blockIdx.x * blockDim.x + threadIdx.x; cid < C; cid += gridDim.x * blockDim.x) {
        uint32_t rem = cid;
        int prev = 0;
        for (int i = 0; i < k; ++i) {
            const uint32_t top = B[i * np1 + prev];
            const int x = unrank_step(B, np1, i, prev, n, top - rem);
            rem -= top - B[i * np1 + x];
            out[(size_t)cid * k + i] = (uint16_t)x;
            prev = x;
        }
    }
}

// Sorted successor ranks of one config in per-warp shared memory (bitonic sort over a
// power-of-two span, padded with 0xFFFFFFFF).  Returns the number of unique entries, which
// are left at buf[0 .. uniq) when compact is set.
template <int K>
__device__ int warp_successors(const uint16_t* __restrict__ cc, const uint32_t* __restrict__ rp,
                               const uint16_t* __restrict__ adj, const uint32_t* __restrict__ B,
                               int np1, uint32_t* buf, int cap, int lane, bool* overflow) {
    int lo[K], dg[K];
    int T = 1;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        int v = cc[i];
        lo[i] = rp[v];
        dg[i] = rp[v + 1] - lo[i];
        T *= dg[i];
    }
    if (T > cap) { *overflow = true; return 0; }
    int P = 1;
    while (P < T) P <<= 1;
    for (int t = lane; t < P; t += 32) {
        uint32_t s = 0xFFFFFFFFu;
        if (t < T) {
            int c[K];
            int rem = t;
#pragma unroll
            for (int i = K - 1; i >= 0; --i) {
                int q = rem / dg[i];
                c[i] = adj[lo[i] + rem - q * dg[i]];
                rem = q;
            }
            sort_small<K>(c);
            s = config_rank<K>(c, B, np1);
        }
        buf[t] = s;
    }
    __syncwarp();
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < P; t += 32) {
                int partner = t ^ stride;
                if (partner > t) {
                    bool up = (t & size) == 0;
                    uint32_t a = buf[t], b = buf[partner];
                    if ((a > b) == up) { buf[t] = b; buf[partner] = a; }
                }
            }
            __syncwarp();
        }
    }
    // unique count: first occurrences among the T real entries
    int uniq = 0;
    for (int t0 = 0; t0 < T; t0 += 32) {
        int t = t0 + lane;
        bool first = t < T && (t == 0 || buf[t] != buf[t - 1]);
        unsigned b = __ballot_sync(0xFFFFFFFFu, first);
        uniq += __popc(b);
    }
    return uniq;
}

template <int K>
__global__ void k_trans(const uint16_t* __restrict__ configs, uint32_t C, int n,
                        const uint32_t* __restrict__ rp, const uint16_t* __restrict__ adj,
                        const uint32_t* __restrict__ B, int cap, unsigned long long* counts,
                        const unsigned long long* __restrict__ heads, unsigned long long* data,
                        unsigned int* err) {
    extern __shared__ uint32_t sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* buf = sm + warp * cap;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    bool overflow = false;
    for (uint32_t cid = blockIdx.x * (blockDim.x >> 5) + warp; cid < C; cid += nwarps) {
        int u = warp_successors<K>(configs + (size_t)cid * K, rp, adj, B, n + 1, buf, cap, lane,
                                   &overflow);
        if (counts) {
            if (lane == 0) counts[cid] = (unsigned long long)u;
        } else {
            // write the unique sorted ranks * n at heads[cid]
            int T = 1;
            for (int i = 0; i < K; ++i) {
                int v = configs[(size_t)cid * K + i];
                T *= rp[v + 1] - rp[v];
            }
            unsigned long long o = heads[cid];
            int written = 0;
            for (int t0 = 0; t0 < T; t0 += 32) {
                int t = t0 + lane;
                bool first = t < T && (t == 0 || buf[t] != buf[t - 1]);
                unsigned b = __ballot_sync(0xFFFFFFFFu, first);
                if (first) {
                    int pos = written + __popc(b & ((1u << lane) - 1u));
                    data[o + pos] = (unsigned long long)buf[t] * (unsigned long long)n;
                }
                written += __popc(b);
            }
        }
        __syncwarp();
    }
    if (overflow) atomicOr(err, kErrBudget);
}

__global__ void k_exclusive_scan_serial(const unsigned long long* in, unsigned long long* out,
                                        uint32_t C) {
    // single-block chunked scan: each thread sums a contiguous chunk, then block scan
    __shared__ unsigned long long part[1024];
    const uint32_t nt = blockDim.x, t = threadIdx.x;
    const uint32_t chunk = (C + nt - 1) / nt;
    const uint32_t b = t * chunk, e = min(C, b + chunk);
    unsigned long long s = 0;
    for (uint32_t i = b; i < e; ++i) s += in[i];
    part[t] = s;
    __syncthreads();
    for (uint32_t off = 1; off < nt; off <<= 1) {
        unsigned long long v = t >= off ? part[t - off] : 0ull;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    unsigned long long run = part[t] - s;
    for (uint32_t i = b; i < e; ++i) { out[i] = run; run += in[i]; }
    if (t == nt - 1) out[C] = part[t];
}

void launch_unrank(const uint32_t* B, int n, int k, uint32_t C, uint16_t* out, int grid, cudaStream_t st) {
    k_unrank<<<grid, 256, 0, st>>>(B, n, k, C, out);
}

int trans_cap(int k, int maxdeg) {
    long long T = 1;
    for (int i = 0; i < k; ++i) T *= maxdeg;
    long long P = 32;
    while (P < T) P <<= 1;
    return (int)P;
}

void launch_trans(int k, const uint16_t* configs, uint32_t C, int n, const uint32_t* rp,
                  const uint16_t* adj, const uint32_t* B, int cap, unsigned long long* counts,
                  const unsigned long long* heads, unsigned long long* data, unsigned int* err,
                  int grid, cudaStream_t st) {
    const int warps = cap <= 1024 ? 8 : (cap <= 4096 ? 2 : 1);
    const size_t sm = (size_t)warps * cap * sizeof(uint32_t);
#define CR_TRANS(KK)                                                                        \
    {                                                                                       \
        raise_smem_limit((const void*)k_trans<KK>, sm); \
        k_trans<KK><<<grid, warps * 32, sm, st>>>(configs, C, n, rp, adj, B, cap, counts, heads, data, err); \
    }
    switch (k) {
        case 1: CR_TRANS(1); break;
        case 2: CR_TRANS(2); break;
        case 3: CR_TRANS(3); break;
        default: CR_TRANS(4); break;
    }
#undef CR_TRANS
}

void launch_scan(const unsigned long long* in, unsigned long long* out, uint32_t C, cudaStream_t st) {
    k_exclusive_scan_serial<<<1, 1024, 0, st>>>(in, out, C);
}


// The perfect game of a solved two-column table (util/perfect_game_extractor.py:67-171
// restated): from the best configuration and the robber vertex with the largest column-0 round,
// the cops move to the first successor that lands on the robber, else to the first successor
// with the smallest marked column-1 round; the robber moves to the first neighbour with the
// largest marked column-0 round; until capture.  One warp: each ply's argmin / argmax runs
// across the lanes and is resolved in list order.  out_c / out_r get the position after each
// ply (index 0 = the start); *count the positions written, *captured 1 when the walk ended in
// a capture.
__device__ __forceinline__ bool cops_hold(const uint16_t* configs, long long cid, int k, int r) {
    bool on = false;
    for (int i = 0; i < k; ++i) on |= configs[cid * k + i] == r;
    return on;
}

__global__ void k_game(const uint8_t* __restrict__ table, const uint16_t* __restrict__ configs,
                       const unsigned long long* __restrict__ heads, const unsigned long long* __restrict__ trans,
                       const uint32_t* __restrict__ rp, const uint16_t* __restrict__ adj, int n, int k,
                       long long best, int cap, long long* out_c, int* out_r, int* count, int* captured) {
    const int lane = threadIdx.x & 31;
    const int cols = 2;
    // the robber's start: the first vertex with the largest column-0 round
    unsigned long long key = ~0ull;
    for (int r = lane; r < n; r += 32) {
        const int rnd = table[((size_t)best * n + r) * cols] >> 1;
        key = min(key, ((unsigned long long)(255 - rnd) << 32) | (unsigned)r);
    }
    // smallest (255 - round, vertex): the largest round, first in vertex order
    unsigned long long kk = key;
    for (int off = 16; off > 0; off >>= 1) kk = min(kk, __shfl_xor_sync(0xFFFFFFFFu, kk, off));
    long long cc = best;
    int rr = (int)(kk & 0xFFFFFFFFu);
    int m = 0, cap_hit = 0;
    if (lane == 0) { out_c[0] = cc; out_r[0] = rr; }
    m = 1;
    while (m < cap) {
        if (cops_hold(configs, cc, k, rr)) { cap_hit = 1; break; }
        // cops: first capture in list order, else the first smallest marked column-1 round
        const unsigned long long t0 = heads[cc], t1 = heads[cc + 1];
        unsigned long long bk = ~0ull;
        for (unsigned long long t = t0 + lane; t < t1; t += 32) {
            const long long nc = (long long)(trans[t] / (unsigned long long)n);
            unsigned long long kv;
            if (cops_hold(configs, nc, k, rr)) {
                kv = (t - t0);                                   // class 0: capture
            } else {
                const uint8_t b = table[((size_t)nc * n + rr) * cols + 1];
                if (!(b & 1)) continue;
                kv = (1ull << 62) | ((unsigned long long)(b >> 1) << 32) | (t - t0);
            }
            bk = min(bk, kv);
        }
        for (int off = 16; off > 0; off >>= 1) bk = min(bk, __shfl_xor_sync(0xFFFFFFFFu, bk, off));
        if (bk != ~0ull) cc = (long long)(trans[t0 + (bk & 0xFFFFFFFFull)] / (unsigned long long)n);
        if (lane == 0) { out_c[m] = cc; out_r[m] = rr; }
        ++m;
        if (m >= cap) break;
        if (cops_hold(configs, cc, k, rr)) { cap_hit = 1; break; }
        // robber: the first neighbour with the largest marked column-0 round
        unsigned long long rk = ~0ull;
        for (uint32_t e = rp[rr] + lane; e < rp[rr + 1]; e += 32) {
            const int v = adj[e];
            const uint8_t b = table[((size_t)cc * n + v) * cols];
            if (!(b & 1)) continue;
            rk = min(rk, ((unsigned long long)(255 - (b >> 1)) << 32) | (e - rp[rr]));
        }
        for (int off = 16; off > 0; off >>= 1) rk = min(rk, __shfl_xor_sync(0xFFFFFFFFu, rk, off));
        if (rk != ~0ull) rr = adj[rp[rr] + (rk & 0xFFFFFFFFull)];
        if (lane == 0) { out_c[m] = cc; out_r[m] = rr; }
        ++m;
    }
    if (lane == 0) {
        *count = m;
        *captured = cap_hit;
    }
}

void launch_game(const uint8_t* table, const uint16_t* configs, const unsigned long long* heads,
                 const unsigned long long* trans, const uint32_t* rp, const uint16_t* adj, int n, int k,
                 long long best, int cap, long long* out_c, int* out_r, int* count, int* captured,
                 cudaStream_t st) {
    k_game<<<1, 32, 0, st>>>(table, configs, heads, trans, rp, adj, n, k, best, cap, out_c, out_r, count, captured);
}


// Marked bit planes from table bytes (a table read from a file): word w of row (col, cid)
// holds the marked bits of robbers 32w .. 32w+31.
__global__ void k_marks_from_table(const uint8_t* __restrict__ table, uint32_t C, int n, int cols, int rwp,
                                   uint32_t* __restrict__ marked) {
    const size_t words = (size_t)cols * C * rwp;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x) {
        const int w = (int)(i % rwp);
        const size_t row = i / rwp;
        const uint32_t cid = (uint32_t)(row % C);
        const int col = (int)(row / C);
        uint32_t bits = 0;
        for (int b = 0; b < 32; ++b) {
            const int r = w * 32 + b;
            if (r < n && (table[((size_t)cid * n + r) * cols + col] & 1u)) bits |= 1u << b;
        }
        marked[i] = bits;
    }
}

void launch_marks_from_table(const uint8_t* table, uint32_t C, int n, int cols, int rwp, uint32_t* marked,
                             int grid, cudaStream_t st) {
    k_marks_from_table<<<grid, 256, 0, st>>>(table, C, n, cols, rwp, marked);
}

}  // namespace crgpu
