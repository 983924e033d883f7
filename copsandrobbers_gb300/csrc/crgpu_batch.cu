// crgpu_batch.cu - many small solves in one persistent launch.
//
// The batched workload is the cop number of many small graphs: for each graph solve k = 1, 2,
// 3 ... in order (v1 rules) and stop at the first WIN.  Solved one launch sequence at a time,
// a small graph costs a few microseconds of work per pass but tens of microseconds of launch
// and synchronisation, so the GPU idles.  Here one persistent kernel owns the whole batch:
// each thread block takes the next graph from a device-side queue (graphs ordered by cost,
// largest first), solves its k = 1, 2, ... sequence itself in a private slot of device memory,
// and writes a result per (graph, k): verdict, pass counts digest and a table digest.  The
// block runs the same frontier bodies as the stand-alone kernels (crgpu_v1_body.cuh) with
// (worker 0 of 1), separated by __syncthreads, so its tables are the same bytes.  No block
// ever waits for another; the only shared state is the queue counter.
//
// The block size and blocks per SM are chosen by a small autotuner that times candidate
// launch shapes on a calibration slice of the batch (cached per device and batch shape).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <tuple>
#include <vector>

#define CR_BODY_NS cta
#define CR_LDG(p) (*(p))
#define CR_RESTRICT
#define CR_BODY_INLINE __noinline__
#include "../../include/crgpu.h"
#include "crgpu_ctx.h"
#include "crgpu_v1_body.cuh"

namespace crgpu {

size_t and_stage_words(int n, int rwp, int nnz);

using namespace cta;

constexpr int kBatchMaxN = 128;
constexpr int kBatchMaxK = 3;

struct BatchDev {
    int count, kmax, p;
    const int32_t* order;
    const int32_t* n;
    const int32_t* maxdeg;
    const uint64_t* rp_off;   // per graph: offset of its n+1 row pointers in rp_all / rrp_all
    const uint64_t* col_off;  // per graph: offset of its neighbour lists in col_all / rcol_all
    const uint32_t* rp_all;
    const uint16_t* col_all;
    const uint32_t* rrp_all;
    const uint16_t* rcol_all;
    unsigned char* slots;
    size_t slot_bytes;
    int* next;
    int32_t* cop;
    cr_batch_result* res;
    unsigned long long* cta_time;  // per block: globaltimer at start and after its last graph
    uint32_t smem_words;           // dynamic shared memory of the launch
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// 64-bit mixer (the splitmix64 finaliser of Steele, Lea and Flood) used by the table digest.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__host__ __device__ inline uint64_t binom_dev(int64_t n, int64_t k) {
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    uint64_t r = 1;
    for (int64_t i = 1; i <= k; ++i) r = r * (uint64_t)(n - i + 1) / (uint64_t)i;
    return r;
}

// Byte offsets of one (n, k, p) solve inside a slot.
struct JobLayout {
    size_t binom, configs, nbr, iso, hop, rhop, cover, table, marked, front, h1, list, clist, fflag, cand,
        cbits, sync, meta, counters, err, total;
};

__host__ __device__ inline JobLayout job_layout(int n, int k, int p, int S) {
    const uint64_t C = binom_dev((int64_t)n + k - 1, k);
    const int rwp = round_words((n + 31) / 32), cols = 2 * p;
    JobLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off += (bytes + 255) & ~size_t(255);
        return at;
    };
    L.binom = take((size_t)k * (n + 1) * 4);
    L.configs = take(C * k * 2);
    L.nbr = take((size_t)n * rwp * 4);
    L.iso = take((size_t)rwp * 4);
    L.hop = take((size_t)n * rwp * 4);
    L.rhop = take((size_t)n * rwp * 4);
    // uncovered-slot masks of the fused first pass (p = 1), up to 4 bytes per mask
    L.cover = take(p == 1 ? 2 * (size_t)n * ((n + 7) & ~7) * 4 : 0);
    L.table = take(C * (size_t)n * cols);
    L.marked = take((size_t)cols * C * rwp * 4);
    L.front = take((size_t)cols * C * S * rwp * 4);
    // k = 3: rows of the separable dense cop turn (written before they are read each pass,
    // so they sit outside the regions the block zeroes)
    L.h1 = take(k == 3 ? (size_t)n * (n + 1) / 2 * n * S * rwp * 4 : 0);
    // frontier row lists and the push-mode candidate list (written before they are read)
    L.list = take((size_t)cols * C * 4);
    L.clist = take(C * 4);
    L.fflag = take((size_t)cols * C);
    L.cand = take(C * S * rwp * 4);
    L.cbits = take(cand_bits_bytes(C));
    L.sync = take(2 * sizeof(unsigned));
    L.meta = take(sizeof(ColMeta) * cols);
    L.counters = take(4 * sizeof(unsigned long long));
    L.err = take(sizeof(unsigned));
    L.total = off;
    return L;
}

// Table digest: sum over 8-byte little-endian words w_j (zero-padded tail) of
// mix64(w_j ^ (j * 0x9E3779B97F4A7C15)), modulo 2^64.
__device__ inline uint64_t digest_word(const uint8_t* t, size_t bytes, size_t j) {
    uint64_t w = 0;
    const size_t at = j * 8;
    if (at + 8 <= bytes && ((uintptr_t)t & 7u) == 0) {
        w = *reinterpret_cast<const uint64_t*>(t + at);   // little-endian: byte b at bits 8b
    } else if (at + 8 <= bytes) {
        for (int b = 0; b < 8; ++b) w |= (uint64_t)t[at + b] << (8 * b);
    } else {
        for (size_t b = 0; at + b < bytes; ++b) w |= (uint64_t)t[at + b] << (8 * b);
    }
    return mix64(w ^ (j * 0x9E3779B97F4A7C15ull));
}

__device__ void block_fill(unsigned char* p, unsigned char v, size_t bytes) {
    // p is 256-byte aligned (slot layout)
    const uint32_t v4 = 0x01010101u * v;
    const uint4 q = make_uint4(v4, v4, v4, v4);
    uint4* p16 = reinterpret_cast<uint4*>(p);
    const size_t n16 = bytes / 16;
    for (size_t i = threadIdx.x; i < n16; i += blockDim.x) p16[i] = q;
    for (size_t i = n16 * 16 + threadIdx.x; i < bytes; i += blockDim.x) p[i] = v;
}

// The uncovered-slot masks of the fused first pass, as the stand-alone solver builds them on the
// host (cover[c][r] bit j: r's j-th neighbour v is neither c nor a neighbour of c; cover[n+c][r]:
// v is not c; a cop's own entry all ones, the rows of a cop without a move zero), W = 1, 2 or 4
// bytes per mask by the largest degree.  Sets d.g.cover, cover_w and npad.
__device__ void build_cover(V1Dev& d, uint8_t* cov, int maxdeg) {
    const int n = d.g.n, rwp = d.g.rwp, npad = (n + 7) & ~7;
    const int W = maxdeg <= 8 ? 1 : (maxdeg <= 16 ? 2 : 4);
    const uint32_t ones = W == 4 ? 0xFFFFFFFFu : ((1u << (8 * W)) - 1u);
    const size_t plane = (size_t)n * npad * W;
    for (int t = threadIdx.x; t < n * npad; t += blockDim.x) {
        const int c = t / npad, r = t - c * npad;
        uint32_t m0 = 0, m1 = 0;
        if (r < n) {
            const uint32_t e0 = d.g.row_ptr[r], deg = d.g.row_ptr[r + 1] - e0;
            for (uint32_t j = 0; j < deg; ++j) {
                const int v = d.g.col[e0 + j];
                if (v == c) continue;
                m1 |= 1u << j;
                if (!((d.g.nbr[(size_t)c * rwp + (v >> 5)] >> (v & 31)) & 1u)) m0 |= 1u << j;
            }
            if (r == c) m0 = ones;
        }
        if ((d.g.isolated[c >> 5] >> (c & 31)) & 1u) m0 = 0;
        for (int q = 0; q < W; ++q) {
            cov[(size_t)t * W + q] = (uint8_t)(m0 >> (8 * q));
            cov[plane + (size_t)t * W + q] = (uint8_t)(m1 >> (8 * q));
        }
    }
    d.g.cover = cov;
    d.g.cover_w = W;
    d.g.npad = npad;
    __syncthreads();
}

// Column col's row list from its flag plane, by the whole block (after the fused first pass).
__device__ void block_list_compact(const V1Dev& d, int col) {
    const uint8_t* f = d.fflag + (size_t)col * d.C;
    uint32_t* out = d.list + (size_t)col * d.C;
    const int lane = threadIdx.x & 31;
    for (uint32_t base = threadIdx.x & ~31u; base < d.C; base += blockDim.x) {
        const uint32_t i = base + lane;
        const bool set = i < d.C && f[i];
        const unsigned b = __ballot_sync(0xFFFFFFFFu, set);
        if (!b) continue;
        int at = 0;
        if (lane == 0) at = atomicAdd(&d.meta[col].len, __popc(b));
        at = __shfl_sync(0xFFFFFFFFu, at, 0);
        if (set) out[at + __popc(b & ((1u << lane) - 1u))] = i;
    }
}

// One (graph, k) solve by the whole block.  Returns 1 on WIN.
template <int K, int RWP, bool P1>
__device__ int solve_job(const BatchDev& b, unsigned char* slot, int gi, int jr, uint64_t* sh) {
    constexpr int G = RWP <= 4 ? 4 : RWP;
    constexpr int NWP = RWP * 2 <= 2 ? 2 : RWP * 2;  // S = 2 slots
    const int n = b.n[gi], p = b.p, cols = 2 * p, S = 2;
    const int rw = (n + 31) / 32, rwp = round_words(rw);
    const uint64_t C = binom_dev((int64_t)n + K - 1, K);
    const JobLayout L = job_layout(n, K, p, S);
    V1Dev d;
    d.g.n = n;
    d.g.maxdeg = b.maxdeg[gi];
    d.g.rw = rw;
    d.g.rwp = rwp;
    d.g.row_ptr = b.rp_all + b.rp_off[gi];
    d.g.col = b.col_all + b.col_off[gi];
    d.g.rrow_ptr = b.rrp_all + b.rp_off[gi];
    d.g.rcol = b.rcol_all + b.col_off[gi];
    d.g.nbr = reinterpret_cast<const uint32_t*>(slot + L.nbr);
    d.g.isolated = reinterpret_cast<const uint32_t*>(slot + L.iso);
    d.g.rhop = reinterpret_cast<const uint32_t*>(slot + L.rhop);
    d.k = K;
    d.cols = cols;
    d.S = S;
    d.C = (uint32_t)C;
    d.binom = reinterpret_cast<const uint32_t*>(slot + L.binom);
    d.configs = reinterpret_cast<const uint16_t*>(slot + L.configs);
    d.hop = reinterpret_cast<const uint32_t*>(slot + L.hop);
    d.table = slot + L.table;
    d.marked = reinterpret_cast<uint32_t*>(slot + L.marked);
    d.front = reinterpret_cast<uint32_t*>(slot + L.front);
    d.fflag = slot + L.fflag;
    d.cand = reinterpret_cast<uint32_t*>(slot + L.cand);
    d.h1 = K == 3 ? reinterpret_cast<uint32_t*>(slot + L.h1) : nullptr;
    d.cbits = reinterpret_cast<uint32_t*>(slot + L.cbits);
    d.list = reinterpret_cast<uint32_t*>(slot + L.list);
    d.clist = reinterpret_cast<uint32_t*>(slot + L.clist);
    d.sync = reinterpret_cast<unsigned*>(slot + L.sync);
    d.meta = reinterpret_cast<ColMeta*>(slot + L.meta);
    d.pass_new = reinterpret_cast<unsigned long long*>(slot + L.counters);
    d.err = reinterpret_cast<unsigned*>(slot + L.err);
    {
        // room past the last-column body's lane groups for staging the graph
        constexpr int CPW = 32 / G;
        const uint32_t groups = (blockDim.x >> 5) * CPW * and_group_words(S, rwp);
        d.and_stage_words = b.smem_words > groups ? b.smem_words - groups : 0u;
    }
    uint32_t* binom = reinterpret_cast<uint32_t*>(slot + L.binom);
    uint32_t* nbr = reinterpret_cast<uint32_t*>(slot + L.nbr);
    uint32_t* iso = reinterpret_cast<uint32_t*>(slot + L.iso);
    uint32_t* hop = reinterpret_cast<uint32_t*>(slot + L.hop);
    uint16_t* configs = reinterpret_cast<uint16_t*>(slot + L.configs);

    // initializeCaptures and pass 1 fused (as the stand-alone p = 1 solve does) when the
    // uncovered-slot masks fit: the first pass then writes every table byte and both marked
    // planes itself
    const int maxdeg = b.maxdeg[gi];
    const bool fused = P1 && maxdeg <= 32;
    // ---- buildAuxGraph: zeroed planes, rank table, neighbour masks, configurations
    block_fill(slot + L.nbr, 0, L.cover - L.nbr);
    if (!fused) {
        block_fill(slot + L.marked, 0, L.front - L.marked);
        block_fill(d.table, kUnmarked, C * (size_t)n * cols);
    }
    block_fill(slot + L.fflag, 0, L.total - L.fflag);
    const int np1 = n + 1;
    for (int t = threadIdx.x; t < K * np1; t += blockDim.x) {
        const int i = t / np1, x = t - i * np1;
        binom[t] = (uint32_t)binom_dev((int64_t)n - x + K - 1 - i, K - i);
    }
    __syncthreads();
    for (int u = threadIdx.x; u < n; u += blockDim.x) {
        const uint32_t e0 = d.g.row_ptr[u], e1 = d.g.row_ptr[u + 1];
        if (e0 == e1) atomicOr(&iso[u >> 5], 1u << (u & 31));
        for (uint32_t e = e0; e < e1; ++e) {
            const int v = d.g.col[e];
            nbr[(size_t)u * rwp + (v >> 5)] |= 1u << (v & 31);
        }
        // transposed 1-hop masks: the in-neighbours of u
        uint32_t* rh = reinterpret_cast<uint32_t*>(slot + L.rhop) + (size_t)u * rwp;
        for (uint32_t e = d.g.rrow_ptr[u]; e < d.g.rrow_ptr[u + 1]; ++e) {
            const int r = d.g.rcol[e];
            rh[r >> 5] |= 1u << (r & 31);
        }
    }
    for (uint32_t cid = threadIdx.x; cid < C; cid += blockDim.x) {
        uint32_t rem = cid;
        int prev = 0;
        for (int i = 0; i < K; ++i) {
            const uint32_t top = binom[i * np1 + prev];
            int lo = prev, hi = n - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (binom[i * np1 + mid] >= top - rem) lo = mid; else hi = mid - 1;
            }
            rem -= top - binom[i * np1 + lo];
            configs[(size_t)cid * K + i] = (uint16_t)lo;
            prev = lo;
        }
    }
    __syncthreads();
    if (!P1) {
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            uint32_t cur[kBatchMaxN / 32], nxt[kBatchMaxN / 32];
            for (int w = 0; w < rwp; ++w) cur[w] = 0u;
            cur[r >> 5] = 1u << (r & 31);
            for (int s = 0; s < p; ++s) {
                for (int w = 0; w < rwp; ++w) nxt[w] = 0u;
                for (int w = 0; w < rwp; ++w) {
                    uint32_t bb = cur[w];
                    while (bb) {
                        const int v = w * 32 + __ffs(bb) - 1;
                        bb &= bb - 1;
                        for (int q = 0; q < rwp; ++q) nxt[q] |= nbr[(size_t)v * rwp + q];
                    }
                }
                for (int w = 0; w < rwp; ++w) cur[w] = nxt[w];
            }
            for (int w = 0; w < rwp; ++w) hop[(size_t)r * rwp + w] = cur[w];
        }
    }
    uint64_t caps = 0, phash = 0;
    int passes = 0;
    bool more = true;
    if (fused) {
        build_cover(d, slot + L.cover, maxdeg);
        if (threadIdx.x == 0) {
            for (int c = 0; c < cols; ++c) d.meta[c] = ColMeta{0, kEmptyLo, -1, 0, 0, 0, 0, 0};
            d.meta[0] = ColMeta{0, 0, 0, 0, (int)C, 0, -1, 1};   // consumed: flags left clear
            d.meta[1] = ColMeta{1, kEmptyLo, -1, 0, 0, 0, 0, 0};
        }
        __syncthreads();
        if (d.g.cover_w == 1) init_pass1_body<K, 1>(d, 0, 1);
        else if (d.g.cover_w == 2) init_pass1_body<K, 2>(d, 0, 1);
        else init_pass1_body<K, 4>(d, 0, 1);
        __syncthreads();
        block_list_compact(d, 1);
        __syncthreads();
        // every configuration's distinct cops: n times the multisets holding a given vertex
        caps = (uint64_t)n * (binom_dev((int64_t)n + K - 1, K) - binom_dev((int64_t)n + K - 2, K));
        const uint64_t found = *d.pass_new;
        const unsigned bits = *d.err;
        __syncthreads();
        passes = 1;
        phash = mix64(found ^ (1ull * 0xD1B54A32D192ED03ull));
        more = found != 0 && !bits;
    } else {
        // ---- initializeCaptures
        if (threadIdx.x == 0) {
            for (int c = 0; c < cols; ++c) d.meta[c] = ColMeta{0, kEmptyLo, -1, 0, 0, 0, 0, 0};
            d.meta[0] = ColMeta{0, 0, 0, 1, (int)C, 0, -1, 0};
            d.meta[1] = ColMeta{0, 0, 0, 0, (int)C, 1, -1, 0};
        }
        __syncthreads();
        init_body(d, K, 0, 1);
        __syncthreads();
        caps = *d.pass_new;
        __syncthreads();
    }
    // ---- mainLoop
    while (more) {
        for (int col = 0; col < cols; ++col) {
            const int nx = (col + 1) % cols;
            prep_body(d, col, nx, 0, 1);
            __syncthreads();
            if (col % 2 == 0) {
                cop_seed_body<K, G>(d, col, nx, 0, 1);
                __syncthreads();
                cop_pull_body<K, NWP, G>(d, col, nx, 0, 1);
                __syncthreads();
                if (K == 3) {
                    pair_h1_body(d, nx, 0, 1);
                    __syncthreads();
                    sep_pull_body<NWP, G>(d, col, nx, 0, 1);
                    __syncthreads();
                }
                cop_push_body<K>(d, col, nx, 0, 1);
                __syncthreads();
                cop_apply_body<G>(d, col, nx, 0, 1);
            } else if (col < cols - 1) {
                direct_body<G>(d, col, nx, 0, 1);
            } else {
                and_body<P1, G>(d, col, 0, 1);
            }
            __syncthreads();
        }
        const uint64_t found = *d.pass_new;
        const unsigned bits = *d.err;
        __syncthreads();
        ++passes;
        phash += mix64(found ^ ((uint64_t)passes * 0xD1B54A32D192ED03ull));
        if (bits || found == 0 || passes >= 4096) break;
    }
    // ---- findFinalResult
    unsigned long long* best = d.pass_new + 1;
    if (threadIdx.x == 0) *best = ~0ull;
    __syncthreads();
    verdict_body(d.table, d.marked, d.C, n, rw, rwp, cols, best, 0, 1);
    // ---- table digest
    const size_t bytes = C * (size_t)n * cols;
    uint64_t part = 0;
    for (size_t j = threadIdx.x; j < (bytes + 7) / 8; j += blockDim.x) part += digest_word(d.table, bytes, j);
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = part;
    __syncthreads();
    int win = 0;
    if (threadIdx.x == 0) {
        uint64_t dg = 0;
        for (unsigned w = 0; w < (blockDim.x >> 5); ++w) dg += sh[w];
        const unsigned long long key = *best;
        cr_batch_result& r = b.res[jr];
        r.solved = 1;
        r.status = *d.err ? CR_ERR_INTERNAL : (passes >= 4096 ? CR_ERR_BUDGET : CR_OK);
        win = (key != ~0ull && (int)(key >> 32) < kMaxRound) ? 1 : 0;
        r.win = win;
        r.capture_plies = win ? (int32_t)(key >> 32) : kMaxRound;
        r.best_config = win ? (int64_t)(key & 0xFFFFFFFFull) : -1;
        r.passes = passes;
        r.base_captures = caps;
        r.states = C * (uint64_t)n * cols;
        r.digest = dg;
        r.pass_hash = phash;
        sh[0] = (uint64_t)win;
    }
    __syncthreads();
    win = (int)sh[0];
    __syncthreads();
    return win;
}

template <int K, bool P1>
__device__ int solve_job_k(const BatchDev& b, unsigned char* slot, int gi, int jr, uint64_t* sh) {
    const int rwp = round_words((b.n[gi] + 31) / 32);
    if (rwp <= 1) return solve_job<K, 1, P1>(b, slot, gi, jr, sh);
    if (rwp <= 2) return solve_job<K, 2, P1>(b, slot, gi, jr, sh);
    return solve_job<K, 4, P1>(b, slot, gi, jr, sh);
}

// Two builds: up to 512 threads per block with up to 128 registers (no spills in the bodies),
// and 1024 threads with 64 (a few spills, twice the threads on each graph).
template <bool P1, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) k_batch(BatchDev b) {
    __shared__ uint64_t sh[32];
    __shared__ int s_job;
    unsigned char* slot = b.slots + (size_t)blockIdx.x * b.slot_bytes;
    if (threadIdx.x == 0) b.cta_time[2 * blockIdx.x] = b.cta_time[2 * blockIdx.x + 1] = global_ns();
    for (;;) {
        if (threadIdx.x == 0) s_job = atomicAdd(b.next, 1);
        __syncthreads();
        const int jj = s_job;
        __syncthreads();
        if (jj >= b.count) break;
        const int gi = b.order[jj];
        int cop = 0;
        for (int k = 1; k <= b.kmax; ++k) {
            const int jr = gi * b.kmax + (k - 1);
            int win;
            if (k == 1) win = solve_job_k<1, P1>(b, slot, gi, jr, sh);
            else if (k == 2) win = solve_job_k<2, P1>(b, slot, gi, jr, sh);
            else win = solve_job_k<3, P1>(b, slot, gi, jr, sh);
            if (win) { cop = k; break; }
        }
        if (threadIdx.x == 0) {
            b.cop[gi] = cop;
            b.cta_time[2 * blockIdx.x + 1] = global_ns();
        }
    }
}

// Grid-wide digest of a stand-alone solver's table (same function as the batch's).
__global__ void k_digest(const uint8_t* table, size_t bytes, unsigned long long* out) {
    uint64_t part = 0;
    for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < (bytes + 7) / 8;
         j += (size_t)gridDim.x * blockDim.x)
        part += digest_word(table, bytes, j);
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, (unsigned long long)part);
}

void launch_digest(const uint8_t* table, size_t bytes, unsigned long long* out, int grid, cudaStream_t st) {
    k_digest<<<grid, 256, 0, st>>>(table, bytes, out);
}

}  // namespace crgpu

using namespace crgpu;

namespace {

// Dynamic shared memory of the batch kernel: the largest need over every vertex count up to
// max_n (lane groups, and so the per-group footprint, change with the row width).
size_t batch_smem(int threads, int max_n) {
    size_t best = 0;
    for (int n = 1; n <= max_n; ++n) {
        const int rwp = round_words((n + 31) / 32);
        const int G = rwp <= 4 ? 4 : rwp, CPW = 32 / G, warps = threads / 32, S = 2;
        const size_t cop = (size_t)warps * CPW * 2 * S * rwp;
        const size_t andb = (size_t)warps * CPW * and_group_words(S, rwp);
        const size_t push = (size_t)warps * S * rwp;
        const size_t pull = cop + rank_table_words(kBatchMaxK, n);
        const size_t pair = (size_t)pair_smem_words(n);
        best = std::max(best, std::max(std::max(pull, pair), std::max(andb, push)) * 4);
    }
    return best;
}

struct Shape {
    int threads, per_sm;
};

std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, Shape> g_tuned;

int fail(cr_context* ctx, int code, const char* msg) {
    if (ctx) ctx->err = msg;
    return code;
}

}  // namespace

#define CR_BCUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                 \
            return e_ == cudaErrorMemoryAllocation ? CR_ERR_NOMEM : CR_ERR_CUDA;           \
        }                                                                                  \
    } while (0)

namespace {

// Device copies of one batch's inputs.
struct BatchInputs {
    std::vector<int32_t> n, maxdeg, order;
    std::vector<uint64_t> rp_off, col_off;
    std::vector<uint32_t> rp, rrp;
    std::vector<uint16_t> col, rcol;
    int max_n = 0;
    size_t max_stage_words = 0;   // the largest graph staging of the last-column body
};

int launch_batch(cr_context* ctx, const BatchInputs& in, const std::vector<int32_t>& order, int kmax,
                 int p, Shape shape, size_t slot_bytes, std::vector<int32_t>* cop,
                 std::vector<cr_batch_result>* res, float* ms,
                 std::vector<unsigned long long>* times = nullptr) {
    const int count = (int)order.size();
    const int nblocks = std::max(1, std::min(count, ctx->num_sms * shape.per_sm));
    void* bufs[13] = {};
    auto cleanup = [&]() {
        for (void* q : bufs)
            if (q) cudaFree(q);
    };
    BatchDev b;
    b.count = count;
    b.kmax = kmax;
    b.p = p;
    size_t sizes[13] = {order.size() * 4, in.n.size() * 4, in.maxdeg.size() * 4, in.rp_off.size() * 8,
                        in.col_off.size() * 8, in.rp.size() * 4, std::max<size_t>(in.col.size(), 1) * 2,
                        in.rrp.size() * 4, std::max<size_t>(in.rcol.size(), 1) * 2,
                        (size_t)nblocks * slot_bytes, sizeof(int) + in.n.size() * 4,
                        in.n.size() * kmax * sizeof(cr_batch_result), (size_t)nblocks * 16};
    for (int i = 0; i < 13; ++i) {
        cudaError_t e = cudaMalloc(&bufs[i], sizes[i]);
        if (e != cudaSuccess) {
            cleanup();
            ctx->err = std::string("batch allocation: ") + cudaGetErrorString(e);
            return e == cudaErrorMemoryAllocation ? CR_ERR_NOMEM : CR_ERR_CUDA;
        }
    }
    cudaStream_t st = ctx->stream;
    const void* src[9] = {order.data(), in.n.data(), in.maxdeg.data(), in.rp_off.data(), in.col_off.data(),
                          in.rp.data(), in.col.data(), in.rrp.data(), in.rcol.data()};
    for (int i = 0; i < 9; ++i) {
        if (i == 6 && in.col.empty()) continue;
        if (i == 8 && in.rcol.empty()) continue;
        cudaMemcpyAsync(bufs[i], src[i], sizes[i], cudaMemcpyHostToDevice, st);
    }
    b.order = (const int32_t*)bufs[0];
    b.n = (const int32_t*)bufs[1];
    b.maxdeg = (const int32_t*)bufs[2];
    b.rp_off = (const uint64_t*)bufs[3];
    b.col_off = (const uint64_t*)bufs[4];
    b.rp_all = (const uint32_t*)bufs[5];
    b.col_all = (const uint16_t*)bufs[6];
    b.rrp_all = (const uint32_t*)bufs[7];
    b.rcol_all = (const uint16_t*)bufs[8];
    b.slots = (unsigned char*)bufs[9];
    b.slot_bytes = slot_bytes;
    b.next = (int*)bufs[10];
    b.cop = (int32_t*)((char*)bufs[10] + sizeof(int));
    b.res = (cr_batch_result*)bufs[11];
    b.cta_time = (unsigned long long*)bufs[12];
    b.smem_words = (uint32_t)((batch_smem(shape.threads, in.max_n) + in.max_stage_words * 4) / 4);
    cudaMemsetAsync(bufs[10], 0, sizes[10], st);
    cudaMemsetAsync(bufs[11], 0, sizes[11], st);
    const size_t sm = batch_smem(shape.threads, in.max_n) + in.max_stage_words * 4;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // the batch launch is captured once as a CUDA graph and replayed
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void (*kern)(BatchDev) = shape.threads > 512 ? k_batch<true, 1024> : k_batch<true, 512>;
    raise_smem_limit((const void*)kern, sm);
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        kern<<<nblocks, shape.threads, sm, st>>>(b);
        e = cudaStreamEndCapture(st, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e == cudaSuccess) {
        cudaEventRecord(e0, st);
        e = cudaGraphLaunch(exec, st);
        cudaEventRecord(e1, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) {
        cudaEventElapsedTime(ms, e0, e1);
        cop->resize(in.n.size());
        res->resize(in.n.size() * kmax);
        cudaMemcpy(cop->data(), b.cop, in.n.size() * 4, cudaMemcpyDeviceToHost);
        e = cudaMemcpy(res->data(), b.res, sizes[11], cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && times) {
            times->resize((size_t)nblocks * 2);
            e = cudaMemcpy(times->data(), b.cta_time, sizes[12], cudaMemcpyDeviceToHost);
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cleanup();
    if (e != cudaSuccess) {
        ctx->err = std::string("batch launch: ") + cudaGetErrorString(e);
        return CR_ERR_CUDA;
    }
    return CR_OK;
}

}  // namespace

extern "C" {

int cr_batch_solve(cr_context* ctx, const cr_graph* graphs, int32_t count, int32_t kmax, int32_t p,
                   int32_t threads_per_cta, int32_t* cop_number, cr_batch_result* results,
                   cr_batch_stats* stats) {
    if (!ctx || !graphs || count <= 0 || !cop_number || !results) return CR_ERR_INVALID;
    if (kmax < 1 || kmax > kBatchMaxK) return fail(ctx, CR_ERR_LIMIT, "batch: kmax outside 1..3");
    if (p != 1) return fail(ctx, CR_ERR_LIMIT, "batch: full visibility (p = 1) only");
    if (threads_per_cta != 0 && threads_per_cta != 256 && threads_per_cta != 512 && threads_per_cta != 1024)
        return fail(ctx, CR_ERR_INVALID, "batch: threads_per_cta must be 0 (autotune), 256, 512 or 1024");
    cudaSetDevice(ctx->device);
    BatchInputs in;
    in.n.resize(count);
    in.maxdeg.resize(count);
    in.rp_off.resize(count);
    in.col_off.resize(count);
    std::vector<double> cost(count);
    for (int i = 0; i < count; ++i) {
        const cr_graph& g = graphs[i];
        if (g.n <= 0 || g.n > kBatchMaxN || !g.row_ptr) return fail(ctx, CR_ERR_LIMIT, "batch: every graph needs 1..128 vertices");
        const uint32_t nnz = g.row_ptr[g.n];
        if (nnz && !g.col_idx) return fail(ctx, CR_ERR_INVALID, "batch: graph arrays missing");
        in.n[i] = g.n;
        in.max_n = std::max(in.max_n, g.n);
        in.rp_off[i] = in.rp.size();
        in.col_off[i] = in.col.size();
        int md = 0;
        std::vector<uint32_t> indeg(g.n + 1, 0);
        for (int v = 0; v < g.n; ++v) {
            if (g.row_ptr[v + 1] < g.row_ptr[v]) return fail(ctx, CR_ERR_INVALID, "batch: row_ptr not monotone");
            md = std::max<int>(md, g.row_ptr[v + 1] - g.row_ptr[v]);
        }
        for (uint32_t e = 0; e < nnz; ++e) {
            if (g.col_idx[e] >= g.n) return fail(ctx, CR_ERR_INVALID, "batch: neighbour index out of range");
            indeg[g.col_idx[e] + 1]++;
        }
        in.maxdeg[i] = md;
        in.max_stage_words = std::max(in.max_stage_words,
                                      and_stage_words(g.n, round_words((g.n + 31) / 32), (int)nnz));
        for (int v = 0; v <= g.n; ++v) in.rp.push_back(g.row_ptr[v]);
        for (uint32_t e = 0; e < nnz; ++e) in.col.push_back(g.col_idx[e]);
        // in-neighbour CSR (ascending sources)
        for (int v = 0; v < g.n; ++v) indeg[v + 1] += indeg[v];
        for (int v = 0; v <= g.n; ++v) in.rrp.push_back(indeg[v]);
        std::vector<uint32_t> fill(indeg.begin(), indeg.end() - 1);
        std::vector<uint16_t> rc(nnz);
        for (int u = 0; u < g.n; ++u)
            for (uint32_t e = g.row_ptr[u]; e < g.row_ptr[u + 1]; ++e) rc[fill[g.col_idx[e]]++] = (uint16_t)u;
        in.rcol.insert(in.rcol.end(), rc.begin(), rc.end());
        cost[i] = (double)binom_dev((int64_t)g.n + kmax - 1, kmax) * g.n;
    }
    std::vector<int32_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return cost[a] > cost[c]; });
    const size_t slot_bytes = job_layout(in.max_n, kmax, p, 2).total;

    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    auto fits = [&](Shape s) {
        return (size_t)std::min(count, ctx->num_sms * s.per_sm) * slot_bytes < free_b / 2;
    };
    Shape shape{threads_per_cta ? threads_per_cta : 512, threads_per_cta == 256 ? 2 : 1};
    if (threads_per_cta == 0) {
        // autotune: time candidate launch shapes on a calibration slice (every 8th graph of
        // the cost order, so the slice has the batch's size mix), once per device and shape
        const auto key = std::make_tuple(ctx->device, in.max_n, kmax, p);
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            shape = it->second;
        } else {
            std::vector<int32_t> calib;
            for (int i = 0; i < count; i += 8) calib.push_back(order[i]);
            // every shape fits the register file: 256 x 2 and 512 x 1 at 128 registers,
            // 1024 x 1 at 64
            const Shape cands[] = {{256, 2}, {512, 1}, {1024, 1}};
            float best = 1e30f;
            for (Shape c : cands) {
                if (!fits(c)) continue;
                std::vector<int32_t> cp;
                std::vector<cr_batch_result> rs;
                float ms = 0;
                if (launch_batch(ctx, in, calib, kmax, p, c, slot_bytes, &cp, &rs, &ms) != CR_OK) continue;
                if (ms < best) {
                    best = ms;
                    shape = c;
                }
            }
            g_tuned[key] = shape;
        }
    }
    while (!fits(shape) && shape.per_sm > 1) shape.per_sm--;
    if (!fits(shape)) return fail(ctx, CR_ERR_NOMEM, "batch: not enough device memory for one slot per SM");
    std::vector<int32_t> cop;
    std::vector<cr_batch_result> res;
    float ms = 0;
    std::vector<unsigned long long> times;
    int rc = launch_batch(ctx, in, order, kmax, p, shape, slot_bytes, &cop, &res, &ms, &times);
    if (rc) return rc;
    memcpy(cop_number, cop.data(), count * sizeof(int32_t));
    memcpy(results, res.data(), res.size() * sizeof(cr_batch_result));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->ms = ms;
        for (const auto& r : res) stats->states += r.solved ? r.states : 0;
        stats->threads = shape.threads;
        stats->ctas = std::min(count, ctx->num_sms * shape.per_sm);
        stats->slot_bytes = (int64_t)slot_bytes;
        // how evenly the blocks were kept busy: mean busy span over the whole span, and the
        // time from the median block's last graph to the last block's
        const size_t nb = times.size() / 2;
        if (nb) {
            unsigned long long t0 = ~0ull, t1 = 0;
            std::vector<double> ends(nb);
            double busy = 0;
            for (size_t i = 0; i < nb; ++i) {
                t0 = std::min(t0, times[2 * i]);
                t1 = std::max(t1, times[2 * i + 1]);
            }
            for (size_t i = 0; i < nb; ++i) {
                busy += (double)(times[2 * i + 1] - times[2 * i]);
                ends[i] = (double)(times[2 * i + 1] - t0);
            }
            std::sort(ends.begin(), ends.end());
            const double span = (double)(t1 - t0);
            stats->busy_frac = span > 0 ? busy / (span * nb) : 0;
            stats->tail_ms = (span - ends[nb / 2]) / 1e6;
        }
    }
    for (const auto& r : res)
        if (r.solved && r.status != CR_OK) return fail(ctx, CR_ERR_INTERNAL, "batch: a solve reported a device error");
    return CR_OK;
}

}  // extern "C"
