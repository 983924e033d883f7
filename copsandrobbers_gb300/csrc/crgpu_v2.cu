// crgpu_v2.cu - snapshot passes of the macro-turn trajectory search
// (solvers/k_cops_visibility_v2.cpp: one plane (C, r), p cop/robber steps per visibility cycle).
//
// The reference decides every unmarked (C0, r) by a branch-and-bound DFS over cop
// trajectories C1..Cp (trajectoryDFS, v2:243-341) against the table as it stood at the start
// of the pass, buffering the marks (v2:437-562).  The DFS value is the minimum, over
// trajectories, of the first event on that trajectory:
//     cop ply d empties the robber cloud          -> 2d - 1        (v2:300-308)
//     robber ply d leaves no robber alive         -> 2d            (v2:312-319)
//     d = p, cloud inside the marked set of C_p   -> 2p + max round (v2:321-334)
// Branch-and-bound order and the two skip filters (v2:450-523) change only the work, not
// that minimum, so these kernels compute it directly, level by level:
//
//   val1[C1][r] = value of the depth-1 node (C1, N(r) \ C1): a warp per (C1, r), lanes over
//                 the successors C2 of C1, each lane running the rest of the trajectory tree
//                 depth first (clouds as multi-word vertex bitmasks, expanded by OR over
//                 neighbour masks held in shared memory);
//   root[C0][r] = min over C1 in T(C0) of (1 if r in C1, 2 if N(r) within C1, else val1).
//
// Only leaves read the table, and a depth-1 node's leaves lie p-1 cop steps away, so after
// the first pass val1 is recomputed only for configs within p-1 cop steps of a config that
// gained marks ("dirty"); the others keep last pass's value, which is exact because the
// snapshot they read has not changed there.
//
// For p >= 3 the depth-2 nodes (C2, V2) repeat heavily: V2 = N(N(r) \ C1 \ C2) \ C2 is the same
// cloud for every predecessor C1 of C2 that misses N(r), so many depth-1 nodes share each
// depth-2 subtree (on a Delaunay graph of 199 vertices with k = 2, one full pass visits 79.3 M
// depth-2 children but only 4.69 M distinct ones).  Each pass therefore dedups the reachable
// depth-2 clouds in a device hash table before any leaf is read:
//   k_v2_hinsert  every dirty depth-1 node inserts its non-terminal children (C2, V2): key =
//                 (rank of C2 + 1) << 32 | 32-bit fingerprint of V2, claimed by atomicCAS with
//                 linear probing; the claiming thread writes the full cloud beside the key;
//   k_v2_heval    one thread per occupied slot takes the exact subtree minimum of its node;
//   k_v2_val1     looks every child up (key equal AND full cloud equal) and takes the stored
//                 value; a child it does not find (probe limit, table full, or a fingerprint
//                 shared by two clouds of the same C2, whose second cloud never got a slot) is
//                 evaluated directly, so the result is exact whatever the table holds.
// The subtree value of a node depends only on (depth, C2, V2) and the pass's snapshot, so the
// table is rebuilt every pass.  When the depth-1 nodes outnumber half the table, they are
// processed in chunks, each with a fresh table.
#include <algorithm>
#include <string>
#include <vector>

#include "crgpu_internal.cuh"
#include "crgpu_v2.h"

namespace crgpu {

void launch_marks_from_table(const uint8_t* table, uint32_t C, int n, int cols, int rwp, uint32_t* marked,
                             int grid, cudaStream_t st);
void launch_verdict_raw(const uint8_t* table, const uint32_t* m0, uint32_t C, int n, int rw,
                        int rwp, int cols, unsigned long long* best, int grid, cudaStream_t st);

constexpr int kV2MaxP = 8;     // visibility periods handled by the device search
constexpr int kV2None = 255;   // "no winning trajectory"

struct V2Solver {
    cudaStream_t st = nullptr;
    int num_sms = 1;
    int n = 0, k = 0, p = 0, rw = 0, rwp = 0, W = 0;
    uint32_t C = 0;
    const uint32_t* rp = nullptr;
    const uint16_t* col = nullptr;
    const uint32_t* binom = nullptr;
    const uint16_t* configs = nullptr;
    uint8_t* table = nullptr;
    uint32_t* marked = nullptr;
    uint32_t* nbr = nullptr;
    uint8_t* val1 = nullptr;
    uint8_t* newval = nullptr;
    uint8_t* changed = nullptr;
    uint8_t* dirty = nullptr;
    uint8_t* tmp = nullptr;
    unsigned long long* counters = nullptr;
    unsigned int* err = nullptr;
    unsigned long long* h_pinned = nullptr;
    // depth-2 cloud table (p >= 3): key words (key and subtree value, see cloud_key) and
    // clouds [hcap][rwp]
    unsigned long long* hkey = nullptr;
    uint32_t* hmask = nullptr;
    uint64_t hcap = 0;
    uint64_t chunk_nodes = 0;   // depth-1 nodes per table fill
    cr_v2_hash_stats hstats{};
    bool first = true;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

struct V2Dev {
    int n, k, p, rwp;
    uint32_t C;
    const uint32_t* rp;
    const uint16_t* col;
    const uint32_t* binom;
    const uint16_t* configs;
    const uint8_t* table;
    const uint32_t* marked;
    const uint32_t* nbr;
    uint8_t* val1;
    uint8_t* newval;
    const uint8_t* dirty;
    unsigned long long* count;     // [0] marks found, [1] depth-2 child visits, [2] table entries
    unsigned long long* hkey;      // null = no cloud table (p < 3)
    uint32_t* hmask;
    uint64_t hcap;                 // power of two
    uint64_t node_lo, node_hi;     // depth-1 nodes (C1 * n + r) of this chunk
};

constexpr int kHashProbes = 64;   // linear-probe limit of an insert or a lookup


template <int W>
struct Mask {
    uint32_t w[W];
};

template <int W>
__device__ __forceinline__ bool mask_empty(const Mask<W>& m) {
    uint32_t x = 0;
#pragma unroll
    for (int i = 0; i < W; ++i) x |= m.w[i];
    return x == 0;
}

template <int W>
__device__ __forceinline__ uint32_t mask_word(const Mask<W>& m, int idx) {
    uint32_t x = 0;
#pragma unroll
    for (int i = 0; i < W; ++i) x = (i == idx) ? m.w[i] : x;
    return x;
}

template <int W, int K>
__device__ __forceinline__ bool mask_hits(const Mask<W>& m, const int (&c)[K]) {
    bool hit = false;
#pragma unroll
    for (int i = 0; i < K; ++i) hit |= (mask_word<W>(m, c[i] >> 5) >> (c[i] & 31)) & 1u;
    return hit;
}

template <int W, int K>
__device__ __forceinline__ void mask_clear(Mask<W>& m, const int (&c)[K]) {
#pragma unroll
    for (int i = 0; i < K; ++i) {
        const int wi = c[i] >> 5;
        const uint32_t b = ~(1u << (c[i] & 31));
#pragma unroll
        for (int j = 0; j < W; ++j)
            if (j == wi) m.w[j] &= b;
    }
}

template <int W>
__device__ __forceinline__ void load_nbr(Mask<W>& m, const uint32_t* snbr, int rwp, int v) {
#pragma unroll
    for (int j = 0; j < W; ++j) m.w[j] = j < rwp ? snbr[v * rwp + j] : 0u;
}

// Robber cloud after one move: OR of the neighbour masks of every vertex of m.
template <int W>
__device__ __forceinline__ Mask<W> expand(const Mask<W>& m, const uint32_t* snbr, int rwp) {
    Mask<W> out;
#pragma unroll
    for (int j = 0; j < W; ++j) out.w[j] = 0u;
#pragma unroll
    for (int i = 0; i < W; ++i) {
        uint32_t b = m.w[i];
        while (b) {
            const int v = i * 32 + __ffs(b) - 1;
            b &= b - 1;
            const uint32_t* row = snbr + v * rwp;
#pragma unroll
            for (int j = 0; j < W; ++j)
                if (j < rwp) out.w[j] |= row[j];
        }
    }
    return out;
}

// Successor enumeration of one config: the product of each cop's neighbour list.
template <int K>
struct Moves {
    int lo[K], dg[K], T;
    int idx[K];   // odometer of the next successor tuple (last cop fastest)
};

template <int K>
__device__ __forceinline__ void moves_of(Moves<K>& mv, const int (&c)[K], const uint32_t* __restrict__ rp) {
    mv.T = 1;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        mv.lo[i] = __ldg(&rp[c[i]]);
        mv.dg[i] = __ldg(&rp[c[i] + 1]) - mv.lo[i];
        mv.T *= mv.dg[i];
        mv.idx[i] = 0;
    }
}

// The successor tuple at the odometer (the same tuple move_target gives for the running
// index), then the odometer steps on: the sequential walks need no division per tuple.
template <int K>
__device__ __forceinline__ uint32_t next_target(Moves<K>& mv, const uint16_t* __restrict__ adj,
                                                const uint32_t* __restrict__ B, int np1, int (&c)[K]) {
#pragma unroll
    for (int i = 0; i < K; ++i) c[i] = __ldg(&adj[mv.lo[i] + mv.idx[i]]);
    bool carry = true;
#pragma unroll
    for (int i = K - 1; i >= 0; --i) {
        if (carry) {
            ++mv.idx[i];
            carry = mv.idx[i] >= mv.dg[i];
            if (carry) mv.idx[i] = 0;
        }
    }
    sort_small<K>(c);
    return config_rank<K>(c, B, np1);
}

template <int K>
__device__ __forceinline__ uint32_t move_target(const Moves<K>& mv, int t, const uint16_t* __restrict__ adj,
                                                const uint32_t* __restrict__ B, int np1, int (&c)[K]) {
    int rem = t;
#pragma unroll
    for (int i = K - 1; i >= 0; --i) {
        const int q = rem / mv.dg[i];
        c[i] = __ldg(&adj[mv.lo[i] + rem - q * mv.dg[i]]);
        rem = q;
    }
    sort_small<K>(c);
    return config_rank<K>(c, B, np1);
}

// Phase D boundary (v2:321-334): cloud within the marked set of config cid -> 2p + max round.
template <int W>
__device__ __forceinline__ int leaf_cost(const V2Dev& d, uint32_t cid, const Mask<W>& V) {
    if (cid >= d.C) return kV2None;  // never taken for a well-formed rank table
    const uint32_t* mrow = d.marked + (size_t)cid * d.rwp;
#pragma unroll
    for (int j = 0; j < W; ++j)
        if (j < d.rwp && (V.w[j] & ~__ldg(&mrow[j]))) return kV2None;
    const uint8_t* trow = d.table + (size_t)cid * d.n;
    int mx = 0;
#pragma unroll
    for (int i = 0; i < W; ++i) {
        uint32_t b = V.w[i];
        while (b) {
            const int v = i * 32 + __ffs(b) - 1;
            b &= b - 1;
            mx = max(mx, (int)(__ldg(&trow[v]) >> 1));
        }
    }
    return 2 * d.p + mx;
}

template <int W, int K>
struct Frame {
    Mask<W> V, E;
    Moves<K> mv;
    int t;
};

// Minimum over the trajectory subtree below node (depth 2, cops c2, cloud V2), p >= 3.
template <int W, int K>
__device__ int subtree_min(const V2Dev& d, const int (&c2)[K], const Mask<W>& V2,
                           const uint32_t* snbr, int best) {
    Frame<W, K> st[kV2MaxP - 2];
    int top = 0;
    st[0].V = V2;
    st[0].E = expand<W>(V2, snbr, d.rwp);
    moves_of<K>(st[0].mv, c2, d.rp);
    st[0].t = 0;
    const int np1 = d.n + 1;
    while (top >= 0) {
        Frame<W, K>& f = st[top];
        const int dc = top + 3;  // depth of the child about to be tried
        if (f.t >= f.mv.T || 2 * dc - 1 >= best) { --top; continue; }
        ++f.t;
        int c[K];
        const uint32_t cid = next_target<K>(f.mv, d.col, d.binom, np1, c);
        Mask<W> nx;
        if (mask_hits<W, K>(f.V, c)) {
            Mask<W> mid = f.V;
            mask_clear<W, K>(mid, c);
            if (mask_empty<W>(mid)) { best = 2 * dc - 1; continue; }
            nx = expand<W>(mid, snbr, d.rwp);
        } else {
            nx = f.E;
        }
        mask_clear<W, K>(nx, c);
        if (mask_empty<W>(nx)) { best = min(best, 2 * dc); continue; }
        if (dc == d.p) { best = min(best, leaf_cost<W>(d, cid, nx)); continue; }
        Frame<W, K>& g = st[top + 1];
        g.V = nx;
        g.E = expand<W>(nx, snbr, d.rwp);
        moves_of<K>(g.mv, c, d.rp);
        g.t = 0;
        ++top;
    }
    return best;
}

// Minimum over the children of depth-2 node (c2, V2) when p = 3 (the children are leaves):
// cop ply 3 empties the cloud -> 5, robber ply 3 leaves nobody -> 6, else the leaf cost.
template <int W, int K>
__device__ int node2_min_p3(const V2Dev& d, const int (&c2)[K], const Mask<W>& V2, const uint32_t* snbr) {
    Moves<K> mv;
    moves_of<K>(mv, c2, d.rp);
    const Mask<W> E = expand<W>(V2, snbr, d.rwp);
    const int np1 = d.n + 1;
    int best = kV2None;
    for (int t = 0; t < mv.T; ++t) {
        int c[K];
        const uint32_t cid = next_target<K>(mv, d.col, d.binom, np1, c);
        Mask<W> nx;
        if (mask_hits<W, K>(V2, c)) {
            Mask<W> mid = V2;
            mask_clear<W, K>(mid, c);
            if (mask_empty<W>(mid)) return 5;   // the smallest value a depth-2 node can take
            nx = expand<W>(mid, snbr, d.rwp);
        } else {
            nx = E;
        }
        mask_clear<W, K>(nx, c);
        if (mask_empty<W>(nx)) { best = 6; continue; }
        if (best > 6) best = min(best, leaf_cost<W>(d, cid, nx));
    }
    return best;
}

// Cloud-table key of depth-2 node (cid, V): the config's rank + 1 above a 24-bit fingerprint of
// the cloud, above a zero byte where the node's subtree value goes once k_v2_heval has it (one
// word per probe holds both; never 0, which marks an empty slot).
template <int W>
__device__ __forceinline__ unsigned long long cloud_key(uint32_t cid, const Mask<W>& V) {
    uint32_t h = 0x9E3779B9u;
#pragma unroll
    for (int j = 0; j < W; ++j) {
        h = (h ^ V.w[j]) * 0x85EBCA6Bu;
        h ^= h >> 13;
    }
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return ((unsigned long long)(cid + 1u) << 32) | ((h & 0xFFFFFFu) << 8);
}

__device__ __forceinline__ uint64_t cloud_slot(unsigned long long key, uint64_t cap) {
    uint64_t z = key + 0x9E3779B97F4A7C15ull;   // splitmix64 finaliser
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (z ^ (z >> 31)) & (cap - 1);
}

// Insert (cid, V) unless its key is present; the thread that claims a slot writes the cloud.
// Returns 1 when this call claimed a new slot.
// Insert (cid, V) unless its key is present; the thread that claims a slot writes the cloud.
// Returns 1 when this call claimed a new slot.
template <int W>
__device__ __forceinline__ unsigned cloud_insert(const V2Dev& d, uint32_t cid, const Mask<W>& V) {
    const unsigned long long key = cloud_key<W>(cid, V);
    uint64_t h = cloud_slot(key, d.hcap);
    for (int probe = 0; probe < kHashProbes; ++probe) {
        const unsigned long long old = atomicCAS(&d.hkey[h], 0ull, key);
        if (old == 0ull) {
            uint32_t* m = d.hmask + h * d.rwp;
#pragma unroll
            for (int j = 0; j < W; ++j)
                if (j < d.rwp) m[j] = V.w[j];
            return 1u;
        }
        if (old == key) return 0u;
        h = (h + 1) & (d.hcap - 1);
    }
    return 0u;   // probe limit: the lookup misses and the node is evaluated directly
}

// Stored value of (cid, V), or -1 when the table does not hold exactly this node.
template <int W>
__device__ __forceinline__ int cloud_lookup(const V2Dev& d, uint32_t cid, const Mask<W>& V) {
    const unsigned long long key = cloud_key<W>(cid, V);
    uint64_t h = cloud_slot(key, d.hcap);
    for (int probe = 0; probe < kHashProbes; ++probe) {
        const unsigned long long k = __ldg(&d.hkey[h]);
        if (k == 0ull) return -1;
        if ((k & ~0xFFull) == key) {
            const uint32_t* m = d.hmask + h * d.rwp;
            bool same = true;
#pragma unroll
            for (int j = 0; j < W; ++j)
                if (j < d.rwp) same &= __ldg(&m[j]) == V.w[j];
            return same ? (int)(k & 0xFFull) : -1;
        }
        h = (h + 1) & (d.hcap - 1);
    }
    return -1;
}

// Depth-1 node (c1, r) of a chunk: its cops and cloud N(r) \ C1; false when the node is
// decided without children (r on a cop, or no robber move left).
template <int W, int K>
__device__ __forceinline__ bool depth1_node(const V2Dev& d, uint32_t c1, int r, const uint32_t* snbr,
                                            int (&cops1)[K], Mask<W>& V1) {
    bool rin = false;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        cops1[i] = d.configs[(size_t)c1 * K + i];
        rin |= cops1[i] == r;
    }
    load_nbr<W>(V1, snbr, d.rwp, r);
    mask_clear<W, K>(V1, cops1);
    return !(rin || mask_empty<W>(V1));
}

// Fill the cloud table with the distinct non-terminal depth-2 children of the chunk's dirty
// depth-1 nodes: a warp per node, lanes over the cop moves.
template <int K, int W>
__global__ void __launch_bounds__(256) k_v2_hinsert(V2Dev d) {
    extern __shared__ uint32_t snbr[];
    for (int i = threadIdx.x; i < d.n * d.rwp; i += blockDim.x) snbr[i] = d.nbr[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t nwarps = (size_t)gridDim.x * (blockDim.x >> 5);
    const int np1 = d.n + 1;
    unsigned visits = 0, fresh = 0;
    for (size_t idx = d.node_lo + (size_t)blockIdx.x * (blockDim.x >> 5) + warp; idx < d.node_hi; idx += nwarps) {
        const uint32_t c1 = (uint32_t)(idx / d.n);
        const int r = (int)(idx - (size_t)c1 * d.n);
        if (!d.dirty[c1]) continue;
        int cops1[K];
        Mask<W> V1;
        if (!depth1_node<W, K>(d, c1, r, snbr, cops1, V1)) continue;
        Moves<K> mv;
        moves_of<K>(mv, cops1, d.rp);
        for (int t = lane; t < mv.T; t += 32) {
            int c2[K];
            const uint32_t cid2 = move_target<K>(mv, t, d.col, d.binom, np1, c2);
            if (cid2 >= d.C) continue;
            Mask<W> mid = V1;
            mask_clear<W, K>(mid, c2);
            if (mask_empty<W>(mid)) continue;
            Mask<W> nx = expand<W>(mid, snbr, d.rwp);
            mask_clear<W, K>(nx, c2);
            if (mask_empty<W>(nx)) continue;
            ++visits;
            fresh += cloud_insert<W>(d, cid2, nx);
        }
    }
    visits = __reduce_add_sync(0xFFFFFFFFu, visits);
    fresh = __reduce_add_sync(0xFFFFFFFFu, fresh);
    if (lane == 0) {
        if (visits) atomicAdd(&d.count[1], (unsigned long long)visits);
        if (fresh) atomicAdd(&d.count[2], (unsigned long long)fresh);
    }
}

// Exact subtree minimum of every node in the cloud table: a thread per slot.
template <int K, int W>
__global__ void __launch_bounds__(256) k_v2_heval(V2Dev d) {
    extern __shared__ uint32_t snbr[];
    for (int i = threadIdx.x; i < d.n * d.rwp; i += blockDim.x) snbr[i] = d.nbr[i];
    __syncthreads();
    for (uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; h < d.hcap;
         h += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long key = d.hkey[h];
        if (key == 0ull) continue;
        const uint32_t cid = (uint32_t)(key >> 32) - 1u;
        int c2[K];
#pragma unroll
        for (int i = 0; i < K; ++i) c2[i] = d.configs[(size_t)cid * K + i];
        Mask<W> V;
#pragma unroll
        for (int j = 0; j < W; ++j) V.w[j] = j < d.rwp ? d.hmask[h * d.rwp + j] : 0u;
        const int v = d.p == 3 ? node2_min_p3<W, K>(d, c2, V, snbr) : subtree_min<W, K>(d, c2, V, snbr, kV2None);
        d.hkey[h] = key | (unsigned long long)min(v, kV2None);   // the value in the key word's low byte
    }
}

template <int K, int W>
__global__ void __launch_bounds__(256) k_v2_val1(V2Dev d) {
    extern __shared__ uint32_t snbr[];
    for (int i = threadIdx.x; i < d.n * d.rwp; i += blockDim.x) snbr[i] = d.nbr[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t nwarps = (size_t)gridDim.x * (blockDim.x >> 5);
    const int np1 = d.n + 1;
    for (size_t idx = d.node_lo + (size_t)blockIdx.x * (blockDim.x >> 5) + warp; idx < d.node_hi; idx += nwarps) {
        const uint32_t c1 = (uint32_t)(idx / d.n);
        const int r = (int)(idx - (size_t)c1 * d.n);
        if (!d.dirty[c1]) continue;
        int cops1[K];
        Mask<W> V1;
        if (!depth1_node<W, K>(d, c1, r, snbr, cops1, V1)) {
            if (lane == 0) d.val1[idx] = kV2None;
            continue;
        }
        int best = kV2None;
        if (d.p == 1) {
            if (lane == 0) best = leaf_cost<W>(d, c1, V1);
        } else {
            Moves<K> mv;
            moves_of<K>(mv, cops1, d.rp);
            for (int t = lane; t < mv.T; t += 32) {
                int c2[K];
                const uint32_t cid2 = move_target<K>(mv, t, d.col, d.binom, np1, c2);
                Mask<W> mid = V1;
                mask_clear<W, K>(mid, c2);
                if (mask_empty<W>(mid)) { best = 3; break; }
                Mask<W> nx = expand<W>(mid, snbr, d.rwp);
                mask_clear<W, K>(nx, c2);
                if (mask_empty<W>(nx)) { best = min(best, 4); continue; }
                if (d.p == 2) best = min(best, leaf_cost<W>(d, cid2, nx));
                else if (best > 5) {
                    // the cloud table holds the node unless an insert gave up on it
                    const int v = d.hkey ? cloud_lookup<W>(d, cid2, nx) : -1;
                    best = v >= 0 ? min(best, v) : subtree_min<W, K>(d, c2, nx, snbr, best);
                }
            }
        }
        best = __reduce_min_sync(0xFFFFFFFFu, best);
        if (lane == 0) d.val1[idx] = (uint8_t)min(best, kV2None);
    }
}

// Root values of the unmarked states; buffered in newval (the snapshot stays intact).
template <int K, int W>
__global__ void __launch_bounds__(256) k_v2_root(V2Dev d) {
    extern __shared__ uint32_t snbr[];
    for (int i = threadIdx.x; i < d.n * d.rwp; i += blockDim.x) snbr[i] = d.nbr[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    const int np1 = d.n + 1;
    unsigned cnt = 0;
    for (uint32_t c0 = blockIdx.x * (blockDim.x >> 5) + warp; c0 < d.C; c0 += nwarps) {
        const uint32_t* mrow = d.marked + (size_t)c0 * d.rwp;
        int cops0[K];
#pragma unroll
        for (int i = 0; i < K; ++i) cops0[i] = d.configs[(size_t)c0 * K + i];
        Moves<K> mv;
        moves_of<K>(mv, cops0, d.rp);
        for (int rb = 0; rb < d.n; rb += 32) {
            const int r = rb + lane;
            const bool live = r < d.n && !((__ldg(&mrow[r >> 5]) >> (r & 31)) & 1u);
            if (!__any_sync(0xFFFFFFFFu, live)) continue;
            int best = kV2None;
            Mask<W> nr;
            if (live) load_nbr<W>(nr, snbr, d.rwp, r);
#pragma unroll
            for (int i = 0; i < K; ++i) mv.idx[i] = 0;
            for (int t = 0; t < mv.T; ++t) {
                int c1[K];
                const uint32_t cid1 = next_target<K>(mv, d.col, d.binom, np1, c1);
                if (!live) continue;
                bool rin = false;
#pragma unroll
                for (int i = 0; i < K; ++i) rin |= c1[i] == r;
                if (rin) { best = 1; continue; }
                Mask<W> v1 = nr;
                mask_clear<W, K>(v1, c1);
                if (mask_empty<W>(v1)) { best = min(best, 2); continue; }
                if (cid1 < d.C) best = min(best, (int)d.val1[(size_t)cid1 * d.n + r]);
            }
            if (live) {
                const int v = best < kMaxRound ? best : kV2None;
                d.newval[(size_t)c0 * d.n + r] = (uint8_t)v;
                cnt += v != kV2None;
            }
        }
    }
    cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
    if (lane == 0 && cnt) atomicAdd(d.count, (unsigned long long)cnt);
}

// Apply the buffered marks (v2:541-557).
__global__ void k_v2_apply(uint8_t* table, uint32_t* marked, uint8_t* newval, uint8_t* changed,
                           uint32_t C, int n, int rwp) {
    const size_t total = (size_t)C * n;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const uint8_t v = newval[i];
        if (v == kV2None) continue;
        newval[i] = kV2None;
        table[i] = (uint8_t)(1 | (v << 1));
        const uint32_t c = (uint32_t)(i / n);
        const int r = (int)(i - (size_t)c * n);
        atomicOr(&marked[(size_t)c * rwp + (r >> 5)], 1u << (r & 31));
        changed[c] = 1;
    }
}

__global__ void k_v2_init(uint8_t* table, uint32_t* marked, const uint16_t* configs, uint32_t C,
                          int n, int k, int rwp, unsigned long long* caps_out) {
    unsigned caps = 0;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        int prev = -1;
        for (int i = 0; i < k; ++i) {
            const int r = configs[(size_t)c * k + i];
            if (r == prev) continue;
            prev = r;
            ++caps;
            table[(size_t)c * n + r] = 1;
            marked[(size_t)c * rwp + (r >> 5)] |= 1u << (r & 31);
        }
    }
    caps = __reduce_add_sync(0xFFFFFFFFu, caps);
    if ((threadIdx.x & 31) == 0 && caps) atomicAdd(caps_out, (unsigned long long)caps);
}

// out[C] = OR over C' in T(C) of in[C']  (one cop step of the dirty-region dilation).
template <int K>
__global__ void k_v2_dilate(const uint8_t* __restrict__ in, uint8_t* out, const uint16_t* configs,
                            uint32_t C, int n, const uint32_t* rp, const uint16_t* adj,
                            const uint32_t* B) {
    const int np1 = n + 1;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        int cops[K];
#pragma unroll
        for (int i = 0; i < K; ++i) cops[i] = configs[(size_t)c * K + i];
        Moves<K> mv;
        moves_of<K>(mv, cops, rp);
        uint8_t any = 0;
        for (int t = 0; t < mv.T && !any; ++t) {
            int cc[K];
            const uint32_t s = next_target<K>(mv, adj, B, np1, cc);
            any = s < C ? in[s] : 0;
        }
        out[c] = any ? 1 : 0;
    }
}

// ------------------------------------------------------------------------------ host ---

// Slots of the depth-2 cloud table: twice the depth-1 nodes (about 1.2 distinct children per
// node on the graphs measured), a power of two between 2^10 and 2^24; 0 below p = 3.
static uint64_t v2_hash_capacity(uint64_t nodes, int p) {
    if (p < 3) return 0;
    uint64_t cap = 1024;
    while (cap < 2 * nodes && cap < (1ull << 24)) cap <<= 1;
    return cap;
}

uint64_t v2_footprint(int n, int k, int p) {
    long double C = 1;
    for (int i = 1; i <= k; ++i) C = C * (n + k - i) / i;
    const uint64_t c = (uint64_t)C;
    const int rwp = round_words((n + 31) / 32);
    const uint64_t hcap = v2_hash_capacity(c * (uint64_t)n, p);
    return c * n * 3 + c * (uint64_t)rwp * 4 + c * 3 + (uint64_t)n * rwp * 4 + c * (uint64_t)k * 2 +
           hcap * (8 + 4 * (uint64_t)rwp) + (1u << 16);
}

static int v2_w(int rwp) { return rwp <= 1 ? 1 : rwp <= 2 ? 2 : rwp <= 4 ? 4 : rwp <= 8 ? 8 : 16; }

static V2Dev v2_view(const V2Solver* s) {
    V2Dev d;
    d.n = s->n; d.k = s->k; d.p = s->p; d.rwp = s->rwp; d.C = s->C;
    d.rp = s->rp; d.col = s->col; d.binom = s->binom; d.configs = s->configs;
    d.table = s->table; d.marked = s->marked; d.nbr = s->nbr;
    d.val1 = s->val1; d.newval = s->newval; d.dirty = s->dirty; d.count = s->counters;
    d.hkey = s->hkey; d.hmask = s->hmask; d.hcap = s->hcap;
    d.node_lo = 0;
    d.node_hi = (uint64_t)s->C * s->n;
    return d;
}

#define V2_CUDA(call)                                                                     \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            if (err) *err = std::string(#call) + ": " + cudaGetErrorString(e_);          \
            return e_ == cudaErrorMemoryAllocation ? CR_ERR_NOMEM : CR_ERR_CUDA;          \
        }                                                                                 \
    } while (0)

int v2_set_hash_capacity(V2Solver* s, uint64_t slots, std::string* err) {
    if (s->p < 3) slots = 0;
    uint64_t cap = 0;
    if (slots) {
        if (slots > (1ull << 40)) {
            if (err) *err = "v2 cloud table: at most 2^40 slots";
            return CR_ERR_LIMIT;
        }
        cap = 1024;
        while (cap < slots) cap <<= 1;
    }
    V2_CUDA(cudaStreamSynchronize(s->st));
    void* old[] = {s->hkey, s->hmask};
    for (void* q : old)
        if (q) cudaFree(q);
    s->hkey = nullptr;
    s->hmask = nullptr;
    s->hcap = 0;
    s->chunk_nodes = 0;
    s->hstats.capacity = 0;
    if (!cap) return CR_OK;
    // a solver whose table could not be allocated keeps working without one (every depth-2
    // node evaluated where it is reached)
    cudaError_t e = cudaMalloc(&s->hkey, cap * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&s->hmask, cap * s->rwp * sizeof(uint32_t));
    if (e != cudaSuccess) {
        void* got[] = {s->hkey, s->hmask};
        for (void* q : got)
            if (q) cudaFree(q);
        s->hkey = nullptr;
        s->hmask = nullptr;
        if (err) *err = std::string("v2 cloud table: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? CR_ERR_NOMEM : CR_ERR_CUDA;
    }
    s->hcap = cap;
    s->chunk_nodes = cap / 2;
    s->hstats.capacity = cap;
    return CR_OK;
}

int v2_create(V2Solver** out, cudaStream_t st, int num_sms, int n, int k, int p,
              const uint32_t* d_rp, const uint16_t* d_col, const uint32_t* h_rp,
              const uint16_t* h_col, const uint32_t* d_binom, const uint16_t* d_configs,
              uint32_t C, std::string* err) {
    if (n > 512) {
        if (err) *err = "v2 rules: clouds are limited to 512 vertices";
        return CR_ERR_LIMIT;
    }
    if (p > kV2MaxP) {
        if (err) *err = "v2 rules: visibility period limited to 8";
        return CR_ERR_LIMIT;
    }
    V2Solver* s = new V2Solver();
    *out = s;
    s->st = st; s->num_sms = num_sms; s->n = n; s->k = k; s->p = p; s->C = C;
    s->rw = (n + 31) / 32;
    s->rwp = round_words(s->rw);
    s->W = v2_w(s->rwp);
    s->rp = d_rp; s->col = d_col; s->binom = d_binom; s->configs = d_configs;
    V2_CUDA(cudaMalloc(&s->table, (size_t)C * n));
    V2_CUDA(cudaMalloc(&s->marked, (size_t)C * s->rwp * 4));
    V2_CUDA(cudaMalloc(&s->nbr, (size_t)n * s->rwp * 4));
    V2_CUDA(cudaMalloc(&s->val1, (size_t)C * n));
    V2_CUDA(cudaMalloc(&s->newval, (size_t)C * n));
    V2_CUDA(cudaMalloc(&s->changed, C));
    V2_CUDA(cudaMalloc(&s->dirty, C));
    V2_CUDA(cudaMalloc(&s->tmp, C));
    V2_CUDA(cudaMalloc(&s->counters, 4 * sizeof(unsigned long long)));
    if (int rc = v2_set_hash_capacity(s, v2_hash_capacity((uint64_t)C * n, p), err)) return rc;
    V2_CUDA(cudaMallocHost(&s->h_pinned, 4 * sizeof(unsigned long long)));
    V2_CUDA(cudaEventCreate(&s->e0));
    V2_CUDA(cudaEventCreate(&s->e1));
    std::vector<uint32_t> nbr((size_t)n * s->rwp, 0);
    for (int v = 0; v < n; ++v)
        for (uint32_t e = h_rp[v]; e < h_rp[v + 1]; ++e) nbr[(size_t)v * s->rwp + (h_col[e] >> 5)] |= 1u << (h_col[e] & 31);
    V2_CUDA(cudaMemcpyAsync(s->nbr, nbr.data(), nbr.size() * 4, cudaMemcpyHostToDevice, st));
    V2_CUDA(cudaStreamSynchronize(st));
    return CR_OK;
}

void v2_destroy(V2Solver* s) {
    if (!s) return;
    void* ptrs[] = {s->table, s->marked, s->nbr, s->val1, s->newval, s->changed, s->dirty, s->tmp, s->counters,
                    s->hkey, s->hmask};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (s->h_pinned) cudaFreeHost(s->h_pinned);
    if (s->e0) cudaEventDestroy(s->e0);
    if (s->e1) cudaEventDestroy(s->e1);
    delete s;
}

int v2_init(V2Solver* s, uint64_t* caps, cr_solve_stats* stats, std::string* err) {
    cudaStream_t st = s->st;
    V2_CUDA(cudaEventRecord(s->e0, st));
    V2_CUDA(cudaMemsetAsync(s->table, kUnmarked, (size_t)s->C * s->n, st));
    V2_CUDA(cudaMemsetAsync(s->marked, 0, (size_t)s->C * s->rwp * 4, st));
    V2_CUDA(cudaMemsetAsync(s->newval, kV2None, (size_t)s->C * s->n, st));
    V2_CUDA(cudaMemsetAsync(s->val1, kV2None, (size_t)s->C * s->n, st));
    V2_CUDA(cudaMemsetAsync(s->changed, 1, s->C, st));
    V2_CUDA(cudaMemsetAsync(s->counters, 0, 4 * sizeof(unsigned long long), st));
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((s->C + 255) / 256, (uint64_t)s->num_sms * 4));
    k_v2_init<<<grid, 256, 0, st>>>(s->table, s->marked, s->configs, s->C, s->n, s->k, s->rwp, s->counters);
    V2_CUDA(cudaGetLastError());
    V2_CUDA(cudaEventRecord(s->e1, st));
    V2_CUDA(cudaMemcpyAsync(s->h_pinned, s->counters, 8, cudaMemcpyDeviceToHost, st));
    V2_CUDA(cudaStreamSynchronize(st));
    *caps = s->h_pinned[0];
    float ms = 0;
    cudaEventElapsedTime(&ms, s->e0, s->e1);
    stats->init_ms = ms;
    stats->kernel_launches = 1;
    s->first = true;
    s->hstats = cr_v2_hash_stats{};
    s->hstats.capacity = s->hcap;
    return CR_OK;
}

// Depth-1 values of the nodes [lo, hi): with a cloud table, fill it and evaluate its nodes
// first.  Returns the kernels launched.
template <int K, int W>
static int launch_v2_val1(V2Solver* s, V2Dev d, uint64_t lo, uint64_t hi, int grid_pairs, size_t sm) {
    cudaStream_t st = s->st;
    raise_smem_limit((const void*)k_v2_val1<K, W>, sm);
    d.node_lo = lo;
    d.node_hi = hi;
    int launches = 0;
    if (d.hkey) {
        raise_smem_limit((const void*)k_v2_hinsert<K, W>, sm);
        raise_smem_limit((const void*)k_v2_heval<K, W>, sm);
        cudaMemsetAsync(d.hkey, 0, d.hcap * sizeof(unsigned long long), st);
        k_v2_hinsert<K, W><<<grid_pairs, 256, sm, st>>>(d);
        const int grid_h = (int)std::max<uint64_t>(1, std::min<uint64_t>((d.hcap + 255) / 256, (uint64_t)s->num_sms * 8));
        k_v2_heval<K, W><<<grid_h, 256, sm, st>>>(d);
        launches += 2;
        ++s->hstats.fills;
    }
    k_v2_val1<K, W><<<grid_pairs, 256, sm, st>>>(d);
    return launches + 1;
}

template <int K, int W>
static int launch_v2_kernels(V2Solver* s, const V2Dev& d, int grid_pairs, int grid_cfg, size_t sm) {
    int launches = 0;
    const uint64_t nodes = (uint64_t)s->C * s->n;
    const uint64_t chunk = d.hkey ? std::max<uint64_t>(1, s->chunk_nodes) : nodes;
    for (uint64_t lo = 0; lo < nodes; lo += chunk)
        launches += launch_v2_val1<K, W>(s, d, lo, std::min(nodes, lo + chunk), grid_pairs, sm);
    raise_smem_limit((const void*)k_v2_root<K, W>, sm);
    k_v2_root<K, W><<<grid_cfg, 256, sm, s->st>>>(d);
    return launches + 1;
}

template <int K>
static int launch_v2_k(V2Solver* s, const V2Dev& d, int W, int grid_pairs, int grid_cfg, size_t sm) {
    switch (W) {
        case 1: return launch_v2_kernels<K, 1>(s, d, grid_pairs, grid_cfg, sm);
        case 2: return launch_v2_kernels<K, 2>(s, d, grid_pairs, grid_cfg, sm);
        case 4: return launch_v2_kernels<K, 4>(s, d, grid_pairs, grid_cfg, sm);
        case 8: return launch_v2_kernels<K, 8>(s, d, grid_pairs, grid_cfg, sm);
        default: return launch_v2_kernels<K, 16>(s, d, grid_pairs, grid_cfg, sm);
    }
}

template <int K>
static void launch_dilate(const V2Solver* s, const uint8_t* in, uint8_t* out, int grid) {
    k_v2_dilate<K><<<grid, 256, 0, s->st>>>(in, out, s->configs, s->C, s->n, s->rp, s->col, s->binom);
}

int v2_pass(V2Solver* s, uint64_t* found, cr_solve_stats* stats, std::string* err) {
    cudaStream_t st = s->st;
    V2_CUDA(cudaEventRecord(s->e0, st));
    V2_CUDA(cudaMemsetAsync(s->counters, 0, 3 * sizeof(unsigned long long), st));
    const int grid_cfg_small = (int)std::max<uint64_t>(1, std::min<uint64_t>((s->C + 255) / 256, (uint64_t)s->num_sms * 4));
    int launches = 0;
    if (s->first || s->p == 1) {
        // first pass: every depth-1 node is evaluated; p = 1: dirty = changed
        V2_CUDA(cudaMemcpyAsync(s->dirty, s->changed, s->C, cudaMemcpyDeviceToDevice, st));
        if (s->first) V2_CUDA(cudaMemsetAsync(s->dirty, 1, s->C, st));
    } else {
        const uint8_t* in = s->changed;
        uint8_t* bufs[2] = {s->dirty, s->tmp};
        // p-1 steps; make the last one land in dirty
        int steps = s->p - 1;
        int cur = (steps % 2 == 1) ? 0 : 1;
        for (int i = 0; i < steps; ++i) {
            uint8_t* out = bufs[cur];
            switch (s->k) {
                case 1: launch_dilate<1>(s, in, out, grid_cfg_small); break;
                case 2: launch_dilate<2>(s, in, out, grid_cfg_small); break;
                case 3: launch_dilate<3>(s, in, out, grid_cfg_small); break;
                default: launch_dilate<4>(s, in, out, grid_cfg_small); break;
            }
            ++launches;
            in = out;
            cur ^= 1;
        }
    }
    s->first = false;
    V2_CUDA(cudaMemsetAsync(s->changed, 0, s->C, st));
    V2Dev d = v2_view(s);
    const size_t sm = (size_t)s->n * s->rwp * 4;
    const uint64_t pairs = (uint64_t)s->C * s->n;
    const int grid_pairs = (int)std::max<uint64_t>(1, std::min<uint64_t>((pairs + 7) / 8, (uint64_t)s->num_sms * 8));
    const int grid_cfg = (int)std::max<uint64_t>(1, std::min<uint64_t>((s->C + 7) / 8, (uint64_t)s->num_sms * 8));
    switch (s->k) {
        case 1: launches += launch_v2_k<1>(s, d, s->W, grid_pairs, grid_cfg, sm); break;
        case 2: launches += launch_v2_k<2>(s, d, s->W, grid_pairs, grid_cfg, sm); break;
        case 3: launches += launch_v2_k<3>(s, d, s->W, grid_pairs, grid_cfg, sm); break;
        default: launches += launch_v2_k<4>(s, d, s->W, grid_pairs, grid_cfg, sm); break;
    }
    const int grid_apply = (int)std::max<uint64_t>(1, std::min<uint64_t>((pairs + 255) / 256, (uint64_t)s->num_sms * 8));
    k_v2_apply<<<grid_apply, 256, 0, st>>>(s->table, s->marked, s->newval, s->changed, s->C, s->n, s->rwp);
    launches += 1;
    V2_CUDA(cudaGetLastError());
    V2_CUDA(cudaEventRecord(s->e1, st));
    V2_CUDA(cudaMemcpyAsync(s->h_pinned, s->counters, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    V2_CUDA(cudaStreamSynchronize(st));
    *found = s->h_pinned[0];
    s->hstats.child_visits += s->h_pinned[1];
    s->hstats.entries += s->h_pinned[2];
    float ms = 0;
    cudaEventElapsedTime(&ms, s->e0, s->e1);
    stats->main_ms += ms;
    stats->kernel_launches += launches;
    return CR_OK;
}

int v2_load_states(V2Solver* s, const uint8_t* states, std::string* err) {
    cudaStream_t st = s->st;
    V2_CUDA(cudaMemcpyAsync(s->table, states, (size_t)s->C * s->n, cudaMemcpyHostToDevice, st));
    launch_marks_from_table(s->table, s->C, s->n, 1, s->rwp, s->marked, s->num_sms * 8, st);
    V2_CUDA(cudaGetLastError());
    V2_CUDA(cudaStreamSynchronize(st));   // the caller's host buffer goes out of scope
    return CR_OK;
}

void v2_verdict(V2Solver* s, unsigned long long* best_key) {
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((s->C + 7) / 8, (uint64_t)s->num_sms * 8));
    launch_verdict_raw(s->table, s->marked, s->C, s->n, s->rw, s->rwp, 1, best_key, grid, s->st);
}

const uint8_t* v2_table(const V2Solver* s) { return s->table; }

cr_v2_hash_stats v2_hash_stats(const V2Solver* s) { return s->hstats; }

}  // namespace crgpu
