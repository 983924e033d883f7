// crgpu_v1.cu - level-synchronous frontier kernels for the v1 rules
// (solvers/k_cops_visibility.cpp: 2p DP columns per visibility cycle).
//
// The reference sweeps all C*N*2p states every pass, column 0 to 2p-1, in place
// (k_cops_visibility.cpp:142-296).  Within one column every state reads only the next
// column, so the order inside a column is irrelevant and one pass is exactly: each column c
// in turn recomputed from column c+1 as it stood before this pass (c+1 is recomputed later
// in the pass), except the last column, which reads column 0 as just recomputed.  These
// kernels run that same schedule, but a column's producer only looks at the states whose
// inputs changed: the marks column c+1's last producer run made (its frontier).
//
//   cop turn (even c)          (C, r, c) = 1 + min over C' in T(C) of marked (C', r, c+1)
//                              k_cops_visibility.cpp:160-197
//   deferred robber (odd c)    (C, r, c) = 1 + (C, r, c+1)           k_cops_visibility.cpp:209-228
//   last column (2p-1)         (C, r, 2p-1) = 1 + max over v p hops from r of (C, v, 0), all
//                              marked                              k_cops_visibility.cpp:235-288
// with values >= 127 left unmarked (lines 189, 220, 280).
//
// Why frontiers suffice: a state left unmarked after its producer ran had no marked input
// then, or every marked input already gave a value >= 127.  Values in a column never
// decrease from one pass to the next, so any input that can now mark it is a new one, and
// the minimum over new inputs equals the minimum over all inputs whenever it is < 127.
// The frontier of a column is split into value slots (one bit plane per value) so that the
// cop-turn minimum is a sequence of bitwise ORs: the lowest slot with a bit gives the value.
//
// The cop turn runs in one of two forms chosen on the device from the frontier's row count:
//   pull (dense)  every configuration ORs the frontier rows of its successors (k_cop_pull);
//   push (sparse) every non-empty frontier row is ORed into the candidate rows of its
//                 predecessors with atomics (k_cop_push), then only those are marked
//                 (k_cop_apply).
// The capture seeds (the frontier of column 1 before pass 1) have a closed form: the OR of
// the seed rows over T(C) is the union of the cops' neighbourhoods.
#include "crgpu_internal.cuh"

namespace crgpu {

#define FULL_MASK 0xFFFFFFFFu
#define CR_MAX_K_DEV 4

__device__ __forceinline__ bool frontier_sparse(const ColMeta& m, uint32_t C) {
    return (unsigned long long)m.rows * kPushRatio < C;
}

// Per-warp running totals a producer reports once at the end of its grid-stride loop.
struct Tally {
    unsigned cnt = 0, err = 0, rows = 0;
    int lo = kEmptyLo, hi = -1;

    __device__ void flush(const V1Dev& d, int col, int lane) {
        cnt = __reduce_add_sync(FULL_MASK, cnt);
        rows = __reduce_add_sync(FULL_MASK, rows);
        lo = __reduce_min_sync(FULL_MASK, lo);
        hi = __reduce_max_sync(FULL_MASK, hi);
        err = __reduce_or_sync(FULL_MASK, err);
        if (lane == 0) {
            if (cnt) atomicAdd(d.pass_new, (unsigned long long)cnt);
            if (rows) atomicAdd(&d.meta[col].rows, (int)rows);
            if (hi >= 0) {
                atomicMin(&d.meta[col].lo, lo);
                atomicMax(&d.meta[col].hi, hi);
            }
            if (err) atomicOr(d.err, err);
        }
    }
};

// Before a producer run of column `col` (whose inputs are column nx): fix the value base of
// its output frontier, reset the range, and clear the frontier flags -- unless the column is
// in append mode (column 0 in pass 1, whose frontier already holds the capture seeds).
__global__ void k_prep(V1Dev d, int col, int nx) {
    ColMeta* mo = d.meta + col;
    const int append = mo->append;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (!append) {
            const ColMeta mi = d.meta[nx];
            mo->base = (mi.hi >= mi.lo) ? mi.lo + 1 : 0;
            mo->lo = kEmptyLo;
            mo->hi = -1;
            mo->rows = 0;
        }
        mo->seed = 0;
        if (col == 0) *d.pass_new = 0ull;
        if (col == d.cols - 1) d.meta[0].append = 0;  // column 0's seeded frontier is consumed
    }
    if (!append) {
        uint8_t* f = d.fflag + (size_t)col * d.C;
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < d.C;
             i += (size_t)gridDim.x * blockDim.x)
            f[i] = 0;
    }
}

// initializeCaptures (k_cops_visibility.cpp:85-127): the table was memset to 0xFE; a robber
// on a cop is a capture of round 0 in columns 0 and 1 only.  The seeds also form the first
// frontiers of columns 0 and 1 (value 0, slot 0); their rows are written whole.
__global__ void k_init(V1Dev d, int K) {
    unsigned caps = 0;
    const int n = d.g.n, rwp = d.g.rwp, S = d.S;
    for (uint32_t cid = blockIdx.x * blockDim.x + threadIdx.x; cid < d.C;
         cid += gridDim.x * blockDim.x) {
        const uint16_t* cc = d.configs + (size_t)cid * K;
        int wi[CR_MAX_K_DEV];
        uint32_t bi[CR_MAX_K_DEV];
        int nb = 0, prev = -1;
        for (int i = 0; i < K; ++i) {
            const int r = cc[i];
            if (r == prev) continue;
            prev = r;
            wi[nb] = r >> 5;
            bi[nb] = 1u << (r & 31);
            ++nb;
            const size_t cell = ((size_t)cid * n + r) * d.cols;
            d.table[cell] = 1;
            d.table[cell + 1] = 1;
        }
        caps += nb;
        // the seed rows of columns 0 and 1: marked rows and slot 0 of the frontier rows,
        // written whole (the other slots zero) with 16-byte stores where rows allow it
        uint32_t* rows[4] = {d.marked + (size_t)cid * rwp, d.marked + ((size_t)d.C + cid) * rwp,
                             d.front + (size_t)cid * S * rwp, d.front + ((size_t)d.C + cid) * S * rwp};
        const int len[4] = {rwp, rwp, S * rwp, S * rwp};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            for (int w0 = 0; w0 < len[q]; w0 += 4) {
                uint32_t x[4];
                for (int j = 0; j < 4; ++j) {
                    x[j] = 0u;
                    for (int b = 0; b < nb; ++b)
                        if (wi[b] == w0 + j) x[j] |= bi[b];
                }
                if ((rwp & 3) == 0) {
                    *reinterpret_cast<uint4*>(rows[q] + w0) = make_uint4(x[0], x[1], x[2], x[3]);
                } else {
                    for (int j = 0; j < 4 && w0 + j < len[q]; ++j) rows[q][w0 + j] = x[j];
                }
            }
        }
        d.fflag[cid] = 1;
        d.fflag[(size_t)d.C + cid] = 1;
    }
    caps = __reduce_add_sync(FULL_MASK, caps);
    if ((threadIdx.x & 31) == 0 && caps) atomicAdd(d.pass_new, (unsigned long long)caps);
}

// ---- lane groups ---------------------------------------------------------------------
// A warp works on CPW = 32 / G configurations at once, G lanes per configuration (G >= rwp,
// so every word of a robber row has its own lane).  All lanes of a warp run the same control
// flow over the same number of rounds (groups without work are predicated off), so warp-wide
// shuffles and ballots stay legal, and the loads of CPW rows are in flight together.
template <int G>
struct Lanes {
    int lane, glane, grp;
    unsigned gmask;
    __device__ explicit Lanes(int l)
        : lane(l), glane(l & (G - 1)), grp(l / G),
          gmask(G == 32 ? FULL_MASK : (((1u << G) - 1u) << ((l / G) * G))) {}
    __device__ bool any(bool p) const { return (__ballot_sync(FULL_MASK, p) & gmask) != 0u; }
    __device__ bool all(bool p) const { return (__ballot_sync(FULL_MASK, p) & gmask) == gmask; }
    __device__ int sum(int v) const {
#pragma unroll
        for (int off = G / 2; off >= 1; off >>= 1) v += __shfl_xor_sync(FULL_MASK, v, off);
        return v;
    }
};

// Mark the states of row cid in column col from wacc = OR of the successors' frontier
// rows (slot s <-> value base_in + s): the lowest slot with a bit gives 1 + min.  Writes the
// table bytes, the marked row, the output frontier row and flag.  All lanes of the warp call
// it; `valid` is the group's predicate.
template <int G>
__device__ __forceinline__ void emit_row(const V1Dev& d, uint32_t cid, bool valid, int col, uint32_t m,
                                         const uint32_t* wacc, uint32_t* wnew, int base_in,
                                         int s_used, int out_base, int append, const Lanes<G>& L,
                                         Tally& t) {
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const int gl = L.glane;
    const uint32_t vm = (valid && gl < rw) ? valid_mask(n, gl) : 0u;
    uint32_t mm = m, any = 0;
    if (valid && gl < rw) {
        for (int s = 0; s < s_used; ++s) {
            const int v = base_in + s + 1;
            const uint32_t nb = (v < kMaxRound) ? (wacc[s * rwp + gl] & ~mm & vm) : 0u;
            mm |= nb;
            wnew[s * rwp + gl] = nb;
            any |= nb;
            if (nb) {
                t.lo = min(t.lo, v);
                t.hi = max(t.hi, v);
                const int so = v - out_base;
                if (so < 0 || so >= S) t.err |= kErrSlot;
            }
        }
    }
    __syncwarp();
    if (L.any(any != 0)) {
        if (gl < rw) {
            d.marked[((size_t)col * d.C + cid) * rwp + gl] = mm;
            t.cnt += __popc(mm ^ m);
        }
        uint32_t* frow = d.front + ((size_t)col * d.C + cid) * S * rwp;
        for (int e = gl; e < S * rwp; e += G) {
            const int so = e / rwp, w = e - so * rwp;
            const int s = out_base + so - base_in - 1;
            const uint32_t val = (s >= 0 && s < s_used && w < rw) ? wnew[s * rwp + w] : 0u;
            frow[e] = append ? (frow[e] | val) : val;
        }
        if (gl == 0) {
            d.fflag[(size_t)col * d.C + cid] = 1;
            t.rows++;
        }
        // table bytes: each lane walks the new bits of its own word (slots are disjoint)
        if (gl < rw) {
            uint8_t* trow = d.table + ((size_t)cid * n + gl * 32) * d.cols + col;
            for (int s = 0; s < s_used; ++s) {
                uint32_t b = wnew[s * rwp + gl];
                const uint8_t val = (uint8_t)(1 | ((base_in + s + 1) << 1));
                while (b) {
                    trow[(size_t)(__ffs(b) - 1) * d.cols] = val;
                    b &= b - 1;
                }
            }
        }
    }
    __syncwarp();
}

// OR-reduce NWP per-lane words across the G lanes of a group by recursive halving: at each
// step a lane keeps one half of its words and receives the partner's copy of that half.
// The group's reduced row lands in out[0 .. nwords).
template <int NWP, int G>
__device__ __forceinline__ void group_or(uint32_t (&acc)[NWP], int gl, uint32_t* out, int nwords) {
    constexpr int STEPS = (NWP < G ? NWP : G) == 1 ? 0 : __builtin_ctz(NWP < G ? NWP : G);
    constexpr int R = NWP >= G ? NWP / G : 1;
    int w = 0;
    int lb = G >> 1;
#pragma unroll
    for (int st = 0; st < STEPS; ++st) {
        const int half = NWP >> (st + 1);
        const bool up = (gl & lb) != 0;
#pragma unroll
        for (int i = 0; i < NWP / 2; ++i) {
            if (i < half) {
                const uint32_t send = up ? acc[i] : acc[i + half];
                const uint32_t keep = up ? acc[i + half] : acc[i];
                acc[i] = keep | __shfl_xor_sync(FULL_MASK, send, lb);
            }
        }
        if (up) w += half;
        lb >>= 1;
    }
    // lanes left sharing the same words (NWP < G)
    for (; lb >= 1; lb >>= 1) acc[0] |= __shfl_xor_sync(FULL_MASK, acc[0], lb);
    const bool writer = NWP >= G || (gl & ((G / NWP) - 1)) == 0;
    if (writer) {
#pragma unroll
        for (int i = 0; i < R; ++i)
            if (w + i < nwords) out[w + i] = acc[i];
    }
}

// Dense cop turn: a lane group per configuration.  Each lane takes its own successor tuples
// (one rank per tuple), ORs whole frontier rows of the flagged successors into NWP per-lane
// words, and the group reduces them by halving.
template <int K, int NWP, int G>
__global__ void __launch_bounds__(256) k_cop_pull(V1Dev d, int col, int nx) {
    extern __shared__ uint32_t sm[];
    constexpr int CPW = 32 / G;
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (mi.hi < mi.lo) return;                              // empty frontier: nothing changes
    if (!mi.seed && frontier_sparse(mi, d.C)) return;      // the push form handles it
    const int base_in = mi.base;
    const int s_used = min(mi.hi - base_in + 1, S);
    const int nwords = s_used * rwp;
    const int out_base = d.meta[col].base;
    const int append = d.meta[col].append;
    uint32_t* wacc = sm + (warp * CPW + L.grp) * (2 * S * rwp);
    uint32_t* wnew = wacc + S * rwp;
    const uint32_t* __restrict__ fin = d.front + (size_t)nx * d.C * S * rwp;
    const uint8_t* __restrict__ fflag_in = d.fflag + (size_t)nx * d.C;
    const uint32_t* __restrict__ rp = d.g.row_ptr;
    const uint16_t* __restrict__ adj = d.g.col;
    const int np1 = n + 1;
    const bool vec4 = (rwp & 3) == 0;
    Tally t;
    const size_t step = (size_t)gridDim.x * (blockDim.x >> 5) * CPW;
    for (size_t cb = ((size_t)blockIdx.x * (blockDim.x >> 5) + warp) * CPW; cb < d.C; cb += step) {
        const uint32_t cid = (uint32_t)(cb + L.grp);
        const bool ok = cid < d.C;
        const uint32_t vm = (ok && gl < rw) ? valid_mask(n, gl) : 0u;
        const uint32_t m = (ok && gl < rw) ? d.marked[((size_t)col * d.C + cid) * rwp + gl] : 0u;
        const bool full = L.all(m == vm);                 // every lane votes (no short circuit)
        const bool need = ok && !full;                    // some robber position still open
        if (!__any_sync(FULL_MASK, need)) continue;
        int lo[K], dg[K];
        int T = 0;
        if (need) {
            const uint16_t* cc = d.configs + (size_t)cid * K;
            T = 1;
#pragma unroll
            for (int i = 0; i < K; ++i) {
                const int v = cc[i];
                lo[i] = __ldg(&rp[v]);
                dg[i] = __ldg(&rp[v + 1]) - lo[i];
                T *= dg[i];
            }
        }
        if (mi.seed) {
            // OR over T(C) of the seed rows {r : r in C'} = union of the cops' neighbourhoods
            if (need && gl < rwp) {
                uint32_t x = 0;
                if (T > 0) {
                    const uint16_t* cc = d.configs + (size_t)cid * K;
#pragma unroll
                    for (int i = 0; i < K; ++i) x |= __ldg(&d.g.nbr[(size_t)cc[i] * rwp + gl]);
                }
                wacc[gl] = x;
            }
        } else {
            uint32_t acc[NWP];
#pragma unroll
            for (int i = 0; i < NWP; ++i) acc[i] = 0u;
            const int Tmax = __reduce_max_sync(FULL_MASK, T);
            for (int t0 = 0; t0 < Tmax; t0 += G) {
                const int tt = t0 + gl;
                if (tt >= T) continue;
                int c[K];
                int rem = tt;
#pragma unroll
                for (int i = K - 1; i >= 0; --i) {
                    const int q = rem / dg[i];
                    c[i] = __ldg(&adj[lo[i] + rem - q * dg[i]]);
                    rem = q;
                }
                sort_small<K>(c);
                const uint32_t s = config_rank<K>(c, d.binom, np1);
                if (s >= d.C) { t.err |= kErrRank; continue; }
                if (!__ldg(&fflag_in[s])) continue;
                const uint32_t* row = fin + (size_t)s * S * rwp;
                if (vec4) {
#pragma unroll
                    for (int w = 0; w < NWP; w += 4) {
                        if (w < nwords) {
                            const uint4 x = __ldg(reinterpret_cast<const uint4*>(row + w));
                            acc[w] |= x.x; acc[w + 1] |= x.y; acc[w + 2] |= x.z; acc[w + 3] |= x.w;
                        }
                    }
                } else {
#pragma unroll
                    for (int w = 0; w < NWP; ++w)
                        if (w < nwords) acc[w] |= __ldg(row + w);
                }
            }
            group_or<NWP, G>(acc, gl, wacc, need ? nwords : 0);
        }
        __syncwarp();
        emit_row<G>(d, cid, need, col, m, wacc, wnew, base_in, s_used, out_base, append, L, t);
    }
    t.flush(d, col, L.lane);
}

// Sparse cop turn, scatter: every non-empty frontier row of column nx is ORed into the
// candidate rows of its predecessors (the product of the cops' in-neighbour lists).
template <int K>
__global__ void __launch_bounds__(256) k_cop_push(V1Dev d, int col, int nx) {
    extern __shared__ uint32_t sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = d.g.n, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (mi.hi < mi.lo || mi.seed || !frontier_sparse(mi, d.C)) return;
    const int s_used = min(mi.hi - mi.base + 1, S);
    const int nwords = s_used * rwp;
    uint32_t* wrow = sm + warp * (S * rwp);
    const uint32_t* __restrict__ fin = d.front + (size_t)nx * d.C * S * rwp;
    const uint8_t* __restrict__ fflag_in = d.fflag + (size_t)nx * d.C;
    const uint32_t* __restrict__ rrp = d.g.rrow_ptr;
    const uint16_t* __restrict__ radj = d.g.rcol;
    const int np1 = n + 1;
    unsigned err = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = (size_t)blockIdx.x * blockDim.x + warp * 32; base < d.C; base += stride) {
        const size_t mine = base + lane;
        unsigned act = __ballot_sync(FULL_MASK, mine < d.C && fflag_in[mine]);
        while (act) {
            const uint32_t cp = (uint32_t)(base + __ffs(act) - 1);
            act &= act - 1;
            const uint32_t* row = fin + (size_t)cp * S * rwp;
            uint32_t nz = 0;
            for (int e = lane; e < nwords; e += 32) {
                wrow[e] = row[e];
                if (wrow[e]) nz = 1;
            }
            const bool any = __any_sync(FULL_MASK, nz != 0);
            __syncwarp();
            if (any) {
                const uint16_t* cc = d.configs + (size_t)cp * K;
                int lo[K], dg[K];
                int T = 1;
#pragma unroll
                for (int i = 0; i < K; ++i) {
                    const int v = cc[i];
                    lo[i] = __ldg(&rrp[v]);
                    dg[i] = __ldg(&rrp[v + 1]) - lo[i];
                    T *= dg[i];
                }
                for (int tt = lane; tt < T; tt += 32) {
                    int c[K];
                    int rem = tt;
#pragma unroll
                    for (int i = K - 1; i >= 0; --i) {
                        const int q = rem / dg[i];
                        c[i] = __ldg(&radj[lo[i] + rem - q * dg[i]]);
                        rem = q;
                    }
                    sort_small<K>(c);
                    const uint32_t pc = config_rank<K>(c, d.binom, np1);
                    if (pc >= d.C) { err |= kErrRank; continue; }
                    uint32_t* crow = d.cand + (size_t)pc * S * rwp;
                    for (int e = 0; e < nwords; ++e)
                        if (wrow[e]) atomicOr(&crow[e], wrow[e]);
                    d.cflag[pc] = 1;
                }
            }
            __syncwarp();
        }
    }
    err = __reduce_or_sync(FULL_MASK, err);
    if (lane == 0 && err) atomicOr(d.err, err);
}

// The flagged configurations of a 32-configuration window, CPW at a time: group g takes the
// g-th remaining flag.  Returns the group's config (valid = false when fewer remain).
template <int G>
__device__ __forceinline__ uint32_t take_flagged(unsigned& act, size_t base, const Lanes<G>& L,
                                                 bool& valid) {
    constexpr int CPW = 32 / G;
    const unsigned pos = __fns(act, 0, L.grp + 1);
    valid = pos < 32u;
#pragma unroll
    for (int i = 0; i < CPW; ++i) act &= act - 1;  // (a no-op once act is empty)
    return valid ? (uint32_t)(base + pos) : 0u;
}

// Sparse cop turn, mark: the configurations that received candidates; their candidate rows
// are consumed and cleared for the next push.
template <int G>
__global__ void __launch_bounds__(256) k_cop_apply(V1Dev d, int col, int nx) {
    extern __shared__ uint32_t sm[];
    constexpr int CPW = 32 / G;
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (mi.hi < mi.lo || mi.seed || !frontier_sparse(mi, d.C)) return;
    const int base_in = mi.base;
    const int s_used = min(mi.hi - base_in + 1, S);
    const int out_base = d.meta[col].base;
    const int append = d.meta[col].append;
    uint32_t* wacc = sm + (warp * CPW + L.grp) * (2 * S * rwp);
    uint32_t* wnew = wacc + S * rwp;
    Tally t;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = (size_t)blockIdx.x * blockDim.x + warp * 32; base < d.C; base += stride) {
        const size_t mine = base + L.lane;
        unsigned act = __ballot_sync(FULL_MASK, mine < d.C && d.cflag[mine]);
        while (act) {
            bool valid;
            const uint32_t cid = take_flagged<G>(act, base, L, valid);
            uint32_t m = 0;
            if (valid) {
                uint32_t* crow = d.cand + (size_t)cid * S * rwp;
                for (int e = gl; e < S * rwp; e += G) {
                    wacc[e] = crow[e];
                    crow[e] = 0u;
                }
                if (gl == 0) d.cflag[cid] = 0;
                if (gl < rw) m = d.marked[((size_t)col * d.C + cid) * rwp + gl];
            }
            __syncwarp();
            emit_row<G>(d, cid, valid, col, m, wacc, wnew, base_in, s_used, out_base, append, L, t);
        }
    }
    t.flush(d, col, L.lane);
}

// Deferred robber turn (odd column below the last): (C, r, c) = 1 + (C, r, c+1), row-local.
template <int G>
__global__ void __launch_bounds__(256) k_direct(V1Dev d, int col, int nx) {
    extern __shared__ uint32_t sm[];
    constexpr int CPW = 32 / G;
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (mi.hi < mi.lo) return;
    const int base_in = mi.base;
    const int s_used = min(mi.hi - base_in + 1, S);
    const int out_base = d.meta[col].base;
    const int append = d.meta[col].append;
    uint32_t* wacc = sm + (warp * CPW + L.grp) * (2 * S * rwp);
    uint32_t* wnew = wacc + S * rwp;
    const uint8_t* __restrict__ fflag_in = d.fflag + (size_t)nx * d.C;
    Tally t;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = (size_t)blockIdx.x * blockDim.x + warp * 32; base < d.C; base += stride) {
        const size_t mine = base + L.lane;
        unsigned act = __ballot_sync(FULL_MASK, mine < d.C && fflag_in[mine]);
        while (act) {
            bool valid;
            const uint32_t cid = take_flagged<G>(act, base, L, valid);
            uint32_t m = 0;
            if (valid) {
                const uint32_t* row = d.front + ((size_t)nx * d.C + cid) * S * rwp;
                for (int e = gl; e < S * rwp; e += G) wacc[e] = e < s_used * rwp ? row[e] : 0u;
                if (gl < rw) m = d.marked[((size_t)col * d.C + cid) * rwp + gl];
            }
            __syncwarp();
            emit_row<G>(d, cid, valid, col, m, wacc, wnew, base_in, s_used, out_base, append, L, t);
        }
    }
    t.flush(d, col, L.lane);
}

// Last column (robber move cashed out over the exact-p-hop cloud) from column 0.
// A lane group per configuration whose column-0 row changed; the work is row-local.  Two
// forms per row, whichever touches fewer vertices:
//   count (p = 1, few column-0 marks): every marked v adds one to the counter of each r with
//          v in N(r) (its in-neighbours); r is complete when its counter reaches deg(r);
//   test  (otherwise): every open r tests hop(r) within column 0's marked row.
// Only the states found complete read column 0's table bytes (for the max).
template <bool P1, int G>
__global__ void __launch_bounds__(256) k_and(V1Dev d, int col) {
    extern __shared__ uint32_t sm[];
    constexpr int CPW = 32 / G;
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S, cols = d.cols;
    const ColMeta mi = d.meta[0];
    if (mi.hi < mi.lo) return;
    const int out_base = d.meta[col].base;
    const int per_grp = 3 * rwp + S * rwp + (n + 3) / 4;
    uint32_t* wm0 = sm + (warp * CPW + L.grp) * per_grp;
    uint32_t* wmc = wm0 + rwp;
    uint32_t* wtouch = wmc + rwp;
    uint32_t* wnew = wtouch + rwp;
    uint32_t* wcnt = wnew + S * rwp;   // n byte counters packed 4 per word
    const uint8_t* __restrict__ fflag0 = d.fflag;
    const uint32_t* __restrict__ rp = d.g.row_ptr;
    const uint16_t* __restrict__ adj = d.g.col;
    const uint32_t* __restrict__ rrp = d.g.rrow_ptr;
    const uint16_t* __restrict__ radj = d.g.rcol;
    const int avg_deg = max(1, (int)((__ldg(&rp[n]) + n - 1) / n));
    Tally t;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = (size_t)blockIdx.x * blockDim.x + warp * 32; base < d.C; base += stride) {
        const size_t mine = base + L.lane;
        unsigned act = __ballot_sync(FULL_MASK, mine < d.C && fflag0[mine]);
        while (act) {
            bool valid;
            const uint32_t cid = take_flagged<G>(act, base, L, valid);
            uint32_t* mrow = d.marked + ((size_t)col * d.C + cid) * rwp;
            const uint32_t vm = (valid && gl < rw) ? valid_mask(n, gl) : 0u;
            const uint32_t mc = (valid && gl < rw) ? mrow[gl] : 0u;
            const bool full = L.all(mc == vm);            // every lane votes (no short circuit)
            const bool need = valid && !full;
            if (!__any_sync(FULL_MASK, need)) continue;
            const uint32_t m0 = (need && gl < rw) ? d.marked[(size_t)cid * rwp + gl] : 0u;
            if (need && gl < rwp) {
                wm0[gl] = m0;
                wmc[gl] = mc;
                wtouch[gl] = 0u;
            }
            if (need)
                for (int e = gl; e < S * rwp; e += G) wnew[e] = 0u;
            const int marked0 = L.sum(__popc(m0));
            const int open = L.sum(__popc(~mc & vm));
            const bool count_form = P1 && d.g.maxdeg <= 255 && marked0 * avg_deg < open;
            if (count_form && need)
                for (int e = gl; e < (n + 3) / 4; e += G) wcnt[e] = 0u;
            __syncwarp();
            if (count_form && need && gl < rw) {
                // every marked v of column 0 counts toward the r that move to it
                uint32_t b = m0;
                while (b) {
                    const int v = gl * 32 + __ffs(b) - 1;
                    b &= b - 1;
                    for (uint32_t e = __ldg(&rrp[v]); e < __ldg(&rrp[v + 1]); ++e) {
                        const int r = __ldg(&radj[e]);
                        atomicAdd(&wcnt[r >> 2], 1u << ((r & 3) * 8));
                        atomicOr(&wtouch[r >> 5], 1u << (r & 31));
                    }
                }
            }
            __syncwarp();
            if (need && gl < rw) {
                const uint8_t* trow = d.table + (size_t)cid * n * cols;
                // candidates: touched and open (count form) or every open state (test form)
                uint32_t cand = ~mc & vm;
                if (count_form) cand &= wtouch[gl] | __ldg(&d.g.isolated[gl]);
                while (cand) {
                    const int r = gl * 32 + __ffs(cand) - 1;
                    cand &= cand - 1;
                    const uint32_t e0 = __ldg(&rp[r]), e1 = __ldg(&rp[r + 1]);
                    bool all;
                    int mx = 0;
                    if (P1) {
                        if (count_form) {
                            all = ((wcnt[r >> 2] >> ((r & 3) * 8)) & 0xFFu) == e1 - e0;
                        } else {
                            all = true;
                            for (uint32_t e = e0; e < e1 && all; ++e) {
                                const int v = __ldg(&adj[e]);
                                all = (wm0[v >> 5] >> (v & 31)) & 1u;
                            }
                        }
                        if (all)
                            for (uint32_t e = e0; e < e1; ++e)
                                mx = max(mx, (int)(trow[(size_t)__ldg(&adj[e]) * cols] >> 1));
                    } else {
                        const uint32_t* h = d.hop + (size_t)r * rwp;
                        all = true;
                        for (int w = 0; w < rw && all; ++w) all = (__ldg(&h[w]) & ~wm0[w]) == 0u;
                        if (all) {
                            for (int w = 0; w < rw; ++w) {
                                uint32_t b = __ldg(&h[w]);
                                while (b) {
                                    const int v = w * 32 + __ffs(b) - 1;
                                    b &= b - 1;
                                    mx = max(mx, (int)(trow[(size_t)v * cols] >> 1));
                                }
                            }
                        }
                    }
                    if (!all) continue;
                    const int v = mx + 1;
                    if (v >= kMaxRound) continue;
                    const int so = v - out_base;
                    if (so < 0 || so >= S) { t.err |= kErrSlot; continue; }
                    wnew[so * rwp + gl] |= 1u << (r & 31);  // this lane owns word r >> 5
                    d.table[((size_t)cid * n + r) * cols + col] = (uint8_t)(1 | (v << 1));
                    t.lo = min(t.lo, v);
                    t.hi = max(t.hi, v);
                }
            }
            __syncwarp();
            uint32_t nb = 0;
            if (need && gl < rw)
                for (int s = 0; s < S; ++s) nb |= wnew[s * rwp + gl];
            if (L.any(nb != 0)) {
                if (gl < rw) {
                    mrow[gl] = mc | nb;
                    t.cnt += __popc(nb);
                }
                uint32_t* frow = d.front + ((size_t)col * d.C + cid) * S * rwp;
                for (int e = gl; e < S * rwp; e += G) frow[e] = wnew[e];
                if (gl == 0) {
                    d.fflag[(size_t)col * d.C + cid] = 1;
                    t.rows++;
                }
            }
            __syncwarp();
        }
    }
    t.flush(d, col, L.lane);
}

// findFinalResult (k_cops_visibility.cpp:301-331): key = worst << 32 | cid, minimised, is the
// first config (lowest id) among those with the strictly smallest worst case.  Each lane
// tests one config's column-0 row; the warp then scans the bytes of the complete rows.
__global__ void k_verdict(const uint8_t* __restrict__ table, const uint32_t* __restrict__ m0,
                          uint32_t C, int n, int rw, int rwp, int cols,
                          unsigned long long* best) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = (size_t)blockIdx.x * blockDim.x + warp * 32; base < C; base += stride) {
        const size_t cid = base + lane;
        bool full = cid < C;
        for (int w = 0; w < rw && full; ++w) full = m0[cid * rwp + w] == valid_mask(n, w);
        unsigned act = __ballot_sync(FULL_MASK, full);
        while (act) {
            const size_t c = base + __ffs(act) - 1;
            act &= act - 1;
            int wc = 0;
            for (int r = lane; r < n; r += 32) wc = max(wc, (int)(table[(c * n + r) * cols] >> 1));
            wc = __reduce_max_sync(FULL_MASK, wc);
            if (lane == 0) atomicMin(best, ((unsigned long long)wc << 32) | c);
        }
    }
}

// ---------------------------------------------------------------- host-side launchers ---

// Lanes per configuration: a power of two covering the robber row (at least 4).
static int group_lanes(int rwp) {
    int g = 4;
    while (g < rwp) g <<= 1;
    return g;
}

size_t cop_smem_bytes(int S, int rwp) {
    return (size_t)8 * (32 / group_lanes(rwp)) * 2 * S * rwp * sizeof(uint32_t);
}
size_t and_smem_bytes(int S, int rwp, int n) {
    return (size_t)8 * (32 / group_lanes(rwp)) * (3 * rwp + S * rwp + (n + 3) / 4) * sizeof(uint32_t);
}

static int pull_words(int S, int rwp) {
    int w = S * rwp, p = 2;
    while (p < w) p <<= 1;
    return p;
}

bool pull_supported(int S, int rwp) { return pull_words(S, rwp) <= 32 && group_lanes(rwp) <= 32; }

template <int K, int G>
static void launch_pull_g(const V1Dev& d, int col, int nx, int grid, cudaStream_t st) {
    const size_t sm = cop_smem_bytes(d.S, d.g.rwp);
    switch (pull_words(d.S, d.g.rwp)) {
        case 2: if (G == 4) k_cop_pull<K, 2, 4><<<grid, 256, sm, st>>>(d, col, nx); break;
        case 4: if (G == 4) k_cop_pull<K, 4, 4><<<grid, 256, sm, st>>>(d, col, nx); break;
        case 8: if (G == 4) k_cop_pull<K, 8, 4><<<grid, 256, sm, st>>>(d, col, nx); break;
        case 16:
            if (G == 4) k_cop_pull<K, 16, 4><<<grid, 256, sm, st>>>(d, col, nx);
            else k_cop_pull<K, 16, 8><<<grid, 256, sm, st>>>(d, col, nx);
            break;
        default:
            if (G == 4) k_cop_pull<K, 32, 4><<<grid, 256, sm, st>>>(d, col, nx);
            else if (G == 8) k_cop_pull<K, 32, 8><<<grid, 256, sm, st>>>(d, col, nx);
            else k_cop_pull<K, 32, 16><<<grid, 256, sm, st>>>(d, col, nx);
            break;
    }
}

template <int G>
static void launch_rows_g(const V1Dev& d, int col, int nx, int direct, int grid, cudaStream_t st) {
    const size_t sm = cop_smem_bytes(d.S, d.g.rwp);
    if (direct) k_direct<G><<<grid, 256, sm, st>>>(d, col, nx);
    else k_cop_apply<G><<<grid, 256, sm, st>>>(d, col, nx);
}

static void launch_rows(const V1Dev& d, int col, int nx, int direct, int grid, cudaStream_t st) {
    switch (group_lanes(d.g.rwp)) {
        case 4: launch_rows_g<4>(d, col, nx, direct, grid, st); break;
        case 8: launch_rows_g<8>(d, col, nx, direct, grid, st); break;
        case 16: launch_rows_g<16>(d, col, nx, direct, grid, st); break;
        default: launch_rows_g<32>(d, col, nx, direct, grid, st); break;
    }
}

template <int K>
static void launch_cop_k(const V1Dev& d, int col, int nx, int grid, cudaStream_t st) {
    switch (group_lanes(d.g.rwp)) {
        case 4: launch_pull_g<K, 4>(d, col, nx, grid, st); break;
        case 8: launch_pull_g<K, 8>(d, col, nx, grid, st); break;
        default: launch_pull_g<K, 16>(d, col, nx, grid, st); break;
    }
    k_cop_push<K><<<grid, 256, (size_t)8 * d.S * d.g.rwp * 4, st>>>(d, col, nx);
    launch_rows(d, col, nx, 0, grid, st);
}

// Cop turn into column col: the pull kernel and the push pair are all enqueued; each reads
// the input frontier's row count on the device and only the matching form does work.
void launch_cop(const V1Dev& d, int col, int nx, int direct, int grid, cudaStream_t st) {
    if (direct) {
        launch_rows(d, col, nx, 1, grid, st);
        return;
    }
    switch (d.k) {
        case 1: launch_cop_k<1>(d, col, nx, grid, st); break;
        case 2: launch_cop_k<2>(d, col, nx, grid, st); break;
        case 3: launch_cop_k<3>(d, col, nx, grid, st); break;
        default: launch_cop_k<4>(d, col, nx, grid, st); break;
    }
}

int cop_launches(int direct) { return direct ? 1 : 3; }

template <bool P1>
static void launch_and_p(const V1Dev& d, int col, int grid, cudaStream_t st) {
    const size_t sm = and_smem_bytes(d.S, d.g.rwp, d.g.n);
    switch (group_lanes(d.g.rwp)) {
        case 4: k_and<P1, 4><<<grid, 256, sm, st>>>(d, col); break;
        case 8: k_and<P1, 8><<<grid, 256, sm, st>>>(d, col); break;
        case 16: k_and<P1, 16><<<grid, 256, sm, st>>>(d, col); break;
        default: k_and<P1, 32><<<grid, 256, sm, st>>>(d, col); break;
    }
}

void launch_and(const V1Dev& d, int col, bool p1, int grid, cudaStream_t st) {
    if (p1) launch_and_p<true>(d, col, grid, st);
    else launch_and_p<false>(d, col, grid, st);
}

void launch_prep(const V1Dev& d, int col, int nx, int grid, cudaStream_t st) {
    k_prep<<<grid, 256, 0, st>>>(d, col, nx);
}

void launch_init(const V1Dev& d, int grid, cudaStream_t st) { k_init<<<grid, 256, 0, st>>>(d, d.k); }

void launch_verdict(const V1Dev& d, int cols, unsigned long long* best, int grid, cudaStream_t st) {
    k_verdict<<<grid, 256, 0, st>>>(d.table, d.marked, d.C, d.g.n, d.g.rw, d.g.rwp, cols, best);
}

void launch_verdict_raw(const uint8_t* table, const uint32_t* m0, uint32_t C, int n, int rw,
                        int rwp, int cols, unsigned long long* best, int grid, cudaStream_t st) {
    k_verdict<<<grid, 256, 0, st>>>(table, m0, C, n, rw, rwp, cols, best);
}

int max_cop_blocks_per_sm(int k, int rwp, int S) {
    // grid-stride kernels: 4 blocks of 256 per SM keep every SM busy whatever the
    // register count of the instance (blocks beyond residency simply queue)
    (void)k; (void)rwp; (void)S;
    return 4;
}

}  // namespace crgpu
